// Transport-speed maximum for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc at the point where
// they need dt: hosts whose device memory is owned by a pool or arena they
// must not bypass, real-time loops that forbid allocation after start-up, and
// embedding frameworks that account for every device byte themselves.  For
// them this file provides oc_transport_speed_noalloc, which computes the same
// value as oc_transport_speed with no allocation at all: its scratch is a
// fixed file-scope device array that exists from library load until process
// exit on every GPU that loads the library.
//
// Limits and sharing:
//  * the scratch holds one partial maximum per 128-cell block, so a mesh may
//    have at most OC_NOALLOC_MAX_CELLS = 4096 * 128 = 524,288 cells; larger
//    meshes are rejected with OC_ERR_UNSUPPORTED before anything is launched;
//  * every call, from any handle, uses the same array; two calls whose kernels
//    overlap on the GPU (different streams, or different host threads) race on
//    it.  Calls on one stream are ordered and safe;
//  * every slot a call reads was written earlier in the same call, so nothing
//    has to start at zero and stale contents of the previous call are never
//    read.
// Set-up: the first call on a device (made with that device current) resolves
// the scratch address with cudaGetSymbolAddress and uploads this file's shape
// tables, once per device and process, under a lock (host threads may make
// first calls concurrently); make that first call before starting any stream
// capture.  A device reset (cudaDeviceReset) after the first call is not
// supported: it discards the uploaded tables, which are not uploaded again.
// Errors: failures set the handle's message (oc_last_error); a CUDA error left
// pending by earlier work of the calling thread is reported and not cleared.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <mutex>
#include <string>

#include "oc_kernels.cuh"
#include "oc_tables.hpp"
#include "oceano_gpu.h"

namespace oc {

constexpr int kNoallocBlock = 128;
constexpr int kNoallocMaxBlocks = 4096;

// block partial maxima (bit patterns of non-negative doubles, or NaN)
static __device__ __align__(256) double g_speed_partials[kNoallocMaxBlocks];

constexpr int kNoallocMaxDevices = 64;
struct NoallocDevice {
  std::atomic<bool> ready{false};
  double *partials = nullptr;  // device address of g_speed_partials (written before ready)
};
static NoallocDevice g_noalloc_dev[kNoallocMaxDevices];
static std::mutex g_noalloc_setup;  // serialises the per-device set-up

static __device__ __forceinline__ double quiet_nan() { return __longlong_as_double(0x7ff8000000000000ll); }

// per-cell maximum of sigma_max(J^-1) sqrt(g h) + |J^-1 u|_inf over the
// Gauss-Lobatto p+2 points (OceanDG.h:2505-2580); a non-finite point speed
// (NaN or infinity, where oc_transport_speed reports OC_ERR_NONFINITE) poisons
// the block result with NaN
__global__ void noalloc_speed_partials(const AuxArgs a, const double *z, const double *q,
                                       double *partials) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double local = 0;
  if (c < a.n_cells) {
    const int p = checked_degree(a.err, a.deg[c]), N = p + 1, G = p + 2;
    const DegTables<double> &tb = tab<double>(p);
    const double *J = a.geo + 11 * (int64_t)c;
    const int n = N * N;
    const int64_t zo = checked(a.err, a.off[c], a.n_dofs - n + 1, BS_OFFSET);
    const double *zb1 = a.sd1 ? a.sd1 + cell_data(a.err, a.sdo1, c, a.n_sd[1], G * G) : nullptr;
    for (int gy = 0; gy < G; ++gy)
      for (int gx = 0; gx < G; ++gx) {
        double zv = 0, q0 = 0, q1 = 0;
        for (int iy = 0; iy < N; ++iy)
          for (int ix = 0; ix < N; ++ix) {
            const double b = tb.BG[gy][iy] * tb.BG[gx][ix];
            zv += b * z[zo + iy * N + ix];
            q0 += b * q[2 * zo + iy * N + ix];
            q1 += b * q[2 * zo + n + iy * N + ix];
          }
        const double zb = zb1 ? zb1[gy * G + gx] : 0.;
        double v0, v1;
        velocity<double>(zv, q0, q1, zb, a.cu4, v0, v1);
        const double cs0 = J[6] * v0 + J[7] * v1, cs1 = J[8] * v0 + J[9] * v1;
        double conv = 0;
        conv = mx<double>(conv, fabs(cs0));
        conv = mx<double>(conv, fabs(cs1));
        const double sos = sqrt(a.g * depth<double>(zv, zb));
        double e0 = 1., e1 = 1.;
        for (int it = 0; it < 5; ++it) {
          const double a0 = J[6] * e0 + J[7] * e1, a1 = J[8] * e0 + J[9] * e1;
          e0 = J[6] * a0 + J[8] * a1;
          e1 = J[7] * a0 + J[9] * a1;
          double nrm = 0;
          nrm = mx<double>(nrm, fabs(e0));
          nrm = mx<double>(nrm, fabs(e1));
          e0 /= nrm;
          e1 /= nrm;
        }
        const double j0 = J[6] * e0 + J[7] * e1, j1 = J[8] * e0 + J[9] * e1;
        const double mev = sqrt((j0 * j0 + j1 * j1) / (e0 * e0 + e1 * e1));
        const double sp = mev * sos + conv;
        local = isfinite(sp) ? mx<double>(local, sp) : quiet_nan();
        if (isnan(local)) break;
      }
  }
  __shared__ double red[kNoallocBlock / 32];
  for (int o = 16; o > 0; o >>= 1) {
    const double other = __shfl_xor_sync(0xffffffffu, local, o);
    local = isnan(other) ? other : (isnan(local) ? local : fmax(local, other));
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = red[0];
    for (int w = 1; w < kNoallocBlock / 32; ++w)
      m = isnan(red[w]) ? red[w] : (isnan(m) ? m : fmax(m, red[w]));
    partials[blockIdx.x] = m;
  }
}

__global__ void noalloc_speed_final(const double *partials, int nblocks, double *out) {
  double m = 0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double v = partials[b];
    m = isnan(v) ? v : (isnan(m) ? m : fmax(m, v));
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double other = __shfl_xor_sync(0xffffffffu, m, o);
    m = isnan(other) ? other : (isnan(m) ? m : fmax(m, other));
  }
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      r = isnan(red[w]) ? red[w] : (isnan(r) ? r : fmax(r, red[w]));
    *out = r;
  }
}

// Fill AuxArgs from the handle, and set its error message (defined with the
// handle in oc_api.cu).
bool noalloc_aux_args(const oc_op *op, AuxArgs *a, cudaStream_t *stream);
void noalloc_set_error(oc_op *op, const std::string &msg);

// Once per device (that device current): scratch address and this unit's shape
// tables.  Returns the scratch address, or nullptr with `why` set.
static double *noalloc_setup(int dev, std::string &why) {
  NoallocDevice &d = g_noalloc_dev[dev];
  if (d.ready.load(std::memory_order_acquire)) return d.partials;
  std::lock_guard<std::mutex> lock(g_noalloc_setup);
  if (d.ready.load(std::memory_order_relaxed)) return d.partials;
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_speed_partials);
  if (e != cudaSuccess || !ptr) {
    why = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
    return nullptr;
  }
  static DegTables<double> td[OC_MAXDEG];  // filled once, under the lock
  static DegTables<float> tf[OC_MAXDEG];
  static bool filled = false;
  if (!filled) {
    for (int p = 1; p <= OC_MAXDEG; ++p) {
      fill_tables(p, 15, td[p - 1]);
      cast_tables(td[p - 1], tf[p - 1]);
    }
    filled = true;
  }
  e = cudaMemcpyToSymbol(c_tabd, td, sizeof(td));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_tabf, tf, sizeof(tf));
  if (e != cudaSuccess) {
    why = std::string("shape tables: ") + cudaGetErrorString(e);
    return nullptr;
  }
  d.partials = static_cast<double *>(ptr);
  d.ready.store(true, std::memory_order_release);
  return d.partials;
}

}  // namespace oc

using namespace oc;

extern "C" oc_status oc_transport_speed_noalloc(oc_op *op, const double *height,
                                               const double *discharge, double *speed) {
  if (!op) return OC_ERR_INVALID_ARG;
  if (!height || !discharge || !speed) {
    noalloc_set_error(op, "oc_transport_speed_noalloc: null vector");
    return OC_ERR_INVALID_ARG;
  }
  AuxArgs a;
  cudaStream_t stream = nullptr;
  if (!noalloc_aux_args(op, &a, &stream)) {
    noalloc_set_error(op, "oc_transport_speed_noalloc: handle without a mesh");
    return OC_ERR_INVALID_ARG;
  }
  const int nblocks = (a.n_cells + kNoallocBlock - 1) / kNoallocBlock;
  if (nblocks > kNoallocMaxBlocks) {
    noalloc_set_error(op, "oc_transport_speed_noalloc: " + std::to_string(a.n_cells) +
                              " cells exceed the fixed scratch (at most " +
                              std::to_string(kNoallocMaxBlocks * kNoallocBlock) + " cells)");
    return OC_ERR_UNSUPPORTED;
  }
  // a pending error of earlier work would be indistinguishable from a launch
  // failure of this call: report it and leave it for the caller
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    noalloc_set_error(op, std::string("oc_transport_speed_noalloc: pending CUDA error: ") +
                              cudaGetErrorString(e));
    return OC_ERR_CUDA;
  }
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kNoallocMaxDevices) {
    noalloc_set_error(op, "oc_transport_speed_noalloc: no usable current device");
    return OC_ERR_CUDA;
  }
  std::string why;
  double *partials = noalloc_setup(dev, why);
  if (!partials) {
    noalloc_set_error(op, "oc_transport_speed_noalloc: set-up failed: " + why);
    return OC_ERR_CUDA;
  }
  noalloc_speed_partials<<<nblocks, kNoallocBlock, 0, stream>>>(a, height, discharge, partials);
  noalloc_speed_final<<<1, 256, 0, stream>>>(partials, nblocks, speed);
  e = cudaPeekAtLastError();  // launch errors of this call (left for the caller too)
  if (e != cudaSuccess) {
    noalloc_set_error(op, std::string("oc_transport_speed_noalloc: launch: ") +
                              cudaGetErrorString(e));
    return OC_ERR_CUDA;
  }
  return OC_OK;
}
