// Transport-speed maximum for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at the point where they need dt: code
// running while a CUDA stream is being captured into a graph, hosts whose
// device memory is owned by a pool or arena they must not bypass, and
// real-time loops that forbid allocation after start-up.  For them this file
// provides oc_transport_speed_noalloc, which computes the same value as
// oc_transport_speed with no allocation at all: its scratch is a fixed
// file-scope device array that exists from library load until process exit
// on every GPU that loads the library.
//
// Limits and sharing:
//  * the scratch holds one partial maximum per 128-cell block, so a mesh may
//    have at most OC_NOALLOC_MAX_CELLS = 4096 * 128 = 524,288 cells; larger
//    meshes are rejected with OC_ERR_UNSUPPORTED;
//  * every call, from any handle, uses the same array; two calls whose kernels
//    overlap on the GPU (different streams, or different host threads) race on
//    it.  Calls on one stream are ordered and safe;
//  * every slot a call reads was written earlier in the same call, so nothing
//    has to start at zero and stale contents of the previous call are never
//    read.
// Set-up: the first call on a device (made with that device current) resolves
// the scratch address with cudaGetSymbolAddress and uploads this file's shape
// tables; make that first call before starting any stream capture.
#include <cuda_runtime.h>

#include <cstring>

#include "oc_kernels.cuh"
#include "oc_tables.hpp"
#include "oceano_gpu.h"

namespace oc {

constexpr int kNoallocBlock = 128;
constexpr int kNoallocMaxBlocks = 4096;

// block partial maxima (bit patterns of non-negative doubles, or NaN)
static __device__ __align__(256) double g_speed_partials[kNoallocMaxBlocks];

struct NoallocDevice {
  bool ready = false;
  double *partials = nullptr;  // device address of g_speed_partials
};
static NoallocDevice g_noalloc_dev[64];

// per-cell maximum of sigma_max(J^-1) sqrt(g h) + |J^-1 u|_inf over the
// Gauss-Lobatto p+2 points (OceanDG.h:2505-2580); a non-finite value poisons
// the block result with NaN
__global__ void noalloc_speed_partials(const AuxArgs a, const double *z, const double *q,
                                       double *partials) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double local = 0;
  if (c < a.n_cells) {
    const int p = a.deg[c], N = p + 1, G = p + 2;
    const DegTables<double> &tb = tab<double>(p);
    const double *J = a.geo + 11 * (int64_t)c;
    const int64_t zo = a.off[c];
    const int n = N * N;
    const double *zb1 = a.sd1 ? a.sd1 + a.sdo1[c] : nullptr;
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
        local = isfinite(sp) ? mx<double>(local, sp) : sp;
        if (!isfinite(local)) break;
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

// Fill AuxArgs from the handle (defined with the handle in oc_api.cu).
bool noalloc_aux_args(const oc_op *op, AuxArgs *a, cudaStream_t *stream);

}  // namespace oc

using namespace oc;

extern "C" oc_status oc_transport_speed_noalloc(oc_op *op, const double *height,
                                               const double *discharge, double *speed) {
  if (!op || !height || !discharge || !speed) return OC_ERR_INVALID_ARG;
  AuxArgs a;
  cudaStream_t stream = nullptr;
  if (!noalloc_aux_args(op, &a, &stream)) return OC_ERR_INVALID_ARG;
  const int nblocks = (a.n_cells + kNoallocBlock - 1) / kNoallocBlock;
  if (nblocks > kNoallocMaxBlocks) return OC_ERR_UNSUPPORTED;  // > 524,288 cells
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return OC_ERR_CUDA;
  NoallocDevice &d = g_noalloc_dev[dev];
  if (!d.ready) {  // once per device: scratch address and this unit's shape tables
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_speed_partials) != cudaSuccess || !ptr) return OC_ERR_CUDA;
    static DegTables<double> td[OC_MAXDEG];
    static DegTables<float> tf[OC_MAXDEG];
    for (int p = 1; p <= OC_MAXDEG; ++p) {
      fill_tables(p, 15, td[p - 1]);
      cast_tables(td[p - 1], tf[p - 1]);
    }
    if (cudaMemcpyToSymbol(c_tabd, td, sizeof(td)) != cudaSuccess) return OC_ERR_CUDA;
    if (cudaMemcpyToSymbol(c_tabf, tf, sizeof(tf)) != cudaSuccess) return OC_ERR_CUDA;
    d.partials = static_cast<double *>(ptr);
    d.ready = true;
  }
  noalloc_speed_partials<<<nblocks, kNoallocBlock, 0, stream>>>(a, height, discharge, d.partials);
  if (cudaGetLastError() != cudaSuccess) return OC_ERR_CUDA;
  noalloc_speed_final<<<1, 256, 0, stream>>>(d.partials, nblocks, speed);
  if (cudaGetLastError() != cudaSuccess) return OC_ERR_CUDA;
  return OC_OK;
}
