// Cell-local kernels around the stage: transport speed (dt), velocity
// projection, vorticity indicator and L2 projection of the vortex.  One
// thread per cell, FP64, runtime degree; tables from this unit's constant copy.
#include "oc_kernels.cuh"

namespace oc {

// values of the nodal tile u (N x N) at the n x n points of the 1D matrix B[n][N]
__device__ inline void eval_tile(int N, int n, const double (*B)[OC_MAXN], const double *u,
                                 double *out /* n*n */) {
  double t[OC_MAXN * (OC_MAXQ + 2)];
  for (int iy = 0; iy < N; ++iy)
    for (int qx = 0; qx < n; ++qx) {
      double s = 0;
      for (int ix = 0; ix < N; ++ix) s += B[qx][ix] * u[iy * N + ix];
      t[iy * n + qx] = s;
    }
  for (int qy = 0; qy < n; ++qy)
    for (int qx = 0; qx < n; ++qx) {
      double s = 0;
      for (int iy = 0; iy < N; ++iy) s += B[qy][iy] * t[iy * n + qx];
      out[qy * n + qx] = s;
    }
}

// out = (Sinv (x) Sinv) in  (transform_from_q_points_to_basis on Gauss p+1)
__device__ inline void from_points(int N, const double (*Si)[OC_MAXN], const double *in,
                                   double *out) {
  double t[OC_MAXN * OC_MAXN];
  for (int qy = 0; qy < N; ++qy)
    for (int ix = 0; ix < N; ++ix) {
      double s = 0;
      for (int qx = 0; qx < N; ++qx) s += Si[ix][qx] * in[qy * N + qx];
      t[qy * N + ix] = s;
    }
  for (int iy = 0; iy < N; ++iy)
    for (int ix = 0; ix < N; ++ix) {
      double s = 0;
      for (int qy = 0; qy < N; ++qy) s += Si[iy][qy] * t[qy * N + ix];
      out[iy * N + ix] = s;
    }
}

// OceanDG.h:2505-2580: max over cells and Gauss-Lobatto p+2 points of
// sigma_max(J^-1) sqrt(g h) + |J^-1 u|_inf; positive doubles are ordered like
// their bit patterns, so the grid maximum is an atomicMax on 64-bit words.
__global__ void transport_speed_kernel(const AuxArgs a, const double *z, const double *q,
                                       unsigned long long *out, double *per_cell) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double local = 0;
  bool nonfinite = false;
  if (c < a.n_cells) {
    const int p = checked_degree(a.err, a.deg[c]), N = p + 1, G = p + 2, n = N * N;
    const DegTables<double> &tb = tab<double>(p);
    const double *J = a.geo + 11 * (int64_t)c;
    const int64_t zo = checked(a.err, a.off[c], a.n_dofs - n + 1, BS_OFFSET);
    double u[OC_MAXN * OC_MAXN], zv[OC_MAXF * OC_MAXF], q0[OC_MAXF * OC_MAXF],
        q1[OC_MAXF * OC_MAXF];
    for (int i = 0; i < n; ++i) u[i] = z[zo + i];
    eval_tile(N, G, tb.BG, u, zv);
    for (int i = 0; i < n; ++i) u[i] = q[2 * zo + i];
    eval_tile(N, G, tb.BG, u, q0);
    for (int i = 0; i < n; ++i) u[i] = q[2 * zo + n + i];
    eval_tile(N, G, tb.BG, u, q1);
    const double *zb1 = a.sd1 ? a.sd1 + cell_data(a.err, a.sdo1, c, a.n_sd[1], G * G) : nullptr;
    for (int k = 0; k < G * G; ++k) {
      const double zb = zb1 ? zb1[k] : 0.;
      double v0, v1;
      velocity<double>(zv[k], q0[k], q1[k], zb, a.cu4, v0, v1);
      const double cs0 = J[6] * v0 + J[7] * v1, cs1 = J[8] * v0 + J[9] * v1;
      double conv = 0;
      conv = mx<double>(conv, fabs(cs0));
      conv = mx<double>(conv, fabs(cs1));
      const double sos = sqrt(a.g * depth<double>(zv[k], zb));
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
      // std::max keeps the running maximum when sp is NaN: check every point
      if (!isfinite(sp)) nonfinite = true;
      local = mx<double>(local, sp);
    }
    if (nonfinite || !isfinite(local)) {
      atomicOr(a.err, ERR_NONFINITE);
      local = 0;
    }
    if (per_cell) per_cell[c] = local;
  }
  for (int o = 16; o > 0; o >>= 1) local = fmax(local, __shfl_xor_sync(OC_FULL, local, o));
  if ((threadIdx.x & 31) == 0 && local > 0)
    atomicMax(out, (unsigned long long)__double_as_longlong(local));
}

// OceanDG.h:2599-2662 (degree >= 1 path): u = S^-1 (velocity at Gauss p+1),
// accumulated point by point into the cell's own output
__global__ void velocity_field_kernel(const AuxArgs a, const double *z, const double *q,
                                      double *u) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.n_cells) return;
  const int p = checked_degree(a.err, a.deg[c]), N = p + 1, n = N * N;
  const DegTables<double> &tb = tab<double>(p);
  const int64_t zo = checked(a.err, a.off[c], a.n_dofs - n + 1, BS_OFFSET);
  const double *zc = z + zo, *q0c = q + 2 * zo, *q1c = q + 2 * zo + n;
  double *u0 = u + 2 * zo, *u1 = u + 2 * zo + n;
  const double *sd = a.sd2 ? a.sd2 + cell_data(a.err, a.sdo2, c, a.n_sd[2], 2 * n) : nullptr;
  for (int i = 0; i < 2 * n; ++i) u0[i] = 0.;
  for (int qy = 0; qy < N; ++qy)
    for (int qx = 0; qx < N; ++qx) {
      double zv = 0, v0 = 0, v1 = 0;
      for (int iy = 0; iy < N; ++iy)
        for (int ix = 0; ix < N; ++ix) {
          const double b = tb.BM[qy][iy] * tb.BM[qx][ix];
          zv += b * zc[iy * N + ix];
          v0 += b * q0c[iy * N + ix];
          v1 += b * q1c[iy * N + ix];
        }
      double w0, w1;
      velocity<double>(zv, v0, v1, sd ? sd[2 * (qy * N + qx)] : 0., a.cu4, w0, w1);
      for (int iy = 0; iy < N; ++iy)
        for (int ix = 0; ix < N; ++ix) {
          const double s = tb.Sinv[iy][qy] * tb.Sinv[ix][qx];
          u0[iy * N + ix] += s * w0;
          u1[iy * N + ix] += s * w1;
        }
    }
}

// hpTuner.h:247-305: max over QGauss(nq) points of |dv/dx - du/dy|;
// B/D: [degree-1][nq*OC_MAXN] values/derivatives of the basis at the points
__global__ void vorticity_kernel(const AuxArgs a, const double *u, int nq, const double *B,
                                 const double *Dm, float *out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.n_cells) return;
  const int p = checked_degree(a.err, a.deg[c]), N = p + 1, n = N * N;
  const double *Bp = B + (p - 1) * 8 * OC_MAXN, *Dp = Dm + (p - 1) * 8 * OC_MAXN;
  const double *J = a.geo + 11 * (int64_t)c;
  const double *uc = u + 2 * checked(a.err, a.off[c], a.n_dofs - n + 1, BS_OFFSET);
  float mv = 0.f;
  for (int qy = 0; qy < nq; ++qy)
    for (int qx = 0; qx < nq; ++qx) {
      double ux = 0, uy = 0, vx = 0, vy = 0;
      for (int iy = 0; iy < N; ++iy)
        for (int ix = 0; ix < N; ++ix) {
          const double bx = Bp[qx * OC_MAXN + ix], by = Bp[qy * OC_MAXN + iy];
          const double dx = Dp[qx * OC_MAXN + ix], dy = Dp[qy * OC_MAXN + iy];
          const double uu = uc[iy * N + ix], vv = uc[n + iy * N + ix];
          ux += dx * by * uu;
          uy += bx * dy * uu;
          vx += dx * by * vv;
          vy += bx * dy * vv;
        }
      const double du_dy = J[7] * ux + J[9] * uy;  // physical d/dy of u
      const double dv_dx = J[6] * vx + J[8] * vy;  // physical d/dx of v
      const float w = (float)fabs(dv_dx - du_dy);
      mv = w > mv ? w : mv;
    }
  out[c] = mv;
}

// OceanDG.h:2241-2352 with the vortex exact solution as the projected function:
// zeta = S^-1 f0, q = S^-1 (f_{1,2} depth(f0, zb)) on Gauss p+1, accumulated
// point by point into the cell's own outputs
__global__ void project_vortex_kernel(const AuxArgs a, double time, double *z, double *q) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.n_cells) return;
  const int p = checked_degree(a.err, a.deg[c]), N = p + 1, n = N * N;
  const DegTables<double> &tb = tab<double>(p);
  const double *J = a.geo + 11 * (int64_t)c;
  const double *sd = a.sd2 ? a.sd2 + cell_data(a.err, a.sdo2, c, a.n_sd[2], 2 * n) : nullptr;
  const int64_t zo = checked(a.err, a.off[c], a.n_dofs - n + 1, BS_OFFSET);
  const VortexParams vp = vortex_params(a.vortex);
  double *zc = z + zo, *q0 = q + 2 * zo, *q1 = q + 2 * zo + n;
  for (int i = 0; i < n; ++i) zc[i] = 0.;
  for (int i = 0; i < 2 * n; ++i) q0[i] = 0.;
  for (int qy = 0; qy < N; ++qy)
    for (int qx = 0; qx < N; ++qx) {
      const double e0 = tb.xM[qx], e1 = tb.xM[qy];
      const double x = J[0] + J[2] * e0 + J[3] * e1, y = J[1] + J[4] * e0 + J[5] * e1;
      const double fz = vortex_value(vp, a.g, x, y, time, 0);
      const double hq = depth<double>(fz, sd ? sd[2 * (qy * N + qx)] : 0.);
      const double f1 = vortex_value(vp, a.g, x, y, time, 1) * hq;
      const double f2 = vortex_value(vp, a.g, x, y, time, 2) * hq;
      for (int iy = 0; iy < N; ++iy)
        for (int ix = 0; ix < N; ++ix) {
          const double s = tb.Sinv[iy][qy] * tb.Sinv[ix][qx];
          zc[iy * N + ix] += s * fz;
          q0[iy * N + ix] += s * f1;
          q1[iy * N + ix] += s * f2;
        }
    }
}

cudaError_t aux_upload_tables(const DegTables<double> *td, const DegTables<float> *tf) {
  cudaError_t e = cudaMemcpyToSymbol(c_tabd, td, sizeof(DegTables<double>) * OC_MAXDEG);
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_tabf, tf, sizeof(DegTables<float>) * OC_MAXDEG);
}

cudaError_t launch_transport_speed(const AuxArgs &a, const double *z, const double *q,
                                   unsigned long long *out, double *per_cell, cudaStream_t st) {
  transport_speed_kernel<<<(a.n_cells + 127) / 128, 128, 0, st>>>(a, z, q, out, per_cell);
  return cudaGetLastError();
}

cudaError_t launch_velocity_field(const AuxArgs &a, const double *z, const double *q, double *u,
                                  cudaStream_t st) {
  velocity_field_kernel<<<(a.n_cells + 127) / 128, 128, 0, st>>>(a, z, q, u);
  return cudaGetLastError();
}

// compute_errors_hydro (OceanDG.h:2380-2459) with the vortex as exact solution:
// per cell the squared L2 errors of depth and discharge on the cell Gauss rule,
// written to part[2c], part[2c+1] (summed by errors_reduce_kernel in a fixed order).
__global__ void errors_kernel(const AuxArgs a, double time, const double *sd0, const int *sdo0,
                              const double *z, const double *q, double *part) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.n_cells) return;
  const int p = checked_degree(a.err, a.deg[c]), N = p + 1, n = N * N;
  const int Q = a.cell_rule ? p + 1 : (3 * p) / 2 + 1;
  const DegTables<double> &tb = tab<double>(p);
  // the cell Gauss rule's tables: floor(1.5 p) + 1 points, or the Gauss p+1 ones
  const double(*BQ)[OC_MAXN] = a.cell_rule ? tb.BM : tb.BQ;
  const double *xQ = a.cell_rule ? tb.xM : tb.xQ, *wQ = a.cell_rule ? tb.wM : tb.wQ;
  const double *J = a.geo + 11 * (int64_t)c;
  const int64_t zo = checked(a.err, a.off[c], a.n_dofs - n + 1, BS_OFFSET);
  const double *zc = z + zo, *q0 = q + 2 * zo, *q1 = q + 2 * zo + n;
  const double *sd = sd0 ? sd0 + cell_data(a.err, sdo0, c, a.n_sd[0], 5 * Q * Q) : nullptr;
  const VortexParams vp = vortex_params(a.vortex);
  double e0 = 0., e1 = 0.;
  for (int qy = 0; qy < Q; ++qy)
    for (int qx = 0; qx < Q; ++qx) {
      double zv = 0., a0 = 0., a1 = 0.;
      for (int iy = 0; iy < N; ++iy)
        for (int ix = 0; ix < N; ++ix) {
          const double b = BQ[qy][iy] * BQ[qx][ix];
          zv += b * zc[iy * N + ix];
          a0 += b * q0[iy * N + ix];
          a1 += b * q1[iy * N + ix];
        }
      const double x = J[0] + J[2] * xQ[qx] + J[3] * xQ[qy];
      const double y = J[1] + J[4] * xQ[qx] + J[5] * xQ[qy];
      const double zb = sd ? sd[5 * (qy * Q + qx)] : 0.;
      const double f0 = vortex_value(vp, a.g, x, y, time, 0);
      const double hq = depth<double>(f0, zb);
      const double jxw = wQ[qx] * wQ[qy] * J[10];
      const double d0 = hq - depth<double>(zv, zb);
      const double u = vortex_value(vp, a.g, x, y, time, 1) * hq - a0;
      const double v = vortex_value(vp, a.g, x, y, time, 2) * hq - a1;
      e0 += d0 * d0 * jxw;
      e1 += (u * u + v * v) * jxw;
    }
  part[2 * (int64_t)c] = e0;
  part[2 * (int64_t)c + 1] = e1;
}

// one block: strided partial sums, then a fixed tree (deterministic order)
__global__ void errors_reduce_kernel(int n, const double *part, double *out) {
  __shared__ double s0[256], s1[256];
  double a0 = 0., a1 = 0.;
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    a0 += part[2 * (int64_t)c];
    a1 += part[2 * (int64_t)c + 1];
  }
  s0[threadIdx.x] = a0;
  s1[threadIdx.x] = a1;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      s0[threadIdx.x] += s0[threadIdx.x + h];
      s1[threadIdx.x] += s1[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sqrt(s0[0]);
    out[1] = sqrt(s1[0]);
  }
}

// prepare_for_conservative_coarsening (OceanDG.h:2732-2778) on marked cells
__global__ void conservative_coarsening_kernel(const AuxArgs a, const unsigned char *mark,
                                               double *z) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.n_cells || !mark[c]) return;
  const int p = checked_degree(a.err, a.deg[c]), N = p + 1, n = N * N, G = p + 2;
  const DegTables<double> &tb = tab<double>(p);
  const double det = a.geo[11 * (int64_t)c + 10];
  double *zc = z + checked(a.err, a.off[c], a.n_dofs - n + 1, BS_OFFSET);
  const double *sd = a.sd1 ? a.sd1 + cell_data(a.err, a.sdo1, c, a.n_sd[1], G * G) : nullptr;
  double area = 0., integral = 0.;
  for (int gy = 0; gy < G; ++gy)
    for (int gx = 0; gx < G; ++gx) {
      double zv = 0.;
      for (int iy = 0; iy < N; ++iy)
        for (int ix = 0; ix < N; ++ix) zv += tb.BG[gy][iy] * tb.BG[gx][ix] * zc[iy * N + ix];
      const double zb = sd ? sd[gy * G + gx] : 0.;
      const double mask = zv <= -zb ? 0. : 1.;
      const double jxw = tb.wG[gx] * tb.wG[gy] * det;
      area += mask * jxw;
      integral += zv * mask * jxw;
    }
  if (area > 0.) {
    const double v = integral * (1. / area);
    for (int i = 0; i < n; ++i) zc[i] = v;
  }
}

// one thread: an index outside its range through the bounds check (no access)
__global__ void bounds_selftest_kernel(int *err) { checked(err, 5, 3, BS_SELFTEST); }

cudaError_t launch_bounds_selftest(int *err, cudaStream_t st) {
  bounds_selftest_kernel<<<1, 1, 0, st>>>(err);
  return cudaGetLastError();
}

cudaError_t launch_errors(const AuxArgs &a, double time, const double *sd0, const int *sdo0,
                          const double *z, const double *q, double *part, double *out,
                          cudaStream_t st) {
  errors_kernel<<<(a.n_cells + 127) / 128, 128, 0, st>>>(a, time, sd0, sdo0, z, q, part);
  errors_reduce_kernel<<<1, 256, 0, st>>>(a.n_cells, part, out);
  return cudaGetLastError();
}

cudaError_t launch_conservative_coarsening(const AuxArgs &a, const unsigned char *mark, double *z,
                                           cudaStream_t st) {
  conservative_coarsening_kernel<<<(a.n_cells + 127) / 128, 128, 0, st>>>(a, mark, z);
  return cudaGetLastError();
}

// Largest vorticity of each member (non-negative floats order like their bits).
__global__ void member_max_kernel(int n, const float *w, const int *info, int n_members,
                                  unsigned *vmax) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int m = info[6 * (int64_t)c + 5];
  if (m >= 0 && m < n_members) atomicMax(&vmax[m], __float_as_uint(fmaxf(w[c], 0.f)));
}

// Indicator features of one cell (see oc_indicator_features in oceano_gpu.h).
__global__ void features_kernel(const AuxArgs a, const double *z, const double *q, const float *w,
                                const int *info, int n_members, const unsigned *vmax, float thr,
                                float *feat, float *flags, float *wn) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.n_cells) return;
  const int p = checked_degree(a.err, a.deg[c]), N = p + 1, n = N * N;
  const DegTables<double> &tb = tab<double>(p);
  // integral weights of the nodal basis on [0,1] (Gauss p+1 is exact for them)
  double mw[OC_MAXN];
  for (int i = 0; i < N; ++i) {
    double s = 0;
    for (int k = 0; k < N; ++k) s += tb.wM[k] * tb.BM[k][i];
    mw[i] = s;
  }
  const int64_t zo = checked(a.err, a.off[c], a.n_dofs - n + 1, BS_OFFSET);
  double zm = 0, q0 = 0, q1 = 0;
  for (int iy = 0; iy < N; ++iy)
    for (int ix = 0; ix < N; ++ix) {
      const double wt = mw[ix] * mw[iy];
      zm += wt * z[zo + iy * N + ix];
      q0 += wt * q[2 * zo + iy * N + ix];
      q1 += wt * q[2 * zo + n + iy * N + ix];
    }
  const int *inf = info + 6 * (int64_t)c;
  const int m = inf[5];
  const float mx = (m >= 0 && m < n_members) ? __uint_as_float(vmax[m]) : 0.f;
  const float inv = mx > 0.f ? 1.f / mx : 0.f;
  const float w0 = w[c] * inv;
  // vorticity magnitudes relative to the member maximum on a log10 scale: the
  // refinement threshold (1e-5 of the maximum) sits many decades below the bulk
  // of the values, where a linear feature is lost in the BF16 inputs
  float nb[4];
  for (int f = 0; f < 4; ++f) nb[f] = log10f(fabsf(inf[f] >= 0 ? w[inf[f]] * inv : w0) + 1e-12f);
  float *o = feat + 12 * (int64_t)c;
  o[0] = (float)zm; o[1] = (float)q0; o[2] = (float)q1;
  o[3] = log10f(fabsf(w0) + 1e-12f);
  o[4] = 0.5f * (nb[1] - nb[0]);  // differences across the cell (faces 1-0, 3-2)
  o[5] = 0.5f * (nb[3] - nb[2]);
  o[6] = nb[0]; o[7] = nb[1]; o[8] = nb[2]; o[9] = nb[3];
  o[10] = (float)inf[4]; o[11] = (float)p;
  if (flags) flags[c] = w0 > thr ? 1.f : 0.f;
  if (wn) wn[c] = w0;
}

cudaError_t launch_features(const AuxArgs &a, const double *z, const double *q, const float *w,
                            const int *info, int n_members, unsigned *vmax, float thr,
                            float *feat, float *flags, float *wn, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(vmax, 0, sizeof(unsigned) * n_members, st);
  if (e != cudaSuccess) return e;
  const int nb = (a.n_cells + 127) / 128;
  member_max_kernel<<<nb, 128, 0, st>>>(a.n_cells, w, info, n_members, vmax);
  features_kernel<<<nb, 128, 0, st>>>(a, z, q, w, info, n_members, vmax, thr, feat, flags, wn);
  return cudaGetLastError();
}

cudaError_t launch_vorticity(const AuxArgs &a, const double *u, int nq, const double *B,
                             const double *D, float *out, cudaStream_t st) {
  vorticity_kernel<<<(a.n_cells + 127) / 128, 128, 0, st>>>(a, u, nq, B, D, out);
  return cudaGetLastError();
}

cudaError_t launch_project_vortex(const AuxArgs &a, double time, double *z, double *q,
                                  cudaStream_t st) {
  project_vortex_kernel<<<(a.n_cells + 127) / 128, 128, 0, st>>>(a, time, z, q);
  return cudaGetLastError();
}

}  // namespace oc
