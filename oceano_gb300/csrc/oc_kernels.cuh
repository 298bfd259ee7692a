// Device code of the GB300 per-stage DG shallow-water operator.
//
// One fused, element-centric kernel per RK stage and degree.  A team of T
// threads (T = max(floor(1.5p)+1, p+2)) owns one cell; 32/T cells share a
// warp, and every synchronisation is a full-warp __syncwarp() executed by all
// lanes (control flow that differs between teams never contains one).  The
// team
//   1. stages its cell's DoFs in shared memory,
//   2. evaluates the L_h cell integrals by sum factorisation (x-passes on
//      node rows, y-passes on point columns, contractions in registers with
//      constant-bank shape coefficients),
//   3. evaluates the numerical flux of every face of the cell (conforming,
//      either side of a hanging face, periodic, boundary) and keeps its own
//      side; both neighbours evaluate a shared face identically,
//   4. forms the zeta right-hand side and runs the wet/dry lumped-mass
//      iteration (FP64: literally, with the batch stop rule; mixed form:
//      the closed form of the same sweeps on fully wet cells, the literal
//      FP64 iteration elsewhere),
//   5. applies the discharge inverse mass and the FP64 Runge-Kutta update,
// and writes only its own cell's outputs.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "oc_layout.h"

namespace oc {

static __constant__ DegTables<double> c_tabd[OC_MAXDEG];
static __constant__ DegTables<float> c_tabf[OC_MAXDEG];

template <typename R>
__device__ __forceinline__ const DegTables<R> &tab(int p);
template <>
__device__ __forceinline__ const DegTables<double> &tab<double>(int p) { return c_tabd[p - 1]; }
template <>
__device__ __forceinline__ const DegTables<float> &tab<float>(int p) { return c_tabf[p - 1]; }

enum { ERR_UNKNOWN_BID = 1 << 2, ERR_NONFINITE = 1 << 3 };
#define OC_FULL 0xffffffffu

template <typename R>
__device__ __forceinline__ R mx(R a, R b) { return a < b ? b : a; }  // std::max
template <typename R>
__device__ __forceinline__ R mn(R a, R b) { return b < a ? b : a; }  // std::min

// ShallowWater.h:312-320
template <typename R>
__device__ __forceinline__ R depth(R z, R zb) { return mx<R>(z + zb, R(1e-12)); }

// ShallowWater.h:322-336, desingularised velocity
template <typename R>
__device__ __forceinline__ void velocity(R z, R q0, R q1, R zb, R cu4, R &v0, R &v1) {
  const R h = depth<R>(z, zb);
  const R h4 = h * h * h * h;
  const R inv = sqrt(R(2.)) * h / sqrt(h4 + mx<R>(h4, cu4));
  v0 = q0 * inv;
  v1 = q1 * inv;
}

// BottomFriction.h:87-137 (linear), :183-213 (Manning)
template <typename R>
__device__ __forceinline__ void friction(int model, R g, R v0, R v1, R cf, R h, R &s0, R &s1) {
  if (model == 1) {
    s0 = cf * h * v0; s1 = cf * h * v1;
  } else if (model == 2) {
    const R inv_depth = R(1.) / (exp(log(h) * R(0.33333333333)));
    const R hcf = g * cf * cf * inv_depth * sqrt(v0 * v0 + v1 * v1);
    s0 = hcf * v0; s1 = hcf * v1;
  } else {
    s0 = 0; s1 = 0;
  }
}

template <typename R>
__device__ __forceinline__ R friction_jac(int model, R g, R v0, R v1, R cf, R h) {
  if (model == 1) return cf;
  if (model == 2) {
    const R inv_depth = R(1.) / (exp(log(h) * R(1.33333333333)));
    return g * cf * cf * inv_depth * sqrt(v0 * v0 + v1 * v1);
  }
  return 0;
}

// LaxFriedrichsModified.h:161-230 and NumericalFluxBase.h:103-126 at one face
// point: mass flux F, advective flux Fa, strong pressure flux of the minus-side
// call (Pm) and of the plus-side call (Pp).
template <typename R>
__device__ __forceinline__ void face_flux(R g, R cu4, R zm, R qm0, R qm1, R zp, R qp0, R qp1,
                                          R n0, R n1, R zbm, R zbp, R &F, R &Fa0, R &Fa1,
                                          R &Pm0, R &Pm1, R &Pp0, R &Pp1) {
  R vm0, vm1, vp0, vp1;
  velocity<R>(zm, qm0, qm1, zbm, cu4, vm0, vm1);
  velocity<R>(zp, qp0, qp1, zbp, cu4, vp0, vp1);
  const R lm = fabs(vm0 * n0 + vm1 * n1) + sqrt(g * depth<R>(zm, zbm));
  const R lp = fabs(vp0 * n0 + vp1 * n1) + sqrt(g * depth<R>(zp, zbp));
  const R lambda = mx<R>(lp, lm);
  const R zbs = mn<R>(zbm, zbp);
  const R hm = depth<R>(zm, zbs), hp = depth<R>(zp, zbs);
  const R hum0 = hm * vm0, hum1 = hm * vm1, hup0 = hp * vp0, hup1 = hp * vp1;
  const R cm = mx<R>(zm, -zbs), cp = mx<R>(zp, -zbs);
  F = R(0.5) * ((hum0 * n0 + hum1 * n1) + (hup0 * n0 + hup1 * n1)) + R(0.5) * lambda * (cm - cp);
  R wm0, wm1, wp0, wp1;  // advective_flux recomputes the velocity from hu
  velocity<R>(zm, hum0, hum1, zbs, cu4, wm0, wm1);
  velocity<R>(zp, hup0, hup1, zbs, cu4, wp0, wp1);
  const R unm = wm0 * n0 + wm1 * n1, unp = wp0 * n0 + wp1 * n1;
  Fa0 = R(0.5) * (hum0 * unm + hup0 * unp) + R(0.5) * lambda * (hum0 - hup0);
  Fa1 = R(0.5) * (hum1 * unm + hup1 * unp) + R(0.5) * lambda * (hum1 - hup1);
  const R s = g * R(0.25) * (hp + hm);
  const R sm = s * (cp - cm), sp = s * (cm - cp);
  Pm0 = sm * n0; Pm1 = sm * n1;
  Pp0 = sp * n0; Pp1 = sp * n1;
}

// Icbc_ShallowWaterVortex.h:139-226 (regularity p=2), FP64
__host__ __device__ inline double vortex_H(double x) {
  const double cosx = cos(x), cos2x = cos(2. * x), sin2x = sin(2. * x), sinx = sin(x);
  const double cosx2 = cosx * cosx, cos2x2 = cos2x * cos2x, x2 = x * x;
  const double c5 = cosx2 * cosx2 * cosx, c6 = c5 * cosx;
  return 0.091145833 * cos2x + 0.182291667 * x * sin2x + c6 * (0.015625 * cosx2 + 0.024305556) +
         0.011393229 * cos2x2 + 0.13671875 * x2 + 0.045572917 * x * cos2x * sin2x +
         0.125 * x * c5 * sinx * (cosx2 + 1.166666667);
}

struct VortexParams {
  double h0, uoo, r0, gamma, x0, y0;
};

__host__ __device__ inline VortexParams vortex_params(const double *v) {
  VortexParams p;
  p.h0 = v[0]; p.uoo = v[1]; p.r0 = v[2]; p.gamma = v[3]; p.x0 = v[4]; p.y0 = v[5];
  return p;
}

// component 0: depth, 1: u, 2: v (3: the passive tracer 0.1 y)
__host__ __device__ inline double vortex_value(const VortexParams vp, double g, double x,
                                               double y, double t, int comp) {
  const double x0 = vp.x0 + vp.uoo * t, y0 = vp.y0;
  const double radius = sqrt((x - x0) * (x - x0) + (y - y0) * (y - y0));
  const double rho_half = 0.5 * M_PI * radius / vp.r0;
  const double c = cos(rho_half), c2 = c * c;
  const double omega = 4. * vp.gamma * c2 * c2;
  if (comp == 0) {
    const double num = 4. * vp.gamma * vp.r0;
    const double Hpi = 4. * vortex_H(0.5 * M_PI), Hrho = 4. * vortex_H(rho_half);
    return radius < vp.r0 ? vp.h0 - 1. / (g * M_PI * M_PI) * num * num * (Hpi - Hrho) : vp.h0;
  }
  if (comp == 1) return radius < vp.r0 ? vp.uoo - (y - y0) * omega : vp.uoo;
  if (comp == 2) return radius < vp.r0 ? (x - x0) * omega : 0.;
  return 0.1 * y;
}

__device__ inline double bc_value(const StageArgs &a, int bid, double x, double y, int comp) {
  if (a.bc_fn[bid] == 1)
    return vortex_value(vortex_params(a.vortex), a.g, x, y, a.dyn->time, comp);
  return comp < 3 ? a.bc_c[bid][comp] : 0.;
}

__device__ __forceinline__ int face_dof(int N, int f, int i) {
  return f == 0 ? i * N : f == 1 ? i * N + N - 1 : f == 2 ? i : (N - 1) * N + i;
}

template <typename R>
__device__ __forceinline__ R load_r(const void *p, int64_t i, int is_float, double ref) {
  if (is_float) return (R)(static_cast<const float *>(p)[i]);
  return (R)(static_cast<const double *>(p)[i] - ref);
}

// stride of the per-variable face point values (>= OC_MAXF and OC_MAXQ)
constexpr int FVS = 8;

template <int P>
struct Dims {
  static constexpr int N = P + 1, Q = (3 * P) / 2 + 1, G = P + 2;
  static constexpr int T = Q > G ? Q : G;
  static constexpr int NN = N * N, NT = N * T;
  static constexpr int CPW = 32 / T;
  // per-cell shared memory: compute-type region and FP64 region (elements)
  static constexpr int SZR = 9 * NN + 6 * NT + 3 * FVS;  // U 3, RES 3, RST 2, BZ 1 tiles; X; FV
  static constexpr int SZD = NN + 3 * NT + T + 2;
  // Team strides: padded so that the 32/T teams of a warp start on different
  // shared-memory banks (stride mod 32 chosen per degree and element size to
  // keep row, column and node-row accesses at most 2-way conflicted).
  static constexpr int pad_f = P == 1 ? 5 : P == 2 ? 5 : P == 3 ? 3 : 8;
  static constexpr int pad_d = P == 1 ? 5 : P == 2 ? 2 : P == 3 ? 3 : 4;
  template <typename R>
  static constexpr int bytes_r() {
    return (((SZR + 31) / 32) * 32 + (sizeof(R) == 4 ? pad_f : pad_d)) * (int)sizeof(R);
  }
  static constexpr int bytes_d() { return (((SZD + 31) / 32) * 32 + pad_d) * 8; }
  // per warp: CPW compute regions, CPW FP64 regions, CPW batch-norm slots
  template <typename R>
  static constexpr int d_offset() { return ((CPW * bytes_r<R>() + 15) / 16) * 16; }
  template <typename R>
  static constexpr int norm_offset() { return d_offset<R>() + CPW * bytes_d(); }
  template <typename R>
  static constexpr int warp_bytes() { return ((norm_offset<R>() + CPW * 8 + 15) / 16) * 16; }
};

// Sum over the T threads of a team; called by all lanes (two full syncs).
template <int T>
__device__ __forceinline__ double team_sum(double *red, int t, bool member, double v) {
  if (member) red[t] = v;
  __syncwarp();
  double s = 0;
  if (member)
#pragma unroll
    for (int k = 0; k < T; ++k) s += red[k];
  __syncwarp();
  return s;
}

template <int T>
__device__ __forceinline__ double team_max(double *red, int t, bool member, double v) {
  if (member) red[t] = v;
  __syncwarp();
  double s = -1.7976931348623157e308;
  if (member)
#pragma unroll
    for (int k = 0; k < T; ++k) s = mx<double>(s, red[k]);
  __syncwarp();
  return s;
}

// Evaluate the FP64 tile DZ at the Gauss-Lobatto (p+2)^2 points, call
// fn(qx, qy, value, o0, o1) per point, integrate o0, o1 back against the basis
// into out0/out1 (rows of thread t < N).  All lanes call; `work` gates arithmetic.
template <int P, class Fn>
__device__ __forceinline__ void gl_eval_apply_integrate(const double *DZ, double *DX, int t,
                                                        bool work, Fn fn, double *out0,
                                                        double *out1) {
  using D = Dims<P>;
  constexpr int N = D::N, G = D::G, T = D::T, NT = D::NT;
  const DegTables<double> &tb = tab<double>(P);
  if (work && t < N) {
#pragma unroll
    for (int gx = 0; gx < G; ++gx) {
      double s = 0;
#pragma unroll
      for (int ix = 0; ix < N; ++ix) s += tb.BG[gx][ix] * DZ[t * N + ix];
      DX[t * T + gx] = s;
    }
  }
  __syncwarp();
  if (work && t < G) {
    double a0[N], a1[N];
#pragma unroll
    for (int i = 0; i < N; ++i) a0[i] = a1[i] = 0;
#pragma unroll
    for (int gy = 0; gy < G; ++gy) {
      double v = 0;
#pragma unroll
      for (int iy = 0; iy < N; ++iy) v += tb.BG[gy][iy] * DX[iy * T + t];
      double o0, o1;
      fn(t, gy, v, o0, o1);
#pragma unroll
      for (int iy = 0; iy < N; ++iy) {
        a0[iy] += tb.BG[gy][iy] * o0;
        a1[iy] += tb.BG[gy][iy] * o1;
      }
    }
#pragma unroll
    for (int iy = 0; iy < N; ++iy) {
      DX[NT + iy * T + t] = a0[iy];
      DX[2 * NT + iy * T + t] = a1[iy];
    }
  }
  __syncwarp();
  if (work && t < N) {
#pragma unroll
    for (int ix = 0; ix < N; ++ix) {
      double s0 = 0, s1 = 0;
#pragma unroll
      for (int gx = 0; gx < G; ++gx) {
        s0 += tb.BG[gx][ix] * DX[NT + t * T + gx];
        s1 += tb.BG[gx][ix] * DX[2 * NT + t * T + gx];
      }
      out0[ix] = s0;
      out1[ix] = s1;
    }
  }
  __syncwarp();
}

// Zeta inverse mass, literally (OceanDG.h:1373-1507, operators.h:276-298):
// epsilon lift of fully dry cells, then at most max_iter sweeps
//   zeta += M_L(mask)^-1 (rhs - int depth(zeta) phi)
// stopped when the l1 norm of the update summed over the cell batch is <= 1e-12.
// DZ holds the initial guess on entry and the result on exit; rhs are the
// rows of thread t < N.  All lanes call; `work` selects the participating teams.
template <int P>
__device__ void zeta_iteration_fp64(const StageArgs &a, int cell, double *DZ, double *DX,
                                    double *DRED, double *warp_norm, int team, int cpw, int t,
                                    bool member, bool work, const double *rhs) {
  using D = Dims<P>;
  constexpr int N = D::N, G = D::G, T = D::T;
  const DegTables<double> &tb = tab<double>(P);
  const double *geo = a.geo + 11 * (int64_t)cell;
  const double det = geo[10];
  const double *zb1 = a.sd1 ? a.sd1 + a.sdo1[cell] : nullptr;
  // epsilon lift (OceanDG.h:1399-1422)
  {
    int ndry = 0;
    double zbmax = -1.7976931348623157e308;
    double d0[N], d1[N];
    gl_eval_apply_integrate<P>(
        DZ, DX, t, work,
        [&](int qx, int qy, double v, double &o0, double &o1) {
          const double zb = zb1 ? zb1[qy * G + qx] : 0.;
          if (v <= -zb) {
            zbmax = mx<double>(zb, zbmax);
            ++ndry;
          }
          o0 = o1 = 0;
        },
        d0, d1);
    const double tot = team_sum<T>(DRED, t, member, (double)ndry);
    const double zmax = team_max<T>(DRED, t, member, zbmax);
    if (work && t < N && tot == (double)(G * G))
#pragma unroll
      for (int ix = 0; ix < N; ++ix) DZ[t * N + ix] = -zmax + 1e-09;
    __syncwarp();
  }
  bool active = work;
  const int W = a.batch;
  for (int k = 0; k < a.max_iter; ++k) {
    if (!__any_sync(OC_FULL, active)) break;
    int ndry = 0;
    double r[N], m[N];
    gl_eval_apply_integrate<P>(
        DZ, DX, t, active,
        [&](int qx, int qy, double v, double &o0, double &o1) {
          const double zb = zb1 ? zb1[qy * G + qx] : 0.;
          const double jxw = tb.wG[qx] * tb.wG[qy] * det;
          const double msk = v <= -zb ? 0. : 1.;
          ndry += msk == 0.;
          o0 = -depth<double>(v, zb) * jxw;
          o1 = msk * jxw;
        },
        r, m);
    const double tot = team_sum<T>(DRED, t, member, (double)ndry);
    double part = 0;
    if (active && t < N) {
#pragma unroll
      for (int ix = 0; ix < N; ++ix) {
        const double old = DZ[t * N + ix];
        const double inc = tot < (double)(G * G) ? 1. / m[ix] * (rhs[ix] + r[ix]) : 0.;
        const double nw = old + inc;
        DZ[t * N + ix] = nw;
        part += fabs(old - nw);
      }
    }
    const double cn = team_sum<T>(DRED, t, member, part);
    if (member && t == 0) warp_norm[team] = active ? cn : 0.0;
    __syncwarp();
    double bn = 0;
    if (member && team < cpw) {  // batches lie inside the first cpw teams
      const int b0 = (team / W) * W;
      for (int j = 0; j < W; ++j) bn += warp_norm[b0 + j];
    }
    __syncwarp();
    active = active && bn > 1e-12;
  }
}

// ---------------------------------------------------------------------------
// The fused stage kernel.
//   MIX = false: FP64 plain form (R = KT = double).
//   MIX = true : mixed form; R = float bulk, KT = type of the k registers.
// ---------------------------------------------------------------------------
template <int P, typename R, typename KT, bool MIX>
__global__ void __launch_bounds__(128) stage_kernel(const StageArgs a) {
  using D = Dims<P>;
  constexpr int N = D::N, Q = D::Q, G = D::G, T = D::T, NN = D::NN, NT = D::NT;
  constexpr int CPWMAX = D::CPW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const DegTables<R> &tb = tab<R>(P);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int team_raw = lane / T, t = lane - team_raw * T;
  const bool member = team_raw < CPWMAX;  // lanes past the last team only synchronise
  const int team = member ? team_raw : 0;
  const int W = a.batch;
  const int cpw = (CPWMAX / W) * W;
  const int wpb = blockDim.x >> 5;
  const int gi = (blockIdx.x * wpb + warp) * cpw + team;
  const bool valid = member && team < cpw && gi < a.n_group;
  const int cell = a.group_cells ? a.group_cells[valid ? gi : 0] : a.group_first + (valid ? gi : 0);

  unsigned char *wbase = smem_raw + warp * D::template warp_bytes<R>();
  R *sm = reinterpret_cast<R *>(wbase + team * D::template bytes_r<R>());
  double *dm = reinterpret_cast<double *>(wbase + D::template d_offset<R>() +
                                          team * D::bytes_d());
  double *warp_norm = reinterpret_cast<double *>(wbase + D::template norm_offset<R>());
  R *U = sm;                  // 3*NN stage input z, q0, q1
  R *RES = U + 3 * NN;        // 3*NN residual
  R *RST = RES + 3 * NN;      // 2*NN stiff residual (ARK)
  R *BZ = RST + 2 * NN;       // NN zeta right-hand side b = sum f k
  R *X = BZ + NN;             // 6 tiles of N*T
  R *FV = X + 6 * NT;         // 3*FVS face point values
  double *DZ = dm;            // NN FP64 iterate
  double *DX = DZ + NN;       // 3 tiles N*T
  double *DRED = DX + 3 * NT; // T+1

  const double *geo = a.geo + 11 * (int64_t)cell;
  const R Ji00 = (R)geo[6], Ji01 = (R)geo[7], Ji10 = (R)geo[8], Ji11 = (R)geo[9];
  const R det = (R)geo[10];
  const int64_t zo = a.off[cell], qo = 2 * zo;
  const double zref = MIX ? a.zeta_ref : 0.0;
  const R g = (R)a.g, cu4 = (R)a.cu4;
  const R zbe_flat = (R)zref;  // zb + zeta_ref where no bathymetry is given
  const int s = a.stage;
  const StageDyn dy = *a.dyn;

  // ---- 1. stage input DoFs ---------------------------------------------------
  if (member && t < N) {
#pragma unroll
    for (int ix = 0; ix < N; ++ix) {
      const int d = t * N + ix;
      U[d] = load_r<R>(a.rz, zo + d, a.r_is_float, zref);
      U[NN + d] = load_r<R>(a.rq, qo + d, a.r_is_float, 0.0);
      U[2 * NN + d] = load_r<R>(a.rq, qo + NN + d, a.r_is_float, 0.0);
    }
  }
  __syncwarp();

  // ---- 2. cell integrals: local_apply_cell_height (OceanDG.h:669-693),
  //         local_apply_cell_discharge / _nonstiff / _stiff (:695-826) ---------
  if (member && t < N) {  // x-pass on rows iy = t
    R z[N], q0[N], q1[N];
#pragma unroll
    for (int ix = 0; ix < N; ++ix) {
      z[ix] = U[t * N + ix];
      q0[ix] = U[NN + t * N + ix];
      q1[ix] = U[2 * NN + t * N + ix];
    }
#pragma unroll
    for (int qx = 0; qx < Q; ++qx) {
      R b0 = 0, d0 = 0, a0 = 0, a1 = 0;
#pragma unroll
      for (int ix = 0; ix < N; ++ix) {
        b0 += tb.BQ[qx][ix] * z[ix];
        d0 += tb.DQ[qx][ix] * z[ix];
        a0 += tb.BQ[qx][ix] * q0[ix];
        a1 += tb.BQ[qx][ix] * q1[ix];
      }
      X[0 * NT + t * T + qx] = b0;
      X[1 * NT + t * T + qx] = d0;
      X[2 * NT + t * T + qx] = a0;
      X[3 * NT + t * T + qx] = a1;
    }
  }
  __syncwarp();
  const bool split = a.ark && !a.last;  // ARK internal stage: stiff part separate
  {
    R Az[N], Cz[N], A0[N], C0[N], A1[N], C1[N];
#pragma unroll
    for (int i = 0; i < N; ++i) Az[i] = Cz[i] = A0[i] = C0[i] = A1[i] = C1[i] = 0;
    if (member && t < Q) {  // y-pass, pointwise model, y-integration on column qx = t
      const double *sd0 = a.sd0 ? a.sd0 + a.sdo0[cell] : nullptr;
      const float *sd0e = a.sd0e ? a.sd0e + a.sdo0[cell] : nullptr;
#pragma unroll
      for (int qy = 0; qy < Q; ++qy) {
        R z = 0, zx = 0, zy = 0, q0 = 0, q1 = 0;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          const R xb = X[0 * NT + iy * T + t], xd = X[1 * NT + iy * T + t];
          z += tb.BQ[qy][iy] * xb;
          zx += tb.BQ[qy][iy] * xd;
          zy += tb.DQ[qy][iy] * xb;
          q0 += tb.BQ[qy][iy] * X[2 * NT + iy * T + t];
          q1 += tb.BQ[qy][iy] * X[3 * NT + iy * T + t];
        }
        const int k = qy * Q + t;
        R zb = MIX ? zbe_flat : R(0), cf = 0, w0 = 0, w1 = 0, fc = 0;
        if (MIX && sd0e) {
          zb = (R)sd0e[5 * k]; cf = (R)sd0e[5 * k + 1]; w0 = (R)sd0e[5 * k + 2];
          w1 = (R)sd0e[5 * k + 3]; fc = (R)sd0e[5 * k + 4];
        } else if (!MIX && sd0) {
          zb = (R)sd0[5 * k]; cf = (R)sd0[5 * k + 1]; w0 = (R)sd0[5 * k + 2];
          w1 = (R)sd0[5 * k + 3]; fc = (R)sd0[5 * k + 4];
        }
        const R w = tb.wQ[t] * tb.wQ[qy] * det;
        // height: int q . grad(phi)   (mass_flux = q, ShallowWater.h:349-357)
        const R gz0 = (Ji00 * q0 + Ji01 * q1) * w, gz1 = (Ji10 * q0 + Ji11 * q1) * w;
        // discharge: advective flux (ShallowWater.h:378-403, nu = 0) and sources (:405-472)
        R v0, v1;
        velocity<R>(z, q0, q1, zb, cu4, v0, v1);
        const R h = depth<R>(z, zb);
        const R dz0 = Ji00 * zx + Ji10 * zy, dz1 = Ji01 * zx + Ji11 * zy;
        R fr0 = 0, fr1 = 0;
        if (a.friction) friction<R>(a.friction, g, v0, v1, cf, h, fr0, fr1);
        const R s0 = -g * h * dz0 - (split ? R(0) : fr0) + w0 + fc * q1;
        const R s1 = -g * h * dz1 - (split ? R(0) : fr1) + w1 - fc * q0;
        const R F00 = q0 * v0, F01 = q0 * v1, F10 = q1 * v0, F11 = q1 * v1;
        const R g00 = (Ji00 * F00 + Ji01 * F01) * w, g01 = (Ji10 * F00 + Ji11 * F01) * w;
        const R g10 = (Ji00 * F10 + Ji01 * F11) * w, g11 = (Ji10 * F10 + Ji11 * F11) * w;
        const R sv0 = s0 * w, sv1 = s1 * w;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          const R b = tb.BQ[qy][iy], d = tb.DQ[qy][iy];
          Az[iy] += b * gz0;
          Cz[iy] += d * gz1;
          A0[iy] += b * g00;
          C0[iy] += d * g01 + b * sv0;
          A1[iy] += b * g10;
          C1[iy] += d * g11 + b * sv1;
        }
      }
    }
    __syncwarp();
    if (member && t < Q) {
#pragma unroll
      for (int iy = 0; iy < N; ++iy) {
        X[0 * NT + iy * T + t] = Az[iy];
        X[1 * NT + iy * T + t] = Cz[iy];
        X[2 * NT + iy * T + t] = A0[iy];
        X[3 * NT + iy * T + t] = C0[iy];
        X[4 * NT + iy * T + t] = A1[iy];
        X[5 * NT + iy * T + t] = C1[iy];
      }
    }
    __syncwarp();
    if (member && t < N) {  // x-integration on rows iy = t
#pragma unroll
      for (int ix = 0; ix < N; ++ix) {
        R rz = 0, r0 = 0, r1 = 0;
#pragma unroll
        for (int qx = 0; qx < Q; ++qx) {
          const R b = tb.BQ[qx][ix], d = tb.DQ[qx][ix];
          rz += d * X[0 * NT + t * T + qx] + b * X[1 * NT + t * T + qx];
          r0 += d * X[2 * NT + t * T + qx] + b * X[3 * NT + t * T + qx];
          r1 += d * X[4 * NT + t * T + qx] + b * X[5 * NT + t * T + qx];
        }
        RES[t * N + ix] = rz;
        RES[NN + t * N + ix] = r0;
        RES[2 * NN + t * N + ix] = r1;
      }
    }
    __syncwarp();
    if (split) {  // warp-uniform: stiff (friction) residual, a second pass over the points
      if (member && t < N) {  // x-pass of the stage input again (X was overwritten)
        R z[N], q0[N], q1[N];
#pragma unroll
        for (int ix = 0; ix < N; ++ix) {
          z[ix] = U[t * N + ix];
          q0[ix] = U[NN + t * N + ix];
          q1[ix] = U[2 * NN + t * N + ix];
        }
#pragma unroll
        for (int qx = 0; qx < Q; ++qx) {
          R b0 = 0, a0 = 0, a1 = 0;
#pragma unroll
          for (int ix = 0; ix < N; ++ix) {
            b0 += tb.BQ[qx][ix] * z[ix];
            a0 += tb.BQ[qx][ix] * q0[ix];
            a1 += tb.BQ[qx][ix] * q1[ix];
          }
          X[2 * NT + t * T + qx] = b0;
          X[3 * NT + t * T + qx] = a0;
          X[4 * NT + t * T + qx] = a1;
        }
      }
      __syncwarp();
      R S0[N], S1[N];
#pragma unroll
      for (int i = 0; i < N; ++i) S0[i] = S1[i] = 0;
      if (member && t < Q) {
        const double *sd0 = a.sd0 ? a.sd0 + a.sdo0[cell] : nullptr;
        const float *sd0e = a.sd0e ? a.sd0e + a.sdo0[cell] : nullptr;
#pragma unroll
        for (int qy = 0; qy < Q; ++qy) {
          R z = 0, q0 = 0, q1 = 0;
#pragma unroll
          for (int iy = 0; iy < N; ++iy) {
            z += tb.BQ[qy][iy] * X[2 * NT + iy * T + t];
            q0 += tb.BQ[qy][iy] * X[3 * NT + iy * T + t];
            q1 += tb.BQ[qy][iy] * X[4 * NT + iy * T + t];
          }
          const int k = qy * Q + t;
          R zb = MIX ? zbe_flat : R(0), cf = 0;
          if (MIX && sd0e) { zb = (R)sd0e[5 * k]; cf = (R)sd0e[5 * k + 1]; }
          else if (!MIX && sd0) { zb = (R)sd0[5 * k]; cf = (R)sd0[5 * k + 1]; }
          R v0, v1, fr0 = 0, fr1 = 0;
          velocity<R>(z, q0, q1, zb, cu4, v0, v1);
          if (a.friction) friction<R>(a.friction, g, v0, v1, cf, depth<R>(z, zb), fr0, fr1);
          const R w = tb.wQ[t] * tb.wQ[qy] * det;
          const R st0 = -fr0 * w, st1 = -fr1 * w;
#pragma unroll
          for (int iy = 0; iy < N; ++iy) {
            S0[iy] += tb.BQ[qy][iy] * st0;
            S1[iy] += tb.BQ[qy][iy] * st1;
          }
        }
      }
      __syncwarp();
      if (member && t < Q) {
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          X[0 * NT + iy * T + t] = S0[iy];
          X[1 * NT + iy * T + t] = S1[iy];
        }
      }
      __syncwarp();
      if (member && t < N) {
#pragma unroll
        for (int ix = 0; ix < N; ++ix) {
          R r0 = 0, r1 = 0;
#pragma unroll
          for (int qx = 0; qx < Q; ++qx) {
            r0 += tb.BQ[qx][ix] * X[0 * NT + t * T + qx];
            r1 += tb.BQ[qx][ix] * X[1 * NT + t * T + qx];
          }
          RST[t * N + ix] = r0;
          RST[NN + t * N + ix] = r1;
        }
      }
      __syncwarp();
    }
  }

  // ---- 3. faces: local_apply_face_* (OceanDG.h:936-1050) and
  //         local_apply_boundary_face_* (:1105-1339) ----------------------------
  const int *slots = a.slots + 8 * (int64_t)cell;
#pragma unroll 1
  for (int sl = 0; sl < 8; ++sl) {
    const int ref = member ? slots[sl] : -1;
    int nfo = 0, fo = 0, tsel = 0;  // own point count, own face number, own table
    if (ref >= 0) {
      const int f = ref >> 1, side = ref & 1;
      const int pk = a.fpack[f];
      const int fm = pk & 15, fp = (pk >> 4) & 15, sub = ((pk >> 8) & 15) - 1,
                orient = (pk >> 12) & 15, nf = (pk >> 16) & 15;
      const int cm = a.fcm[f], cp = a.fcp[f];
      const int pm = a.deg[cm], pp = a.deg[cp];
      const int Nm = pm + 1, Np = pp + 1;
      const DegTables<R> &tm = tab<R>(pm);
      const DegTables<R> &tp = tab<R>(pp);
      const int64_t zom = a.off[cm], zop = a.off[cp];
      const int64_t nm = (int64_t)Nm * Nm, np = (int64_t)Np * Np;
      const R n0 = (R)a.fnrm[2 * f], n1 = (R)a.fnrm[2 * f + 1];
      const R len = (R)a.flen[f];
      const int sdo = a.fsd[f];
      nfo = nf;
      fo = side ? fp : fm;
      tsel = side ? sub + 1 : 0;
      for (int k = t; k < nf; k += T) {
        const int kp = orient ? nf - 1 - k : k;
        R zm = 0, qm0 = 0, qm1 = 0, zp = 0, qp0 = 0, qp1 = 0;
        for (int i = 0; i < Nm; ++i) {
          const int d = face_dof(Nm, fm, i);
          const R l = tm.F[0][nf][k][i];
          zm += l * load_r<R>(a.rz, zom + d, a.r_is_float, zref);
          qm0 += l * load_r<R>(a.rq, 2 * zom + d, a.r_is_float, 0.0);
          qm1 += l * load_r<R>(a.rq, 2 * zom + nm + d, a.r_is_float, 0.0);
        }
        for (int i = 0; i < Np; ++i) {
          const int d = face_dof(Np, fp, i);
          const R l = tp.F[sub + 1][nf][kp][i];
          zp += l * load_r<R>(a.rz, zop + d, a.r_is_float, zref);
          qp0 += l * load_r<R>(a.rq, 2 * zop + d, a.r_is_float, 0.0);
          qp1 += l * load_r<R>(a.rq, 2 * zop + np + d, a.r_is_float, 0.0);
        }
        R zbm = MIX ? zbe_flat : R(0), zbp = zbm;
        if (MIX && a.sdfe) {
          zbm = (R)a.sdfe[sdo + 2 * k]; zbp = (R)a.sdfe[sdo + 2 * k + 1];
        } else if (!MIX && a.sdf) {
          zbm = (R)a.sdf[sdo + 2 * k]; zbp = (R)a.sdf[sdo + 2 * k + 1];
        }
        R F, Fa0, Fa1, Pm0, Pm1, Pp0, Pp1;
        face_flux<R>(g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, zbm, zbp, F, Fa0, Fa1, Pm0,
                     Pm1, Pp0, Pp1);
        const R jxw = tb.wF[nf][k] * len;
        const int ko = side ? kp : k;
        if (side == 0) {
          FV[ko] = -F * jxw;
          FV[FVS + ko] = (-Fa0 - Pm0) * jxw;
          FV[2 * FVS + ko] = (-Fa1 - Pm1) * jxw;
        } else {
          FV[ko] = F * jxw;
          FV[FVS + ko] = (Fa0 + Pp0) * jxw;
          FV[2 * FVS + ko] = (Fa1 + Pp1) * jxw;
        }
      }
    } else if (ref < -1) {  // boundary face
      const int b = -ref - 2;
      const int f = a.n_inner + b;
      const int fm = a.fpack[f] & 15;
      const R n0 = (R)a.fnrm[2 * f], n1 = (R)a.fnrm[2 * f + 1];
      const R len = (R)a.flen[f];
      const int bid = a.bbid[b];
      const int kind = (bid >= 0 && bid < OC_MAXBID) ? a.bc_kind[bid] : 0;
      if (kind == 0 && t == 0) atomicOr(a.err, ERR_UNKNOWN_BID);
      const int sdo = a.fsd[f];
      nfo = Q;
      fo = fm;
      tsel = -1;
      if (t < Q) {
        const int k = t;
        R zm = 0, qm0 = 0, qm1 = 0;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const int d = face_dof(N, fm, i);
          const R l = tb.BQ[k][i];
          zm += l * U[d];
          qm0 += l * U[NN + d];
          qm1 += l * U[2 * NN + d];
        }
        R zbm = MIX ? zbe_flat : R(0);
        double zb_abs = 0.;
        if (a.sdb) zb_abs = a.sdb[sdo + k];
        if (MIX && a.sdbe) zbm = (R)a.sdbe[sdo + k];
        else if (!MIX && a.sdb) zbm = (R)zb_abs;
        const double sx = tab<double>(P).xQ[k];
        const double e0 = fm == 0 ? 0. : fm == 1 ? 1. : sx;
        const double e1 = fm < 2 ? sx : fm == 2 ? 0. : 1.;
        const double px = geo[0] + geo[2] * e0 + geo[3] * e1;
        const double py = geo[1] + geo[4] * e0 + geo[5] * e1;
        const R un = qm0 * n0 + qm1 * n1;
        R zp = zm, qp0 = qm0, qp1 = qm1;
        bool at_outflow = false;
        if (kind == 1) {  // wall
          qp0 = qm0 - R(2.) * un * n0;
          qp1 = qm1 - R(2.) * un * n1;
        } else if (kind == 2) {  // supercritical inflow
          const double zd = bc_value(a, bid, px, py, 0);
          zp = (R)(zd - zref);
          const R hh = depth<R>(zp, zbm);
          qp0 = (R)bc_value(a, bid, px, py, 1) * hh;
          qp1 = (R)bc_value(a, bid, px, py, 2) * hh;
        } else if (kind == 3) {  // supercritical outflow
          at_outflow = true;
        } else if (kind == 4) {  // height inflow
          zp = (R)(bc_value(a, bid, px, py, 0) - zref);
        } else if (kind == 5) {  // discharge inflow
          const R qn = (R)bc_value(a, bid, px, py, 1);
          qp0 = qn * -n0;
          qp1 = qn * -n1;
        } else if (kind == 6) {  // absorbing outflow (Riemann invariants)
          const R zf = (R)(bc_value(a, bid, px, py, 0) - zref);
          const R hf = depth<R>(zf, zbm);
          const R qf0 = (R)bc_value(a, bid, px, py, 1) * hf;
          const R qf1 = (R)bc_value(a, bid, px, py, 2) * hf;
          R v0, v1, u0, u1;
          velocity<R>(zm, qm0, qm1, zbm, cu4, v0, v1);
          const R rp = v0 * n0 + v1 * n1 + R(2.) * sqrt(g * depth<R>(zm, zbm));
          velocity<R>(zf, qf0, qf1, zbm, cu4, u0, u1);
          const R rm = u0 * n0 + u1 * n1 - R(2.) * sqrt(g * depth<R>(zf, zbm));
          const R cb = R(0.25) * (rp - rm), hb = cb * cb / g, ub = R(0.5) * (rp + rm);
          zp = hb - zbm;
          const R hd = depth<R>(zp, zbm);
          qp0 = ub * hd * n0;
          qp1 = ub * hd * n1;
        }
        R F, Fa0, Fa1, Pm0, Pm1, Pp0, Pp1;
        face_flux<R>(g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, zbm, zbm, F, Fa0, Fa1, Pm0,
                     Pm1, Pp0, Pp1);
        Fa0 += Pm0;
        Fa1 += Pm1;
        if (at_outflow && un < R(-1e-12)) Fa0 = Fa1 = 0;
        const R jxw = tb.wQ[k] * len;
        FV[k] = -F * jxw;
        FV[FVS + k] = -Fa0 * jxw;
        FV[2 * FVS + k] = -Fa1 * jxw;
      }
    }
    __syncwarp();
    if (nfo > 0 && t < N) {  // integrate the own-side values against the own basis
      R cz = 0, c0 = 0, c1 = 0;
      for (int k = 0; k < nfo; ++k) {
        const R l = tsel < 0 ? tb.BQ[k][t] : tb.F[tsel][nfo][k][t];
        cz += l * FV[k];
        c0 += l * FV[FVS + k];
        c1 += l * FV[2 * FVS + k];
      }
      const int d = face_dof(N, fo, t);
      RES[d] += cz;
      RES[NN + d] += c0;
      RES[2 * NN + d] += c1;
    }
    __syncwarp();
  }

  // ---- apply(): dst = M^-1 L_h(src), exact Gauss p+1 inverse for all variables ----
  if (a.apply_mode) {
    if (member && t < N) {
#pragma unroll
      for (int e = 0; e < 3; ++e)
#pragma unroll
        for (int qx = 0; qx < N; ++qx) {
          R v = 0;
#pragma unroll
          for (int ix = 0; ix < N; ++ix) v += tb.Sinv[ix][qx] * RES[e * NN + t * N + ix];
          X[e * NT + t * T + qx] = v;
        }
    }
    __syncwarp();
    if (member && t < N) {
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        R bq[N];
#pragma unroll
        for (int qy = 0; qy < N; ++qy) {
          R v = 0;
#pragma unroll
          for (int iy = 0; iy < N; ++iy) v += tb.Sinv[iy][qy] * X[e * NT + iy * T + t];
          bq[qy] = v / (tb.wM[t] * tb.wM[qy] * det);
        }
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          R v = 0;
#pragma unroll
          for (int qy = 0; qy < N; ++qy) v += tb.Sinv[iy][qy] * bq[qy];
          X[(3 + e) * NT + iy * T + t] = v;
        }
      }
    }
    __syncwarp();
    if (valid && t < N) {
#pragma unroll
      for (int e = 0; e < 3; ++e)
#pragma unroll
        for (int ix = 0; ix < N; ++ix) {
          R v = 0;
#pragma unroll
          for (int qx = 0; qx < N; ++qx) v += tb.Sinv[ix][qx] * X[(3 + e) * NT + t * T + qx];
          if (e == 0) a.out_z[zo + t * N + ix] = (double)v;
          else a.out_q[qo + (e - 1) * NN + t * N + ix] = (double)v;
        }
    }
    return;
  }

  // ---- 4. zeta: pre-lambda + local_apply_cell_mass_height (OceanDG.h:1830-1849)
  //         and local_apply_inverse_mass_matrix_height (:1373-1507) ------------
  KT *kz_out = static_cast<KT *>(a.kz[s + 1]);
  if (valid && t < N) {
#pragma unroll
    for (int ix = 0; ix < N; ++ix) {
      const int d = t * N + ix;
      const R res = RES[d];
      kz_out[zo + d] = (KT)res;
      R bsum = (R)dy.f[0] * (s == 0 ? res : (R) static_cast<const KT *>(a.kz[1])[zo + d]);
      for (int j = 1; j < s + 1; ++j)
        bsum += (R)dy.f[j] * (j == s ? res : (R) static_cast<const KT *>(a.kz[j + 1])[zo + d]);
      BZ[d] = bsum;
    }
  }
  __syncwarp();
  double znext[N];  // FP64 result rows of thread t < N
  bool need_fp64 = !MIX;
  if (MIX) {
    // wet check of u^n at the Gauss-Lobatto points (FP32 estimate)
    bool wet = true;
    if (member && t < N) {
#pragma unroll
      for (int ix = 0; ix < N; ++ix) X[t * N + ix] = (R)(a.un_z[zo + t * N + ix] - zref);
    }
    __syncwarp();
    if (member && t < N) {
#pragma unroll
      for (int gx = 0; gx < G; ++gx) {
        R v = 0;
#pragma unroll
        for (int ix = 0; ix < N; ++ix) v += tb.BG[gx][ix] * X[t * N + ix];
        X[NT + t * T + gx] = v;
      }
    }
    __syncwarp();
    if (member && t < G) {
      const float *zb1e = a.sd1e ? a.sd1e + a.sdo1[cell] : nullptr;
#pragma unroll
      for (int gy = 0; gy < G; ++gy) {
        R v = 0;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) v += tb.BG[gy][iy] * X[NT + iy * T + t];
        const R zb = zb1e ? (R)zb1e[gy * G + t] : zbe_flat;
        wet = wet && (v + zb > (R)a.wet_threshold);
      }
    }
    // team AND through the FP64 reduction slots
    const double dryc = team_sum<T>(DRED, t, member, wet ? 0. : 1.);
    const bool team_wet = dryc == 0.;
    // closed form of max_iter sweeps on fully wet cells: delta = A_K b
    if (member && t < N) {
#pragma unroll
      for (int ap = 0; ap < N; ++ap) {
        R v = 0;
#pragma unroll
        for (int ix = 0; ix < N; ++ix) v += tb.W1[ap][ix] * BZ[t * N + ix];
        X[t * T + ap] = v;
      }
    }
    __syncwarp();
    if (member && t < N) {
      R c[N];
#pragma unroll
      for (int aa = 0; aa < N; ++aa) {
        R v = 0;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) v += tb.W1[aa][iy] * X[iy * T + t];
        c[aa] = v * tb.Gk[aa][t] / det;
      }
#pragma unroll
      for (int iy = 0; iy < N; ++iy) {
        R v = 0;
#pragma unroll
        for (int aa = 0; aa < N; ++aa) v += tb.W2[iy][aa] * c[aa];
        X[NT + iy * T + t] = v;
      }
    }
    __syncwarp();
    if (member && t < N) {
#pragma unroll
      for (int ix = 0; ix < N; ++ix) {
        R dl = 0;
#pragma unroll
        for (int ap = 0; ap < N; ++ap) dl += tb.W2[ix][ap] * X[NT + t * T + ap];
        znext[ix] = a.un_z[zo + t * N + ix] + (double)dl;
        X[2 * NT + t * N + ix] = X[t * N + ix] + dl;  // zeta' of the result (wet check)
      }
    }
    __syncwarp();
    // the closed form is the literal iteration only while every point stays wet:
    // check the result too, else redo the cell with the FP64 literal iteration
    bool wet2 = true;
    if (member && t < N) {
#pragma unroll
      for (int gx = 0; gx < G; ++gx) {
        R v = 0;
#pragma unroll
        for (int ix = 0; ix < N; ++ix) v += tb.BG[gx][ix] * X[2 * NT + t * N + ix];
        X[3 * NT + t * T + gx] = v;
      }
    }
    __syncwarp();
    if (member && t < G) {
      const float *zb1e = a.sd1e ? a.sd1e + a.sdo1[cell] : nullptr;
#pragma unroll
      for (int gy = 0; gy < G; ++gy) {
        R v = 0;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) v += tb.BG[gy][iy] * X[3 * NT + iy * T + t];
        const R zb = zb1e ? (R)zb1e[gy * G + t] : zbe_flat;
        wet2 = wet2 && (v + zb > (R)a.wet_threshold);
      }
    }
    const double dry2 = team_sum<T>(DRED, t, member, wet2 ? 0. : 1.);
    need_fp64 = !(team_wet && dry2 == 0.);
  }
  if (__any_sync(OC_FULL, valid && need_fp64)) {
    // literal FP64 iteration (all lanes; teams with work = valid && need_fp64)
    const bool work = valid && need_fp64;
    if (member && t < N) {
#pragma unroll
      for (int ix = 0; ix < N; ++ix) DZ[t * N + ix] = a.un_z[zo + t * N + ix];
    }
    __syncwarp();
    // rhs = b + int depth(zeta^n) phi over Gauss-Lobatto p+2 (OceanDG.h:828-855)
    double rhs[N], dummy[N];
    {
      const double det_d = geo[10];
      const double *zb1 = a.sd1 ? a.sd1 + a.sdo1[cell] : nullptr;
      const DegTables<double> &td = tab<double>(P);
      gl_eval_apply_integrate<P>(
          DZ, DX, t, work,
          [&](int qx, int qy, double v, double &o0, double &o1) {
            const double zb = zb1 ? zb1[qy * G + qx] : 0.;
            o0 = depth<double>(v, zb) * (td.wG[qx] * td.wG[qy] * det_d);
            o1 = 0;
          },
          rhs, dummy);
      if (work && t < N)
#pragma unroll
        for (int ix = 0; ix < N; ++ix) rhs[ix] = (double)BZ[t * N + ix] + rhs[ix];
    }
    zeta_iteration_fp64<P>(a, cell, DZ, DX, DRED, warp_norm, team, cpw, t, member, work, rhs);
    if (work && t < N)
#pragma unroll
      for (int ix = 0; ix < N; ++ix) znext[ix] = DZ[t * N + ix];
    __syncwarp();
  }
  if (valid && t < N) {
#pragma unroll
    for (int ix = 0; ix < N; ++ix) {
      const int d = t * N + ix;
      if (a.out_z) a.out_z[zo + d] = znext[ix];
      if (MIX && a.out_rz) a.out_rz[zo + d] = (float)(znext[ix] - zref);
    }
  }

  // ---- 5. discharge: local_apply_inverse_mass_matrix_discharge (OceanDG.h:1532-1571)
  //         + post-lambda (:1878-1909); ARK: :2052-2116 ----------------------------
  // b = sum of weighted residual registers (ARK), or the ERK residual itself
  if (split) {
    // rhs of the modified mass: b = sum_j (f_j kex_j + ft_j kim_j)
    if (member && t < N) {
#pragma unroll
      for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int ix = 0; ix < N; ++ix) {
          const int d = t * N + ix;
          const int64_t gidx = qo + e * NN + d;
          const R kex = RES[(1 + e) * NN + d], kim = RST[e * NN + d];
          if (valid) {
            static_cast<KT *>(a.kq[2 * s + 1])[gidx] = (KT)kex;
            static_cast<KT *>(a.kq[2 * s + 2])[gidx] = (KT)kim;
          }
          R bsum = s == 0 ? (R)dy.f[0] * kex + (R)dy.ft[0] * kim
                          : (R)dy.f[0] * (R) static_cast<const KT *>(a.kq[1])[gidx] +
                                (R)dy.ft[0] * (R) static_cast<const KT *>(a.kq[2])[gidx];
          for (int j = 1; j < s + 1; ++j) {
            const R ke = j == s ? kex : (R) static_cast<const KT *>(a.kq[2 * j + 1])[gidx];
            const R ki = j == s ? kim : (R) static_cast<const KT *>(a.kq[2 * j + 2])[gidx];
            bsum += (R)dy.f[j] * ke + (R)dy.ft[j] * ki;
          }
          RES[(1 + e) * NN + d] = bsum;
        }
    }
    __syncwarp();
  } else if (a.ark) {  // ARK last stage: b = f0 kex0 + sum_j (f_j kex_j + f_{j-1} kim_{j-1})
    if (member && t < N) {
#pragma unroll
      for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int ix = 0; ix < N; ++ix) {
          const int d = t * N + ix;
          const int64_t gidx = qo + e * NN + d;
          const R kex = RES[(1 + e) * NN + d];
          if (valid) static_cast<KT *>(a.kq[2 * s + 1])[gidx] = (KT)kex;
          R bsum = (R)dy.f[0] * (s == 0 ? kex : (R) static_cast<const KT *>(a.kq[1])[gidx]);
          for (int j = 1; j < s + 1; ++j) {
            const R ke = j == s ? kex : (R) static_cast<const KT *>(a.kq[2 * j + 1])[gidx];
            const R ki = (R) static_cast<const KT *>(a.kq[2 * j])[gidx];
            bsum += (R)dy.f[j] * ke + (R)dy.f[j - 1] * ki;
          }
          RES[(1 + e) * NN + d] = bsum;
        }
    }
    __syncwarp();
  }
  // coefficient of the diagonal (JxW)^-1 at Gauss p+1; ARK internal: modified mass
  // (OceanDG.h:1573-1645): (JxW (1 + fm J_fric(r)))^-1
  R coef[N];  // column qx = t: coef[qy]
  R corr[2][N];  // mixed ARK: S^T diag(JxW fm J) S q^n, rows of t < N (y-integrated per column)
#pragma unroll
  for (int i = 0; i < N; ++i) {
    coef[i] = 0;
    corr[0][i] = corr[1][i] = 0;
  }
  if (member && t < N) {
#pragma unroll
    for (int qy = 0; qy < N; ++qy) coef[qy] = R(1) / (tb.wM[t] * tb.wM[qy] * det);
  }
  if (split) {
    // stage input and u^n at Gauss p+1: x-pass on rows
    if (member && t < N) {
#pragma unroll
      for (int qx = 0; qx < N; ++qx) {
        R vz = 0, v0 = 0, v1 = 0, n0 = 0, n1 = 0;
#pragma unroll
        for (int ix = 0; ix < N; ++ix) {
          const R bm = tb.BM[qx][ix];
          vz += bm * U[t * N + ix];
          v0 += bm * U[NN + t * N + ix];
          v1 += bm * U[2 * NN + t * N + ix];
          n0 += bm * (R)a.un_q[qo + t * N + ix];
          n1 += bm * (R)a.un_q[qo + NN + t * N + ix];
        }
        X[0 * NT + t * T + qx] = vz;
        X[1 * NT + t * T + qx] = v0;
        X[2 * NT + t * T + qx] = v1;
        X[3 * NT + t * T + qx] = n0;
        X[4 * NT + t * T + qx] = n1;
      }
    }
    __syncwarp();
    R m0[N], m1[N];  // MIX: y-integrated correction; FP64: y-integrated M q^n
#pragma unroll
    for (int i = 0; i < N; ++i) m0[i] = m1[i] = 0;
    if (member && t < N) {
      const double *sd2 = a.sd2 ? a.sd2 + a.sdo2[cell] : nullptr;
      const float *sd2e = a.sd2e ? a.sd2e + a.sdo2[cell] : nullptr;
#pragma unroll
      for (int qy = 0; qy < N; ++qy) {
        R vz = 0, v0 = 0, v1 = 0, n0 = 0, n1 = 0;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          const R bm = tb.BM[qy][iy];
          vz += bm * X[0 * NT + iy * T + t];
          v0 += bm * X[1 * NT + iy * T + t];
          v1 += bm * X[2 * NT + iy * T + t];
          n0 += bm * X[3 * NT + iy * T + t];
          n1 += bm * X[4 * NT + iy * T + t];
        }
        const int k = qy * N + t;
        R zb = MIX ? zbe_flat : R(0), cf = 0;
        if (MIX && sd2e) { zb = (R)sd2e[2 * k]; cf = (R)sd2e[2 * k + 1]; }
        else if (!MIX && sd2) { zb = (R)sd2[2 * k]; cf = (R)sd2[2 * k + 1]; }
        R u0, u1;
        velocity<R>(vz, v0, v1, zb, cu4, u0, u1);
        const R jf = friction_jac<R>(a.friction, g, u0, u1, cf, depth<R>(vz, zb));
        const R jxw = tb.wM[t] * tb.wM[qy] * det;
        coef[qy] = R(1) / jxw;
        coef[qy] *= R(1) / (R(1) + (R)dy.fm * jf);
        const R wq = MIX ? jxw * (R)dy.fm * jf : jxw;  // MIX: correction; FP64: mass of q^n
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          m0[iy] += tb.BM[qy][iy] * (wq * n0);
          m1[iy] += tb.BM[qy][iy] * (wq * n1);
        }
      }
    }
    __syncwarp();
    if (member && t < N) {
#pragma unroll
      for (int iy = 0; iy < N; ++iy) {
        X[0 * NT + iy * T + t] = m0[iy];
        X[1 * NT + iy * T + t] = m1[iy];
      }
    }
    __syncwarp();
    if (member && t < N) {  // x-integration, then add/subtract into the rhs rows
#pragma unroll
      for (int ix = 0; ix < N; ++ix) {
        R c0 = 0, c1 = 0;
#pragma unroll
        for (int qx = 0; qx < N; ++qx) {
          c0 += tb.BM[qx][ix] * X[0 * NT + t * T + qx];
          c1 += tb.BM[qx][ix] * X[1 * NT + t * T + qx];
        }
        if (MIX) {
          RES[NN + t * N + ix] -= c0;
          RES[2 * NN + t * N + ix] -= c1;
        } else {
          RES[NN + t * N + ix] += c0;
          RES[2 * NN + t * N + ix] += c1;
        }
      }
    }
    __syncwarp();
  }
  // S^-1 diag(coef) S^-T applied to the two discharge components of RES
  if (member && t < N) {  // x-pass: A[iy][qx] = sum_ix Sinv[ix][qx] in[iy][ix]
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
      for (int qx = 0; qx < N; ++qx) {
        R v = 0;
#pragma unroll
        for (int ix = 0; ix < N; ++ix) v += tb.Sinv[ix][qx] * RES[(1 + e) * NN + t * N + ix];
        X[e * NT + t * T + qx] = v;
      }
  }
  __syncwarp();
  if (member && t < N) {  // y on column qx = t: scale, back-transform in y
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      R bq[N];
#pragma unroll
      for (int qy = 0; qy < N; ++qy) {
        R v = 0;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) v += tb.Sinv[iy][qy] * X[e * NT + iy * T + t];
        bq[qy] = v * coef[qy];
      }
#pragma unroll
      for (int iy = 0; iy < N; ++iy) {
        R v = 0;
#pragma unroll
        for (int qy = 0; qy < N; ++qy) v += tb.Sinv[iy][qy] * bq[qy];
        X[(2 + e) * NT + iy * T + t] = v;
      }
    }
  }
  __syncwarp();
  if (valid && t < N) {  // x back-transform, registers, RK update in FP64
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
      for (int ix = 0; ix < N; ++ix) {
        R v = 0;
#pragma unroll
        for (int qx = 0; qx < N; ++qx) v += tb.Sinv[ix][qx] * X[(2 + e) * NT + t * T + qx];
        const int64_t gidx = qo + e * NN + t * N + ix;
        double nxt;
        if (!a.ark) {
          // ERK: k_q[s+1] = M^-1 L_h q; next = q^n + sum_j f_j k_q[j+1]
          if (!a.last || a.write_kq_last) static_cast<KT *>(a.kq[s + 1])[gidx] = (KT)v;
          const double kc = (double)(KT)v;
          double acc = a.un_q[gidx] + dy.f[0] * (s == 0 ? kc : (double)static_cast<const KT *>(a.kq[1])[gidx]);
          for (int j = 1; j < s + 1; ++j)
            acc += dy.f[j] * (j == s ? kc : (double)static_cast<const KT *>(a.kq[j + 1])[gidx]);
          nxt = acc;
          if (a.out_q) a.out_q[gidx] = nxt;
        } else if (!a.last) {
          nxt = MIX ? a.un_q[gidx] + (double)v : (double)v;
          if (a.out_q) a.out_q[gidx] = nxt;
        } else {
          if (a.aux_q) a.aux_q[gidx] = (double)v;
          nxt = a.un_q[gidx] + (double)v;
          a.out_q[gidx] = nxt;
        }
        if (MIX && a.out_rq) a.out_rq[gidx] = (float)nxt;
      }
  }
}

}  // namespace oc
