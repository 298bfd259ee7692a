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
//   3. integrates the face contributions of its four faces (conforming, either
//      side of a hanging face, periodic, boundary): the FP64 form integrates
//      the values the stage's face pass (oc_face.cu) evaluated once per face
//      and left per side; the mixed form evaluates each face point itself
//      from the neighbour's trace, the flux of an inner face once per side,
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

// ---------------------------------------------------------------------------
// Bounds-checked build (OC_BOUNDS_CHECK).  Every index a kernel reads from a
// mesh table -- cell ids, degrees, DoF offsets, face records, static-data and
// face-pass offsets -- is range-checked where it is loaded.  An index outside
// its range sets ERR_BOUNDS, records the site and the index in err[1..3] (the
// first failure only) and is replaced by 0, so that the accesses it feeds stay
// in bounds; the host then reports OC_ERR_BOUNDS with the site and the index.
// Without the macro the checks compile to nothing.
// ---------------------------------------------------------------------------
#ifdef OC_BOUNDS_CHECK
static __device__ __noinline__ void bounds_fail(int *err, int site, int64_t i) {
  atomicOr(err, ERR_BOUNDS);
  if (atomicCAS(err + 1, 0, site) == 0) {
    err[2] = (int)(uint32_t)(uint64_t)i;
    err[3] = (int)(uint32_t)((uint64_t)i >> 32);
  }
}
#endif
// index i, valid in [0, n); an offset followed by `extent` elements of an
// array of `size` elements is checked with n = size - extent + 1
__device__ __forceinline__ int64_t checked(int *err, int64_t i, int64_t n, int site) {
#ifdef OC_BOUNDS_CHECK
  if (i < 0 || i >= n) {
    bounds_fail(err, site, i);
    return 0;
  }
#else
  (void)err; (void)n; (void)site;
#endif
  return i;
}
// degree p of a cell, valid in [1, OC_MAXDEG] (replaced by 1)
__device__ __forceinline__ int checked_degree(int *err, int p) {
  return 1 + (int)checked(err, p - 1, OC_MAXDEG, BS_DEGREE);
}

// offset of a cell's block of `extent` static-data values (sd0: 5 Q^2, sd1:
// (p+2)^2, sd2: 2 (p+1)^2) in an array of n elements
__device__ __forceinline__ int64_t cell_data(int *err, const int *sdo, int cell, int64_t n,
                                             int extent) {
  return checked(err, __ldg(sdo + cell), n - extent + 1, BS_CELL_DATA);
}
// boundary kinds (values of OC_BC_* in oceano_gpu.h)
enum { OC_BC_WALL_ = 1, OC_BC_SUPIN_ = 2, OC_BC_SUPOUT_ = 3, OC_BC_HEIGHT_ = 4,
       OC_BC_DISCHARGE_ = 5, OC_BC_ABSORB_ = 6 };
#define OC_FULL 0xffffffffu

// math in the compute type, with the single-precision functions named explicitly
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_abs(float x) { return fabsf(x); }
__device__ __forceinline__ double m_abs(double x) { return fabs(x); }
__device__ __forceinline__ float m_exp(float x) { return expf(x); }
__device__ __forceinline__ double m_exp(double x) { return exp(x); }
__device__ __forceinline__ float m_log(float x) { return logf(x); }
__device__ __forceinline__ double m_log(double x) { return log(x); }
__device__ __forceinline__ float m_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double m_fma(double a, double b, double c) { return fma(a, b, c); }
// two independent fused multiply-adds, x += a0 b0 and y += a1 b1: one packed
// FFMA2 instruction in FP32 (sm_100 and later), two DFMAs in FP64; each lane's
// result is the scalar fma's
__device__ __forceinline__ void fma2(float &x, float &y, float a0, float b0, float a1, float b1) {
  const float2 r = __ffma2_rn(make_float2(a0, a1), make_float2(b0, b1), make_float2(x, y));
  x = r.x;
  y = r.y;
}
__device__ __forceinline__ void fma2(double &x, double &y, double a0, double b0, double a1,
                                     double b1) {
  x = fma(a0, b0, x);
  y = fma(a1, b1, y);
}

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
  const R inv = R(1.4142135623730951) * h / m_sqrt(h4 + mx<R>(h4, cu4));
  v0 = q0 * inv;
  v1 = q1 * inv;
}

// BottomFriction.h:87-137 (linear), :183-213 (Manning)
template <typename R>
__device__ __forceinline__ void friction(int model, R g, R v0, R v1, R cf, R h, R &s0, R &s1) {
  if (model == 1) {
    s0 = cf * h * v0; s1 = cf * h * v1;
  } else if (model == 2) {
    const R inv_depth = R(1.) / (m_exp(m_log(h) * R(0.33333333333)));
    const R hcf = g * cf * cf * inv_depth * m_sqrt(v0 * v0 + v1 * v1);
    s0 = hcf * v0; s1 = hcf * v1;
  } else {
    s0 = 0; s1 = 0;
  }
}

template <typename R>
__device__ __forceinline__ R friction_jac(int model, R g, R v0, R v1, R cf, R h) {
  if (model == 1) return cf;
  if (model == 2) {
    const R inv_depth = R(1.) / (m_exp(m_log(h) * R(1.33333333333)));
    return g * cf * cf * inv_depth * m_sqrt(v0 * v0 + v1 * v1);
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
  const R lm = m_abs(vm0 * n0 + vm1 * n1) + m_sqrt(g * depth<R>(zm, zbm));
  const R lp = m_abs(vp0 * n0 + vp1 * n1) + m_sqrt(g * depth<R>(zp, zbp));
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

// ---------------------------------------------------------------------------
// Mixed form: discharge carried as a deviation from a constant reference state.
// The FP32 state is (zeta - zeta_ref, q - q_r); depth = h_r + dh with
// dh = (zeta - zeta_ref) + (zbe - h_r) (zbe = zb + zeta_ref).  The fluxes are
// evaluated minus their value at the reference state (q_r, u_r): a constant
// flux has no weak divergence (cell Gauss and face Gauss-Lobatto rules are
// exact for it), so this changes nothing in exact arithmetic, but the FP32
// rounding now scales with |q - q_r| instead of |q|.
// ---------------------------------------------------------------------------
// (RefStateF, oc_layout.h: set on the host, read from the kernel parameter bank)
template <typename R>
using RefState = RefStateF;

// du = u - u_r for q = q_r + dq at depth h = h_r + dh (ShallowWater.h:322-336,
// desingularised below Threshold_for_wetdry); also returns h and 1/h on wet
// points (wet = h^4 >= cu^4, where the velocity is q / h; rh = 0 otherwise).
template <typename R>
__device__ __forceinline__ void vel_dev(const RefState<R> &rf, R cu4, R dh, R dq0, R dq1, R &du0,
                                        R &du1, R &h, R &rh) {
  h = mx<R>(rf.hr + dh, R(1e-12));
  const R h2 = h * h, h4 = h2 * h2;
  if (h4 >= cu4) {  // sqrt(2) h / sqrt(h^4 + max(h^4, cu^4)) = 1 / h
    rh = R(1) / h;
    du0 = (dq0 + (rf.rr0 - rf.ur0 * dh)) * rh;
    du1 = (dq1 + (rf.rr1 - rf.ur1 * dh)) * rh;
  } else {
    rh = R(0);
    const R s = R(1.4142135623730951) * h / m_sqrt(h4 + cu4);
    du0 = s * (rf.qr0 + dq0) - rf.ur0;
    du1 = s * (rf.qr1 + dq1) - rf.ur1;
  }
}
template <typename R>
__device__ __forceinline__ void vel_dev(const RefState<R> &rf, R cu4, R dh, R dq0, R dq1, R &du0,
                                        R &du1, R &h) {
  R rh;
  vel_dev<R>(rf, cu4, dh, dq0, dq1, du0, du1, h, rh);
}

// face_flux on deviations: F - q_r.n, Fa - q_r (u_r.n), P unchanged.  zm, zp are
// zeta - zeta_ref, dq* = q - q_r, zbm, zbp = zb + zeta_ref.  flat: zbm == zbp
// (no bathymetry data), where the hydrostatic reconstruction leaves the states
// unchanged (hu = q, velocity recomputed from hu = velocity).
template <typename R>
__device__ __forceinline__ void face_flux_dev(const RefState<R> &rf, R g, R cu4, R zm, R dqm0,
                                              R dqm1, R zp, R dqp0, R dqp1, R n0, R n1, R zbm,
                                              R zbp, R &F, R &Fa0, R &Fa1, R &Pm0, R &Pm1,
                                              R &Pp0, R &Pp1, bool flat = false) {
  const R dzbm = zbm - rf.hr, dzbp = zbp - rf.hr;
  R dvm0, dvm1, hmo, rhm, dvp0, dvp1, hpo, rhp;  // own-bathymetry velocities and depths
  vel_dev<R>(rf, cu4, zm + dzbm, dqm0, dqm1, dvm0, dvm1, hmo, rhm);
  vel_dev<R>(rf, cu4, zp + dzbp, dqp0, dqp1, dvp0, dvp1, hpo, rhp);
  const R urn = rf.ur0 * n0 + rf.ur1 * n1;
  if (flat) {
    const R dunm = dvm0 * n0 + dvm1 * n1, dunp = dvp0 * n0 + dvp1 * n1;
    const R lambda = mx<R>(m_abs(urn + dunp) + m_sqrt(g * hpo), m_abs(urn + dunm) + m_sqrt(g * hmo));
    const R cm = mx<R>(zm, -zbm), cp = mx<R>(zp, -zbm);
    F = R(0.5) * ((dqm0 * n0 + dqm1 * n1) + (dqp0 * n0 + dqp1 * n1)) + R(0.5) * lambda * (cm - cp);
    const R Xm0 = rf.qr0 * dunm + dqm0 * (urn + dunm), Xm1 = rf.qr1 * dunm + dqm1 * (urn + dunm);
    const R Xp0 = rf.qr0 * dunp + dqp0 * (urn + dunp), Xp1 = rf.qr1 * dunp + dqp1 * (urn + dunp);
    Fa0 = R(0.5) * (Xm0 + Xp0) + R(0.5) * lambda * (dqm0 - dqp0);
    Fa1 = R(0.5) * (Xm1 + Xp1) + R(0.5) * lambda * (dqm1 - dqp1);
    const R sg = g * R(0.25) * (hpo + hmo);
    const R sm = sg * (cp - cm), sp = sg * (cm - cp);
    Pm0 = sm * n0; Pm1 = sm * n1;
    Pp0 = sp * n0; Pp1 = sp * n1;
    return;
  }
  const R vm0 = rf.ur0 + dvm0, vm1 = rf.ur1 + dvm1, vp0 = rf.ur0 + dvp0, vp1 = rf.ur1 + dvp1;
  const R lm = m_abs(vm0 * n0 + vm1 * n1) + m_sqrt(g * hmo);
  const R lp = m_abs(vp0 * n0 + vp1 * n1) + m_sqrt(g * hpo);
  const R lambda = mx<R>(lp, lm);
  const R zbs = mn<R>(zbm, zbp), dzbs = zbs - rf.hr;
  const R dhm = zm + dzbs, dhp = zp + dzbs;
  const R hm = mx<R>(rf.hr + dhm, R(1e-12)), hp = mx<R>(rf.hr + dhp, R(1e-12));
  // reconstructed discharge deviations hu - q_r, hu = h_s u (hydrostatic reconstruction)
  R dhum0, dhum1, dhup0, dhup1;
  const R cu = R(1e-12);
  if (rhm > R(0) && hm > cu) {  // wet: u = q / h_own, hu = (h_s / h_own) q
    const R r = hm * rhm, c = (dzbs - dzbm) * rhm;
    dhum0 = r * dqm0 + rf.qr0 * c;
    dhum1 = r * dqm1 + rf.qr1 * c;
  } else {
    dhum0 = hm * vm0 - rf.qr0;
    dhum1 = hm * vm1 - rf.qr1;
  }
  if (rhp > R(0) && hp > cu) {
    const R r = hp * rhp, c = (dzbs - dzbp) * rhp;
    dhup0 = r * dqp0 + rf.qr0 * c;
    dhup1 = r * dqp1 + rf.qr1 * c;
  } else {
    dhup0 = hp * vp0 - rf.qr0;
    dhup1 = hp * vp1 - rf.qr1;
  }
  const R cm = mx<R>(zm, -zbs), cp = mx<R>(zp, -zbs);
  F = R(0.5) * ((dhum0 * n0 + dhum1 * n1) + (dhup0 * n0 + dhup1 * n1)) + R(0.5) * lambda * (cm - cp);
  // advective flux: velocity recomputed from hu at the reconstructed depth
  R dwm0, dwm1, dwp0, dwp1, hh;
  vel_dev<R>(rf, cu4, dhm, dhum0, dhum1, dwm0, dwm1, hh);
  vel_dev<R>(rf, cu4, dhp, dhup0, dhup1, dwp0, dwp1, hh);
  const R dunm = dwm0 * n0 + dwm1 * n1, dunp = dwp0 * n0 + dwp1 * n1;
  // hu (w.n) - q_r (u_r.n) = q_r (dw.n) + d(hu) ((u_r + dw).n)
  const R Xm0 = rf.qr0 * dunm + dhum0 * (urn + dunm), Xm1 = rf.qr1 * dunm + dhum1 * (urn + dunm);
  const R Xp0 = rf.qr0 * dunp + dhup0 * (urn + dunp), Xp1 = rf.qr1 * dunp + dhup1 * (urn + dunp);
  Fa0 = R(0.5) * (Xm0 + Xp0) + R(0.5) * lambda * (dhum0 - dhup0);
  Fa1 = R(0.5) * (Xm1 + Xp1) + R(0.5) * lambda * (dhum1 - dhup1);
  const R sg = g * R(0.25) * (hp + hm);
  const R sm = sg * (cp - cm), sp = sg * (cm - cp);
  Pm0 = sm * n0; Pm1 = sm * n1;
  Pp0 = sp * n0; Pp1 = sp * n1;
}

// face_flux_dev with bathymetry (zb- != zb+): the well-balanced differences of
// the hydrostatic reconstruction (LaxFriedrichsModified.h:161-192) and of the
// pressure jump (NumericalFluxBase.h:103-126) in FP64 -- zb* = min(zb-, zb+),
// the reconstructed depths h* = zeta + zb*, the bathymetry differences
// zb* - zb of the reconstructed discharge, max(zeta, -zb*) of both sides and
// the depth sum of the pressure term -- from the FP64 bathymetry (absolute zb)
// and the FP32 free-surface deviations zm, zp (zeta - zeta_ref).  Velocities,
// wave speeds, fluxes and the remaining products stay FP32.  (GB300 runs FP64
// at 1/64 of the FP32 rate: no FP64 division or product is needed here; on wet
// points h*/h = 1 + (zb* - zb)/h.)  zbme, zbpe: FP32 zb + zeta_ref.
template <typename R>
__device__ __forceinline__ void face_flux_dev_wb(const RefState<R> &rf, R g, R cu4, double zref,
                                                 R zm, R dqm0, R dqm1, R zp, R dqp0, R dqp1,
                                                 R n0, R n1, double zbm, double zbp, R zbme,
                                                 R zbpe, R &F, R &Fa0, R &Fa1, R &Pm0, R &Pm1,
                                                 R &Pp0, R &Pp1) {
  // own-bathymetry depths for the velocities and wave speeds (FP32)
  R dvm0, dvm1, hmo, rhm, dvp0, dvp1, hpo, rhp;
  vel_dev<R>(rf, cu4, zm + (zbme - rf.hr), dqm0, dqm1, dvm0, dvm1, hmo, rhm);
  vel_dev<R>(rf, cu4, zp + (zbpe - rf.hr), dqp0, dqp1, dvp0, dvp1, hpo, rhp);
  const R vm0 = rf.ur0 + dvm0, vm1 = rf.ur1 + dvm1, vp0 = rf.ur0 + dvp0, vp1 = rf.ur1 + dvp1;
  const R lm = m_abs(vm0 * n0 + vm1 * n1) + m_sqrt(g * hmo);
  const R lp = m_abs(vp0 * n0 + vp1 * n1) + m_sqrt(g * hpo);
  const R lambda = mx<R>(lp, lm);
  const R urn = rf.ur0 * n0 + rf.ur1 * n1;
  // FP64 differences
  const double zma = (double)zm + zref, zpa = (double)zp + zref;  // absolute free surface
  const double zbs = fmin(zbm, zbp);
  const double hm64 = fmax(zma + zbs, 1e-12), hp64 = fmax(zpa + zbs, 1e-12);
  const R dbm = (R)(zbs - zbm), dbp = (R)(zbs - zbp);
  const R dc = (R)(fmax(zma, -zbs) - fmax(zpa, -zbs));  // c- - c+
  const R hsum = (R)(hp64 + hm64);
  const R hm = (R)hm64, hp = (R)hp64;
  // reconstructed discharge deviations hu - q_r, hu = h* u
  R dhum0, dhum1, dhup0, dhup1;
  if (rhm > R(0) && hm64 > 1e-12) {  // wet: hu = (1 + (zb* - zb)/h) q
    const R c = dbm * rhm, r = R(1) + c;
    dhum0 = r * dqm0 + rf.qr0 * c;
    dhum1 = r * dqm1 + rf.qr1 * c;
  } else {
    dhum0 = hm * vm0 - rf.qr0;
    dhum1 = hm * vm1 - rf.qr1;
  }
  if (rhp > R(0) && hp64 > 1e-12) {
    const R c = dbp * rhp, r = R(1) + c;
    dhup0 = r * dqp0 + rf.qr0 * c;
    dhup1 = r * dqp1 + rf.qr1 * c;
  } else {
    dhup0 = hp * vp0 - rf.qr0;
    dhup1 = hp * vp1 - rf.qr1;
  }
  F = R(0.5) * ((dhum0 * n0 + dhum1 * n1) + (dhup0 * n0 + dhup1 * n1)) + R(0.5) * lambda * dc;
  // advective flux: velocity recomputed from hu at the reconstructed depth
  R dwm0, dwm1, dwp0, dwp1, hh;
  vel_dev<R>(rf, cu4, (R)(hm64 - (double)rf.hr), dhum0, dhum1, dwm0, dwm1, hh);
  vel_dev<R>(rf, cu4, (R)(hp64 - (double)rf.hr), dhup0, dhup1, dwp0, dwp1, hh);
  const R dunm = dwm0 * n0 + dwm1 * n1, dunp = dwp0 * n0 + dwp1 * n1;
  const R Xm0 = rf.qr0 * dunm + dhum0 * (urn + dunm), Xm1 = rf.qr1 * dunm + dhum1 * (urn + dunm);
  const R Xp0 = rf.qr0 * dunp + dhup0 * (urn + dunp), Xp1 = rf.qr1 * dunp + dhup1 * (urn + dunp);
  Fa0 = R(0.5) * (Xm0 + Xp0) + R(0.5) * lambda * (dhum0 - dhup0);
  Fa1 = R(0.5) * (Xm1 + Xp1) + R(0.5) * lambda * (dhum1 - dhup1);
  const R sm = -(g * R(0.25)) * hsum * dc;  // g/4 (h+ + h-) (c+ - c-), minus-side call
  Pm0 = sm * n0; Pm1 = sm * n1;
  Pp0 = -sm * n0; Pp1 = -sm * n1;
}

// face_flux_dev_wb kept out of line where it is called inside the fused face loop
// of the mixed stage kernel (bathymetry only): the common flat-bathymetry loop
// keeps its small instruction footprint
template <typename R>
__device__ __noinline__ void face_flux_dev_wb_call(const RefState<R> &rf, R g, R cu4, double zref,
                                                   R zm, R dqm0, R dqm1, R zp, R dqp0, R dqp1,
                                                   R n0, R n1, double zbm, double zbp, R zbme,
                                                   R zbpe, R &F, R &Fa0, R &Fa1, R &Pm0,
                                                   R &Pm1, R &Pp0, R &Pp1) {
  face_flux_dev_wb<R>(rf, g, cu4, zref, zm, dqm0, dqm1, zp, dqp0, dqp1, n0, n1, zbm, zbp, zbme,
                      zbpe, F, Fa0, Fa1, Pm0, Pm1, Pp0, Pp1);
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

// stage-input load with the input precision fixed at compile time (a runtime
// switch would let the compiler evaluate both branches).  Read-only loads
// (ld.global.nc): the stage inputs are not written during the launch, and the
// compiler may then issue the loads of several elements ahead of the shared-memory
// stores of the earlier ones (one memory round trip instead of one per element).
template <typename RIN, typename R>
__device__ __forceinline__ R load_in(const void *p, int64_t i, double ref) {
  if constexpr (sizeof(RIN) == 4) {
    return (R)__ldg(static_cast<const float *>(p) + i);
  } else {
    return (R)(__ldg(static_cast<const double *>(p) + i) - ref);
  }
}

// asynchronous global -> shared copy of one element (cp.async, no register
// staging), and the wait of the calling thread for all of its copies
template <typename T>
__device__ __forceinline__ void cp_async(T *smem, const T *gmem) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// read-only load of a stage register (FP32 or FP64)
template <typename KT>
__device__ __forceinline__ KT ldro(const void *p, int64_t i) {
  return __ldg(static_cast<const KT *>(p) + i);
}

// stride of the per-variable face point values (>= OC_MAXF and OC_MAXQ)
constexpr int FVS = 8;

// QR: the cell Gauss rule (the reference's n_points_1d, main.cc:216 /
// OceanDG.h:448): 0 floor(1.5 P) + 1 points per direction, 1 P + 1 points
template <int P, int QR = 0>
struct Dims {
  static constexpr int N = P + 1, Q = QR ? P + 1 : (3 * P) / 2 + 1, G = P + 2;
  static constexpr int T = Q > G ? Q : G;
  static constexpr int NN = N * N, NT = N * T;
  static constexpr int CPW = 32 / T;
  // scratch tiles of the sum factorisation, the zeta solve and the discharge
  // inverse.  Between the cell integrals and the zeta solve they hold the face
  // data: in the mixed form (FP32 compute type) the neighbour traces of the 8
  // face slots ([slot][var][OC_MAXN]) and one face's point values (3 FVS); in
  // the FP64 form the face pass's point values of the 8 slots ([slot][var][FVS]).
  // A smaller team region leaves more of the SM's shared memory to the L1 cache.
  template <typename R>
  static constexpr int xs() {
    constexpr int f = sizeof(R) == 4 ? 8 * 3 * OC_MAXN + 3 * FVS : 8 * 3 * FVS;
    return 6 * NT > f ? 6 * NT : f;
  }
  // per-cell shared memory: compute-type region and FP64 region (elements)
  template <typename R>
  static constexpr int szr() { return 10 * NN + xs<R>(); }  // U 3, RES 3, RST 2, BZ 1, ZN 1; X
  static constexpr int SZD = NN + 3 * NT + T + 2;
  // Team strides: padded so that the 32/T teams of a warp start on different
  // shared-memory banks (stride mod 32 chosen per degree and element size to
  // keep row, column and node-row accesses at most 2-way conflicted).  FP32,
  // counted over the sum-factorisation rows and columns, the face traces read by
  // a whole team and the face values: degree 4 (4 teams of 7 lanes) is free of
  // conflicts with a stride of 24 mod 32 (with 16 mod 32 every access was 2-way),
  // degree 1 (10 teams of 3) has at most 2-way conflicts with 29 mod 32.
  static constexpr int pad_f = P == 1 ? 5 : P == 2 ? 29 : P == 3 ? 3 : 8;
  static constexpr int pad_d = P == 1 ? 5 : P == 2 ? 2 : P == 3 ? 3 : 4;
  template <typename R>
  static constexpr int bytes_r() {
    return (((szr<R>() + 7) / 8) * 8 + (sizeof(R) == 4 ? pad_f : pad_d)) * (int)sizeof(R);
  }
  static constexpr int bytes_d() { return (((SZD + 31) / 32) * 32 + pad_d) * 8; }
  static_assert(SZD <= OC_DSTRIDE, "FP64 zeta work area exceeds its global stride");
  // the FP64 team region lives in shared memory in the FP64 form only; the mixed
  // form (FP32 compute type) keeps it in the per-cell global work area
  template <typename R>
  static constexpr int bytes_d_smem() { return sizeof(R) == 4 ? 0 : bytes_d(); }
  // per warp: CPW compute regions, CPW FP64 regions, CPW batch-norm slots, int area
  template <typename R>
  static constexpr int d_offset() { return ((CPW * bytes_r<R>() + 15) / 16) * 16; }
  template <typename R>
  static constexpr int norm_offset() { return d_offset<R>() + CPW * bytes_d_smem<R>(); }
  template <typename R>
  static constexpr int int_offset() { return norm_offset<R>() + CPW * 8; }
  static constexpr int INTS = 2 + 16 + 8 + 1 + 8;  // cell, offset, 8 slot records, 8 sdo, flag,
                                                   // 8 face-pass offsets
  template <typename R>
  static constexpr int warp_bytes() { return ((int_offset<R>() + CPW * INTS * 4 + 15) / 16) * 16; }
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
template <int P, int QR, class Fn>
__device__ __forceinline__ void gl_eval_apply_integrate(const double *DZ, double *DX, int t,
                                                        bool work, Fn fn, double *out0,
                                                        double *out1) {
  using D = Dims<P, QR>;
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
// (out of line: the mixed form runs it only for cells that are not fully wet,
// and a smaller kernel body keeps the common path in the instruction cache)
template <int P, int QR>
__device__ __noinline__ void zeta_iteration_fp64(const StageArgs &a, int cell, double *DZ,
                                                 double *DX, double *DRED, double *warp_norm,
                                                 int team, int cpw, int t, bool member, bool work,
                                                 const double *rhs) {
  using D = Dims<P, QR>;
  constexpr int N = D::N, G = D::G, T = D::T;
  const DegTables<double> &tb = tab<double>(P);
  const double *geo = a.geo + 11 * (int64_t)cell;
  const double det = geo[10];
  const double *zb1 = a.sd1 ? a.sd1 + cell_data(a.err, a.sdo1, cell, a.n_sd[1], G * G) : nullptr;
  // epsilon lift (OceanDG.h:1399-1422)
  {
    int ndry = 0;
    double zbmax = -1.7976931348623157e308;
    double d0[N], d1[N];
    gl_eval_apply_integrate<P, QR>(
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
    gl_eval_apply_integrate<P, QR>(
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

// Mixed form's exact wetness check of one cell (all lanes of the warp call): the
// nodal values vals ([row][node], FP32 deviations from zeta_ref) at the
// Gauss-Lobatto (p+2)^2 points, through the scratch tile Xs; lane t < G of a
// team with `check` set tests column t: zeta + zb > threshold at every point.
template <int P, int QR, typename R>
__device__ __forceinline__ bool gl_wet(const R *vals, R *Xs, int t, bool member, bool check,
                                       const float *zb1e, R zbe_flat, R wet_thr) {
  using D = Dims<P, QR>;
  constexpr int N = D::N, G = D::G, T = D::T;
  const DegTables<R> &tb = tab<R>(P);
  if (member && t < N) {
#pragma unroll
    for (int gx = 0; gx < G; ++gx) {
      R v = 0;
#pragma unroll
      for (int ix = 0; ix < N; ++ix) v += tb.BG[gx][ix] * vals[t * N + ix];
      Xs[t * T + gx] = v;
    }
  }
  __syncwarp();
  bool wet = true;
  if (check && member && t < G) {
#pragma unroll
    for (int gy = 0; gy < G; ++gy) {
      R v = 0;
#pragma unroll
      for (int iy = 0; iy < N; ++iy) v += tb.BG[gy][iy] * Xs[iy * T + t];
      const R zb = zb1e ? (R)zb1e[gy * G + t] : zbe_flat;
      wet = wet && (v + zb > wet_thr);
    }
  }
  __syncwarp();
  return wet;
}

// gl_wet out of line, for the lean variants: without bathymetry data the check runs
// only where the Lebesgue bound cannot prove wetness, so its code stays out of
// the instruction cache of the common path (with bathymetry it runs every time and
// stays inline)
template <int P, int QR, typename R>
__device__ __noinline__ bool gl_wet_call(const R *vals, R *Xs, int t, bool member, bool check,
                                         const float *zb1e, R zbe_flat, R wet_thr) {
  return gl_wet<P, QR, R>(vals, Xs, t, member, check, zb1e, zbe_flat, wet_thr);
}

// The zeta solve of a stage literally in FP64 (all lanes of the warp call; `work`
// selects the teams): zeta^n into DZ, rhs = b + int depth(zeta^n) phi over
// Gauss-Lobatto p+2 (OceanDG.h:828-855), then zeta_iteration_fp64.  The FP64
// form runs it for every cell, the mixed form only for cells that are not fully
// wet; out of line, so that the mixed kernel's common path stays small in the
// instruction cache.
template <int P, int QR, typename R>
__device__ __noinline__ void zeta_literal_fp64(const StageArgs &a, int cell, int64_t zo,
                                               const R *BZ, const double *sd1_p, double *DZ,
                                               double *DX, double *DRED, double *warp_norm,
                                               int team, int cpw, int t, bool member, bool work) {
  using D = Dims<P, QR>;
  constexpr int N = D::N, G = D::G;
  if (member && t < N) {
#pragma unroll
    for (int ix = 0; ix < N; ++ix) DZ[t * N + ix] = a.un_z[zo + t * N + ix];
  }
  __syncwarp();
  double rhs[N], dummy[N];
  {
    const double det_d = a.geo[11 * (int64_t)cell + 10];
    const double *zb1 = sd1_p ? sd1_p + cell_data(a.err, a.sdo1, cell, a.n_sd[1], G * G) : nullptr;
    const DegTables<double> &td = tab<double>(P);
    gl_eval_apply_integrate<P, QR>(
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
  zeta_iteration_fp64<P, QR>(a, cell, DZ, DX, DRED, warp_norm, team, cpw, t, member, work, rhs);
}

// Boundary face point (OceanDG.h:1105-1339): ghost state of the boundary kind
// and the numerical fluxes.  Kept out of line so that none of its FP64 work
// (boundary data functions at the point coordinates) is hoisted into the
// face loop of the cells that have no boundary face.
template <typename R, bool MIX>
__device__ __noinline__ void boundary_flux(const StageArgs &a, int bid, int bkind, int fo,
                                           double sx, const double *geo, double zref, int sdk,
                                           R g, R cu4, R zm, R qm0, R qm1, R n0, R n1, R &F,
                                           R &Fa0, R &Fa1) {
  R zbm = MIX ? (R)a.zreff : R(0);
  if (MIX && a.sdbe) zbm = (R)a.sdbe[sdk];
  else if (!MIX && a.sdb) zbm = (R)a.sdb[sdk];
  const double e0 = fo == 0 ? 0. : fo == 1 ? 1. : sx;
  const double e1 = fo < 2 ? sx : fo == 2 ? 0. : 1.;
  const double px = geo[0] + geo[2] * e0 + geo[3] * e1;
  const double py = geo[1] + geo[4] * e0 + geo[5] * e1;
  // MIX: qm0, qm1 arrive as q - q_r; the ghost state is built on absolute values
  // and its deviation kept exact where the ghost copies or reflects the inner state
  const RefStateF &rf = a.ref;
  const R dqm0 = qm0, dqm1 = qm1;
  if constexpr (MIX) {
    qm0 += rf.qr0;
    qm1 += rf.qr1;
  }
  const R un = qm0 * n0 + qm1 * n1;
  R zp = zm, qp0 = qm0, qp1 = qm1;
  bool at_outflow = false, ghost_abs = false;  // ghost_abs: deviation from the absolute ghost
  if (bkind == OC_BC_WALL_) {
    qp0 = qm0 - R(2.) * un * n0;
    qp1 = qm1 - R(2.) * un * n1;
  } else if (bkind == OC_BC_SUPIN_) {
    ghost_abs = true;
    const double zd = bc_value(a, bid, px, py, 0);
    zp = (R)(zd - zref);
    const R hh = depth<R>(zp, zbm);
    qp0 = (R)bc_value(a, bid, px, py, 1) * hh;
    qp1 = (R)bc_value(a, bid, px, py, 2) * hh;
  } else if (bkind == OC_BC_SUPOUT_) {
    at_outflow = true;
  } else if (bkind == OC_BC_HEIGHT_) {
    zp = (R)(bc_value(a, bid, px, py, 0) - zref);
  } else if (bkind == OC_BC_DISCHARGE_) {
    ghost_abs = true;
    const R qn = (R)bc_value(a, bid, px, py, 1);
    qp0 = qn * -n0;
    qp1 = qn * -n1;
  } else if (bkind == OC_BC_ABSORB_) {
    ghost_abs = true;
    const R zf = (R)(bc_value(a, bid, px, py, 0) - zref);
    const R hf = depth<R>(zf, zbm);
    const R qf0 = (R)bc_value(a, bid, px, py, 1) * hf;
    const R qf1 = (R)bc_value(a, bid, px, py, 2) * hf;
    R v0, v1, u0, u1;
    velocity<R>(zm, qm0, qm1, zbm, cu4, v0, v1);
    const R rp = v0 * n0 + v1 * n1 + R(2.) * m_sqrt(g * depth<R>(zm, zbm));
    velocity<R>(zf, qf0, qf1, zbm, cu4, u0, u1);
    const R rm = u0 * n0 + u1 * n1 - R(2.) * m_sqrt(g * depth<R>(zf, zbm));
    const R cb = R(0.25) * (rp - rm), hb = cb * cb / g, ub = R(0.5) * (rp + rm);
    zp = hb - zbm;
    const R hd = depth<R>(zp, zbm);
    qp0 = ub * hd * n0;
    qp1 = ub * hd * n1;
  }
  R Pm0, Pm1, Pp0, Pp1;
  if constexpr (MIX) {  // fluxes minus the reference flux (q_r.n, q_r (u_r.n))
    R dqp0 = dqm0 - R(2.) * un * n0, dqp1 = dqm1 - R(2.) * un * n1;  // wall
    if (ghost_abs) {
      dqp0 = qp0 - rf.qr0;
      dqp1 = qp1 - rf.qr1;
    } else if (bkind != OC_BC_WALL_) {  // ghost discharge = inner discharge
      dqp0 = dqm0;
      dqp1 = dqm1;
    }
    face_flux_dev<R>(rf, g, cu4, zm, dqm0, dqm1, zp, dqp0, dqp1, n0, n1, zbm, zbm, F, Fa0, Fa1,
                     Pm0, Pm1, Pp0, Pp1, true);
  } else {
    face_flux<R>(g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, zbm, zbm, F, Fa0, Fa1, Pm0, Pm1,
                 Pp0, Pp1);
  }
  Fa0 += Pm0;
  Fa1 += Pm1;
  if (at_outflow && un < R(-1e-12)) {  // no advective or pressure flux through the outflow
    if constexpr (MIX) {
      const R urn = rf.ur0 * n0 + rf.ur1 * n1;
      Fa0 = -rf.qr0 * urn;
      Fa1 = -rf.qr1 * urn;
    } else {
      Fa0 = Fa1 = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// Face records of a cell (built on the host, 8 per cell: 2 per face number):
//   rec[0] inner: zeta offset of the other cell; boundary: boundary face index
//   rec[1] bits 0-1 own face number, 2-3 other face number, 4-6 other degree,
//          7-8 subface+1, 9 orientation, 10 side (0 minus, 1 plus),
//          11-13 face points (inner), 14-15 kind (0 none, 1 inner, 2 boundary),
//          16-19 boundary id
// ---------------------------------------------------------------------------
struct FaceRec {
  int other, pk;
  __device__ __forceinline__ int own_face() const { return pk & 3; }
  __device__ __forceinline__ int nb_face() const { return (pk >> 2) & 3; }
  __device__ __forceinline__ int nb_deg() const { return (pk >> 4) & 7; }
  __device__ __forceinline__ int sub() const { return ((pk >> 7) & 3) - 1; }
  __device__ __forceinline__ int orient() const { return (pk >> 9) & 1; }
  __device__ __forceinline__ int side() const { return (pk >> 10) & 1; }
  __device__ __forceinline__ int nf() const { return (pk >> 11) & 7; }
  __device__ __forceinline__ int kind() const { return (pk >> 14) & 3; }
  __device__ __forceinline__ int bid() const { return (pk >> 16) & 15; }
};

#ifdef OC_BOUNDS_CHECK
// Face record of a slot of a cell with q boundary-face points (bounds-checked build): packed
// fields in range, the neighbour's DoFs or the boundary face, the static face
// data (sdo) and the face-pass values (fo) of the slot inside their arrays.  A
// malformed record becomes an empty slot; a bad offset becomes 0.
static __device__ __noinline__ void check_record(const StageArgs &a, FaceRec &r, int q,
                                                 int *sdo, int *fo) {
  const int kind = r.kind();
  if (kind == 0) return;
  bool ok = kind <= 2;
  if (kind == 1)
    ok = ok && r.nb_deg() >= 1 && r.nb_deg() <= OC_MAXDEG && r.nf() >= 2 && r.nf() <= OC_MAXF &&
         r.sub() <= 1;
  if (!ok) {
    checked(a.err, r.pk, 0, BS_RECORD);
    r.pk = 0;
    r.other = 0;
    return;
  }
  const int nfo = kind == 1 ? r.nf() : q;
  if (kind == 1) {
    const int nn = (r.nb_deg() + 1) * (r.nb_deg() + 1);
    r.other = (int)checked(a.err, r.other, a.n_dofs - nn + 1, BS_NEIGHBOUR);
  } else {
    r.other = (int)checked(a.err, r.other, a.n_bnd_faces, BS_BOUNDARY);
  }
  if (sdo)
    *sdo = (int)checked(a.err, *sdo, kind == 1 ? a.n_sd[3] - 2 * nfo + 1 : a.n_sd[4] - nfo + 1,
                        BS_FACE_DATA);
  if (fo) *fo = (int)checked(a.err, *fo, a.n_fout - 3 * nfo + 1, BS_FACE_OUT);
}
#endif

// Boundary face of a cell slot in the mixed form's face phase: lane t < Q of the
// team evaluates Gauss point t (the own trace, the ghost state of the boundary
// kind and the fluxes, boundary_flux) and writes the point's values times the
// outward sign and JxW into FV ([var][FVS]).
template <int P, int QR, typename R, bool MIX>
__device__ __forceinline__ void boundary_slot(const StageArgs &a, int bid, int fo, int sdo, R n0,
                                              R n1, R len, const double *geo, double zref, R g,
                                              R cu4, const R *U, R *FV, int t) {
  using D = Dims<P, QR>;
  constexpr int N = D::N, NN = D::NN, Q = D::Q;
  const DegTables<R> &tb = tab<R>(P);
  const auto &cBQ = QR ? tb.BM : tb.BQ;
  const auto &cwQ = QR ? tb.wM : tb.wQ;
  const int bkind = a.bc_kind[bid];
  if (bkind == 0 && t == 0) atomicOr(a.err, ERR_UNKNOWN_BID);
  if (t < Q) {
    const int k = t;
    R zm = 0, qm0 = 0, qm1 = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const int d = face_dof(N, fo, i);
      const R l = cBQ[k][i];
      zm += l * U[d];
      qm0 += l * U[NN + d];
      qm1 += l * U[2 * NN + d];
    }
    R F, Fa0, Fa1;
    const double sx = QR ? tab<double>(P).xM[k] : tab<double>(P).xQ[k];
    boundary_flux<R, MIX>(a, bid, bkind, fo, sx, geo, zref, sdo + k, g, cu4, zm, qm0, qm1, n0, n1,
                          F, Fa0, Fa1);
    const R jxw = cwQ[k] * len;
    FV[k] = -F * jxw;
    FV[FVS + k] = -Fa0 * jxw;
    FV[2 * FVS + k] = -Fa1 * jxw;
  }
}

// boundary_slot out of line, for the lean variants (only the teams of boundary
// cells run it; the common path keeps a smaller instruction footprint)
template <int P, int QR, typename R, bool MIX>
__device__ __noinline__ void boundary_slot_call(const StageArgs &a, int bid, int fo, int sdo,
                                                R n0, R n1, R len, const double *geo, double zref,
                                                R g, R cu4, const R *U, R *FV, int t) {
  boundary_slot<P, QR, R, MIX>(a, bid, fo, sdo, n0, n1, len, geo, zref, g, cu4, U, FV, t);
}

// Stage coefficients in the compute type: the FP32 copies for the FP32 bulk (one
// 16-byte read-only load, no FP64 conversion), the FP64 values otherwise.
template <typename R>
__device__ __forceinline__ void load_coefs(const float *ff, const double *fd,
                                           R (&o)[OC_MAXSTAGES]) {
  static_assert(OC_MAXSTAGES == 4, "one float4 of coefficients");
  if constexpr (sizeof(R) == 4) {
    const float4 f4 = __ldg(reinterpret_cast<const float4 *>(ff));
    o[0] = f4.x; o[1] = f4.y; o[2] = f4.z; o[3] = f4.w;
  } else {
#pragma unroll
    for (int j = 0; j < OC_MAXSTAGES; ++j) o[j] = (R)__ldg(&fd[j]);
  }
}

// One flag word per warp: OC_ERR_NONFINITE when any lane stored a non-finite
// u^{n+1} (read by the host at its next synchronising call).
__device__ __forceinline__ void report_nonfinite(const StageArgs &a, bool bad) {
  if (__any_sync(OC_FULL, bad) && (threadIdx.x & 31) == 0) atomicOr(a.err, ERR_NONFINITE);
}

// ---------------------------------------------------------------------------
// The fused stage kernel.
//   MIX = false: FP64 plain form (R = KT = double).
//   MIX = true : mixed form; R = float bulk, KT = type of the k registers.
// Memory flow: warp-cooperative prologue (stage input, face records, partial
// zeta right-hand side), team-local face contributions (FP64: the face pass's
// point values of the cell's face sides; mixed: after the cell integrals, from
// the neighbour traces), team-local cell integrals, zeta and discharge solves,
// warp-cooperative epilogue (RK update and stores).  Global accesses of the
// prologue/epilogue are lane-contiguous over the warp's cells.
// ---------------------------------------------------------------------------
// resident 4-warp blocks per SM the mixed kernels are compiled for (register cap)
#ifndef OC_MIXED_MIN_BLOCKS
#define OC_MIXED_MIN_BLOCKS 5
#endif
// One block of the stage: `blk` is the block index within the degree group of
// n_group cells (listed by group_cells, or group_first + i when NULL); the FP64
// work-area slots of the mixed form are indexed by the launch-wide block index.
template <int P, typename R, typename KT, bool MIX, typename RIN, bool LEAN, int QR, bool CONF>
__device__ __forceinline__ void stage_body(const StageArgs &a, unsigned char *smem_raw,
                                           const int blk, const int n_group,
                                           const int *group_cells, const int group_first) {
  using D = Dims<P, QR>;
  constexpr int N = D::N, Q = D::Q, G = D::G, T = D::T, NN = D::NN, NT = D::NT;
  constexpr int CPWMAX = D::CPW;
  static_assert(CPWMAX <= OC_MAXCPW, "cells per warp above the work-area slot stride");
  const DegTables<R> &tb = tab<R>(P);
  // cell Gauss rule: the floor(1.5 P) + 1 point tables, or (QR = 1) the P + 1 point
  // tables of the discharge mass
  const auto &cBQ = QR ? tb.BM : tb.BQ;
  const auto &cDQ = QR ? tb.DM : tb.DQ;
  const auto &cwQ = QR ? tb.wM : tb.wQ;

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int team_raw = lane / T, t = lane - team_raw * T;
  const bool member = team_raw < CPWMAX;  // lanes past the last team only help and synchronise
  const int team = member ? team_raw : 0;
  const int W = a.batch;
  const int cpw = (CPWMAX / W) * W;
  const int wpb = blockDim.x >> 5;
  const int gi0 = (blk * wpb + warp) * cpw;
  const int nvalid = max(0, min(cpw, n_group - gi0));  // cells of this warp
  const bool valid = member && team < nvalid;
  const int s = a.stage;
  // programmatic dependent launch: the next launch in the stream may be scheduled
  // now; it waits (griddepcontrol.wait) for this grid to complete before it reads
  // what this one writes
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  // the mixed time-step path (FP32 registers) forms internal stage inputs in FP32
  constexpr bool fast = MIX && sizeof(KT) == 4;
  // FP64 form: faces from the stage's face pass (each face once, oc_face.cu);
  // mixed form: faces evaluated here by both neighbours, which costs fewer
  // instructions than a separate pass in FP32 (where FP64's 1/64 rate does not
  // make the flux the bottleneck)
  constexpr bool FPASS = !MIX;
  // LEAN: a workload without static data (bathymetry, friction coefficients,
  // sources), friction model or ARK scheme (the host checks this); the branches
  // of those features are compiled out of the variant.  The per-cell time scale
  // of ensembles stays in (a few multiplies; 0.5% on the vortex step)
  const bool ark = !LEAN && a.ark;
  const int friction_m = LEAN ? 0 : a.friction;
  const double *sd0_p = LEAN ? nullptr : a.sd0, *sd1_p = LEAN ? nullptr : a.sd1,
               *sd2_p = LEAN ? nullptr : a.sd2, *sdf_p = LEAN ? nullptr : a.sdf;
  const float *sd0e_p = LEAN ? nullptr : a.sd0e, *sd1e_p = LEAN ? nullptr : a.sd1e,
              *sd2e_p = LEAN ? nullptr : a.sd2e, *sdfe_p = LEAN ? nullptr : a.sdfe;
  const int *cfsdo_p = LEAN ? nullptr : a.cfsdo;
  // CONF: every cell of degree P, no hanging face, standard orientation (the host
  // checks this): every inner face takes the register-row path
  const double *cscale_p = a.cscale;
  const float *cscalef_p = a.cscalef;
  static_assert(MIX == (sizeof(R) == 4), "the scratch layout assumes FP32 exactly in the mixed form");
  const double zref = MIX ? a.zeta_ref : 0.0;
  const R g = MIX ? (R)a.gf : (R)a.g, cu4 = MIX ? (R)a.cu4f : (R)a.cu4;
  const R zbe_flat = MIX ? (R)a.zreff : R(0);  // zb + zeta_ref where no bathymetry is given
  // mixed form: discharge stored as q - q_r (reference state (h_r, q_r))
  const RefStateF &rf = a.ref;
  const double qref0 = MIX ? a.q_ref[0] : 0.0, qref1 = MIX ? a.q_ref[1] : 0.0;

  unsigned char *wbase = smem_raw + warp * D::template warp_bytes<R>();
  auto Rreg = [&](int j) { return reinterpret_cast<R *>(wbase + j * D::template bytes_r<R>()); };
  int *ints = reinterpret_cast<int *>(wbase + D::template int_offset<R>());
  int *w_cell = ints, *w_off = ints + CPWMAX, *w_rec = ints + 2 * CPWMAX,
      *w_sdo = ints + 18 * CPWMAX, *w_flag = ints + 26 * CPWMAX, *w_fo = ints + 27 * CPWMAX;
  double *warp_norm = reinterpret_cast<double *>(wbase + D::template norm_offset<R>());
  R *U = Rreg(team);          // 3*NN stage input z, q0, q1
  R *RES = U + 3 * NN;        // 3*NN residual; later the discharge result
  R *RST = RES + 3 * NN;      // 2*NN stiff residual (ARK)
  R *BZ = RST + 2 * NN;       // NN zeta right-hand side b = sum f k (mixed: then delta)
  R *ZN = BZ + NN;            // NN mixed form: zeta^n - zeta_ref
  R *X = ZN + NN;             // scratch tiles
  auto Dreg = [&](int j) {  // FP64 team region of team j: shared (FP64 form) or global slot
    if constexpr (MIX)
      return a.dscratch + ((int64_t)(blockIdx.x * wpb + warp) * OC_MAXCPW + j) * OC_DSTRIDE;
    else
      return reinterpret_cast<double *>(wbase + D::template d_offset<R>() + j * D::bytes_d());
  };

  // ---- 0. prologue: cells, stage input, face records, partial rhs ------------
  if (lane < CPWMAX) {
    const int j = lane;
    const int gi = nvalid > 0 ? gi0 + (j < nvalid ? j : 0) : 0;  // idle warps read cell 0
    const int c = (int)checked(a.err, group_cells ? group_cells[gi] : group_first + gi,
                               a.n_cells, BS_CELL);
    w_cell[j] = c;
    w_off[j] = (int)checked(a.err, a.uniform_nn ? (int64_t)c * a.uniform_nn : a.off[c],
                            a.n_dofs - NN + 1, BS_OFFSET);
    w_flag[j] = 0;
  }
  __syncwarp();
  const int cell = w_cell[team];
  const int64_t zo = w_off[team], qo = 2 * zo;
  double *DZ = Dreg(team);        // NN FP64 iterate
  double *DX = DZ + NN;           // 3 tiles N*T
  double *DRED = DX + 3 * NT;     // T+1
  const double *geo = a.geo + 11 * (int64_t)cell;
  R gR[11];  // geometry in the compute type (FP32 copy in the mixed form); loads issued early
#pragma unroll
  for (int k = 0; k < 11; ++k) {
    if constexpr (MIX) gR[k] = (R)__ldg(a.geof + 11 * (int64_t)cell + k);
    else gR[k] = (R)__ldg(geo + k);
  }
#pragma unroll
  for (int i = 0; i < (CPWMAX * 16 + 31) / 32; ++i) {  // face records (invalid teams: empty)
    const int e = lane + 32 * i;
    if (e < nvalid * 16) {
      const int j = e >> 4, k = e & 15;
      w_rec[j * 16 + k] = __ldg(a.cfrec + 16 * (int64_t)w_cell[j] + k);
    }
  }
  for (int e = lane; e < (CPWMAX - nvalid) * 16; e += 32) {
    const int j = nvalid + (e >> 4);
    w_rec[j * 16 + (e & 15)] = (e & 1) ? 0 : -1;
  }
  if (cfsdo_p)
    for (int e = lane; e < nvalid * 8; e += 32)
      w_sdo[e] = cfsdo_p[8 * (int64_t)w_cell[e >> 3] + (e & 7)];
  if (FPASS)
    for (int e = lane; e < nvalid * 8; e += 32)
      w_fo[e] = __ldg(a.cfofs + 8 * (int64_t)w_cell[e >> 3] + (e & 7));
#ifdef OC_BOUNDS_CHECK
  __syncwarp();
  for (int e = lane; e < nvalid * 8; e += 32)
    check_record(a, reinterpret_cast<FaceRec *>(w_rec)[e], Q, cfsdo_p ? w_sdo + e : nullptr,
                 FPASS ? w_fo + e : nullptr);
#endif
  // Everything above reads only the mesh (written before the stream's first stage
  // launch); from here on the kernel reads the previous launch's results and
  // writes buffers it may still read, so it waits for that launch to complete.
  // Without a programmatic launch the wait returns at once.
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  __syncwarp();
  // the face pass's point values of the team's 8 face slots, copied asynchronously
  // into the scratch tiles ([slot][var][FVS]; free until the cell integrals) while
  // the stage input below is loaded: one memory round trip for both
  const FaceRec *recs = reinterpret_cast<const FaceRec *>(w_rec + 16 * team);
  if (FPASS && member) {
    const R *fout = static_cast<const R *>(a.fout);
#pragma unroll
    for (int sl = 0; sl < 8; ++sl) {
      const FaceRec r = recs[sl];
      const int kind = r.kind();
      const int nfo = kind == 1 ? r.nf() : kind == 2 ? Q : 0;
      const int64_t fo = w_fo[8 * team + sl];
      for (int k = t; k < nfo; k += T)
#pragma unroll
        for (int v = 0; v < 3; ++v)
          cp_async(X + (sl * 3 + v) * FVS + k, fout + fo + v * nfo + k);
    }
  }
  R fR[OC_MAXSTAGES];  // coefficients in the compute type (mixed form: the FP32 copies)
  load_coefs<R>(a.dyn->ff, a.dyn->f, fR);
  R fRs = fR[0];  // f_s
#pragma unroll
  for (int j = 1; j < OC_MAXSTAGES; ++j)
    if (j == a.stage) fRs = fR[j];
  // stage input: element e = lane + 32 i of the warp's cells (compile-time trip
  // count, so that the loads of all elements are issued before the stores)
#pragma unroll
  for (int i = 0; i < (CPWMAX * NN + 31) / 32; ++i) {
    const int e = lane + 32 * i;
    if (e >= nvalid * NN) break;
    const int j = e / NN, d = e - j * NN;
    const int64_t oz = w_off[j] + d, oq = 2 * (int64_t)w_off[j] + d;
    R *Uj = Rreg(j);
    Uj[d] = load_in<RIN, R>(a.rz, oz, zref);
    const R uq0 = load_in<RIN, R>(a.rq, oq, qref0), uq1 = load_in<RIN, R>(a.rq, oq + NN, qref1);
    Uj[NN + d] = uq0;
    Uj[2 * NN + d] = uq1;
    // fast ERK path: the discharge part of the update known before this stage,
    // QB = (last stage ? 0 : q^n) + sum_{j<s} f_j k_q[j+1] (RST region, unused by
    // the explicit stage), loaded with the stage input so that the epilogue loads nothing
    if (fast && !ark && (LEAN || !a.apply_mode)) {
      R qb0 = 0, qb1 = 0;
#pragma unroll
      for (int jj = 0; jj < OC_MAXSTAGES; ++jj)
        if (jj < s) {
          qb0 += fR[jj] * (R)ldro<KT>(a.kq[jj + 1], oq);
          qb1 += fR[jj] * (R)ldro<KT>(a.kq[jj + 1], oq + NN);
        }
      if (!a.last) {
        qb0 += s == 0 ? uq0 : (R)__ldg(a.un_qf + oq);
        qb1 += s == 0 ? uq1 : (R)__ldg(a.un_qf + oq + NN);
      }
      Uj[6 * NN + d] = qb0;
      Uj[7 * NN + d] = qb1;
    }
    if (LEAN || !a.apply_mode) {
      R bprev = 0;  // sum_{j<s} f_j kz_j in the reference's order
#pragma unroll
      for (int jj = 0; jj < OC_MAXSTAGES; ++jj)  // compile-time indices: fR stays in registers
        if (jj < s)
          bprev = jj == 0 ? fR[0] * (R)ldro<KT>(a.kz[1], oz)
                          : bprev + fR[jj] * (R)ldro<KT>(a.kz[jj + 1], oz);
      Uj[8 * NN + d] = bprev;
      if constexpr (fast) {
        Uj[9 * NN + d] = s == 0 ? Uj[d] : (R)__ldg(a.un_zf + oz);
      } else if constexpr (MIX) {
        Uj[9 * NN + d] = (R)(__ldg(a.un_z + oz) - zref);
      }
    }
  }
  cp_async_wait_all();
  __syncwarp();
  const R Ji00 = gR[6], Ji01 = gR[7], Ji10 = gR[8], Ji11 = gR[9];
  const R det = gR[10];

  // ---- 1. faces: local_apply_face_* (OceanDG.h:936-1050) and
  //         local_apply_boundary_face_* (:1105-1339) ----------------------------
  // The face pass of this stage (oc_face.cu) evaluated every face's flux once and
  // left, per face side, the point values times sign and JxW; the record of a
  // slot holds the offset of this side's values.  Each slot's values are
  // integrated against the own basis: the trace rows of the own side (full face,
  // or the subface rows on the coarse side of a hanging face), Gauss rows on
  // boundary faces.
  // integration column of node t on a full face of this degree, in registers
  R pcol[G];
  {
    const int tt = t < N ? t : 0;
#pragma unroll
    for (int k = 0; k < G; ++k) pcol[k] = tb.F[0][G][k][tt];
  }
  const DegTables<R> *pgt = reinterpret_cast<const DegTables<R> *>(
      sizeof(R) == 4 ? (const void *)a.gtabf : (const void *)a.gtabd);
  const DegTables<R> &ptb = pgt[P - 1];
  // the values of all slots were copied into the scratch tiles by the prologue
  R *FVA = X;
  if (member && t < N) {
#pragma unroll
    for (int e = 0; e < 3; ++e)
#pragma unroll
      for (int ix = 0; ix < N; ++ix) RES[e * NN + t * N + ix] = R(0);
  }
  __syncwarp();
  if constexpr (FPASS) {
#pragma unroll 1
  for (int sl = 0; sl < 8; ++sl) {
    const FaceRec r = recs[sl];
    const int kind = member ? r.kind() : 0;
    // second slots of conforming faces are empty in every team of most warps
    if (!__any_sync(OC_FULL, kind != 0)) continue;
    const int fo = r.own_face();
    // DoF of node i on face fo: fbase + i * fstride (face_dof)
    const int fbase = fo == 0 ? 0 : fo == 1 ? N - 1 : fo == 2 ? 0 : (N - 1) * N;
    const int fstride = fo < 2 ? N : 1;
    int nfo = 0, tsel = 0;
    if (kind == 1) {
      nfo = r.nf();
      tsel = r.side() ? r.sub() + 1 : 0;
    } else if (kind == 2) {
      nfo = Q;
      tsel = -1;
    }
    const R *FV = FVA + sl * 3 * FVS;
    // integration rows: registers when every face of the warp in this slot is a full
    // face of this degree's point set, else the global table copy (boundary faces:
    // Gauss rows; inner faces: the trace rows of the own side)
    const bool reg_cols = __all_sync(OC_FULL, nfo == 0 || (tsel == 0 && nfo == G));
    if (nfo > 0 && t < N) {  // integrate the own-side values against the own basis
      R cz = 0, c0 = 0, c1 = 0;
      if (reg_cols) {
#pragma unroll
        for (int k = 0; k < G; ++k) {
          cz += pcol[k] * FV[k];
          c0 += pcol[k] * FV[FVS + k];
          c1 += pcol[k] * FV[2 * FVS + k];
        }
      } else {
        const R *col = tsel < 0 ? (QR ? &ptb.BM[0][t] : &ptb.BQ[0][t]) : &ptb.F[tsel][nfo][0][t];  // stride OC_MAXN
#pragma unroll
        for (int k = 0; k < (Q > OC_MAXF ? Q : OC_MAXF); ++k) {  // nfo <= max(Q, OC_MAXF)
          if (k < nfo) {
            const R l = __ldg(col + k * OC_MAXN);
            fma2(cz, c0, l, FV[k], l, FV[FVS + k]);
            c1 += l * FV[2 * FVS + k];
          }
        }
      }
      const int d = fbase + t * fstride;
      RES[d] += cz;
      RES[NN + d] += c0;
      RES[2 * NN + d] += c1;
    }
    __syncwarp();
  }
  }

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
        fma2(b0, a0, cBQ[qx][ix], z[ix], cBQ[qx][ix], q0[ix]);
        fma2(d0, a1, cDQ[qx][ix], z[ix], cBQ[qx][ix], q1[ix]);
      }
      X[0 * NT + t * T + qx] = b0;
      X[1 * NT + t * T + qx] = d0;
      X[2 * NT + t * T + qx] = a0;
      X[3 * NT + t * T + qx] = a1;
    }
  }
  __syncwarp();
  const bool split = ark && !a.last;  // ARK internal stage: stiff part separate
  {
    R Az[N], Cz[N], A0[N], C0[N], A1[N], C1[N];
#pragma unroll
    for (int i = 0; i < N; ++i) Az[i] = Cz[i] = A0[i] = C0[i] = A1[i] = C1[i] = 0;
    if (member && t < Q) {  // y-pass, pointwise model, y-integration on column qx = t
      const int64_t so0 = sd0_p ? cell_data(a.err, a.sdo0, cell, a.n_sd[0], 5 * Q * Q) : 0;
      const double *sd0 = sd0_p ? sd0_p + so0 : nullptr;
      const float *sd0e = sd0e_p ? sd0e_p + so0 : nullptr;
      // not unrolled: the point loop is the largest block of the kernel, and a
      // smaller instruction footprint leaves fewer warps waiting on instruction
      // fetch (the shape coefficients become uniform constant loads)
#pragma unroll 1
      for (int qy = 0; qy < Q; ++qy) {
        R z = 0, zx = 0, zy = 0, q0 = 0, q1 = 0;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          const R xb = X[0 * NT + iy * T + t], xd = X[1 * NT + iy * T + t];
          const R b = cBQ[qy][iy];
          fma2(z, zx, b, xb, b, xd);
          fma2(q0, q1, b, X[2 * NT + iy * T + t], b, X[3 * NT + iy * T + t]);
          zy += cDQ[qy][iy] * xb;
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
        const R w = cwQ[t] * cwQ[qy] * det;
        // height: int q . grad(phi)   (mass_flux = q, ShallowWater.h:349-357)
        const R gz0 = (Ji00 * q0 + Ji01 * q1) * w, gz1 = (Ji10 * q0 + Ji11 * q1) * w;
        // discharge: advective flux (ShallowWater.h:378-403, nu = 0) and sources (:405-472)
        R v0, v1, h, F00, F01, F10, F11, qa0 = q0, qa1 = q1;
        if constexpr (MIX) {  // q0, q1 are q - q_r: flux minus the reference flux q_r u_r
          R du0, du1;
          vel_dev<R>(rf, cu4, z + (zb - rf.hr), q0, q1, du0, du1, h);
          v0 = rf.ur0 + du0; v1 = rf.ur1 + du1;
          qa0 = rf.qr0 + q0; qa1 = rf.qr1 + q1;
          F00 = rf.qr0 * du0 + q0 * v0; F01 = rf.qr0 * du1 + q0 * v1;
          F10 = rf.qr1 * du0 + q1 * v0; F11 = rf.qr1 * du1 + q1 * v1;
        } else {
          velocity<R>(z, q0, q1, zb, cu4, v0, v1);
          h = depth<R>(z, zb);
          F00 = q0 * v0; F01 = q0 * v1; F10 = q1 * v0; F11 = q1 * v1;
        }
        const R dz0 = Ji00 * zx + Ji10 * zy, dz1 = Ji01 * zx + Ji11 * zy;
        R fr0 = 0, fr1 = 0;
        if (friction_m && !split) friction<R>(friction_m, g, v0, v1, cf, h, fr0, fr1);
        // -g h grad(zeta) (ShallowWater.h:405-432); with bathymetry the mixed form
        // forms the depth h = zeta + zb of the source in FP64
        R hs = h;
        if constexpr (MIX) {
          if (sd0) hs = (R)fmax((double)z + (zref + sd0[5 * k]), 1e-12);
        }
        const R pg0 = -g * hs * dz0, pg1 = -g * hs * dz1;
        const R s0 = pg0 - fr0 + w0 + fc * qa1;
        const R s1 = pg1 - fr1 + w1 - fc * qa0;
        const R g00 = (Ji00 * F00 + Ji01 * F01) * w, g01 = (Ji10 * F00 + Ji11 * F01) * w;
        const R g10 = (Ji00 * F10 + Ji01 * F11) * w, g11 = (Ji10 * F10 + Ji11 * F11) * w;
        const R sv0 = s0 * w, sv1 = s1 * w;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          const R b = cBQ[qy][iy], d = cDQ[qy][iy];
          fma2(Az[iy], Cz[iy], b, gz0, d, gz1);
          fma2(A0[iy], A1[iy], b, g00, b, g10);
          fma2(C0[iy], C1[iy], d, g01, d, g11);
          fma2(C0[iy], C1[iy], b, sv0, b, sv1);
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
          const R b = cBQ[qx][ix], d = cDQ[qx][ix];
          fma2(r0, r1, d, X[2 * NT + t * T + qx], d, X[4 * NT + t * T + qx]);
          fma2(r0, r1, b, X[3 * NT + t * T + qx], b, X[5 * NT + t * T + qx]);
          rz += d * X[0 * NT + t * T + qx];
          rz += b * X[1 * NT + t * T + qx];
        }
        RES[t * N + ix] += rz;
        RES[NN + t * N + ix] += r0;
        RES[2 * NN + t * N + ix] += r1;
      }
    }
    __syncwarp();
  }
  if (split) {  // warp-uniform: stiff (friction) residual, a second pass over the points
    if (member && t < N) {
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
          b0 += cBQ[qx][ix] * z[ix];
          a0 += cBQ[qx][ix] * q0[ix];
          a1 += cBQ[qx][ix] * q1[ix];
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
      const int64_t so0 = sd0_p ? cell_data(a.err, a.sdo0, cell, a.n_sd[0], 5 * Q * Q) : 0;
      const double *sd0 = sd0_p ? sd0_p + so0 : nullptr;
      const float *sd0e = sd0e_p ? sd0e_p + so0 : nullptr;
#pragma unroll
      for (int qy = 0; qy < Q; ++qy) {
        R z = 0, q0 = 0, q1 = 0;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          z += cBQ[qy][iy] * X[2 * NT + iy * T + t];
          q0 += cBQ[qy][iy] * X[3 * NT + iy * T + t];
          q1 += cBQ[qy][iy] * X[4 * NT + iy * T + t];
        }
        const int k = qy * Q + t;
        R zb = MIX ? zbe_flat : R(0), cf = 0;
        if (MIX && sd0e) { zb = (R)sd0e[5 * k]; cf = (R)sd0e[5 * k + 1]; }
        else if (!MIX && sd0) { zb = (R)sd0[5 * k]; cf = (R)sd0[5 * k + 1]; }
        R v0, v1, fr0 = 0, fr1 = 0;
        if constexpr (MIX) velocity<R>(z, rf.qr0 + q0, rf.qr1 + q1, zb, cu4, v0, v1);
        else velocity<R>(z, q0, q1, zb, cu4, v0, v1);
        if (friction_m) friction<R>(friction_m, g, v0, v1, cf, depth<R>(z, zb), fr0, fr1);
        const R w = cwQ[t] * cwQ[qy] * det;
        const R st0 = -fr0 * w, st1 = -fr1 * w;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          S0[iy] += cBQ[qy][iy] * st0;
          S1[iy] += cBQ[qy][iy] * st1;
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
          r0 += cBQ[qx][ix] * X[0 * NT + t * T + qx];
          r1 += cBQ[qx][ix] * X[1 * NT + t * T + qx];
        }
        RST[t * N + ix] = r0;
        RST[NN + t * N + ix] = r1;
      }
    }
    __syncwarp();
  }

  if constexpr (!FPASS) {
  R *NB = X;                      // neighbour traces [slot][var][node]
  R *FV = X + 8 * 3 * OC_MAXN;    // 3*FVS face point values
  // ---- 3. faces of the mixed form, in this kernel: local_apply_face_* (OceanDG.h:936-1050)
  //         and local_apply_boundary_face_* (:1105-1339); each face evaluated
  //         identically by both neighbours, own side kept ------------------------
  // 2a. neighbour traces of every inner slot: [slot][var][node], in the scratch
  // tiles (free between the cell integrals and the zeta solve); a smaller team
  // region leaves more of the SM's shared memory / L1 to the L1 cache
  if (member) {
#pragma unroll
    for (int ii = 0; ii < (8 * OC_MAXN + T - 1) / T; ++ii) {
      const int e = t + ii * T;
      if (e >= 8 * OC_MAXN) break;
      const int sl = e / OC_MAXN, i = e - sl * OC_MAXN;
      const FaceRec r = recs[sl];
      const int Nn = CONF ? N : r.nb_deg() + 1;
      if (r.kind() == 1 && i < Nn) {
        const int d = face_dof(Nn, r.nb_face(), i);
        const int64_t oz = r.other, oq = 2 * (int64_t)r.other;
        NB[(sl * 3 + 0) * OC_MAXN + i] = load_in<RIN, R>(a.rz, oz + d, zref);
        NB[(sl * 3 + 1) * OC_MAXN + i] = load_in<RIN, R>(a.rq, oq + d, qref0);
        NB[(sl * 3 + 2) * OC_MAXN + i] = load_in<RIN, R>(a.rq, oq + Nn * Nn + d, qref1);
      }
    }
  }
  __syncwarp();
  // own outward normals and face lengths of the affine cell
  const R J00 = gR[2], J01 = gR[3], J10 = gR[4], J11 = gR[5];
  // Conforming faces between cells of this degree (the common case): the trace
  // row of point k = t (both sides: no subface, standard orientation) and the
  // integration column of node t, held in registers so that the face loop reads
  // no lane-dependent constant-bank address.
  R frow[N], fcol[G], fw;
  {
    const int kk = t < G ? t : 0, tt = t < N ? t : 0;
#pragma unroll
    for (int i = 0; i < N; ++i) frow[i] = tb.F[0][G][kk][i];
#pragma unroll
    for (int k = 0; k < G; ++k) fcol[k] = tb.F[0][G][k][tt];
    fw = tb.wF[G][kk];
  }
  // lane-dependent table entries of the hanging / degree-jump face paths come
  // from the global copy (L1), where divergent addresses cost a few wavefronts
  // instead of one constant-bank replay per distinct address
  const DegTables<R> *gt = reinterpret_cast<const DegTables<R> *>(
      sizeof(R) == 4 ? (const void *)a.gtabf : (const void *)a.gtabd);
  const DegTables<R> &tbg = gt[P - 1];
#pragma unroll 1
  for (int sl = 0; sl < 8; ++sl) {
    const FaceRec r = recs[sl];
    const int kind = member ? r.kind() : 0;
    // second slots of conforming faces are empty in every team of most warps
    if (!__any_sync(OC_FULL, kind != 0)) continue;
    // Warp-uniform choice of the inner-face path: the register-row path when every
    // inner face of the warp in this slot joins two cells of this degree in standard
    // orientation, else the table path for all of them (one path per warp: on hp
    // meshes the teams of a warp meet different neighbour degrees, and two paths
    // would run one after the other)
    const bool reg_path =
        CONF || __all_sync(OC_FULL, kind != 1 || (r.nb_deg() == P && r.orient() == 0));
    const int fo = r.own_face();
    // DoF of node i on face fo: fbase + i * fstride (face_dof)
    const int fbase = fo == 0 ? 0 : fo == 1 ? N - 1 : fo == 2 ? 0 : (N - 1) * N;
    const int fstride = fo < 2 ? N : 1;
    int nfo = 0, tsel = 0;
    if (kind != 0) {
      // outward normal of the own face: J^-T n_ref / |.|; tangent length |J t_ref|
      const R nr0 = fo == 0 ? R(-1) : fo == 1 ? R(1) : R(0);
      const R nr1 = fo == 2 ? R(-1) : fo == 3 ? R(1) : R(0);
      R on0 = Ji00 * nr0 + Ji10 * nr1, on1 = Ji01 * nr0 + Ji11 * nr1;
      const R inv = R(1) / m_sqrt(on0 * on0 + on1 * on1);
      on0 *= inv; on1 *= inv;
      const R tx = fo < 2 ? J01 : J00, ty = fo < 2 ? J11 : J10;
      R len = m_sqrt(tx * tx + ty * ty);
      if (kind == 1) {
        const int side = r.side(), sub = CONF ? -1 : r.sub(), orient = r.orient(), nf = r.nf();
        const int pn = CONF ? P : r.nb_deg(), Nn = pn + 1;
        const DegTables<R> &tn = gt[pn - 1];
        if (side == 1 && sub >= 0) len *= R(0.5);  // coarse side: the fine half-face
        const R n0 = side ? -on0 : on0, n1 = side ? -on1 : on1;  // minus normal
        const int sdo = cfsdo_p ? w_sdo[8 * team + sl] : 0;
        nfo = nf;
        tsel = side ? sub + 1 : 0;
        if (reg_path) {  // same degree: nf == G <= T, point k on both sides
          if (t < G) {
            const int k = t;
            // trace rows: full face from registers; the coarse side of a hanging
            // face (own on the plus side, the neighbour's on the minus side) reads
            // the subface rows
            const int nsel = side ? 0 : sub + 1;
            R lo[N], ln[N];
            if (tsel == 0) {
#pragma unroll
              for (int i = 0; i < N; ++i) lo[i] = frow[i];
            } else {
#pragma unroll
              for (int i = 0; i < N; ++i) lo[i] = __ldg(&tbg.F[tsel][G][k][i]);
            }
            if (nsel == 0) {
#pragma unroll
              for (int i = 0; i < N; ++i) ln[i] = frow[i];
            } else {
#pragma unroll
              for (int i = 0; i < N; ++i) ln[i] = __ldg(&tbg.F[nsel][G][k][i]);
            }
            R zo_ = 0, qo0 = 0, qo1 = 0, zn = 0, qn0 = 0, qn1 = 0;
#pragma unroll
            for (int i = 0; i < N; ++i) {
              const int d = fbase + i * fstride;
              fma2(zo_, qo0, lo[i], U[d], lo[i], U[NN + d]);
              fma2(qo1, zn, lo[i], U[2 * NN + d], ln[i], NB[(sl * 3 + 0) * OC_MAXN + i]);
              fma2(qn0, qn1, ln[i], NB[(sl * 3 + 1) * OC_MAXN + i], ln[i],
                   NB[(sl * 3 + 2) * OC_MAXN + i]);
            }
            const R zm = side ? zn : zo_, qm0 = side ? qn0 : qo0, qm1 = side ? qn1 : qo1;
            const R zp = side ? zo_ : zn, qp0 = side ? qo0 : qn0, qp1 = side ? qo1 : qn1;
            R zbm = MIX ? zbe_flat : R(0), zbp = zbm;
            if (!MIX && sdf_p) {
              zbm = (R)sdf_p[sdo + 2 * k]; zbp = (R)sdf_p[sdo + 2 * k + 1];
            }
            R F, Fa0, Fa1, Pm0, Pm1, Pp0, Pp1;
            if constexpr (MIX) {
              if (sdf_p)  // bathymetry: well-balanced differences in FP64
                face_flux_dev_wb_call<R>(rf, g, cu4, zref, zm, qm0, qm1, zp, qp0, qp1, n0, n1,
                                    sdf_p[sdo + 2 * k], sdf_p[sdo + 2 * k + 1],
                                    sdfe_p[sdo + 2 * k], sdfe_p[sdo + 2 * k + 1], F, Fa0, Fa1,
                                    Pm0, Pm1, Pp0, Pp1);
              else
                face_flux_dev<R>(rf, g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, zbm, zbp, F,
                                 Fa0, Fa1, Pm0, Pm1, Pp0, Pp1, true);
            } else
              face_flux<R>(g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, zbm, zbp, F, Fa0, Fa1,
                           Pm0, Pm1, Pp0, Pp1);
            const R jxw = fw * len;
            const R sg = side ? R(1) : R(-1);
            FV[k] = sg * F * jxw;
            FV[FVS + k] = sg * (Fa0 + (side ? Pp0 : Pm0)) * jxw;
            FV[2 * FVS + k] = sg * (Fa1 + (side ? Pp1 : Pm1)) * jxw;
          }
        } else
        for (int k = t; k < nf; k += T) {
          const int kp = orient ? nf - 1 - k : k;  // point index on the plus side
          const int ko = side ? kp : k, kn = side ? k : kp;
          R zo_ = 0, qo0 = 0, qo1 = 0, zn = 0, qn0 = 0, qn1 = 0;
#pragma unroll
          for (int i = 0; i < N; ++i) {  // own trace
            const int d = face_dof(N, fo, i);
            const R l = __ldg(&tbg.F[tsel][nf][ko][i]);
            fma2(zo_, qo0, l, U[d], l, U[NN + d]);
            qo1 += l * U[2 * NN + d];
          }
          const int nsel = side ? 0 : sub + 1;
#pragma unroll
          for (int i = 0; i < OC_MAXN; ++i) {  // neighbour trace (Nn <= OC_MAXN nodes)
            if (i < Nn) {
              const R l = __ldg(&tn.F[nsel][nf][kn][i]);
              fma2(zn, qn0, l, NB[(sl * 3 + 0) * OC_MAXN + i], l, NB[(sl * 3 + 1) * OC_MAXN + i]);
              qn1 += l * NB[(sl * 3 + 2) * OC_MAXN + i];
            }
          }
          const R zm = side ? zn : zo_, qm0 = side ? qn0 : qo0, qm1 = side ? qn1 : qo1;
          const R zp = side ? zo_ : zn, qp0 = side ? qo0 : qn0, qp1 = side ? qo1 : qn1;
          R zbm = MIX ? zbe_flat : R(0), zbp = zbm;
          if (!MIX && sdf_p) {
            zbm = (R)sdf_p[sdo + 2 * k]; zbp = (R)sdf_p[sdo + 2 * k + 1];
          }
          R F, Fa0, Fa1, Pm0, Pm1, Pp0, Pp1;
          if constexpr (MIX) {
            if (sdf_p)  // bathymetry: well-balanced differences in FP64
              face_flux_dev_wb_call<R>(rf, g, cu4, zref, zm, qm0, qm1, zp, qp0, qp1, n0, n1,
                                  sdf_p[sdo + 2 * k], sdf_p[sdo + 2 * k + 1],
                                  sdfe_p[sdo + 2 * k], sdfe_p[sdo + 2 * k + 1], F, Fa0, Fa1, Pm0,
                                  Pm1, Pp0, Pp1);
            else
              face_flux_dev<R>(rf, g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, zbm, zbp, F, Fa0,
                               Fa1, Pm0, Pm1, Pp0, Pp1, true);
          } else
            face_flux<R>(g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, zbm, zbp, F, Fa0, Fa1, Pm0,
                         Pm1, Pp0, Pp1);
          const R jxw = __ldg(&tbg.wF[nf][k]) * len;
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
      } else {  // boundary face
        const int sdo = cfsdo_p ? w_sdo[8 * team + sl] : 0;
        nfo = Q;
        tsel = -1;
        if constexpr (LEAN)
          boundary_slot_call<P, QR, R, MIX>(a, r.bid(), fo, sdo, on0, on1, len, geo, zref, g, cu4,
                                            U, FV, t);
        else
          boundary_slot<P, QR, R, MIX>(a, r.bid(), fo, sdo, on0, on1, len, geo, zref, g, cu4, U,
                                       FV, t);
      }
    }
    __syncwarp();
    // integration rows: registers when every face of the warp in this slot is a full
    // face of this degree's point set, else the global table copy (boundary faces:
    // Gauss rows; inner faces: the trace rows of the own side)
    const bool reg_cols = __all_sync(OC_FULL, nfo == 0 || (tsel == 0 && nfo == G));
    if (nfo > 0 && t < N) {  // integrate the own-side values against the own basis
      R cz = 0, c0 = 0, c1 = 0;
      if (reg_cols) {
#pragma unroll
        for (int k = 0; k < G; ++k) {
          fma2(cz, c0, fcol[k], FV[k], fcol[k], FV[FVS + k]);
          c1 += fcol[k] * FV[2 * FVS + k];
        }
      } else {
        const R *col = tsel < 0 ? (QR ? &tbg.BM[0][t] : &tbg.BQ[0][t]) : &tbg.F[tsel][nfo][0][t];  // stride OC_MAXN
#pragma unroll
        for (int k = 0; k < (Q > OC_MAXF ? Q : OC_MAXF); ++k) {  // nfo <= max(Q, OC_MAXF)
          if (k < nfo) {
            const R l = __ldg(col + k * OC_MAXN);
            fma2(cz, c0, l, FV[k], l, FV[FVS + k]);
            c1 += l * FV[2 * FVS + k];
          }
        }
      }
      const int d = fbase + t * fstride;
      RES[d] += cz;
      RES[NN + d] += c0;
      RES[2 * NN + d] += c1;
    }
    __syncwarp();
  }

  }

  // ---- apply(): dst = M^-1 L_h(src), exact Gauss p+1 inverse for all variables
  //      (not in the lean variants: apply() launches the general ones) ----
  if (!LEAN && a.apply_mode) {
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

  // independent instances with their own step size (time-step path): the cell's
  // residual scaled by dt_c / dt, so that every later sum f_j k_j carries it
  if (cscale_p) {
    if (member && t < N) {
      const R sc = MIX ? (R)__ldg(cscalef_p + cell) : (R)__ldg(cscale_p + cell);
#pragma unroll
      for (int e = 0; e < 3; ++e)
#pragma unroll
        for (int ix = 0; ix < N; ++ix) RES[e * NN + t * N + ix] *= sc;
    }
    __syncwarp();
  }

  // ---- 3. zeta: pre-lambda + local_apply_cell_mass_height (OceanDG.h:1830-1849)
  //         and local_apply_inverse_mass_matrix_height (:1373-1507) ------------
  // b = sum_{j<s} f_j kz_j (prologue) + f_s L_h zeta, in the reference's order
  if (member && t < N) {
#pragma unroll
    for (int ix = 0; ix < N; ++ix) {
      const int d = t * N + ix;
      BZ[d] = s == 0 ? fR[0] * RES[d] : BZ[d] + fRs * RES[d];
    }
  }
  __syncwarp();
  bool need_fp64 = !MIX;
  if (MIX) {
    const R wet_thr = (R)a.wet_thrf;
    const unsigned team_mask = ((1u << T) - 1u) << (team * T);
    // Without bathymetry data every Gauss-Lobatto point is wet when the nodal
    // |zeta - zeta_ref| stay below (zb + zeta_ref - threshold) / Lambda (Lambda: the
    // Lebesgue constant of the nodal basis at those points, with a margin for the
    // FP32 evaluation); only warps where that bound fails evaluate the points.
    const bool flat_zb = sd1e_p == nullptr;
    const R wet_lim = flat_zb ? (zbe_flat - wet_thr) / tb.lebG * R(0.999) : R(0);
    auto bound_wet = [&](const R *vals) {  // team-uniform
      bool ok = flat_zb;
      if (ok && member && t < N)
#pragma unroll
        for (int ix = 0; ix < N; ++ix) ok = ok && m_abs(vals[t * N + ix]) < wet_lim;
      return (__ballot_sync(OC_FULL, member && !ok) & team_mask) == 0u;
    };
    // wet check of u^n at the Gauss-Lobatto points (FP32 estimate)
    bool wet = true;
    const bool sure0 = bound_wet(ZN);
    const bool exact0 = __any_sync(OC_FULL, member && !sure0);
    const float *zb1e = sd1e_p ? sd1e_p + cell_data(a.err, a.sdo1, cell, a.n_sd[1], G * G) : nullptr;
    if (exact0)
      wet = LEAN ? gl_wet_call<P, QR, R>(ZN, X + NT, t, member, !sure0, zb1e, zbe_flat, wet_thr)
                 : gl_wet<P, QR, R>(ZN, X + NT, t, member, !sure0, zb1e, zbe_flat, wet_thr);
    // closed form of max_iter sweeps on fully wet cells: delta = A_K b (the 1D
    // factors applied to two output rows at a time in packed FMAs)
    if (member && t < N) {
#pragma unroll
      for (int ap = 0; ap < N; ap += 2) {
        R v0 = 0, v1 = 0;
#pragma unroll
        for (int ix = 0; ix < N; ++ix) {
          const R b = BZ[t * N + ix];
          if (ap + 1 < N) fma2(v0, v1, tb.W1[ap][ix], b, tb.W1[ap + 1][ix], b);
          else v0 += tb.W1[ap][ix] * b;
        }
        X[t * T + ap] = v0;
        if (ap + 1 < N) X[t * T + ap + 1] = v1;
      }
    }
    __syncwarp();
    if (member && t < N) {
      R c[N];
#pragma unroll
      for (int aa = 0; aa < N; aa += 2) {
        R v0 = 0, v1 = 0;
#pragma unroll
        for (int iy = 0; iy < N; ++iy) {
          const R x = X[iy * T + t];
          if (aa + 1 < N) fma2(v0, v1, tb.W1[aa][iy], x, tb.W1[aa + 1][iy], x);
          else v0 += tb.W1[aa][iy] * x;
        }
        c[aa] = v0 * tb.Gk[aa][t] / det;
        if (aa + 1 < N) c[aa + 1] = v1 * tb.Gk[aa + 1][t] / det;
      }
#pragma unroll
      for (int iy = 0; iy < N; iy += 2) {
        R v0 = 0, v1 = 0;
#pragma unroll
        for (int aa = 0; aa < N; ++aa) {
          if (iy + 1 < N) fma2(v0, v1, tb.W2[iy][aa], c[aa], tb.W2[iy + 1][aa], c[aa]);
          else v0 += tb.W2[iy][aa] * c[aa];
        }
        X[2 * NT + iy * T + t] = v0;
        if (iy + 1 < N) X[2 * NT + (iy + 1) * T + t] = v1;
      }
    }
    __syncwarp();
    if (member && t < N) {  // delta rows into tile 3, zeta' of the result into tile 4
#pragma unroll
      for (int ix = 0; ix < N; ix += 2) {
        R d0 = 0, d1 = 0;
#pragma unroll
        for (int ap = 0; ap < N; ++ap) {
          const R x = X[2 * NT + t * T + ap];
          if (ix + 1 < N) fma2(d0, d1, tb.W2[ix][ap], x, tb.W2[ix + 1][ap], x);
          else d0 += tb.W2[ix][ap] * x;
        }
        X[3 * NT + t * N + ix] = d0;
        X[4 * NT + t * N + ix] = ZN[t * N + ix] + d0;
        if (ix + 1 < N) {
          X[3 * NT + t * N + ix + 1] = d1;
          X[4 * NT + t * N + ix + 1] = ZN[t * N + ix + 1] + d1;
        }
      }
    }
    __syncwarp();
    // the closed form is the literal iteration only while every point stays wet:
    // check the result too, else redo the cell with the FP64 literal iteration
    const bool sure1 = bound_wet(X + 4 * NT);
    const bool exact1 = __any_sync(OC_FULL, member && !sure1);
    if (exact1) {  // all lanes call (the helper synchronises the warp)
      const bool w1 =
          LEAN ? gl_wet_call<P, QR, R>(X + 4 * NT, X + 5 * NT, t, member, !sure1, zb1e, zbe_flat,
                                       wet_thr)
               : gl_wet<P, QR, R>(X + 4 * NT, X + 5 * NT, t, member, !sure1, zb1e, zbe_flat,
                                  wet_thr);
      wet = wet && w1;
    }
    const unsigned drym = __ballot_sync(OC_FULL, member && !wet);  // team OR of "not wet"
    need_fp64 = ((drym >> (team * T)) & ((1u << T) - 1u)) != 0u;
  }
  if (__any_sync(OC_FULL, valid && need_fp64)) {
    // literal FP64 iteration (all lanes; teams with work = valid && need_fp64)
    const bool work = valid && need_fp64;
    zeta_literal_fp64<P, QR, R>(a, cell, zo, BZ, sd1_p, DZ, DX, DRED, warp_norm, team, cpw, t,
                                member, work);
    if (work && t == 0) w_flag[team] = 1;
  }
  if (MIX && member && t < N && !need_fp64) {  // wet: keep delta (FP32) in BZ
#pragma unroll
    for (int ix = 0; ix < N; ++ix) BZ[t * N + ix] = X[3 * NT + t * N + ix];
  }
  __syncwarp();

  // last stage of the mixed time step: u^n of the FP64 accumulation, loaded here
  // so that the loads overlap the discharge passes (lane element e = lane + 32 i)
  constexpr int EZ = (CPWMAX * NN + 31) / 32, EQ = (2 * CPWMAX * NN + 31) / 32;
  double unz[fast ? EZ : 1], unq[fast ? EQ : 1];
  if constexpr (fast) {
    if (a.out_z) {
#pragma unroll
      for (int i = 0; i < EZ; ++i) {
        const int e = lane + 32 * i;
        if (e < nvalid * NN) {
          const int j = e / NN, d = e - j * NN;
          unz[i] = a.un_z[w_off[j] + d];
        }
      }
    }
    if (!ark && a.out_q) {
#pragma unroll
      for (int i = 0; i < EQ; ++i) {
        const int e = lane + 32 * i;
        if (e < nvalid * 2 * NN) {
          const int j = e / (2 * NN), d = e - j * 2 * NN;
          unq[i] = a.un_q[2 * (int64_t)w_off[j] + d];
        }
      }
    }
  }

  // ---- 4. discharge: local_apply_inverse_mass_matrix_discharge (OceanDG.h:1532-1571);
  //         ARK: cell_mass_discharge + inverse_modified_mass (:1573-1645, :2086-2116) ----
  if (split) {
    // b = sum_j (f_j kex_j + ft_j kim_j); stores kex_s, kim_s
    R ftR[OC_MAXSTAGES];
    load_coefs<R>(a.dyn->fft, a.dyn->ft, ftR);
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
          R bsum = s == 0 ? fR[0] * kex + ftR[0] * kim
                          : fR[0] * (R) static_cast<const KT *>(a.kq[1])[gidx] +
                                ftR[0] * (R) static_cast<const KT *>(a.kq[2])[gidx];
#pragma unroll
          for (int j = 1; j < OC_MAXSTAGES; ++j) {
            if (j > s) break;
            const R ke = j == s ? kex : (R) static_cast<const KT *>(a.kq[2 * j + 1])[gidx];
            const R ki = j == s ? kim : (R) static_cast<const KT *>(a.kq[2 * j + 2])[gidx];
            bsum += fR[j] * ke + ftR[j] * ki;
          }
          RES[(1 + e) * NN + d] = bsum;
        }
    }
    __syncwarp();
  } else if (ark) {  // ARK last stage: b = f0 kex0 + sum_j (f_j kex_j + f_{j-1} kim_{j-1})
    if (member && t < N) {
#pragma unroll
      for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int ix = 0; ix < N; ++ix) {
          const int d = t * N + ix;
          const int64_t gidx = qo + e * NN + d;
          const R kex = RES[(1 + e) * NN + d];
          if (valid) static_cast<KT *>(a.kq[2 * s + 1])[gidx] = (KT)kex;
          R bsum = fR[0] * (s == 0 ? kex : (R) static_cast<const KT *>(a.kq[1])[gidx]);
#pragma unroll
          for (int j = 1; j < OC_MAXSTAGES; ++j) {
            if (j > s) break;
            const R ke = j == s ? kex : (R) static_cast<const KT *>(a.kq[2 * j + 1])[gidx];
            const R ki = (R) static_cast<const KT *>(a.kq[2 * j])[gidx];
            bsum += fR[j] * ke + fR[j - 1] * ki;
          }
          RES[(1 + e) * NN + d] = bsum;
        }
    }
    __syncwarp();
  }
  // coefficient of the diagonal (JxW)^-1 at Gauss p+1; ARK internal: modified mass
  // (OceanDG.h:1573-1645): (JxW (1 + fm J_fric(r)))^-1
  R coef[N];  // column qx = t: coef[qy]
#pragma unroll
  for (int i = 0; i < N; ++i) coef[i] = 0;
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
    const R fmR = sizeof(R) == 4 ? (R)__ldg(&a.dyn->ffm) : (R)__ldg(&a.dyn->fm);
    R m0[N], m1[N];  // MIX: y-integrated correction; FP64: y-integrated M q^n
#pragma unroll
    for (int i = 0; i < N; ++i) m0[i] = m1[i] = 0;
    if (member && t < N) {
      const int64_t so2 = sd2_p ? cell_data(a.err, a.sdo2, cell, a.n_sd[2], 2 * NN) : 0;
      const double *sd2 = sd2_p ? sd2_p + so2 : nullptr;
      const float *sd2e = sd2e_p ? sd2e_p + so2 : nullptr;
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
        if constexpr (MIX) velocity<R>(vz, rf.qr0 + v0, rf.qr1 + v1, zb, cu4, u0, u1);
        else velocity<R>(vz, v0, v1, zb, cu4, u0, u1);
        const R jf = friction_jac<R>(friction_m, g, u0, u1, cf, depth<R>(vz, zb));
        const R jxw = tb.wM[t] * tb.wM[qy] * det;
        coef[qy] = R(1) / jxw;
        coef[qy] *= R(1) / (R(1) + fmR * jf);
        const R wq = MIX ? jxw * fmR * jf : jxw;  // MIX: correction; FP64: mass of q^n
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
  // S^-1 diag(coef) S^-T applied to the two discharge components of RES (in place);
  // both components in one pass, their sums paired in packed FMAs
  if (member && t < N) {  // x-pass: A[iy][qx] = sum_ix Sinv[ix][qx] in[iy][ix]
#pragma unroll
    for (int qx = 0; qx < N; ++qx) {
      R v0 = 0, v1 = 0;
#pragma unroll
      for (int ix = 0; ix < N; ++ix)
        fma2(v0, v1, tb.Sinv[ix][qx], RES[NN + t * N + ix], tb.Sinv[ix][qx],
             RES[2 * NN + t * N + ix]);
      X[0 * NT + t * T + qx] = v0;
      X[1 * NT + t * T + qx] = v1;
    }
  }
  __syncwarp();
  if (member && t < N) {  // y on column qx = t: scale, back-transform in y
    R b0[N], b1[N];
#pragma unroll
    for (int qy = 0; qy < N; ++qy) {
      R v0 = 0, v1 = 0;
#pragma unroll
      for (int iy = 0; iy < N; ++iy)
        fma2(v0, v1, tb.Sinv[iy][qy], X[0 * NT + iy * T + t], tb.Sinv[iy][qy],
             X[1 * NT + iy * T + t]);
      b0[qy] = v0 * coef[qy];
      b1[qy] = v1 * coef[qy];
    }
#pragma unroll
    for (int iy = 0; iy < N; ++iy) {
      R v0 = 0, v1 = 0;
#pragma unroll
      for (int qy = 0; qy < N; ++qy) fma2(v0, v1, tb.Sinv[iy][qy], b0[qy], tb.Sinv[iy][qy], b1[qy]);
      X[2 * NT + iy * T + t] = v0;
      X[3 * NT + iy * T + t] = v1;
    }
  }
  __syncwarp();
  if (member && t < N) {  // x back-transform into RES_q
#pragma unroll
    for (int ix = 0; ix < N; ++ix) {
      R v0 = 0, v1 = 0;
#pragma unroll
      for (int qx = 0; qx < N; ++qx)
        fma2(v0, v1, tb.Sinv[ix][qx], X[2 * NT + t * T + qx], tb.Sinv[ix][qx],
             X[3 * NT + t * T + qx]);
      RES[NN + t * N + ix] = v0;
      RES[2 * NN + t * N + ix] = v1;
    }
  }
  __syncwarp();

  // ---- 5. epilogue: warp-cooperative RK update and stores ------------------------
  // FP64 form and the reference-ABI stage: next = u^n + sum_j f_j k_j in FP64.
  // Mixed time step (fast): delta = sum_j f_j k_j in FP32; internal stages store
  // u^n_f32 + delta (FP32), the last stage accumulates u^n + delta in FP64.
  KT *kz_out = static_cast<KT *>(a.kz[s + 1]);
  bool nonfinite = false;  // a non-finite value in u^{n+1} (last stage)
  if constexpr (fast) {
    // FP32 stage input u^n_f32 + delta; FP64 result only at the last stage (its
    // own loop, so that no FP64 work is issued at the internal stages)
    const bool anyflag = __any_sync(OC_FULL, lane < CPWMAX && lane < nvalid && w_flag[lane]);
#pragma unroll 2
    for (int e = lane; e < nvalid * NN; e += 32) {
      const int j = e / NN, d = e - j * NN;
      const int64_t gz = w_off[j] + d;
      const R *Rj = Rreg(j);
      kz_out[gz] = (KT)Rj[3 * NN + d];
      if (s == 0 && a.out_unzf) a.out_unzf[gz] = (float)Rj[9 * NN + d];
      if (a.out_rz) a.out_rz[gz] = (float)(Rj[9 * NN + d] + Rj[8 * NN + d]);
    }
    if (a.out_z) {
#pragma unroll
      for (int i = 0; i < EZ; ++i) {
        const int e = lane + 32 * i;
        if (e < nvalid * NN) {
          const int j = e / NN, d = e - j * NN;
          const double v = unz[i] + (double)Rreg(j)[8 * NN + d];
          a.out_z[w_off[j] + d] = v;
          nonfinite |= !isfinite(v);
        }
      }
    }
    if (anyflag) {  // cells that took the FP64 literal iteration (rare)
      for (int e = lane; e < nvalid * NN; e += 32) {
        const int j = e / NN, d = e - j * NN;
        if (!w_flag[j]) continue;
        const int64_t gz = w_off[j] + d;
        const double *DZj = Dreg(j);
        if (a.out_z) a.out_z[gz] = DZj[d];
        if (a.out_rz) a.out_rz[gz] = (float)(DZj[d] - zref);
        nonfinite |= a.last && !isfinite(DZj[d]);
      }
    }
  } else {
#pragma unroll 2
    for (int e = lane; e < nvalid * NN; e += 32) {  // zeta
      const int j = e / NN, d = e - j * NN;
      const int64_t gz = w_off[j] + d;
      const R *Rj = Rreg(j);
      kz_out[gz] = (KT)Rj[3 * NN + d];
      double zn;
      if (w_flag[j]) {
        const double *DZj = Dreg(j);
        zn = DZj[d];
      } else {
        zn = a.un_z[gz] + (double)Rj[8 * NN + d];
      }
      if (a.out_z) a.out_z[gz] = zn;
      nonfinite |= a.last && !isfinite(zn);
      if (MIX && a.out_rz) a.out_rz[gz] = (float)(zn - zref);
    }
  }
  const bool wkq = !ark && (!a.last || a.write_kq_last);
  if (fast && !ark) {
    // delta = sum_j f_j k_q[j+1] in FP32 (kept in smem for the FP64 loop)
#pragma unroll 2
    for (int e = lane; e < nvalid * 2 * NN; e += 32) {
      const int j = e / (2 * NN), d = e - j * 2 * NN;
      const int64_t gq = 2 * (int64_t)w_off[j] + d;
      R *Rj = Rreg(j);
      const R v = Rj[4 * NN + d];
      if (wkq) static_cast<KT *>(a.kq[s + 1])[gq] = (KT)v;
      // QB (prologue) = q^n + sum_{j<s} f_j k_q[j+1] (internal stages) or the sum alone
      const R up = Rj[6 * NN + d] + fRs * v;
      if (s == 0 && a.out_unqf) a.out_unqf[gq] = (float)Rj[NN + d];
      if (a.out_rq) a.out_rq[gq] = (float)up;
      Rj[4 * NN + d] = up;  // last stage: delta for the FP64 accumulation
    }
    if (a.out_q) {
#pragma unroll
      for (int i = 0; i < EQ; ++i) {
        const int e = lane + 32 * i;
        if (e < nvalid * 2 * NN) {
          const int j = e / (2 * NN), d = e - j * 2 * NN;
          const double v = unq[i] + (double)Rreg(j)[4 * NN + d];
          a.out_q[2 * (int64_t)w_off[j] + d] = v;
          nonfinite |= !isfinite(v);
        }
      }
    }
    report_nonfinite(a, nonfinite);
    return;
  }
  // (the lean mixed variant always returned above: no unreachable-loop warning)
#pragma nv_diag_suppress 128
#pragma unroll 2
  for (int e = lane; e < nvalid * 2 * NN; e += 32) {  // discharge
    const int j = e / (2 * NN), d = e - j * 2 * NN;
    const int64_t gq = 2 * (int64_t)w_off[j] + d;
    const R v = Rreg(j)[4 * NN + d];  // RES[NN + d] of team j
    double nxt;
    if (!ark) {
      // ERK: k_q[s+1] = M^-1 L_h q; next = q^n + sum_j f_j k_q[j+1]
      const double kc = (double)(KT)v;
      if (wkq) static_cast<KT *>(a.kq[s + 1])[gq] = (KT)v;
      const double *fd = a.dyn->f;
      double acc = a.un_q[gq] + fd[0] * (s == 0 ? kc : (double)static_cast<const KT *>(a.kq[1])[gq]);
#pragma unroll
      for (int jj = 1; jj < OC_MAXSTAGES; ++jj)
        if (jj <= s) acc += fd[jj] * (jj == s ? kc : (double)static_cast<const KT *>(a.kq[jj + 1])[gq]);
      nxt = acc;
    } else if (!a.last) {
      nxt = MIX ? a.un_q[gq] + (double)v : (double)v;
    } else {
      if (a.aux_q) a.aux_q[gq] = (double)v;
      nxt = a.un_q[gq] + (double)v;
    }
    if (a.out_q) a.out_q[gq] = nxt;
    nonfinite |= a.last && !isfinite(nxt);
    if (MIX && a.out_rq) a.out_rq[gq] = (float)(nxt - (d < NN ? qref0 : qref1));
  }
  report_nonfinite(a, nonfinite);
}

// Launch of a stage kernel with programmatic stream serialization: its blocks may
// be scheduled while the previous kernel of the stream drains (that kernel lets
// them with griddepcontrol.launch_dependents); the kernel reads only mesh data
// before its griddepcontrol.wait.  Valid inside stream capture (the graph keeps
// a programmatic edge).
template <typename K>
static cudaError_t launch_programmatic(K kernel, int grid, int threads, int smem,
                                       cudaStream_t st, const StageArgs &a) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, a);
}

// One degree group per launch.
template <int P, typename R, typename KT, bool MIX, typename RIN, bool LEAN, int QR, bool CONF>
__global__ void __launch_bounds__(128, MIX ? OC_MIXED_MIN_BLOCKS : 1) stage_kernel(const StageArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  stage_body<P, R, KT, MIX, RIN, LEAN, QR, CONF>(a, smem_raw, blockIdx.x, a.n_group,
                                                 a.group_cells, a.group_first);
}

// Every degree group of an hp mesh in one launch: the grid is the concatenation
// of the groups' block ranges, most expensive degree first (a.hp_first_block[p],
// a.hp_blocks[p]); each block runs the body of its degree.
#ifndef OC_HP_MIN_BLOCKS
#define OC_HP_MIN_BLOCKS 4
#endif
template <typename R, typename KT, bool MIX, typename RIN, bool LEAN>
__global__ void __launch_bounds__(128, MIX ? OC_HP_MIN_BLOCKS : 1) stage_kernel_hp(const StageArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int b = blockIdx.x;
#define OC_HP_CASE(P)                                                                          \
  if (b >= a.hp_first_block[P] && b < a.hp_first_block[P] + a.hp_blocks[P]) {                 \
    stage_body<P, R, KT, MIX, RIN, LEAN, 0, false>(a, smem_raw, b - a.hp_first_block[P],      \
                                                   a.hp_n[P], a.hp_cells[P], 0);               \
    return;                                                                                    \
  }
  OC_HP_CASE(4)
  OC_HP_CASE(3)
  OC_HP_CASE(2)
  OC_HP_CASE(1)
#undef OC_HP_CASE
}

}  // namespace oc
