// Face pass of a stage: the numerical flux of every face evaluated once.
//
// local_apply_face_height / _discharge (OceanDG.h:936-1050) and
// local_apply_boundary_face_* (:1105-1339) are face integrals: the reference's
// MatrixFree::loop visits every face once and submits the flux to both sides.
// Here one thread evaluates one face: it loads both sides' face nodes once and,
// at every quadrature point, interpolates the two traces (Gauss-Lobatto nodes
// on the face, subface rows on the coarse side of a hanging face), evaluates the
// Lax-Friedrichs mass and advective fluxes with hydrostatic reconstruction and
// the pressure jump of each side, and writes, per side, the three point values
// (mass, x and y discharge) already multiplied by the side's sign and JxW.  The
// stage kernel then integrates each side's values against its own basis.  The
// output of inner face f starts at fofs[f]: minus side [3][nf], then plus side
// [3][nf] in the plus side's point order; boundary face values [3][Q].
#include "oc_kernels.cuh"

namespace oc {

// Point values of one inner face (minus side at point k, plus side at point kp)
template <typename R, bool MIX>
__device__ __forceinline__ void face_point(const StageArgs &a, R g, R cu4, double zref, int fsd,
                                           int k, int kp, int nf, R n0, R n1, R jxw, R zm,
                                           R qm0, R qm1, R zp, R qp0, R qp1, R *outm, R *outp) {
  const RefStateF &rf = a.ref;
  R F, Fa0, Fa1, Pm0, Pm1, Pp0, Pp1;
  if constexpr (MIX) {
    if (a.sdf)  // bathymetry: well-balanced differences in FP64
      face_flux_dev_wb<R>(rf, g, cu4, zref, zm, qm0, qm1, zp, qp0, qp1, n0, n1,
                          __ldg(a.sdf + fsd + 2 * k), __ldg(a.sdf + fsd + 2 * k + 1),
                          __ldg(a.sdfe + fsd + 2 * k), __ldg(a.sdfe + fsd + 2 * k + 1), F, Fa0,
                          Fa1, Pm0, Pm1, Pp0, Pp1);
    else
      face_flux_dev<R>(rf, g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, (R)a.zreff, (R)a.zreff, F,
                       Fa0, Fa1, Pm0, Pm1, Pp0, Pp1, true);
  } else {
    const R zbm = a.sdf ? (R)__ldg(a.sdf + fsd + 2 * k) : R(0);
    const R zbp = a.sdf ? (R)__ldg(a.sdf + fsd + 2 * k + 1) : R(0);
    face_flux<R>(g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, zbm, zbp, F, Fa0, Fa1, Pm0, Pm1, Pp0,
                 Pp1);
  }
  outm[k] = -F * jxw;
  outm[nf + k] = -(Fa0 + Pm0) * jxw;
  outm[2 * nf + k] = -(Fa1 + Pm1) * jxw;
  outp[kp] = F * jxw;
  outp[nf + kp] = (Fa0 + Pp0) * jxw;
  outp[2 * nf + kp] = (Fa1 + Pp1) * jxw;
}

// One thread per face: the face nodes of both sides are loaded once, then every
// quadrature point of the face is evaluated.  P > 0: every cell has degree P
// (shape rows from the constant bank, compile-time loops); P = 0: any degrees
// (rows from the global table copy).  Inner faces first, then boundary faces.
template <int P, typename R, bool MIX, typename RIN>
__global__ void __launch_bounds__(128) face_kernel(const StageArgs a) {
  // the stage kernel of this stage may be scheduled now; it waits for this grid
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int nfaces = a.n_inner + a.n_bnd_faces;
  if (f >= nfaces) {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    return;
  }
  // mesh data only before the wait (written before the stream's first stage)
  const int fpk = __ldg(a.fpack + f);
  const int cm = __ldg(a.fcm + f);
  const int pm = P ? P : __ldg(a.deg + cm), Nm = pm + 1;
  const int64_t om = a.uniform_nn ? (int64_t)cm * a.uniform_nn : (int64_t)__ldg(a.off + cm);
  R *out = static_cast<R *>(a.fout) + __ldg(a.fofs + f);
  const int fsd = __ldg(a.fsd + f);
  R n0, n1, len;
  if constexpr (MIX) {
    n0 = __ldg(a.fnrmf + 2 * f); n1 = __ldg(a.fnrmf + 2 * f + 1); len = __ldg(a.flenf + f);
  } else {
    n0 = __ldg(a.fnrm + 2 * f); n1 = __ldg(a.fnrm + 2 * f + 1); len = __ldg(a.flen + f);
  }
  const DegTables<R> *gt = reinterpret_cast<const DegTables<R> *>(
      sizeof(R) == 4 ? (const void *)a.gtabf : (const void *)a.gtabd);
  const double zref = MIX ? a.zeta_ref : 0.0;
  const double qref0 = MIX ? a.q_ref[0] : 0.0, qref1 = MIX ? a.q_ref[1] : 0.0;
  const R g = MIX ? (R)a.gf : (R)a.g, cu4 = MIX ? (R)a.cu4f : (R)a.cu4;
  const int fm = fpk & 15;
  constexpr int NMAX = P ? P + 1 : OC_MAXN;
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  // minus-side face nodes
  R zmn[NMAX], qm0n[NMAX], qm1n[NMAX];
#pragma unroll
  for (int n = 0; n < NMAX; ++n) {
    zmn[n] = qm0n[n] = qm1n[n] = R(0);
    if (P || n < Nm) {
      const int d = face_dof(Nm, fm, n);
      zmn[n] = load_in<RIN, R>(a.rz, om + d, zref);
      qm0n[n] = load_in<RIN, R>(a.rq, 2 * om + d, qref0);
      qm1n[n] = load_in<RIN, R>(a.rq, 2 * om + Nm * Nm + d, qref1);
    }
  }
  if (f < a.n_inner) {
    const int fp = (fpk >> 4) & 15, sub = ((fpk >> 8) & 15) - 1, orient = (fpk >> 12) & 15;
    const int nf = P ? P + 2 : (fpk >> 16) & 15;
    const int cp = __ldg(a.fcp + f);
    const int pp = P ? P : __ldg(a.deg + cp), Np = pp + 1;
    const int64_t op = a.uniform_nn ? (int64_t)cp * a.uniform_nn : (int64_t)__ldg(a.off + cp);
    R zpn[NMAX], qp0n[NMAX], qp1n[NMAX];
#pragma unroll
    for (int n = 0; n < NMAX; ++n) {
      zpn[n] = qp0n[n] = qp1n[n] = R(0);
      if (P || n < Np) {
        const int d = face_dof(Np, fp, n);
        zpn[n] = load_in<RIN, R>(a.rz, op + d, zref);
        qp0n[n] = load_in<RIN, R>(a.rq, 2 * op + d, qref0);
        qp1n[n] = load_in<RIN, R>(a.rq, 2 * op + Np * Np + d, qref1);
      }
    }
    R *outm = out, *outp = out + 3 * nf;
    const DegTables<R> &tm = gt[pm - 1], &tp = gt[pp - 1];
    if constexpr (P > 0) {
      constexpr int G = P + 2;
      const DegTables<R> &tc = tab<R>(P);
      const bool plain = sub < 0 && orient == 0;  // conforming, standard orientation
#pragma unroll
      for (int k = 0; k < G; ++k) {
        const int kp = orient ? G - 1 - k : k;
        R zm = 0, qm0 = 0, qm1 = 0, zp = 0, qp0 = 0, qp1 = 0;
#pragma unroll
        for (int n = 0; n < P + 1; ++n) {
          const R l = tc.F[0][G][k][n];
          zm += l * zmn[n]; qm0 += l * qm0n[n]; qm1 += l * qm1n[n];
          const R lp = plain ? l : __ldg(&tp.F[sub + 1][G][kp][n]);
          zp += lp * zpn[n]; qp0 += lp * qp0n[n]; qp1 += lp * qp1n[n];
        }
        face_point<R, MIX>(a, g, cu4, zref, fsd, k, kp, G, n0, n1, tc.wF[G][k] * len, zm, qm0,
                           qm1, zp, qp0, qp1, outm, outp);
      }
    } else {
#pragma unroll 1
      for (int k = 0; k < nf; ++k) {
        const int kp = orient ? nf - 1 - k : k;
        R zm = 0, qm0 = 0, qm1 = 0, zp = 0, qp0 = 0, qp1 = 0;
#pragma unroll
        for (int n = 0; n < OC_MAXN; ++n) {
          if (n < Nm) {
            const R l = __ldg(&tm.F[0][nf][k][n]);
            zm += l * zmn[n]; qm0 += l * qm0n[n]; qm1 += l * qm1n[n];
          }
          if (n < Np) {
            const R l = __ldg(&tp.F[sub + 1][nf][kp][n]);
            zp += l * zpn[n]; qp0 += l * qp0n[n]; qp1 += l * qp1n[n];
          }
        }
        face_point<R, MIX>(a, g, cu4, zref, fsd, k, kp, nf, n0, n1, __ldg(&tm.wF[nf][k]) * len,
                           zm, qm0, qm1, zp, qp0, qp1, outm, outp);
      }
    }
  } else {  // boundary face: Gauss n_q points of the cell
    const int b = f - a.n_inner;
    const int bid = __ldg(a.bbid + b);
    const int bkind = a.bc_kind[bid];
    if (bkind == 0) {
      atomicOr(a.err, ERR_UNKNOWN_BID);
      return;
    }
    const int Q = (3 * pm) / 2 + 1;
    const DegTables<R> &tm = gt[pm - 1];
    const DegTables<double> &td = reinterpret_cast<const DegTables<double> *>(a.gtabd)[pm - 1];
    const double *geo = a.geo + 11 * (int64_t)cm;
#pragma unroll 1
    for (int k = 0; k < Q; ++k) {
      R zm = 0, qm0 = 0, qm1 = 0;
#pragma unroll
      for (int n = 0; n < NMAX; ++n) {
        if (P || n < Nm) {
          const R l = __ldg(&tm.BQ[k][n]);
          zm += l * zmn[n]; qm0 += l * qm0n[n]; qm1 += l * qm1n[n];
        }
      }
      R F, Fa0, Fa1;
      boundary_flux<R, MIX>(a, bid, bkind, fm, __ldg(&td.xQ[k]), geo, zref, fsd + k, g, cu4, zm,
                            qm0, qm1, n0, n1, F, Fa0, Fa1);
      const R jxw = __ldg(&tm.wQ[k]) * len;
      out[k] = -F * jxw;
      out[Q + k] = -Fa0 * jxw;
      out[2 * Q + k] = -Fa1 * jxw;
    }
  }
}

// FP32 deviations of the FP64 state, (zeta - zeta_ref, q - q_ref): the stage
// input of the first stage of the mixed time step, and the copy of u^n its later
// stages read.  One thread per (cell, node) slot of the largest degree.
__global__ void __launch_bounds__(256) unf32_kernel(const StageArgs a, const double *z,
                                                    const double *q, float *zf, float *qf) {
  constexpr int S = OC_MAXN * OC_MAXN;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c = i / S;
  const int d = (int)(i - c * S);
  if (c >= a.n_cells) return;
  const int N = __ldg(a.deg + c) + 1, NN = N * N;
  if (d >= NN) return;
  const int64_t o = a.uniform_nn ? c * a.uniform_nn : (int64_t)__ldg(a.off + c);
  zf[o + d] = (float)(__ldg(z + o + d) - a.zeta_ref);
  qf[2 * o + d] = (float)(__ldg(q + 2 * o + d) - a.q_ref[0]);
  qf[2 * o + NN + d] = (float)(__ldg(q + 2 * o + NN + d) - a.q_ref[1]);
}

cudaError_t launch_unf32(const StageArgs &a, const double *z, const double *q, float *zf,
                         float *qf, cudaStream_t st) {
  const int64_t n = (int64_t)a.n_cells * OC_MAXN * OC_MAXN;
  unf32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a, z, q, zf, qf);
  return cudaGetLastError();
}

template <int P>
static cudaError_t launch_face_p(const StageArgs &a, int variant, int grid, int threads,
                                 cudaStream_t st) {
  if (variant == 0)
    return launch_programmatic(face_kernel<P, double, false, double>, grid, threads, 0, st, a);
  if (a.r_is_float)
    return launch_programmatic(face_kernel<P, float, true, float>, grid, threads, 0, st, a);
  return launch_programmatic(face_kernel<P, float, true, double>, grid, threads, 0, st, a);
}

// variant 0: FP64; 1: mixed with FP32 stage input; 2: mixed with FP64 stage input.
// uniform_p: the degree of every cell, 0 for mixed degrees.
cudaError_t launch_face_pass(const StageArgs &a, int variant, int uniform_p, cudaStream_t st) {
  const int nfaces = a.n_inner + a.n_bnd_faces;
  if (nfaces == 0) return cudaSuccess;
  const int threads = 128;
  const int grid = (nfaces + threads - 1) / threads;
  switch (uniform_p) {
    case 1: return launch_face_p<1>(a, variant, grid, threads, st);
    case 2: return launch_face_p<2>(a, variant, grid, threads, st);
    case 3: return launch_face_p<3>(a, variant, grid, threads, st);
    case 4: return launch_face_p<4>(a, variant, grid, threads, st);
    default: return launch_face_p<0>(a, variant, grid, threads, st);
  }
}

cudaError_t face_upload_tables(const DegTables<double> *td, const DegTables<float> *tf) {
  cudaError_t e = cudaMemcpyToSymbol(c_tabd, td, sizeof(DegTables<double>) * OC_MAXDEG);
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_tabf, tf, sizeof(DegTables<float>) * OC_MAXDEG);
}

}  // namespace oc
