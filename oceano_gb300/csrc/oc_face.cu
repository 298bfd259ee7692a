// Face pass of an FP64 stage: the numerical flux of every face evaluated once.
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
// The FP64 form is bound by the FP64 pipe, so evaluating each flux once instead
// of once per side pays for the extra pass; the mixed form evaluates its faces
// in the stage kernel.
#include "oc_kernels.cuh"

namespace oc {

// Point values of one inner face (minus side at point k, plus side at point kp)
using R = double;
__device__ __forceinline__ void face_point(const StageArgs &a, R g, R cu4, int fsd, int k, int kp,
                                           int nf, R n0, R n1, R jxw, R zm, R qm0, R qm1, R zp,
                                           R qp0, R qp1, R *outm, R *outp) {
  R F, Fa0, Fa1, Pm0, Pm1, Pp0, Pp1;
  const R zbm = a.sdf ? __ldg(a.sdf + fsd + 2 * k) : R(0);
  const R zbp = a.sdf ? __ldg(a.sdf + fsd + 2 * k + 1) : R(0);
  face_flux<R>(g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, zbm, zbp, F, Fa0, Fa1, Pm0, Pm1, Pp0,
               Pp1);
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
template <int P>
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
  const int cm = (int)checked(a.err, __ldg(a.fcm + f), a.n_cells, BS_FACE_CELL);
  const int pm = P ? P : checked_degree(a.err, __ldg(a.deg + cm)), Nm = pm + 1;
  const int64_t om = checked(
      a.err, a.uniform_nn ? (int64_t)cm * a.uniform_nn : (int64_t)__ldg(a.off + cm),
      a.n_dofs - Nm * Nm + 1, BS_OFFSET);
  const bool inner = f < a.n_inner;
  const int nf = P ? P + 2 : (fpk >> 16) & 15;  // points of an inner face
  const int Qm = a.cell_rule ? pm + 1 : (3 * pm) / 2 + 1;  // points of a boundary face
#ifdef OC_BOUNDS_CHECK
  if (inner && (nf < 2 || nf > OC_MAXF || ((fpk >> 8) & 15) > 2)) {  // pack word: nf, subface
    checked(a.err, fpk, 0, BS_RECORD);
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    return;
  }
#endif
  const int64_t fo =
      checked(a.err, __ldg(a.fofs + f), a.n_fout - (inner ? 6 * nf : 3 * Qm) + 1, BS_FACE_OUT);
  R *out = static_cast<R *>(a.fout) + fo;
  int fsd = __ldg(a.fsd + f);
  if (inner ? a.sdf != nullptr : a.sdb != nullptr)
    fsd = (int)checked(a.err, fsd, inner ? a.n_sd[3] - 2 * nf + 1 : a.n_sd[4] - Qm + 1,
                       BS_FACE_DATA);
  const R n0 = __ldg(a.fnrm + 2 * f), n1 = __ldg(a.fnrm + 2 * f + 1), len = __ldg(a.flen + f);
  const DegTables<R> *gt = reinterpret_cast<const DegTables<R> *>(a.gtabd);
  const R g = a.g, cu4 = a.cu4;
  const double *rz = static_cast<const double *>(a.rz), *rq = static_cast<const double *>(a.rq);
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
      zmn[n] = __ldg(rz + om + d);
      qm0n[n] = __ldg(rq + 2 * om + d);
      qm1n[n] = __ldg(rq + 2 * om + Nm * Nm + d);
    }
  }
  if (inner) {
    const int fp = (fpk >> 4) & 15, sub = ((fpk >> 8) & 15) - 1, orient = (fpk >> 12) & 15;
    const int cp = (int)checked(a.err, __ldg(a.fcp + f), a.n_cells, BS_FACE_CELL);
    const int pp = P ? P : checked_degree(a.err, __ldg(a.deg + cp)), Np = pp + 1;
    const int64_t op = checked(
        a.err, a.uniform_nn ? (int64_t)cp * a.uniform_nn : (int64_t)__ldg(a.off + cp),
        a.n_dofs - Np * Np + 1, BS_OFFSET);
    R zpn[NMAX], qp0n[NMAX], qp1n[NMAX];
#pragma unroll
    for (int n = 0; n < NMAX; ++n) {
      zpn[n] = qp0n[n] = qp1n[n] = R(0);
      if (P || n < Np) {
        const int d = face_dof(Np, fp, n);
        zpn[n] = __ldg(rz + op + d);
        qp0n[n] = __ldg(rq + 2 * op + d);
        qp1n[n] = __ldg(rq + 2 * op + Np * Np + d);
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
        face_point(a, g, cu4, fsd, k, kp, G, n0, n1, tc.wF[G][k] * len, zm, qm0, qm1, zp, qp0,
                   qp1, outm, outp);
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
        face_point(a, g, cu4, fsd, k, kp, nf, n0, n1, __ldg(&tm.wF[nf][k]) * len, zm, qm0, qm1,
                   zp, qp0, qp1, outm, outp);
      }
    }
  } else {  // boundary face: Gauss n_q points of the cell
    const int b = f - a.n_inner;
    const int bid = (int)checked(a.err, __ldg(a.bbid + b), OC_MAXBID, BS_BOUNDARY);
    const int bkind = a.bc_kind[bid];
    if (bkind == 0) {
      atomicOr(a.err, ERR_UNKNOWN_BID);
      return;
    }
    const int Q = Qm;
    const DegTables<R> &tm = gt[pm - 1];
    // the cell Gauss rule's rows: floor(1.5 p) + 1 points, or the Gauss p+1 tables
    const R(*BQ)[OC_MAXN] = a.cell_rule ? tm.BM : tm.BQ;
    const R *wQ = a.cell_rule ? tm.wM : tm.wQ;
    const R *xQ = a.cell_rule ? tm.xM : tm.xQ;
    const double *geo = a.geo + 11 * (int64_t)cm;
#pragma unroll 1
    for (int k = 0; k < Q; ++k) {
      R zm = 0, qm0 = 0, qm1 = 0;
#pragma unroll
      for (int n = 0; n < NMAX; ++n) {
        if (P || n < Nm) {
          const R l = __ldg(&BQ[k][n]);
          zm += l * zmn[n]; qm0 += l * qm0n[n]; qm1 += l * qm1n[n];
        }
      }
      R F, Fa0, Fa1;
      boundary_flux<R, false>(a, bid, bkind, fm, __ldg(&xQ[k]), geo, 0.0, fsd + k, g, cu4, zm,
                              qm0, qm1, n0, n1, F, Fa0, Fa1);
      const R jxw = __ldg(&wQ[k]) * len;
      out[k] = -F * jxw;
      out[Q + k] = -Fa0 * jxw;
      out[2 * Q + k] = -Fa1 * jxw;
    }
  }
}

// uniform_p: the degree of every cell, 0 for mixed degrees.
cudaError_t launch_face_pass(const StageArgs &a, int uniform_p, cudaStream_t st) {
  const int nfaces = a.n_inner + a.n_bnd_faces;
  if (nfaces == 0) return cudaSuccess;
  const int threads = 128;
  const int grid = (nfaces + threads - 1) / threads;
  switch (uniform_p) {
    case 1: return launch_programmatic(face_kernel<1>, grid, threads, 0, st, a);
    case 2: return launch_programmatic(face_kernel<2>, grid, threads, 0, st, a);
    case 3: return launch_programmatic(face_kernel<3>, grid, threads, 0, st, a);
    case 4: return launch_programmatic(face_kernel<4>, grid, threads, 0, st, a);
    default: return launch_programmatic(face_kernel<0>, grid, threads, 0, st, a);
  }
}

cudaError_t face_upload_tables(const DegTables<double> *td, const DegTables<float> *tf) {
  cudaError_t e = cudaMemcpyToSymbol(c_tabd, td, sizeof(DegTables<double>) * OC_MAXDEG);
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_tabf, tf, sizeof(DegTables<float>) * OC_MAXDEG);
}

}  // namespace oc
