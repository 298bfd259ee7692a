// Face pass of a stage: the numerical flux of every face evaluated once.
//
// local_apply_face_height / _discharge (OceanDG.h:936-1050) and
// local_apply_boundary_face_* (:1105-1339) are face integrals: the reference's
// MatrixFree::loop visits every face once and submits the flux to both sides.
// Here one thread evaluates one quadrature point of one face: it interpolates
// both sides' face traces from the stage input (Gauss-Lobatto nodes on the
// face, subface rows on the coarse side of a hanging face), evaluates the
// Lax-Friedrichs mass and advective fluxes with hydrostatic reconstruction and
// the pressure jump of each side, and writes, per side, the three point values
// (mass, x and y discharge) already multiplied by the side's sign and JxW.  The
// stage kernel then integrates each side's values against its own basis.  The
// output of inner face f starts at fofs[f]: minus side [3][nf], then plus side
// [3][nf] in the plus side's point order; boundary face values [3][Q].
#include "oc_kernels.cuh"

namespace oc {

template <typename R, bool MIX, typename RIN>
__global__ void __launch_bounds__(256) face_kernel(const StageArgs a) {
  // the stage kernel of this stage may be scheduled now; it waits for this grid
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= a.n_fpts) {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    return;
  }
  // mesh data only before the wait (written before the stream's first stage)
  const int item = __ldg(a.fpts + i);
  const int f = item >> 3, k = item & 7;
  const int fpk = __ldg(a.fpack + f);
  const int cm = __ldg(a.fcm + f);
  const int pm = __ldg(a.deg + cm), Nm = pm + 1;
  const int64_t om = a.uniform_nn ? (int64_t)cm * a.uniform_nn : (int64_t)__ldg(a.off + cm);
  const int64_t base = __ldg(a.fofs + f);
  const int fsd = __ldg(a.fsd + f);
  R n0, n1, len;
  if constexpr (MIX) {
    n0 = __ldg(a.fnrmf + 2 * f); n1 = __ldg(a.fnrmf + 2 * f + 1); len = __ldg(a.flenf + f);
  } else {
    n0 = __ldg(a.fnrm + 2 * f); n1 = __ldg(a.fnrm + 2 * f + 1); len = __ldg(a.flen + f);
  }
  const DegTables<R> *gt = reinterpret_cast<const DegTables<R> *>(
      sizeof(R) == 4 ? (const void *)a.gtabf : (const void *)a.gtabd);
  const DegTables<R> &tm = gt[pm - 1];
  const double zref = MIX ? a.zeta_ref : 0.0;
  const double qref0 = MIX ? a.q_ref[0] : 0.0, qref1 = MIX ? a.q_ref[1] : 0.0;
  const R g = MIX ? (R)a.gf : (R)a.g, cu4 = MIX ? (R)a.cu4f : (R)a.cu4;
  const RefStateF &rf = a.ref;
  R *out = static_cast<R *>(a.fout);
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  const int fm = fpk & 15;
  if (f < a.n_inner) {
    const int fp = (fpk >> 4) & 15, sub = ((fpk >> 8) & 15) - 1, orient = (fpk >> 12) & 15,
              nf = (fpk >> 16) & 15;
    const int cp = __ldg(a.fcp + f);
    const int pp = __ldg(a.deg + cp), Np = pp + 1;
    const int64_t op = a.uniform_nn ? (int64_t)cp * a.uniform_nn : (int64_t)__ldg(a.off + cp);
    const DegTables<R> &tp = gt[pp - 1];
    const int kp = orient ? nf - 1 - k : k;  // the point's index on the plus side
    // traces: minus side on its full face, plus side on the subface (hanging) or full face
    R zm = 0, qm0 = 0, qm1 = 0, zp = 0, qp0 = 0, qp1 = 0;
#pragma unroll
    for (int n = 0; n < OC_MAXN; ++n) {
      if (n < Nm) {
        const R l = __ldg(&tm.F[0][nf][k][n]);
        const int d = face_dof(Nm, fm, n);
        zm += l * load_in<RIN, R>(a.rz, om + d, zref);
        qm0 += l * load_in<RIN, R>(a.rq, 2 * om + d, qref0);
        qm1 += l * load_in<RIN, R>(a.rq, 2 * om + Nm * Nm + d, qref1);
      }
      if (n < Np) {
        const R l = __ldg(&tp.F[sub + 1][nf][kp][n]);
        const int d = face_dof(Np, fp, n);
        zp += l * load_in<RIN, R>(a.rz, op + d, zref);
        qp0 += l * load_in<RIN, R>(a.rq, 2 * op + d, qref0);
        qp1 += l * load_in<RIN, R>(a.rq, 2 * op + Np * Np + d, qref1);
      }
    }
    R F, Fa0, Fa1, Pm0, Pm1, Pp0, Pp1;
    if constexpr (MIX) {
      if (a.sdf)  // bathymetry: well-balanced differences in FP64
        face_flux_dev_wb<R>(rf, g, cu4, zref, zm, qm0, qm1, zp, qp0, qp1, n0, n1,
                            __ldg(a.sdf + fsd + 2 * k), __ldg(a.sdf + fsd + 2 * k + 1),
                            __ldg(a.sdfe + fsd + 2 * k), __ldg(a.sdfe + fsd + 2 * k + 1), F,
                            Fa0, Fa1, Pm0, Pm1, Pp0, Pp1);
      else
        face_flux_dev<R>(rf, g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, (R)a.zreff, (R)a.zreff,
                         F, Fa0, Fa1, Pm0, Pm1, Pp0, Pp1, true);
    } else {
      const R zbm = a.sdf ? (R)__ldg(a.sdf + fsd + 2 * k) : R(0);
      const R zbp = a.sdf ? (R)__ldg(a.sdf + fsd + 2 * k + 1) : R(0);
      face_flux<R>(g, cu4, zm, qm0, qm1, zp, qp0, qp1, n0, n1, zbm, zbp, F, Fa0, Fa1, Pm0, Pm1,
                   Pp0, Pp1);
    }
    // JxW of the point: the minus (finer) face's length, which is also the
    // covered half of a coarse plus face
    const R jxw = __ldg(&tm.wF[nf][k]) * len;
    out[base + k] = -F * jxw;
    out[base + nf + k] = -(Fa0 + Pm0) * jxw;
    out[base + 2 * nf + k] = -(Fa1 + Pm1) * jxw;
    const int64_t bp = base + 3 * nf;
    out[bp + kp] = F * jxw;
    out[bp + nf + kp] = (Fa0 + Pp0) * jxw;
    out[bp + 2 * nf + kp] = (Fa1 + Pp1) * jxw;
  } else {  // boundary face: Gauss n_q points of the cell
    const int b = f - a.n_inner;
    const int bid = __ldg(a.bbid + b);
    const int bkind = a.bc_kind[bid];
    if (bkind == 0) {
      if (k == 0) atomicOr(a.err, ERR_UNKNOWN_BID);
      return;
    }
    const int Q = (3 * pm) / 2 + 1;
    R zm = 0, qm0 = 0, qm1 = 0;
#pragma unroll
    for (int n = 0; n < OC_MAXN; ++n) {
      if (n < Nm) {
        const R l = __ldg(&tm.BQ[k][n]);
        const int d = face_dof(Nm, fm, n);
        zm += l * load_in<RIN, R>(a.rz, om + d, zref);
        qm0 += l * load_in<RIN, R>(a.rq, 2 * om + d, qref0);
        qm1 += l * load_in<RIN, R>(a.rq, 2 * om + Nm * Nm + d, qref1);
      }
    }
    const DegTables<double> &td = reinterpret_cast<const DegTables<double> *>(a.gtabd)[pm - 1];
    R F, Fa0, Fa1;
    boundary_flux<R, MIX>(a, bid, bkind, fm, __ldg(&td.xQ[k]), a.geo + 11 * (int64_t)cm, zref,
                          fsd + k, g, cu4, zm, qm0, qm1, n0, n1, F, Fa0, Fa1);
    const R jxw = __ldg(&tm.wQ[k]) * len;
    out[base + k] = -F * jxw;
    out[base + Q + k] = -Fa0 * jxw;
    out[base + 2 * Q + k] = -Fa1 * jxw;
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

// variant 0: FP64; 1: mixed with FP32 stage input; 2: mixed with FP64 stage input
cudaError_t launch_face_pass(const StageArgs &a, int variant, cudaStream_t st) {
  if (a.n_fpts == 0) return cudaSuccess;
  const int threads = 256;
  const int grid = (int)((a.n_fpts + threads - 1) / threads);
  if (variant == 0) return launch_programmatic(face_kernel<double, false, double>, grid, threads, 0, st, a);
  if (a.r_is_float) return launch_programmatic(face_kernel<float, true, float>, grid, threads, 0, st, a);
  return launch_programmatic(face_kernel<float, true, double>, grid, threads, 0, st, a);
}

}  // namespace oc
