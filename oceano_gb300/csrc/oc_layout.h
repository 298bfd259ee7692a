// Shared host/device layout of the GPU operator: table sizes, per-degree
// shape tables and the argument block of the stage kernels.
#pragma once
#include <cstdint>

#define OC_MAXN 5      // nodes per direction, p <= 4
#define OC_MAXQ 7      // floor(1.5*4)+1 Gauss points per direction
#define OC_MAXF 6      // Gauss-Lobatto points per face, max(p-,p+)+2 <= 6
#define OC_MAXBID 16   // boundary ids
#define OC_MAXSTAGES 4
#define OC_MAXDEG 4
#define OC_MAXCPW 10    // cells per warp at p = 1 (the most of any degree)
#define OC_DSTRIDE 144  // doubles per cell of the FP64 zeta work area, >= N^2 + 3 N T + T + 2

// Device error word (StageArgs::err, AuxArgs::err): err[0] holds flags, err[1]
// the site of the first failed bounds check of the bounds-checked build
// (OC_BOUNDS_CHECK) and err[2], err[3] the low and high 32 bits of its index.
constexpr int kErrWords = 4;
enum ErrFlag { ERR_UNKNOWN_BID = 1 << 2, ERR_NONFINITE = 1 << 3, ERR_BOUNDS = 1 << 4 };
enum BoundsSite {
  BS_SELFTEST = 1,  // oc_bounds_selftest
  BS_CELL,          // cell id of a degree group
  BS_DEGREE,        // cell degree
  BS_OFFSET,        // DoF offset of a cell
  BS_RECORD,        // packed fields of a face record / face pack word
  BS_NEIGHBOUR,     // DoF offset of a face neighbour
  BS_BOUNDARY,      // boundary face index or boundary id
  BS_FACE_DATA,     // static face-data offset
  BS_FACE_OUT,      // face-pass output offset
  BS_CELL_DATA,     // static cell-data offset
  BS_FACE_CELL      // cell id of a face side
};
inline const char *bounds_site_name(int s) {
  static const char *names[] = {"none", "self-test", "cell id", "cell degree", "cell DoF offset",
                                "face record", "neighbour DoF offset", "boundary face",
                                "face static-data offset", "face-pass output offset",
                                "cell static-data offset", "face cell id"};
  return s >= 0 && s <= BS_FACE_CELL ? names[s] : "unknown site";
}

// Per-degree tables; matrices are [point][node] on [0,1].
template <typename R>
struct DegTables {
  R BQ[OC_MAXQ][OC_MAXN], DQ[OC_MAXQ][OC_MAXN], wQ[OC_MAXQ], xQ[OC_MAXQ];  // Gauss floor(1.5p)+1
  R BG[OC_MAXF][OC_MAXN], wG[OC_MAXF];                        // Gauss-Lobatto p+2
  // Gauss p+1: mass of the discharge and, with DM, the cell rule n_points_1d = p + 1
  // (rows sized like the BQ rows so that a kernel selects either rule's arrays)
  R BM[OC_MAXQ][OC_MAXN], DM[OC_MAXQ][OC_MAXN], wM[OC_MAXQ], xM[OC_MAXQ];
  R Sinv[OC_MAXN][OC_MAXN];
  R F[3][OC_MAXF + 1][OC_MAXF][OC_MAXN];  // [0 full face | 1,2 subface 0,1][nf][k][node]
  R wF[OC_MAXF + 1][OC_MAXF];             // Gauss-Lobatto nf weights
  R lump[OC_MAXN];                        // 1D lumped GL(p+2) mass
  R W1[OC_MAXN][OC_MAXN], W2[OC_MAXN][OC_MAXN], Gk[OC_MAXN][OC_MAXN];  // closed-form sweeps
  R lebG;  // max over the Gauss-Lobatto (p+2)^2 points of sum_ij |phi_i(x) phi_j(y)|
};

template <typename R>
inline void cast_tables(const DegTables<double> &a, DegTables<R> &b) {
  const double *s = reinterpret_cast<const double *>(&a);
  R *d = reinterpret_cast<R *>(&b);
  for (unsigned i = 0; i < sizeof(DegTables<double>) / sizeof(double); ++i) d[i] = (R)s[i];
}

// Per-call coefficients, read by the kernels from device memory so that a
// captured CUDA graph stays valid when dt or the time change.
struct alignas(16) StageDyn {
  float ff[OC_MAXSTAGES], fft[OC_MAXSTAGES];  // FP32 copies of f, ft (mixed form: one 16-byte load each)
  double f[OC_MAXSTAGES], ft[OC_MAXSTAGES];
  double fm, time;
  float ffm, pad_[3];
};

// Fill the FP32 copies of a coefficient block from its FP64 values.
inline void stage_dyn_round(StageDyn &d) {
  for (int j = 0; j < OC_MAXSTAGES; ++j) { d.ff[j] = (float)d.f[j]; d.fft[j] = (float)d.ft[j]; }
  d.ffm = (float)d.fm;
}

// FP32 reference state of the mixed form: depth, discharge, velocity q/h and the
// residual q - u h of the rounded pair (computed with one fused multiply-add).
struct RefStateF {
  float hr, qr0, qr1, ur0, ur1, rr0, rr1;
};

// Face references of a cell slot: >= 0: 2*inner_face + side (0 minus, 1 plus);
// < -1: boundary face b encoded as -(b+2); -1: empty.
struct StageArgs {
  // mesh
  int n_cells;
  int n_group;                 // cells processed by this launch
  const int *group_cells;      // their ids (NULL: identity starting at group_first)
  int group_first;
  int uniform_nn;              // (p+1)^2 when every cell has degree p: offset = cell * uniform_nn
  const int *deg;              // [n_cells]
  const int *off;              // [n_cells] zeta offset (discharge: 2*off)
  const double *geo;           // [n_cells*11]: x0,y0,J00,J01,J10,J11,Ji00,Ji01,Ji10,Ji11,det
  const int *slots;            // [n_cells*8]: 2 refs per face number (host bookkeeping)
  const int *cfrec;            // [n_cells*16]: 8 face records (other, packed word)
  const int *cfsdo;            // [n_cells*8]: static face-data offsets, NULL without data
  const int *cfofs;            // [n_cells*8]: face-pass output offset of each slot side
  const int *fcm, *fcp;        // [n_inner+n_bnd], [n_inner]
  const int *fpack;            // fm | fp<<4 | (sub+1)<<8 | orient<<12 | nf<<16
  const double *fnrm;          // [n_faces*2] minus normal
  const double *flen;          // [n_faces]
  const int *fsd;              // inner: offset into sdf; boundary: offset into sdb
  const int *bbid;             // [n_bnd] boundary id
  int n_inner;
  // face pass: boundary faces, the offset of every face's output
  // (inner: minus [3][nf] then plus [3][nf]; boundary: [3][Q]) and the output
  // (R values: double in the FP64 form, float in the mixed form)
  int n_bnd_faces;
  const int *fofs;
  void *fout;
  int cell_rule;  // Gauss points of boundary faces: 0 floor(1.5 p) + 1, 1 p + 1
  // static data (NULL = zero); *e arrays are FP32 copies with zeta_reference folded into zb
  const double *sd0, *sd1, *sd2, *sdf, *sdb;
  const float *sd0e, *sd1e, *sd2e, *sdfe, *sdbe;
  const int *sdo0, *sdo1, *sdo2; // per cell offsets
  // stage vectors
  const void *rz, *rq, *rvel;  // stage input (double, or float deviations in mixed mode)
  int r_is_float;
  const double *un_z, *un_q;   // solution u^n (FP64)
  void *kz[OC_MAXSTAGES + 1];  // residual registers (double or float)
  void *kq[2 * OC_MAXSTAGES];
  double *out_z, *out_q;       // next_ri or solution (FP64)
  float *out_rz, *out_rq;      // mixed: FP32 stage input of the next stage (may be NULL)
  // mixed time-step path: FP32 copies of u^n (zeta - zeta_ref, q), written at
  // stage 0 (out_un*) and read by the later stages (un_*f); internal stage
  // inputs are then formed as u^n_f32 + delta in FP32 and only the last stage
  // accumulates in FP64
  const float *un_zf, *un_qf;
  float *out_unzf, *out_unqf;
  int fast_mixed;
  const float *geof;           // [n_cells*11] FP32 copy of geo (mixed form)
  // mixed form: FP64 work area of the literal zeta iteration, OC_DSTRIDE doubles
  // per (launch-wide warp, team) slot, OC_MAXCPW slots per warp (only cells that
  // are not fully wet touch it)
  double *dscratch;
  // global-memory copies of the per-degree tables (index p - 1), read through
  // the L1 cache where lanes need different entries (hanging and degree-jump faces)
  const DegTables<double> *gtabd;
  const DegTables<float> *gtabf;
  // mixed form: reference state (depth h_ref, discharge q_ref); the FP32 discharge
  // is q - q_ref and the fluxes are evaluated minus their reference value
  double h_ref, q_ref[2];
  RefStateF ref;  // the same state in FP32 with u_ref = q_ref / h_ref (read from the parameter bank)
  // FP32 copies of g, cu4, the wet threshold and zeta_ref (no conversions in the kernels)
  float gf, cu4f, wet_thrf, zreff;
  // one-launch hp stage (stage_kernel_hp): per degree p the first block, the
  // number of blocks, the cells and the cell list of the group
  int hp_first_block[OC_MAXDEG + 1], hp_blocks[OC_MAXDEG + 1], hp_n[OC_MAXDEG + 1];
  const int *hp_cells[OC_MAXDEG + 1];
  double *aux_q;              // ARK last stage: next_ri_discharge receives M^-1 rhs
  const struct StageDyn *dyn;  // device copy of the per-call coefficients
  int stage, n_stages, ark, last, write_kq_last, apply_mode;
  // model
  double g, cu4, nu, zeta_ref, wet_threshold;
  int friction, max_iter, batch;
  // boundary conditions
  int bc_kind[OC_MAXBID], bc_fn[OC_MAXBID];
  double bc_c[OC_MAXBID][3];
  double vortex[8];
  // per-cell step-size scale of the time-step path (NULL: 1): the residual of
  // cell c is multiplied by cscale[c] before the Runge-Kutta update
  const float *cscalef;
  const double *cscale;
  // extents checked by the bounds-checked build (OC_BOUNDS_CHECK): DoFs per
  // variable, elements of the face-pass output and of sd0, sd1, sd2, sdf, sdb
  int64_t n_dofs, n_fout, n_sd[5];
  // status word: err[0] bit flags of oc_status codes; err[1..3] the site and
  // the index of the first failed bounds check (bounds-checked build)
  int *err;
};

// Arguments of the cell-local auxiliary kernels (transport speed, velocity,
// vorticity, projection).
struct AuxArgs {
  int n_cells;
  const int *deg, *off;
  const double *geo;
  const double *sd1, *sd2;  // zb at Gauss-Lobatto p+2; (zb, cf) at Gauss p+1
  const int *sdo1, *sdo2;
  double g, cu4;
  double vortex[8];
  int64_t n_dofs, n_sd[5];  // extents checked by the bounds-checked build
  int cell_rule;            // cell Gauss rule of the errors: 0 floor(1.5 p) + 1, 1 p + 1
  int *err;
};
