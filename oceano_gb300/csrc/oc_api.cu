// C ABI of the GB300 operator (include/oceano_gpu.h): handle, mesh tables,
// static data, stage and time-step drivers with host or device vectors.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "oceano_gpu.h"
#include "oc_layout.h"
#include "oc_tables.hpp"

namespace oc {
cudaError_t launch_stage_p1(const StageArgs &, int, int, int, cudaStream_t);
cudaError_t launch_stage_p2(const StageArgs &, int, int, int, cudaStream_t);
cudaError_t launch_stage_p3(const StageArgs &, int, int, int, cudaStream_t);
cudaError_t launch_stage_p4(const StageArgs &, int, int, int, cudaStream_t);
cudaError_t configure_stage_p1();
cudaError_t configure_stage_p2();
cudaError_t configure_stage_p3();
cudaError_t configure_stage_p4();
int stage_cells_per_warp_p1();
int stage_cells_per_warp_p2();
int stage_cells_per_warp_p3();
int stage_cells_per_warp_p4();
cudaError_t upload_tables_p1(const DegTables<double> *, const DegTables<float> *);
cudaError_t upload_tables_p2(const DegTables<double> *, const DegTables<float> *);
cudaError_t upload_tables_p3(const DegTables<double> *, const DegTables<float> *);
cudaError_t upload_tables_p4(const DegTables<double> *, const DegTables<float> *);
// the same entry points for the cell Gauss rule p + 1 (OC_CELL_RULE_P1)
cudaError_t launch_stage_p1_r1(const StageArgs &, int, int, int, cudaStream_t);
cudaError_t configure_stage_p1_r1();
int stage_cells_per_warp_p1_r1();
cudaError_t upload_tables_p1_r1(const DegTables<double> *, const DegTables<float> *);
cudaError_t launch_stage_p2_r1(const StageArgs &, int, int, int, cudaStream_t);
cudaError_t configure_stage_p2_r1();
int stage_cells_per_warp_p2_r1();
cudaError_t upload_tables_p2_r1(const DegTables<double> *, const DegTables<float> *);
cudaError_t launch_stage_p3_r1(const StageArgs &, int, int, int, cudaStream_t);
cudaError_t configure_stage_p3_r1();
int stage_cells_per_warp_p3_r1();
cudaError_t upload_tables_p3_r1(const DegTables<double> *, const DegTables<float> *);
cudaError_t launch_stage_p4_r1(const StageArgs &, int, int, int, cudaStream_t);
cudaError_t configure_stage_p4_r1();
int stage_cells_per_warp_p4_r1();
cudaError_t upload_tables_p4_r1(const DegTables<double> *, const DegTables<float> *);

cudaError_t configure_stage_hp_v0();
cudaError_t configure_stage_hp_v1();
cudaError_t configure_stage_hp_v2();
cudaError_t launch_stage_hp_v0(const StageArgs &, int, int, bool, cudaStream_t);
cudaError_t launch_stage_hp_v1(const StageArgs &, int, int, bool, cudaStream_t);
cudaError_t launch_stage_hp_v2(const StageArgs &, int, int, bool, cudaStream_t);
cudaError_t upload_tables_hp_v0(const DegTables<double> *, const DegTables<float> *);
cudaError_t upload_tables_hp_v1(const DegTables<double> *, const DegTables<float> *);
cudaError_t upload_tables_hp_v2(const DegTables<double> *, const DegTables<float> *);

cudaError_t launch_bounds_selftest(int *, cudaStream_t);
cudaError_t aux_upload_tables(const DegTables<double> *, const DegTables<float> *);
cudaError_t launch_face_pass(const StageArgs &, int, cudaStream_t);
cudaError_t face_upload_tables(const DegTables<double> *, const DegTables<float> *);
cudaError_t launch_transport_speed(const AuxArgs &, const double *, const double *,
                                   unsigned long long *, double *, cudaStream_t);
cudaError_t launch_velocity_field(const AuxArgs &, const double *, const double *, double *,
                                  cudaStream_t);
cudaError_t launch_vorticity(const AuxArgs &, const double *, int, const double *,
                             const double *, float *, cudaStream_t);
cudaError_t launch_project_vortex(const AuxArgs &, double, double *, double *, cudaStream_t);
cudaError_t launch_errors(const AuxArgs &, double, const double *, const int *, const double *,
                          const double *, double *, double *, cudaStream_t);
cudaError_t launch_conservative_coarsening(const AuxArgs &, const unsigned char *, double *,
                                           cudaStream_t);
cudaError_t launch_features(const AuxArgs &, const double *, const double *, const float *,
                            const int *, int, unsigned *, float, float *, float *, float *,
                            cudaStream_t);
}  // namespace oc

using namespace oc;

static const int kWarpsPerBlock = 4;

// Butcher tableaux of time_stepping.h:136-379 (a rows, b, c; d~ for TR-BDF2)
struct Scheme {
  int s;
  double a[OC_MAXSTAGES][OC_MAXSTAGES], b[OC_MAXSTAGES], c[OC_MAXSTAGES];
  double at[OC_MAXSTAGES][OC_MAXSTAGES], dt[OC_MAXSTAGES];
  bool ark;
};

static bool make_scheme(int id, Scheme &sc) {
  std::memset(&sc, 0, sizeof(sc));
  const double chi = 2.0 - std::sqrt(2.0);
  switch (id) {
    case OC_ERK_FORWARD_EULER:
      sc.s = 1; sc.b[0] = 1; break;
    case OC_ERK_SSP22:
      sc.s = 2; sc.a[0][0] = 1; sc.b[0] = sc.b[1] = 0.5; sc.c[1] = 1; break;
    case OC_ERK_SSP33:
      sc.s = 3; sc.a[0][0] = 1; sc.a[1][0] = sc.a[1][1] = 0.25;
      sc.b[0] = sc.b[1] = 1.0 / 6.0; sc.b[2] = 2.0 / 3.0; sc.c[1] = 1; sc.c[2] = 0.5; break;
    case OC_ERK_RK4:
      sc.s = 4; sc.a[0][0] = 0.5; sc.a[1][1] = 0.5; sc.a[2][2] = 1;
      sc.b[0] = 1.0 / 6.0; sc.b[1] = sc.b[2] = 1.0 / 3.0; sc.b[3] = 1.0 / 6.0;
      sc.c[1] = sc.c[2] = 0.5; sc.c[3] = 1; break;
    case OC_ERK_STAGE3_ORDER2:
    case OC_ARK_STAGE3_ORDER2:
      sc.s = 3; sc.a[0][0] = chi; sc.a[1][0] = sc.a[1][1] = 0.5;
      sc.b[0] = sc.b[1] = 0.5 - chi / 4.0; sc.b[2] = chi / 2.0; sc.c[1] = chi; sc.c[2] = 1;
      if (id == OC_ARK_STAGE3_ORDER2) {
        sc.ark = true;
        sc.at[0][0] = chi / 2.0;
        sc.at[1][0] = sc.at[1][1] = 1.0 / (2.0 * std::sqrt(2.0));
        sc.dt[0] = chi / 2.0; sc.dt[1] = 1.0 - 1.0 / std::sqrt(2.0);
      }
      break;
    default: return false;
  }
  return true;
}

struct oc_op {
  int n_cells = 0, n_inner = 0, n_bnd = 0;
  int64_t n_dofs = 0;
  oc_params prm{};
  std::string err;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  // host copies
  std::vector<int> deg, off, slots, fcm, fcp, fpack, fsd, bbid, sdo[3];
  std::vector<double> geo, fnrm, flen;
  int64_t sd_size[5] = {0, 0, 0, 0, 0};
  // device copies
  int *d_deg = nullptr, *d_off = nullptr, *d_slots = nullptr, *d_fcm = nullptr,
      *d_fcp = nullptr, *d_fpack = nullptr, *d_fsd = nullptr, *d_bbid = nullptr;
  int *d_sdo[3] = {nullptr, nullptr, nullptr};
  std::vector<int> cfrec, cfsdo, cfofs;        // per-cell face records for the kernels
  int *d_cfrec = nullptr, *d_cfsdo = nullptr, *d_cfofs = nullptr;
  double *d_geo = nullptr, *d_fnrm = nullptr, *d_flen = nullptr;
  // face pass: output offsets, output buffer, FP32 face geometry
  std::vector<int> fofs;
  int *d_fofs = nullptr;
  void *d_fout = nullptr;
  int64_t n_fout = 0;  // elements of the face-pass output
  float *d_geof = nullptr;
  double *d_dscratch = nullptr;  // mixed form: FP64 zeta work area per (warp, team) slot
  DegTables<double> *d_tabd = nullptr;  // table copies in global memory (divergent reads)
  DegTables<float> *d_tabf = nullptr;
  double *d_sd[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  float *d_sde[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // degree groups
  int group_n[OC_MAXDEG + 1] = {0, 0, 0, 0, 0};
  int *d_group[OC_MAXDEG + 1] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // the same groups in index order, where d_group is sorted (mixed form): the last
  // stage of a host-vector step writes u^{n+1} over the host link in this order
  int *d_group_idx[OC_MAXDEG + 1] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int uniform_deg = 0;
  int conforming = 0;  // uniform degree, no hanging face, standard orientation
  // boundary conditions
  int bc_kind[OC_MAXBID] = {0}, bc_fn[OC_MAXBID] = {0};
  double bc_c[OC_MAXBID][3] = {{0}};
  double vortex[8] = {0};
  // scratch
  int *d_err = nullptr;
  unsigned long long *d_speed = nullptr;
  StageDyn *d_dyn = nullptr;    // per-stage coefficient blocks (OC_MAXSTAGES + 1)
  StageDyn *h_dyn = nullptr;    // pageable host mirror (safe to reuse once a copy is enqueued)
  // host-memory staging and time-step registers
  std::vector<void *> bufs;
  double *st_rz = nullptr, *st_rq = nullptr, *st_rv = nullptr, *st_sz = nullptr, *st_sq = nullptr,
         *st_nz = nullptr, *st_nq = nullptr;
  double *st_kz[OC_MAXSTAGES + 1] = {nullptr}, *st_kq[2 * OC_MAXSTAGES] = {nullptr};
  void *ts_kz[OC_MAXSTAGES + 1] = {nullptr}, *ts_kq[2 * OC_MAXSTAGES] = {nullptr};
  void *ts_rz[2] = {nullptr, nullptr}, *ts_rq[2] = {nullptr, nullptr};
  double *ts_z = nullptr, *ts_q = nullptr;  // solution when the caller passes host memory
  double *ts_z0 = nullptr, *ts_q0 = nullptr;  // one-stage schemes: copy of u^n (stage input)
  double *d_cscale = nullptr;  // per-cell step-size scale (NULL: 1)
  float *d_cscalef = nullptr;
  double *ts_aux = nullptr;
  float *ts_unzf = nullptr, *ts_unqf = nullptr;  // FP32 copies of u^n (mixed time step)
  // mixed form reference state (FP32-representable values)
  double ref_h = 1.0, ref_q[2] = {0.0, 0.0};
  // launch configuration: OC_LAUNCH_AUTO tunes it at the first time step
  int launch_mode = OC_LAUNCH_AUTO;
  int tuned = 0;
  int use_hp = 0;                           // one launch for all degree groups
  int hp_wpb = 4;                           // warps per block of that launch
  int wpb[OC_MAXDEG + 1] = {4, 4, 4, 4, 4}; // warps per block per degree group
  float tune_ms[2] = {0.f, 0.f};            // measured stage time: per-group, one launch
  // vorticity: basis values / derivatives at QGauss(nq) per degree (cached per nq)
  double *d_vtab[9] = {nullptr};
  // indicator features: velocity and vorticity scratch, per-member maxima
  double *d_ivel = nullptr;
  float *d_ivort = nullptr;
  unsigned *d_imax = nullptr;
  double *d_epart = nullptr;  // per-cell squared errors + the two results
  int imax_n = 0;
  // timing by the reference's TimerOutput scope names (oc_set_timing)
  int timing = 0;
  struct Scope {
    const char *name;
    int64_t calls = 0;
    double seconds = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
  };
  Scope scopes[3] = {{"rk_stage hydro - integrals L_h + inv mass + vec upd"},
                     {"rk time stepping total"},
                     {"compute transport speed"}};
  // graph cache of oc_perform_time_step
  int64_t graph_launches = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_scheme = -1;
  const void *graph_z = nullptr, *graph_q = nullptr;
  const void *graph_oz = nullptr, *graph_oq = nullptr;  // last-stage outputs of the graph
  const void *graph_hz = nullptr, *graph_hq = nullptr;  // host vectors the graph copies in
  // Host-vector time step on a mesh of one degree (mixed form): u^n is copied in
  // by pieces on a second stream, and stage 0 runs by chunks of cells, each
  // launched once the DoFs that its cells and their face neighbours read have
  // arrived, so that the transfer in overlaps stage 0.  Three chunks: the chunk
  // launches follow one another on the stream, and each lasts at least the
  // lifetime of one warp (about a third of a stage on the 320x160 degree-3 vortex),
  // so more chunks lengthen stage 0 again (measured per step: 1 chunk 0.350 ms,
  // 2 0.335, 3 0.323, 4 0.329, 8 0.373).
  static constexpr int kChunks = 3;
  cudaStream_t cstream = nullptr;
  cudaEvent_t cev[kChunks + 1] = {nullptr};
  // per-group launches on a mesh of several degrees: one stream per degree group,
  // forked from and joined back into the handle's stream (gev[0]: fork)
  cudaStream_t gstream[OC_MAXDEG + 1] = {nullptr};
  cudaEvent_t gev[OC_MAXDEG + 1] = {nullptr};
  int n_chunks = 0;                    // 0: not set up yet; 1: no chunking
  int chunk_first[kChunks + 1] = {0};  // cell range [first[k], first[k + 1]) of chunk k
  int64_t chunk_reach[kChunks] = {0};  // zeta DoFs [0, reach[k]) read by chunks 0..k
};

#define OC_TRY(call)                                                              \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      op->err = std::string(#call) + ": " + cudaGetErrorString(e_);               \
      return OC_ERR_CUDA;                                                         \
    }                                                                             \
  } while (0)

static oc_status fail(oc_op *op, oc_status s, const std::string &msg) {
  if (op) op->err = msg;
  return s;
}

// A timed region of the handle's stream: events recorded around the enqueued GPU
// work of one call (no-ops unless timing is on), and an NVTX range around the call.
enum { SCOPE_STAGE = 0, SCOPE_STEP = 1, SCOPE_SPEED = 2 };
struct TimedScope {
  oc_op *op;
  int scope;
  cudaEvent_t e0 = nullptr;
  TimedScope(oc_op *o, int sc) : op(o), scope(sc) {
    nvtxRangePushA(o->scopes[sc].name);
    if (o->timing && cudaEventCreate(&e0) == cudaSuccess) cudaEventRecord(e0, o->stream);
  }
  ~TimedScope() {
    if (e0) {
      cudaEvent_t e1 = nullptr;
      if (cudaEventCreate(&e1) == cudaSuccess && cudaEventRecord(e1, op->stream) == cudaSuccess) {
        op->scopes[scope].pending.emplace_back(e0, e1);
      } else {
        cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
      }
    }
    nvtxRangePop();
  }
};

// fold the recorded event pairs into the scope totals (waits for them)
static void resolve_timers(oc_op *op) {
  for (auto &sc : op->scopes) {
    for (auto &ev : sc.pending) {
      float ms = 0.f;
      if (cudaEventSynchronize(ev.second) == cudaSuccess &&
          cudaEventElapsedTime(&ms, ev.first, ev.second) == cudaSuccess) {
        sc.calls += 1;
        sc.seconds += 1e-3 * ms;
      }
      cudaEventDestroy(ev.first);
      cudaEventDestroy(ev.second);
    }
    sc.pending.clear();
  }
}

template <typename T>
static cudaError_t upload(oc_op *op, T **dst, const T *src, size_t n) {
  if (n == 0) { *dst = nullptr; return cudaSuccess; }
  cudaError_t e = cudaMalloc((void **)dst, n * sizeof(T));
  if (e != cudaSuccess) return e;
  op->bufs.push_back(*dst);
  return cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

static cudaError_t alloc(oc_op *op, void **dst, size_t bytes) {
  cudaError_t e = cudaMalloc(dst, bytes);
  if (e == cudaSuccess) op->bufs.push_back(*dst);
  return e;
}

static int n_groups(const oc_op *op) {
  int k = 0;
  for (int p = 1; p <= OC_MAXDEG; ++p) k += op->group_n[p] > 0;
  return k;
}

// the one-launch hp kernel: several degree groups, built for the default cell rule only
static bool hp_possible(const oc_op *op) {
  return n_groups(op) > 1 && op->prm.cell_quadrature == OC_CELL_RULE_DEFAULT;
}

// Gauss points per direction of the cell integrals and boundary faces of degree p
static int cell_q(const oc_op *op, int p) {
  return op->prm.cell_quadrature == OC_CELL_RULE_P1 ? p + 1 : (3 * p) / 2 + 1;
}

static int cells_per_warp(const oc_op *op, int p) {
  if (op->prm.cell_quadrature == OC_CELL_RULE_P1) switch (p) {
      case 1: return stage_cells_per_warp_p1_r1();
      case 2: return stage_cells_per_warp_p2_r1();
      case 3: return stage_cells_per_warp_p3_r1();
      default: return stage_cells_per_warp_p4_r1();
    }
  switch (p) {
    case 1: return stage_cells_per_warp_p1();
    case 2: return stage_cells_per_warp_p2();
    case 3: return stage_cells_per_warp_p3();
    default: return stage_cells_per_warp_p4();
  }
}

static cudaError_t launch_stage(const oc_op *op, int p, const StageArgs &a, int variant, int grid,
                                int wpb, cudaStream_t s) {
  if (op->prm.cell_quadrature == OC_CELL_RULE_P1) switch (p) {
      case 1: return launch_stage_p1_r1(a, variant, grid, wpb, s);
      case 2: return launch_stage_p2_r1(a, variant, grid, wpb, s);
      case 3: return launch_stage_p3_r1(a, variant, grid, wpb, s);
      default: return launch_stage_p4_r1(a, variant, grid, wpb, s);
    }
  switch (p) {
    case 1: return launch_stage_p1(a, variant, grid, wpb, s);
    case 2: return launch_stage_p2(a, variant, grid, wpb, s);
    case 3: return launch_stage_p3(a, variant, grid, wpb, s);
    default: return launch_stage_p4(a, variant, grid, wpb, s);
  }
}

static cudaError_t launch_stage_hp(int hv, const StageArgs &a, int grid, int wpb, bool lean,
                                   cudaStream_t s) {
  switch (hv) {
    case 0: return launch_stage_hp_v0(a, grid, wpb, false, s);
    case 1: return launch_stage_hp_v1(a, grid, wpb, lean, s);
    default: return launch_stage_hp_v2(a, grid, wpb, lean, s);
  }
}

static oc_status read_error(oc_op *op);

extern "C" {

const char *oc_last_error(const oc_op *op) { return op ? op->err.c_str() : "null handle"; }
int64_t oc_n_dofs(const oc_op *op) { return op ? op->n_dofs : -1; }
int64_t oc_launch_count(const oc_op *op) { return op ? op->launches : -1; }
void *oc_stream(oc_op *op) { return op ? (void *)op->stream : nullptr; }

oc_status oc_set_reference_state(oc_op *op, double depth, double qx, double qy) {
  if (!op || !(depth > 0.) || !std::isfinite(qx) || !std::isfinite(qy))
    return OC_ERR_INVALID_ARG;
  op->ref_h = (double)(float)depth;
  op->ref_q[0] = (double)(float)qx;
  op->ref_q[1] = (double)(float)qy;
  if (op->graph) { cudaGraphExecDestroy(op->graph); op->graph = nullptr; }
  return OC_OK;
}

oc_status oc_set_launch_mode(oc_op *op, int32_t mode) {
  if (!op) return OC_ERR_INVALID_ARG;
  if (mode < OC_LAUNCH_AUTO || mode > OC_LAUNCH_ONE)
    return fail(op, OC_ERR_INVALID_ARG, "unknown launch mode");
  op->launch_mode = mode;
  op->tuned = 0;
  op->use_hp = mode == OC_LAUNCH_ONE && hp_possible(op);
  if (op->graph) { cudaGraphExecDestroy(op->graph); op->graph = nullptr; }
  return OC_OK;
}

oc_status oc_launch_config(const oc_op *op, int32_t *out) {
  if (!op || !out) return OC_ERR_INVALID_ARG;
  out[0] = op->use_hp; out[1] = op->hp_wpb;
  for (int p = 1; p <= OC_MAXDEG; ++p) out[1 + p] = op->wpb[p];
  out[6] = op->tuned;
  return OC_OK;
}

oc_status oc_synchronize(oc_op *op) {
  if (!op) return OC_ERR_INVALID_ARG;
  return read_error(op);  // waits for the stream, reports and clears the device flags
}

void oc_destroy(oc_op *op) {
  if (!op) return;
  if (op->stream) cudaStreamSynchronize(op->stream);
  resolve_timers(op);
  if (op->graph) cudaGraphExecDestroy(op->graph);
  for (void *p : op->bufs) cudaFree(p);
  delete[] op->h_dyn;
  for (cudaEvent_t e : op->cev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : op->gev)
    if (e) cudaEventDestroy(e);
  for (cudaStream_t g : op->gstream)
    if (g) cudaStreamDestroy(g);
  if (op->cstream) cudaStreamDestroy(op->cstream);
  if (op->stream) cudaStreamDestroy(op->stream);
  delete op;
}

oc_status oc_create(const oc_mesh_desc *m, const oc_params *prm, oc_op **out) {
  if (!out) return OC_ERR_INVALID_ARG;
  *out = nullptr;
  if (!m || !prm || m->n_cells <= 0 || !m->degree || !m->vertices || m->n_inner_faces < 0 ||
      m->n_boundary_faces < 0)
    return OC_ERR_INVALID_ARG;
  oc_op *op = new oc_op();
  op->prm = *prm;
  if (op->prm.batch_width <= 0) op->prm.batch_width = 1;
  if (op->prm.max_iteration_height < 0) op->prm.max_iteration_height = 0;
  const int nc = m->n_cells, ni = m->n_inner_faces, nb = m->n_boundary_faces;
  op->n_cells = nc; op->n_inner = ni; op->n_bnd = nb;
  auto bad = [&](oc_status s, const std::string &msg) {
    oc_status r = fail(op, s, msg);
    *out = op;  // keep the handle so that the caller can read the message
    return r;
  };
  if (prm->horizontal_viscosity != 0.0)
    return bad(OC_ERR_UNSUPPORTED, "horizontal_viscosity != 0 is not implemented on the GPU");
  if (prm->cell_quadrature != OC_CELL_RULE_DEFAULT && prm->cell_quadrature != OC_CELL_RULE_P1)
    return bad(OC_ERR_INVALID_ARG, "unknown cell quadrature rule");
  if (prm->precision != OC_PREC_FP64 && prm->precision != OC_PREC_MIXED)
    return bad(OC_ERR_INVALID_ARG, "unknown precision");
  // cells: degree, offsets, affine geometry
  op->deg.assign(m->degree, m->degree + nc);
  op->off.resize(nc);
  op->geo.resize(11 * (size_t)nc);
  for (int k = 0; k < 3; ++k) op->sdo[k].resize(nc);
  int64_t off = 0, s0 = 0, s1 = 0, s2 = 0;
  int first_deg = m->degree[0];
  bool uniform = true;
  for (int c = 0; c < nc; ++c) {
    const int p = m->degree[c];
    if (p < 1 || p > OC_MAXDEG) return bad(OC_ERR_UNSUPPORTED, "degree must be 1..4");
    uniform = uniform && p == first_deg;
    const int Q = cell_q(op, p);
    op->off[c] = (int)off;
    op->sdo[0][c] = (int)s0; op->sdo[1][c] = (int)s1; op->sdo[2][c] = (int)s2;
    off += (p + 1) * (p + 1);
    s0 += 5 * Q * Q; s1 += (p + 2) * (p + 2); s2 += 2 * (p + 1) * (p + 1);
    const double *v = m->vertices + 8 * (size_t)c;
    double *J = &op->geo[11 * (size_t)c];
    J[0] = v[0]; J[1] = v[1];
    J[2] = v[2] - v[0]; J[3] = v[4] - v[0];
    J[4] = v[3] - v[1]; J[5] = v[5] - v[1];
    const double scale = std::fabs(J[2]) + std::fabs(J[3]) + std::fabs(J[4]) + std::fabs(J[5]);
    const double ex = v[6] - (v[2] + v[4] - v[0]), ey = v[7] - (v[3] + v[5] - v[1]);
    if (std::fabs(ex) + std::fabs(ey) > 1e-12 * scale)
      return bad(OC_ERR_UNSUPPORTED, "cell " + std::to_string(c) + " is not affine");
    const double det = J[2] * J[5] - J[3] * J[4];
    if (!(det > 0)) return bad(OC_ERR_INVALID_ARG, "cell " + std::to_string(c) + " has det <= 0");
    J[6] = J[5] / det; J[7] = -J[3] / det; J[8] = -J[4] / det; J[9] = J[2] / det; J[10] = det;
  }
  if (off >= (int64_t)1 << 30) return bad(OC_ERR_UNSUPPORTED, "more than 2^30 DoFs per variable");
  op->n_dofs = off;
  op->sd_size[0] = s0; op->sd_size[1] = s1; op->sd_size[2] = s2;
  op->uniform_deg = uniform ? first_deg : 0;
  // faces
  const int nf = ni + nb;
  op->fcm.resize(nf); op->fcp.assign(std::max(ni, 1), 0); op->fpack.resize(nf);
  op->fsd.resize(nf); op->bbid.assign(std::max(nb, 1), 0);
  op->fnrm.resize(2 * (size_t)nf); op->flen.resize(nf);
  op->slots.assign(8 * (size_t)nc, -1);
  int64_t sf = 0, sb = 0;
  bool nonconforming = false;
  static const double rn[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
  for (int f = 0; f < nf; ++f) {
    const int cm = m->cell_m[f];
    const int fm = m->face_m[f];
    if (cm < 0 || cm >= nc || fm < 0 || fm > 3) return bad(OC_ERR_INVALID_ARG, "bad face " + std::to_string(f));
    const double *J = &op->geo[11 * (size_t)cm];
    double nx = J[6] * rn[fm][0] + J[8] * rn[fm][1], ny = J[7] * rn[fm][0] + J[9] * rn[fm][1];
    const double nn = std::sqrt(nx * nx + ny * ny);
    op->fnrm[2 * f] = nx / nn; op->fnrm[2 * f + 1] = ny / nn;
    const double t0 = fm < 2 ? 0 : 1, t1 = fm < 2 ? 1 : 0;
    const double tx = J[2] * t0 + J[3] * t1, ty = J[4] * t0 + J[5] * t1;
    op->flen[f] = std::sqrt(tx * tx + ty * ty);
    op->fcm[f] = cm;
    if (f < ni) {
      const int cp = m->cell_p[f], fp = m->face_p[f], sub = m->subface[f];
      const int orient = m->orientation ? m->orientation[f] : 0;
      if (cp < 0 || cp >= nc || fp < 0 || fp > 3 || sub < -1 || sub > 1 || orient < 0 || orient > 1)
        return bad(OC_ERR_INVALID_ARG, "bad inner face " + std::to_string(f));
      const int nfq = std::max(m->degree[cm], m->degree[cp]) + 2;
      op->fcp[f] = cp;
      op->fpack[f] = fm | (fp << 4) | ((sub + 1) << 8) | (orient << 12) | (nfq << 16);
      if (sub >= 0 || orient != 0) nonconforming = true;
      op->fsd[f] = (int)sf;
      sf += 2 * nfq;
      int *sm = &op->slots[8 * (size_t)cm + 2 * fm];
      if (sm[0] != -1) return bad(OC_ERR_INVALID_ARG, "cell face listed twice (minus side)");
      sm[0] = 2 * f;
      int *sp = &op->slots[8 * (size_t)cp + 2 * fp];
      const int pos = sub < 0 ? 0 : sub;
      if (sp[pos] != -1) return bad(OC_ERR_INVALID_ARG, "cell face listed twice (plus side)");
      sp[pos] = 2 * f + 1;
    } else {
      const int b = f - ni;
      const int bid = m->boundary_id[b];
      if (bid < 0 || bid >= OC_MAXBID) return bad(OC_ERR_UNKNOWN_BOUNDARY_ID, "boundary id out of range");
      op->bbid[b] = bid;
      op->fpack[f] = fm;
      op->fsd[f] = (int)sb;
      sb += cell_q(op, m->degree[cm]);
      int *sm = &op->slots[8 * (size_t)cm + 2 * fm];
      if (sm[0] != -1) return bad(OC_ERR_INVALID_ARG, "cell face listed twice (boundary)");
      sm[0] = -(b + 2);
    }
  }
  for (int c = 0; c < nc; ++c)
    for (int fno = 0; fno < 4; ++fno) {
      const int *sl = &op->slots[8 * (size_t)c + 2 * fno];
      if (sl[0] == -1 && sl[1] == -1)
        return bad(OC_ERR_INVALID_ARG, "cell " + std::to_string(c) + " face " + std::to_string(fno) + " has no face");
      if (sl[0] == -1) return bad(OC_ERR_INVALID_ARG, "hanging face without subface 0");
    }
  op->sd_size[3] = sf; op->sd_size[4] = sb;
  op->conforming = op->uniform_deg != 0 && !nonconforming;
  // face pass: output offset of every face
  op->fofs.resize(nf);
  int64_t fo_total = 0;
  for (int f = 0; f < nf; ++f) {
    const int npt = f < ni ? (op->fpack[f] >> 16) & 15 : cell_q(op, op->deg[op->fcm[f]]);
    op->fofs[f] = (int)fo_total;
    fo_total += (f < ni ? 6 : 3) * npt;
  }
  if (fo_total >= (int64_t)1 << 31 || (int64_t)nf >= (int64_t)1 << 27)
    return bad(OC_ERR_UNSUPPORTED, "too many faces for the face pass");
  // per-cell face records: (other zeta offset | boundary index, packed description),
  // and the face-pass output offset of each slot side
  op->cfrec.assign(16 * (size_t)nc, 0);
  op->cfsdo.assign(8 * (size_t)nc, 0);
  op->cfofs.assign(8 * (size_t)nc, -1);
  for (int c = 0; c < nc; ++c)
    for (int sl = 0; sl < 8; ++sl) {
      const int ref = op->slots[8 * (size_t)c + sl];
      int other = -1, pk = 0, sdo = 0, fofs = -1;
      if (ref >= 0) {
        const int f = ref >> 1, side = ref & 1;
        const int fpk = op->fpack[f];
        const int fm = fpk & 15, fp = (fpk >> 4) & 15, sub1 = (fpk >> 8) & 15,
                  orient = (fpk >> 12) & 15, nfq = (fpk >> 16) & 15;
        const int oc = side ? op->fcm[f] : op->fcp[f];
        other = op->off[oc];
        fofs = op->fofs[f] + side * 3 * nfq;
        pk = (side ? fp : fm) | ((side ? fm : fp) << 2) | (op->deg[oc] << 4) | (sub1 << 7) |
             (orient << 9) | (side << 10) | (nfq << 11) | (1 << 14);
        sdo = op->fsd[f];
      } else if (ref < -1) {
        const int b = -ref - 2, f = ni + b;
        other = b;
        fofs = op->fofs[f];
        pk = (op->fpack[f] & 15) | (2 << 14) | (op->bbid[b] << 16);
        sdo = op->fsd[f];
      }
      op->cfrec[16 * (size_t)c + 2 * sl] = other;
      op->cfrec[16 * (size_t)c + 2 * sl + 1] = pk;
      op->cfsdo[8 * (size_t)c + sl] = sdo;
      op->cfofs[8 * (size_t)c + sl] = fofs;
    }
  // device
  OC_TRY(cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking));
  OC_TRY(upload(op, &op->d_deg, op->deg.data(), nc));
  OC_TRY(upload(op, &op->d_off, op->off.data(), nc));
  OC_TRY(upload(op, &op->d_geo, op->geo.data(), op->geo.size()));
  {
    std::vector<float> gf(op->geo.begin(), op->geo.end());
    OC_TRY(upload(op, &op->d_geof, gf.data(), gf.size()));
  }
  OC_TRY(upload(op, &op->d_slots, op->slots.data(), op->slots.size()));
  OC_TRY(upload(op, &op->d_fcm, op->fcm.data(), op->fcm.size()));
  OC_TRY(upload(op, &op->d_fcp, op->fcp.data(), op->fcp.size()));
  OC_TRY(upload(op, &op->d_fpack, op->fpack.data(), op->fpack.size()));
  OC_TRY(upload(op, &op->d_fsd, op->fsd.data(), op->fsd.size()));
  OC_TRY(upload(op, &op->d_bbid, op->bbid.data(), op->bbid.size()));
  OC_TRY(upload(op, &op->d_fnrm, op->fnrm.data(), op->fnrm.size()));
  OC_TRY(upload(op, &op->d_flen, op->flen.data(), op->flen.size()));
  OC_TRY(upload(op, &op->d_fofs, op->fofs.data(), op->fofs.size()));
  op->n_fout = fo_total;
  OC_TRY(alloc(op, &op->d_fout, std::max<size_t>(fo_total, 1) * sizeof(double)));
  for (int k = 0; k < 3; ++k) OC_TRY(upload(op, &op->d_sdo[k], op->sdo[k].data(), nc));
  OC_TRY(upload(op, &op->d_cfrec, op->cfrec.data(), op->cfrec.size()));
  OC_TRY(upload(op, &op->d_cfsdo, op->cfsdo.data(), op->cfsdo.size()));
  OC_TRY(upload(op, &op->d_cfofs, op->cfofs.data(), op->cfofs.size()));
  for (int p = 1; p <= OC_MAXDEG; ++p) {
    std::vector<int> g;
    for (int c = 0; c < nc; ++c)
      if (m->degree[c] == p) g.push_back(c);
    // Mixed form: cells of a group in the order of their face records (kind,
    // neighbour degree, face points, side, subface, orientation, boundary id of
    // each slot; the neighbour's face number aside): the cells of a warp then
    // mostly take the same face paths, and fewer lanes idle on divergent branches
    // (random hp mesh 0.383 -> 0.363 ms, ensemble 3.10 -> 3.00 ms per step, A/B).
    // Cells are independent within a stage, so the order changes no result,
    // except through the batches of the zeta stop rule (batch_width > 1: cells
    // batched in index order, as the oracle does), where it is kept.  The FP64
    // form keeps the index order: its stage kernel copies the face pass's values,
    // which neighbouring cells share (hp mesh 1.61 -> 1.24 G DoF-stage/s sorted).
    if (!uniform && op->prm.batch_width == 1 && op->prm.precision == OC_PREC_MIXED) {
      OC_TRY(upload(op, &op->d_group_idx[p], g.data(), g.size()));
      auto key = [&](int c, int sl) { return op->cfrec[16 * (size_t)c + 2 * sl + 1] & ~0xC; };
      std::stable_sort(g.begin(), g.end(), [&](int x, int y) {
        for (int sl = 0; sl < 8; ++sl) {
          const int kx = key(x, sl), ky = key(y, sl);
          if (kx != ky) return kx < ky;
        }
        return false;
      });
    }
    op->group_n[p] = (int)g.size();
    if (!uniform && !g.empty()) OC_TRY(upload(op, &op->d_group[p], g.data(), g.size()));
  }
  if (op->prm.precision == OC_PREC_MIXED) {
    // FP64 zeta work area of the mixed kernels: one slot per (warp, team) of
    // every group's warps, each group rounded up to whole blocks of at most
    // kWarpsPerBlock warps: the one-launch hp grid, or the concurrent per-group
    // launches side by side (launch_groups gives each group its part)
    size_t warps = 0;
    for (int p = 1; p <= OC_MAXDEG; ++p) {
      const int cpw = (cells_per_warp(op, p) / op->prm.batch_width) * op->prm.batch_width;
      if (op->group_n[p] == 0 || cpw == 0) continue;
      warps += (op->group_n[p] + cpw - 1) / cpw + kWarpsPerBlock;
    }
    const size_t slots = warps * OC_MAXCPW;
    OC_TRY(alloc(op, (void **)&op->d_dscratch, std::max<size_t>(slots, 1) * OC_DSTRIDE * 8));
  }
  // tables
  std::vector<DegTables<double>> td(OC_MAXDEG);
  std::vector<DegTables<float>> tf(OC_MAXDEG);
  for (int p = 1; p <= OC_MAXDEG; ++p) {
    fill_tables(p, op->prm.max_iteration_height, td[p - 1]);
    cast_tables(td[p - 1], tf[p - 1]);
  }
  OC_TRY(upload_tables_p1(td.data(), tf.data()));
  OC_TRY(upload_tables_p2(td.data(), tf.data()));
  OC_TRY(upload_tables_p3(td.data(), tf.data()));
  OC_TRY(upload_tables_p4(td.data(), tf.data()));
  OC_TRY(upload_tables_p1_r1(td.data(), tf.data()));
  OC_TRY(upload_tables_p2_r1(td.data(), tf.data()));
  OC_TRY(upload_tables_p3_r1(td.data(), tf.data()));
  OC_TRY(upload_tables_p4_r1(td.data(), tf.data()));
  OC_TRY(upload(op, &op->d_tabd, td.data(), td.size()));
  OC_TRY(upload(op, &op->d_tabf, tf.data(), tf.size()));
  OC_TRY(upload_tables_hp_v0(td.data(), tf.data()));
  OC_TRY(upload_tables_hp_v1(td.data(), tf.data()));
  OC_TRY(upload_tables_hp_v2(td.data(), tf.data()));
  OC_TRY(aux_upload_tables(td.data(), tf.data()));
  OC_TRY(face_upload_tables(td.data(), tf.data()));
  OC_TRY(alloc(op, (void **)&op->d_err, kErrWords * sizeof(int)));
  OC_TRY(alloc(op, (void **)&op->d_speed, sizeof(unsigned long long)));
  OC_TRY(alloc(op, (void **)&op->d_dyn, sizeof(StageDyn) * (OC_MAXSTAGES + 1)));
  op->h_dyn = new StageDyn[OC_MAXSTAGES + 1];
  OC_TRY(configure_stage_p1());
  OC_TRY(configure_stage_p2());
  OC_TRY(configure_stage_p3());
  OC_TRY(configure_stage_p4());
  OC_TRY(configure_stage_p1_r1());
  OC_TRY(configure_stage_p2_r1());
  OC_TRY(configure_stage_p3_r1());
  OC_TRY(configure_stage_p4_r1());
  OC_TRY(configure_stage_hp_v0());
  OC_TRY(configure_stage_hp_v1());
  OC_TRY(configure_stage_hp_v2());
  OC_TRY(cudaMemset(op->d_err, 0, kErrWords * sizeof(int)));
  OC_TRY(cudaDeviceSynchronize());
  *out = op;
  return OC_OK;
}

oc_status oc_set_boundary(oc_op *op, int32_t bid, int32_t kind, int32_t fn, const double *v) {
  if (!op) return OC_ERR_INVALID_ARG;
  if (bid < 0 || bid >= OC_MAXBID) return fail(op, OC_ERR_UNKNOWN_BOUNDARY_ID, "boundary id out of range");
  if (kind < OC_BC_NONE || kind > OC_BC_ABSORBING_OUTFLOW || fn < 0 || fn > 1)
    return fail(op, OC_ERR_INVALID_ARG, "bad boundary kind or function");
  op->bc_kind[bid] = kind;
  op->bc_fn[bid] = fn;
  for (int k = 0; k < 3; ++k) op->bc_c[bid][k] = v ? v[k] : 0.0;
  op->graph_scheme = -1;
  return OC_OK;
}

oc_status oc_set_vortex(oc_op *op, const double *v) {
  if (!op || !v) return OC_ERR_INVALID_ARG;
  for (int k = 0; k < 6; ++k) op->vortex[k] = v[k];
  op->graph_scheme = -1;
  return OC_OK;
}

int64_t oc_static_data_size(const oc_op *op, int32_t which) {
  if (!op || which < 0 || which > 4) return -1;
  return op->sd_size[which];
}

oc_status oc_quadrature_points(const oc_op *op, int32_t which, double *xy) {
  if (!op || !xy || which < 0 || which > 4) return OC_ERR_INVALID_ARG;
  int64_t k = 0;
  auto map = [&](int c, double e0, double e1, double *o) {
    const double *J = &op->geo[11 * (size_t)c];
    o[0] = J[0] + J[2] * e0 + J[3] * e1;
    o[1] = J[1] + J[4] * e0 + J[5] * e1;
  };
  auto fpoint = [](int f, double s, double &e0, double &e1) {
    e0 = f == 0 ? 0. : f == 1 ? 1. : s;
    e1 = f < 2 ? s : f == 2 ? 0. : 1.;
  };
  double x[16], w[16];
  if (which <= 2) {
    for (int c = 0; c < op->n_cells; ++c) {
      const int p = op->deg[c];
      const int n = which == 0 ? cell_q(op, p) : which == 1 ? p + 2 : p + 1;
      if (which == 1) lobatto_rule(n, x, w); else gauss_rule(n, x, w);
      for (int qy = 0; qy < n; ++qy)
        for (int qx = 0; qx < n; ++qx) { map(c, x[qx], x[qy], xy + 2 * k); ++k; }
    }
  } else if (which == 3) {
    for (int f = 0; f < op->n_inner; ++f) {
      const int nfq = (op->fpack[f] >> 16) & 15, fm = op->fpack[f] & 15;
      lobatto_rule(nfq, x, w);
      for (int q = 0; q < nfq; ++q) {
        double e0, e1, pt[2];
        fpoint(fm, x[q], e0, e1);
        map(op->fcm[f], e0, e1, pt);
        const double nx = op->fnrm[2 * f], ny = op->fnrm[2 * f + 1];
        xy[2 * k] = pt[0] - 1e-12 * nx; xy[2 * k + 1] = pt[1] - 1e-12 * ny; ++k;
        xy[2 * k] = pt[0] + 1e-12 * nx; xy[2 * k + 1] = pt[1] + 1e-12 * ny; ++k;
      }
    }
  } else {
    for (int b = 0; b < op->n_bnd; ++b) {
      const int f = op->n_inner + b, c = op->fcm[f], fm = op->fpack[f] & 15;
      const int n = cell_q(op, op->deg[c]);
      gauss_rule(n, x, w);
      for (int q = 0; q < n; ++q) {
        double e0, e1;
        fpoint(fm, x[q], e0, e1);
        map(c, e0, e1, xy + 2 * k);
        ++k;
      }
    }
  }
  return OC_OK;
}

oc_status oc_set_static_data(oc_op *op, const double *c0, const double *c1, const double *c2,
                             const double *fc, const double *bn) {
  if (!op) return OC_ERR_INVALID_ARG;
  const double *src[5] = {c0, c1, c2, fc, bn};
  const double zref = op->prm.precision == OC_PREC_MIXED ? op->prm.zeta_reference : 0.0;
  OC_TRY(cudaStreamSynchronize(op->stream));
  for (int k = 0; k < 5; ++k) {
    if (op->d_sd[k]) { cudaFree(op->d_sd[k]); op->bufs.erase(std::find(op->bufs.begin(), op->bufs.end(), (void *)op->d_sd[k])); op->d_sd[k] = nullptr; }
    if (op->d_sde[k]) { cudaFree(op->d_sde[k]); op->bufs.erase(std::find(op->bufs.begin(), op->bufs.end(), (void *)op->d_sde[k])); op->d_sde[k] = nullptr; }
    if (!src[k] || op->sd_size[k] == 0) continue;
    const int64_t n = op->sd_size[k];
    OC_TRY(upload(op, &op->d_sd[k], src[k], n));
    // FP32 copy with zeta_reference folded into zb (the mixed form works on zeta - zref)
    std::vector<float> e(n);
    const int stride = k == 0 ? 5 : k == 2 ? 2 : 1;
    for (int64_t i = 0; i < n; ++i) {
      const bool is_zb = k == 3 || (i % stride) == 0;
      e[i] = (float)(is_zb ? src[k][i] + zref : src[k][i]);
    }
    OC_TRY(upload(op, &op->d_sde[k], e.data(), n));
  }
  op->graph_scheme = -1;
  return OC_OK;
}

}  // extern "C"

// --------------------------------------------------------------------------
// stage launches
// --------------------------------------------------------------------------

static void fill_common(oc_op *op, StageArgs &a) {
  std::memset(&a, 0, sizeof(a));
  a.n_cells = op->n_cells;
  a.deg = op->d_deg; a.off = op->d_off; a.geo = op->d_geo; a.slots = op->d_slots;
  a.fcm = op->d_fcm; a.fcp = op->d_fcp; a.fpack = op->d_fpack; a.fnrm = op->d_fnrm;
  a.flen = op->d_flen; a.fsd = op->d_fsd; a.bbid = op->d_bbid; a.n_inner = op->n_inner;
  a.sd0 = op->d_sd[0]; a.sd1 = op->d_sd[1]; a.sd2 = op->d_sd[2]; a.sdf = op->d_sd[3];
  a.sdb = op->d_sd[4];
  a.sd0e = op->d_sde[0]; a.sd1e = op->d_sde[1]; a.sd2e = op->d_sde[2]; a.sdfe = op->d_sde[3];
  a.sdbe = op->d_sde[4];
  a.sdo0 = op->d_sdo[0]; a.sdo1 = op->d_sdo[1]; a.sdo2 = op->d_sdo[2];
  a.cfrec = op->d_cfrec;
  a.cfofs = op->d_cfofs;
  a.n_bnd_faces = op->n_bnd; a.fofs = op->d_fofs;
  a.fout = op->d_fout;
  a.cell_rule = op->prm.cell_quadrature;
  a.n_dofs = op->n_dofs; a.n_fout = op->n_fout;
  for (int k = 0; k < 5; ++k) a.n_sd[k] = op->sd_size[k];
  a.geof = op->prm.precision == OC_PREC_MIXED ? op->d_geof : nullptr;
  a.uniform_nn = op->uniform_deg ? (op->uniform_deg + 1) * (op->uniform_deg + 1) : 0;
  a.h_ref = op->ref_h;
  a.q_ref[0] = op->ref_q[0];
  a.q_ref[1] = op->ref_q[1];
  a.ref.hr = (float)op->ref_h;
  a.ref.qr0 = (float)op->ref_q[0];
  a.ref.qr1 = (float)op->ref_q[1];
  a.ref.ur0 = a.ref.qr0 / a.ref.hr;
  a.ref.ur1 = a.ref.qr1 / a.ref.hr;
  a.ref.rr0 = std::fmaf(-a.ref.ur0, a.ref.hr, a.ref.qr0);  // exact residual (IEEE fma)
  a.ref.rr1 = std::fmaf(-a.ref.ur1, a.ref.hr, a.ref.qr1);
  a.dscratch = op->d_dscratch;
  a.gtabd = op->d_tabd;
  a.gtabf = op->d_tabf;
  a.cfsdo = (op->d_sd[3] || op->d_sd[4]) ? op->d_cfsdo : nullptr;
  const double cu = op->prm.threshold_wetdry;
  a.g = op->prm.g; a.cu4 = cu * cu * cu * cu; a.nu = op->prm.horizontal_viscosity;
  a.zeta_ref = op->prm.precision == OC_PREC_MIXED ? op->prm.zeta_reference : 0.0;
  a.wet_threshold = 1e-3;
  a.gf = (float)a.g; a.cu4f = (float)a.cu4; a.wet_thrf = (float)a.wet_threshold;
  a.zreff = (float)a.zeta_ref;
  a.friction = op->prm.friction_model; a.max_iter = op->prm.max_iteration_height;
  a.batch = op->prm.batch_width;
  for (int b = 0; b < OC_MAXBID; ++b) {
    a.bc_kind[b] = op->bc_kind[b]; a.bc_fn[b] = op->bc_fn[b];
    for (int k = 0; k < 3; ++k) a.bc_c[b][k] = op->bc_c[b][k];
  }
  for (int k = 0; k < 8; ++k) a.vortex[k] = op->vortex[k];
  a.err = op->d_err;
}

static oc_status check_boundaries(oc_op *op) {
  for (int b = 0; b < op->n_bnd; ++b)
    if (op->bc_kind[op->bbid[b]] == OC_BC_NONE)
      return fail(op, OC_ERR_UNKNOWN_BOUNDARY_ID,
                  "Unknown boundary id " + std::to_string(op->bbid[b]) +
                      ", did you set a boundary condition for this part of the domain boundary?");
  return OC_OK;
}

// launch the fused kernel over every degree group: one launch per group, or
// (hp meshes, use_hp) one launch whose grid concatenates the groups, highest
// degree first; variant 2 (the mixed reference-ABI stage) always per group
// index_order: the groups in cell-index order (d_group_idx) where they are sorted
static oc_status launch_groups(oc_op *op, StageArgs a, int variant, bool index_order = false) {
  auto group = [&](int p) {
    return index_order && op->d_group_idx[p] ? op->d_group_idx[p] : op->d_group[p];
  };
  const int batch = op->prm.batch_width;
  for (int p = 1; p <= OC_MAXDEG; ++p)
    if (op->group_n[p] && (cells_per_warp(op, p) / batch) * batch == 0)
      return fail(op, OC_ERR_UNSUPPORTED, "batch_width larger than the cells of a warp");
  // face pass of the FP64 stage: every face's flux once, both sides' values (the
  // mixed stage kernels evaluate their faces themselves)
  if (variant == 0) {
    OC_TRY(launch_face_pass(a, op->uniform_deg, op->stream));
    op->launches++;
  }
  if (op->use_hp && variant != 2 && n_groups(op) > 1) {
    const int wpb = op->hp_wpb;
    int b0 = 0;
    for (int p = OC_MAXDEG; p >= 1; --p) {
      const int n = op->group_n[p];
      const int cpw = (cells_per_warp(op, p) / batch) * batch;
      a.hp_first_block[p] = b0;
      a.hp_n[p] = n;
      a.hp_cells[p] = group(p);
      a.hp_blocks[p] = n ? (n + wpb * cpw - 1) / (wpb * cpw) : 0;
      b0 += a.hp_blocks[p];
    }
    const int hv = variant == 0 ? 0 : (a.r_is_float ? 1 : 2);
    OC_TRY(launch_stage_hp(hv, a, b0, wpb, variant >= 3, op->stream));
    op->launches++;
    return OC_OK;
  }
  // Per-group launches.  With several groups they run concurrently, one stream
  // per group (no drain between the groups, each group with its own registers and
  // block size; each group's launch gets its own part of the FP64 work area,
  // which the kernels index by block): hp step 0.480 -> 0.388 ms against the
  // groups one after the other on the handle's stream (A/B).
  const bool conc = n_groups(op) > 1;
  if (conc) {
    if (!op->gstream[1]) {
      for (int p = 1; p <= OC_MAXDEG; ++p)
        OC_TRY(cudaStreamCreateWithFlags(&op->gstream[p], cudaStreamNonBlocking));
      for (int p = 0; p <= OC_MAXDEG; ++p)
        OC_TRY(cudaEventCreateWithFlags(&op->gev[p], cudaEventDisableTiming));
    }
    OC_TRY(cudaEventRecord(op->gev[0], op->stream));
  }
  double *const dbase = a.dscratch;
  size_t woff = 0;  // warps of the work area taken by the groups before (sized in oc_create)
  for (int p = 1; p <= OC_MAXDEG; ++p) {
    const int n = op->group_n[p];
    if (n == 0) continue;
    const int cpw = (cells_per_warp(op, p) / batch) * batch;
    const int wpb = op->wpb[p];
    a.n_group = n;
    a.group_cells = op->uniform_deg ? nullptr : group(p);
    a.group_first = 0;
    const int grid = (n + wpb * cpw - 1) / (wpb * cpw);
    if (conc) {
      a.dscratch = dbase ? dbase + woff * OC_MAXCPW * OC_DSTRIDE : nullptr;
      OC_TRY(cudaStreamWaitEvent(op->gstream[p], op->gev[0], 0));
      OC_TRY(launch_stage(op, p, a, variant, grid, wpb, op->gstream[p]));
      OC_TRY(cudaEventRecord(op->gev[p], op->gstream[p]));
    } else {
      OC_TRY(launch_stage(op, p, a, variant, grid, wpb, op->stream));
    }
    woff += (size_t)(n + cpw - 1) / cpw + kWarpsPerBlock;
    op->launches++;
  }
  if (conc)
    for (int p = 1; p <= OC_MAXDEG; ++p)
      if (op->group_n[p]) OC_TRY(cudaStreamWaitEvent(op->stream, op->gev[p], 0));
  return OC_OK;
}

static oc_status read_error(oc_op *op) {
  int e[kErrWords] = {0, 0, 0, 0};
  OC_TRY(cudaMemcpyAsync(e, op->d_err, sizeof(e), cudaMemcpyDeviceToHost, op->stream));
  OC_TRY(cudaStreamSynchronize(op->stream));
  if (e[0]) {
    OC_TRY(cudaMemset(op->d_err, 0, sizeof(e)));
    if (e[0] & ERR_BOUNDS) {  // bounds-checked build: site and index of the first failure
      const int64_t idx = (int64_t)(((uint64_t)(uint32_t)e[3] << 32) | (uint32_t)e[2]);
      return fail(op, OC_ERR_BOUNDS, std::string("bounds check failed: ") + bounds_site_name(e[1]) +
                                         " index " + std::to_string(idx));
    }
    if (e[0] & ERR_UNKNOWN_BID) return fail(op, OC_ERR_UNKNOWN_BOUNDARY_ID, "unknown boundary id in a kernel");
    if (e[0] & ERR_NONFINITE) return fail(op, OC_ERR_NONFINITE, "non-finite value detected");
    return fail(op, OC_ERR_CUDA, "device error flag " + std::to_string(e[0]));
  }
  return OC_OK;
}

static oc_status ensure(oc_op *op, double **p, size_t n) {
  if (*p) return OC_OK;
  OC_TRY(alloc(op, (void **)p, n * sizeof(double)));
  return OC_OK;
}

extern "C" oc_status oc_perform_stage_hydro(oc_op *op, uint32_t stage, uint32_t n_stages,
                                            double time, const double *fr, const double *ftr,
                                            double fmat, const oc_stage_vectors *v,
                                            int32_t memory) {
  if (!op || !v || !fr) return OC_ERR_INVALID_ARG;
  if (n_stages < 1 || n_stages > OC_MAXSTAGES || stage >= n_stages)
    return fail(op, OC_ERR_INVALID_ARG, "stage out of range");
  const bool ark = ftr != nullptr;
  const int nkz = n_stages + 1, nkq = ark ? 2 * n_stages : n_stages + 1;
  if (v->n_ki_height < nkz || v->n_ki_discharge < nkq || !v->ki_height || !v->ki_discharge)
    return fail(op, OC_ERR_INVALID_ARG, "too few k vectors");
  if (!v->ri_height || !v->ri_discharge || !v->solution_height || !v->solution_discharge ||
      !v->next_height || !v->next_discharge)
    return fail(op, OC_ERR_INVALID_ARG, "null vector");
  oc_status st = check_boundaries(op);
  if (st != OC_OK) return st;
  const bool last = stage == n_stages - 1;
  const size_t nz = op->n_dofs, nq = 2 * nz;
  const bool mixed = op->prm.precision == OC_PREC_MIXED;
  StageArgs a;
  fill_common(op, a);
  StageDyn &dy = op->h_dyn[0];
  std::memset(&dy, 0, sizeof(dy));
  for (uint32_t j = 0; j <= stage; ++j) { dy.f[j] = fr[j]; dy.ft[j] = ark ? ftr[j] : 0.0; }
  dy.fm = fmat;
  dy.time = time;
  stage_dyn_round(dy);
  a.dyn = op->d_dyn;
  a.stage = (int)stage; a.n_stages = (int)n_stages; a.ark = ark; a.last = last;
  a.write_kq_last = 1;
  a.r_is_float = 0;
  // vectors: device pointers as given, or staged copies of host vectors
  const double *rz = v->ri_height, *rq = v->ri_discharge;
  double *sz = v->solution_height, *sq = v->solution_discharge;
  double *nzp = v->next_height, *nqp = v->next_discharge;
  double *kz[OC_MAXSTAGES + 1], *kq[2 * OC_MAXSTAGES];
  for (int j = 0; j < nkz; ++j) kz[j] = v->ki_height[j];
  for (int j = 0; j < nkq; ++j) kq[j] = v->ki_discharge[j];
  const bool host = memory == OC_MEM_HOST;
  if (host) {
    if (ensure(op, &op->st_rz, nz) || ensure(op, &op->st_rq, nq) || ensure(op, &op->st_sz, nz) ||
        ensure(op, &op->st_sq, nq) || ensure(op, &op->st_nz, nz) || ensure(op, &op->st_nq, nq))
      return OC_ERR_CUDA;
    for (int j = 0; j < nkz; ++j) if (ensure(op, &op->st_kz[j], nz)) return OC_ERR_CUDA;
    for (int j = 0; j < nkq; ++j) if (ensure(op, &op->st_kq[j], nq)) return OC_ERR_CUDA;
    cudaStream_t s = op->stream;
    OC_TRY(cudaMemcpyAsync(op->st_rz, rz, nz * 8, cudaMemcpyHostToDevice, s));
    OC_TRY(cudaMemcpyAsync(op->st_rq, rq, nq * 8, cudaMemcpyHostToDevice, s));
    OC_TRY(cudaMemcpyAsync(op->st_sz, sz, nz * 8, cudaMemcpyHostToDevice, s));
    OC_TRY(cudaMemcpyAsync(op->st_sq, sq, nq * 8, cudaMemcpyHostToDevice, s));
    if (ark && last) OC_TRY(cudaMemcpyAsync(op->st_nq, nqp, nq * 8, cudaMemcpyHostToDevice, s));
    // only the registers the stage reads are copied in
    for (uint32_t j = 1; j <= stage; ++j) {
      OC_TRY(cudaMemcpyAsync(op->st_kz[j], kz[j], nz * 8, cudaMemcpyHostToDevice, s));
      if (!ark) OC_TRY(cudaMemcpyAsync(op->st_kq[j], kq[j], nq * 8, cudaMemcpyHostToDevice, s));
    }
    if (ark)
      for (int j = 1; j < (int)(2 * stage + 1); ++j)
        OC_TRY(cudaMemcpyAsync(op->st_kq[j], kq[j], nq * 8, cudaMemcpyHostToDevice, s));
    rz = op->st_rz; rq = op->st_rq; sz = op->st_sz; sq = op->st_sq;
    nzp = op->st_nz; nqp = op->st_nq;
    for (int j = 0; j < nkz; ++j) kz[j] = op->st_kz[j];
    for (int j = 0; j < nkq; ++j) kq[j] = op->st_kq[j];
  }
  OC_TRY(cudaMemcpyAsync(op->d_dyn, &dy, sizeof(StageDyn), cudaMemcpyHostToDevice, op->stream));
  a.rz = rz; a.rq = rq;
  a.un_z = sz; a.un_q = sq;
  for (int j = 0; j < nkz; ++j) a.kz[j] = kz[j];
  for (int j = 0; j < nkq; ++j) a.kq[j] = kq[j];
  a.out_z = last ? sz : nzp;
  a.out_q = (last && !ark) ? sq : (ark && last ? sq : nqp);
  a.aux_q = (ark && last) ? nqp : nullptr;
  a.out_rz = nullptr; a.out_rq = nullptr;
  {
    TimedScope ts(op, SCOPE_STAGE);
    st = launch_groups(op, a, mixed ? 2 : 0);
  }
  if (st != OC_OK) return st;
  if (host) {
    cudaStream_t s = op->stream;
    OC_TRY(cudaMemcpyAsync(v->ki_height[stage + 1], op->st_kz[stage + 1], nz * 8,
                           cudaMemcpyDeviceToHost, s));
    if (!ark) {
      OC_TRY(cudaMemcpyAsync(v->ki_discharge[stage + 1], op->st_kq[stage + 1], nq * 8, cudaMemcpyDeviceToHost, s));
    } else {
      OC_TRY(cudaMemcpyAsync(v->ki_discharge[2 * stage + 1], op->st_kq[2 * stage + 1], nq * 8, cudaMemcpyDeviceToHost, s));
      if (!last) OC_TRY(cudaMemcpyAsync(v->ki_discharge[2 * stage + 2], op->st_kq[2 * stage + 2], nq * 8, cudaMemcpyDeviceToHost, s));
    }
    if (last) {
      OC_TRY(cudaMemcpyAsync(v->solution_height, op->st_sz, nz * 8, cudaMemcpyDeviceToHost, s));
      OC_TRY(cudaMemcpyAsync(v->solution_discharge, op->st_sq, nq * 8, cudaMemcpyDeviceToHost, s));
      if (ark) OC_TRY(cudaMemcpyAsync(v->next_discharge, op->st_nq, nq * 8, cudaMemcpyDeviceToHost, s));
    } else {
      OC_TRY(cudaMemcpyAsync(v->next_height, op->st_nz, nz * 8, cudaMemcpyDeviceToHost, s));
      OC_TRY(cudaMemcpyAsync(v->next_discharge, op->st_nq, nq * 8, cudaMemcpyDeviceToHost, s));
    }
  }
  return read_error(op);
}

// ---------------------------------------------------------------------------
// whole time steps with handle-owned registers, replayed as a CUDA graph
// ---------------------------------------------------------------------------

static oc_status ensure_ts(oc_op *op, const Scheme &sc) {
  const size_t nz = op->n_dofs, nq = 2 * nz;
  const bool mixed = op->prm.precision == OC_PREC_MIXED;
  const size_t ks = mixed ? 4 : 8;
  const int nkq = sc.ark ? 2 * sc.s : sc.s + 1;
  for (int j = 1; j <= sc.s; ++j)
    if (!op->ts_kz[j]) OC_TRY(alloc(op, &op->ts_kz[j], nz * ks));
  for (int j = 1; j < nkq; ++j)
    if (!op->ts_kq[j]) OC_TRY(alloc(op, &op->ts_kq[j], nq * ks));
  const size_t rs = mixed ? 4 : 8;
  for (int j = 0; j < 2; ++j) {
    if (!op->ts_rz[j]) OC_TRY(alloc(op, &op->ts_rz[j], nz * rs));
    if (!op->ts_rq[j]) OC_TRY(alloc(op, &op->ts_rq[j], nq * rs));
  }
  if (sc.ark && !op->ts_aux) OC_TRY(alloc(op, (void **)&op->ts_aux, nq * 8));
  if (sc.s == 1 && !op->ts_z0) {  // the single stage writes u^{n+1} over u^n
    OC_TRY(alloc(op, (void **)&op->ts_z0, nz * 8));
    OC_TRY(alloc(op, (void **)&op->ts_q0, nq * 8));
  }
  if (mixed && !op->ts_unzf) {
    OC_TRY(alloc(op, (void **)&op->ts_unzf, nz * 4));
    OC_TRY(alloc(op, (void **)&op->ts_unqf, nq * 4));
  }
  return OC_OK;
}

// arguments of stage st of a time step on the solution (z, q)
static void step_stage_args(oc_op *op, const Scheme &sc, int st, double *z, double *q,
                            StageArgs &a, double *oz = nullptr, double *oq = nullptr) {
  const bool mixed = op->prm.precision == OC_PREC_MIXED;
  fill_common(op, a);
  {
    const bool last = st == sc.s - 1;
    a.dyn = op->d_dyn + st;
    a.stage = st; a.n_stages = sc.s; a.ark = sc.ark; a.last = last; a.write_kq_last = 0;
    if (st == 0) {
      // a one-stage scheme overwrites u^n in place: its stage input is a copy
      // (neighbour traces must not see outputs of other blocks)
      a.rz = sc.s == 1 ? op->ts_z0 : z; a.rq = sc.s == 1 ? op->ts_q0 : q;
      a.r_is_float = 0;
    } else {
      a.rz = op->ts_rz[(st - 1) & 1]; a.rq = op->ts_rq[(st - 1) & 1];
      a.r_is_float = mixed ? 1 : 0;
    }
    a.un_z = z; a.un_q = q;
    a.cscale = op->d_cscale; a.cscalef = op->d_cscalef;
    a.fast_mixed = mixed ? 1 : 0;
    a.un_zf = (mixed && st > 0) ? op->ts_unzf : nullptr;
    a.un_qf = (mixed && st > 0) ? op->ts_unqf : nullptr;
    // stage 0 of the mixed step leaves the FP32 deviations of u^n for the later stages
    a.out_unzf = (mixed && st == 0) ? op->ts_unzf : nullptr;
    a.out_unqf = (mixed && st == 0) ? op->ts_unqf : nullptr;
    for (int j = 0; j <= sc.s; ++j) a.kz[j] = op->ts_kz[j];
    for (int j = 0; j < 2 * OC_MAXSTAGES; ++j) a.kq[j] = op->ts_kq[j];
    if (last) {  // u^{n+1} in place, or into (oz, oq) when given
      a.out_z = oz ? oz : z; a.out_q = oq ? oq : q; a.out_rz = nullptr; a.out_rq = nullptr;
      a.aux_q = sc.ark ? op->ts_aux : nullptr;
    } else if (mixed) {
      a.out_z = nullptr; a.out_q = nullptr;
      a.out_rz = (float *)op->ts_rz[st & 1]; a.out_rq = (float *)op->ts_rq[st & 1];
      a.aux_q = nullptr;
    } else {
      a.out_z = (double *)op->ts_rz[st & 1]; a.out_q = (double *)op->ts_rq[st & 1];
      a.out_rz = nullptr; a.out_rq = nullptr; a.aux_q = nullptr;
    }
  }
}

// kernel variant of the time-step path: 0 FP64; 1 mixed; 3 the mixed kernel
// compiled without static data, friction and ARK scheme, for workloads that
// use none of them; 4 the same on a conforming single-degree mesh
static int step_variant(const oc_op *op, const Scheme &sc) {
  if (op->prm.precision != OC_PREC_MIXED) return 0;
  bool lean = !sc.ark && op->prm.friction_model == 0;
  for (int k = 0; k < 5; ++k) lean = lean && !op->d_sd[k];
  return lean ? (op->conforming ? 4 : 3) : 1;
}

// Chunks of the host-vector time step (mixed form, one degree, u^n of at least
// kChunkMinBytes; otherwise n_chunks = 1): kChunks equal cell ranges and, per
// chunk, the prefix of u^n that chunks 0..k read (own DoFs and those of the
// inner-face neighbours; the last prefix is every DoF).  A smaller u^n arrives
// sooner than the chunk launches add to stage 0 (the 2,500-cell channel, 0.5 MB:
// e2e step 0.13 ms in one piece, 0.20 ms in three).
static constexpr int64_t kChunkMinBytes = (int64_t)8 << 20;
static oc_status setup_chunks(oc_op *op) {
  if (op->n_chunks) return OC_OK;
  const int nc = op->n_cells, p = op->uniform_deg, K = oc_op::kChunks;
  if (!p || op->prm.precision != OC_PREC_MIXED || 24 * op->n_dofs < kChunkMinBytes) {
    op->n_chunks = 1;
    return OC_OK;
  }
  OC_TRY(cudaStreamCreateWithFlags(&op->cstream, cudaStreamNonBlocking));
  for (int k = 0; k <= K; ++k) OC_TRY(cudaEventCreateWithFlags(&op->cev[k], cudaEventDisableTiming));
  const int64_t nn = (int64_t)(p + 1) * (p + 1);
  int64_t reach = 0;
  for (int k = 0; k < K; ++k) {
    op->chunk_first[k] = (int)((int64_t)nc * k / K);
    op->chunk_first[k + 1] = (int)((int64_t)nc * (k + 1) / K);
    for (int c = op->chunk_first[k]; c < op->chunk_first[k + 1]; ++c) {
      reach = std::max(reach, (int64_t)op->off[c] + nn);
      for (int sl = 0; sl < 8; ++sl) {
        const int other = op->cfrec[16 * (size_t)c + 2 * sl], pk = op->cfrec[16 * (size_t)c + 2 * sl + 1];
        if (((pk >> 14) & 3) == 1) reach = std::max(reach, (int64_t)other + nn);
      }
    }
    op->chunk_reach[k] = reach;
  }
  op->n_chunks = K;
  return OC_OK;
}

// enqueue the stages of one time step on op->stream (capturable; the chunked step
// and concurrent degree groups fork other streams from it and join them back)
static oc_status enqueue_step(oc_op *op, const Scheme &sc, double *z, double *q,
                              double *oz = nullptr, double *oq = nullptr,
                              const double *hz = nullptr, const double *hq = nullptr) {
  const bool mixed = op->prm.precision == OC_PREC_MIXED;
  if (sc.s == 1) {
    const size_t nz = op->n_dofs;
    OC_TRY(cudaMemcpyAsync(op->ts_z0, z, nz * 8, cudaMemcpyDeviceToDevice, op->stream));
    OC_TRY(cudaMemcpyAsync(op->ts_q0, q, 2 * nz * 8, cudaMemcpyDeviceToDevice, op->stream));
  }
  // host vectors hz, hq (chunked step): copied into z, q by pieces on the second
  // stream, one event per chunk once its prefix is in
  const bool chunked = hz && hq && op->n_chunks > 1;
  if (chunked) {
    OC_TRY(cudaEventRecord(op->cev[oc_op::kChunks], op->stream));
    OC_TRY(cudaStreamWaitEvent(op->cstream, op->cev[oc_op::kChunks], 0));
    int64_t done = 0;
    for (int k = 0; k < op->n_chunks; ++k) {
      const int64_t r = op->chunk_reach[k];
      if (r > done) {
        OC_TRY(cudaMemcpyAsync(z + done, hz + done, (r - done) * 8, cudaMemcpyHostToDevice,
                               op->cstream));
        OC_TRY(cudaMemcpyAsync(q + 2 * done, hq + 2 * done, 2 * (r - done) * 8,
                               cudaMemcpyHostToDevice, op->cstream));
        done = r;
      }
      OC_TRY(cudaEventRecord(op->cev[k], op->cstream));
    }
  }
  for (int st = 0; st < sc.s; ++st) {
    StageArgs a;
    step_stage_args(op, sc, st, z, q, a, oz, oq);
    const int variant = step_variant(op, sc);
    if (chunked && st == 0) {
      const int p = op->uniform_deg, batch = op->prm.batch_width;
      const int cpw = (cells_per_warp(op, p) / batch) * batch, wpb = op->wpb[p];
      a.group_cells = nullptr;
      for (int k = 0; k < op->n_chunks; ++k) {
        OC_TRY(cudaStreamWaitEvent(op->stream, op->cev[k], 0));
        a.group_first = op->chunk_first[k];
        a.n_group = op->chunk_first[k + 1] - op->chunk_first[k];
        OC_TRY(launch_stage(op, p, a, variant, (a.n_group + wpb * cpw - 1) / (wpb * cpw), wpb,
                            op->stream));
        op->launches++;
      }
      continue;
    }
    // the last stage writing into page-locked host vectors: cells in index order,
    // so that each warp's writes over the host link are close together (ensemble
    // e2e step 4.80 ms with the sorted order throughout, 4.55 with this, 4.63
    // unsorted; A/B)
    oc_status s = launch_groups(op, a, variant, oz != nullptr && st == sc.s - 1);
    if (s != OC_OK) return s;
  }
  return OC_OK;
}

// mean time (ms) of `reps` launches of stage 1 of a time step (stage 0 first,
// to fill its inputs); the stage reads (z, q) and writes only time-step registers
static oc_status time_stage(oc_op *op, const Scheme &sc, double *z, double *q, int reps,
                            float *ms) {
  const bool mixed = op->prm.precision == OC_PREC_MIXED;
  StageArgs a0, a1;
  step_stage_args(op, sc, 0, z, q, a0);
  step_stage_args(op, sc, sc.s > 2 ? 1 : 0, z, q, a1);
  const int variant = step_variant(op, sc);
  oc_status s = launch_groups(op, a0, variant);
  if (s != OC_OK) return s;
  cudaEvent_t e0, e1;
  OC_TRY(cudaEventCreate(&e0));
  OC_TRY(cudaEventCreate(&e1));
  for (int r = 0; r < 2 && s == OC_OK; ++r) s = launch_groups(op, a1, variant);  // warm-up
  cudaEventRecord(e0, op->stream);
  for (int r = 0; r < reps && s == OC_OK; ++r) s = launch_groups(op, a1, variant);
  cudaEventRecord(e1, op->stream);
  cudaError_t ce = cudaEventSynchronize(e1);
  float t = 0.f;
  if (ce == cudaSuccess) ce = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != OC_OK) return s;
  if (ce != cudaSuccess) return fail(op, OC_ERR_CUDA, cudaGetErrorString(ce));
  *ms = t / reps;
  return OC_OK;
}

// Launch autotuner (first time step, before the graph is captured): warps per
// block {1, 2, 4} per degree group for per-group launches and {2, 4} for the
// one-launch hp stage, each timed on a scratch copy of the solution; keeps the
// fastest configuration.  OC_LAUNCH_PER_GROUP / OC_LAUNCH_ONE fix the mode and
// tune only its block size.
static oc_status autotune(oc_op *op, const Scheme &sc, const double *z, const double *q) {
  const size_t nz = op->n_dofs, nq = 2 * nz;
  double *tz = nullptr, *tq = nullptr;
  OC_TRY(cudaMalloc((void **)&tz, nz * 8));
  OC_TRY(cudaMalloc((void **)&tq, nq * 8));
  oc_status st = OC_OK;
  cudaError_t ce = cudaMemcpyAsync(tz, z, nz * 8, cudaMemcpyDeviceToDevice, op->stream);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(tq, q, nq * 8, cudaMemcpyDeviceToDevice, op->stream);
  if (ce == cudaSuccess && sc.s == 1)  // stage input of one-stage schemes
    ce = cudaMemcpyAsync(op->ts_z0, z, nz * 8, cudaMemcpyDeviceToDevice, op->stream);
  if (ce == cudaSuccess && sc.s == 1)
    ce = cudaMemcpyAsync(op->ts_q0, q, nq * 8, cudaMemcpyDeviceToDevice, op->stream);
  if (ce != cudaSuccess) st = fail(op, OC_ERR_CUDA, cudaGetErrorString(ce));
  const int64_t launches = op->launches;
  const int reps = 5;
  const int cand[3] = {1, 2, 4};
  // per-group launches: each group alone, best block size per degree
  float per_group = 0.f;
  if (st == OC_OK && op->launch_mode != OC_LAUNCH_ONE) {
    op->use_hp = 0;
    int saved[OC_MAXDEG + 1];
    for (int p = 0; p <= OC_MAXDEG; ++p) saved[p] = op->group_n[p];
    for (int p = 1; p <= OC_MAXDEG && st == OC_OK; ++p) {
      if (!saved[p]) continue;
      for (int k = 0; k <= OC_MAXDEG; ++k) op->group_n[k] = k == p ? saved[k] : 0;
      float best = 3.4e38f;
      int bw = 4;
      for (int c = 0; c < 3 && st == OC_OK; ++c) {
        op->wpb[p] = cand[c];
        float t = 0.f;
        st = time_stage(op, sc, tz, tq, reps, &t);
        if (st == OC_OK && t < best) { best = t; bw = cand[c]; }
      }
      op->wpb[p] = bw;
      per_group += best;
    }
    for (int p = 0; p <= OC_MAXDEG; ++p) op->group_n[p] = saved[p];
    // several groups run concurrently (launch_groups): time them together
    if (st == OC_OK && n_groups(op) > 1) st = time_stage(op, sc, tz, tq, reps, &per_group);
  }
  op->tune_ms[0] = per_group;
  float one = 3.4e38f;
  if (st == OC_OK && op->launch_mode != OC_LAUNCH_PER_GROUP && hp_possible(op)) {
    op->use_hp = 1;
    int bw = 4;
    for (int c = 1; c < 3 && st == OC_OK; ++c) {
      op->hp_wpb = cand[c];
      float t = 0.f;
      st = time_stage(op, sc, tz, tq, reps, &t);
      if (st == OC_OK && t < one) { one = t; bw = cand[c]; }
    }
    op->hp_wpb = bw;
    op->tune_ms[1] = one;
  }
  op->use_hp = op->launch_mode == OC_LAUNCH_ONE ? hp_possible(op)
               : op->launch_mode == OC_LAUNCH_PER_GROUP ? 0
               : (hp_possible(op) && one < per_group);
  op->launches = launches;
  cudaStreamSynchronize(op->stream);
  cudaFree(tz);
  cudaFree(tq);
  if (st != OC_OK) return st;
  op->tuned = 1;
  return read_error(op);
}

// Device address of a page-locked host buffer (cudaHostAlloc / cudaHostRegister),
// or NULL for pageable memory.
static double *mapped_host(double *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // pageable memory may report an error on older drivers
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return static_cast<double *>(at.devicePointer);
}

extern "C" oc_status oc_perform_time_step(oc_op *op, int32_t scheme, double time, double dt,
                                          double *z, double *q, int32_t memory) {
  if (!op || !z || !q) return OC_ERR_INVALID_ARG;
  Scheme sc;
  if (!make_scheme(scheme, sc)) return fail(op, OC_ERR_INVALID_ARG, "unknown scheme");
  if (sc.ark && op->d_cscale)
    return fail(op, OC_ERR_UNSUPPORTED, "per-cell time scales with the additive scheme");
  oc_status st = check_boundaries(op);
  if (st != OC_OK) return st;
  st = ensure_ts(op, sc);
  if (st != OC_OK) return st;
  const size_t nz = op->n_dofs, nq = 2 * nz;
  double *dz = z, *dq = q;
  // host vectors: copied in; the last stage writes u^{n+1} straight into them when
  // both are page-locked host memory the GPU can address (over NVLink-C2C on
  // Grace-Blackwell, overlapping the transfer with the stage), else copied out
  double *oz = nullptr, *oq = nullptr;
  const double *hz = nullptr, *hq = nullptr;  // copied in by the graph (chunked step)
  if (memory == OC_MEM_HOST) {
    if (ensure(op, &op->ts_z, nz) || ensure(op, &op->ts_q, nq)) return OC_ERR_CUDA;
    dz = op->ts_z; dq = op->ts_q;
    oz = mapped_host(z); oq = mapped_host(q);
    if (!oz || !oq) oz = oq = nullptr;
    // page-locked vectors on a tuned operator of one degree: the graph copies u^n
    // in by pieces, overlapped with stage 0 (setup_chunks); otherwise one copy here
    if (oz && op->tuned && sc.s > 1) {
      st = setup_chunks(op);
      if (st != OC_OK) return st;
      if (op->n_chunks > 1) { hz = z; hq = q; }
    }
    if (!hz) {
      OC_TRY(cudaMemcpyAsync(op->ts_z, z, nz * 8, cudaMemcpyHostToDevice, op->stream));
      OC_TRY(cudaMemcpyAsync(op->ts_q, q, nq * 8, cudaMemcpyHostToDevice, op->stream));
    }
  }
  // coefficients: rows a_i[stage] (b_i at the last stage) times dt
  for (int s = 0; s < sc.s; ++s) {
    StageDyn &d = op->h_dyn[s];
    std::memset(&d, 0, sizeof(d));
    const bool last = s == sc.s - 1;
    for (int j = 0; j <= s; ++j) {
      d.f[j] = (last ? sc.b[j] : sc.a[s][j]) * dt;
      d.ft[j] = sc.ark ? (last ? sc.b[j] : sc.at[s][j]) * dt : 0.0;
    }
    d.fm = sc.ark && s < 2 ? sc.dt[s] * dt : 0.0;
    d.time = time + sc.c[s] * dt;
    stage_dyn_round(d);
  }
  OC_TRY(cudaMemcpyAsync(op->d_dyn, op->h_dyn, sizeof(StageDyn) * sc.s, cudaMemcpyHostToDevice,
                         op->stream));
  if (!op->tuned) {
    st = autotune(op, sc, dz, dq);
    if (st != OC_OK) return st;
  }
  if (!op->graph || op->graph_scheme != scheme || op->graph_z != dz || op->graph_q != dq ||
      op->graph_oz != oz || op->graph_oq != oq || op->graph_hz != hz || op->graph_hq != hq) {
    if (op->graph) { cudaGraphExecDestroy(op->graph); op->graph = nullptr; }
    cudaGraph_t g;
    OC_TRY(cudaStreamBeginCapture(op->stream, cudaStreamCaptureModeThreadLocal));
    const int64_t before = op->launches;
    st = enqueue_step(op, sc, dz, dq, oz, oq, hz, hq);
    cudaError_t ce = cudaStreamEndCapture(op->stream, &g);
    op->graph_launches = op->launches - before;
    op->launches = before;
    if (st != OC_OK) return st;
    if (ce != cudaSuccess) return fail(op, OC_ERR_CUDA, cudaGetErrorString(ce));
    OC_TRY(cudaGraphInstantiate(&op->graph, g, 0));
    cudaGraphDestroy(g);
    op->graph_scheme = scheme; op->graph_z = dz; op->graph_q = dq;
    op->graph_oz = oz; op->graph_oq = oq;
    op->graph_hz = hz; op->graph_hq = hq;
  }
  {
    TimedScope ts(op, SCOPE_STEP);
    OC_TRY(cudaGraphLaunch(op->graph, op->stream));
  }
  op->launches += op->graph_launches;
  if (memory == OC_MEM_HOST) {
    if (!oz) {
      OC_TRY(cudaMemcpyAsync(z, op->ts_z, nz * 8, cudaMemcpyDeviceToHost, op->stream));
      OC_TRY(cudaMemcpyAsync(q, op->ts_q, nq * 8, cudaMemcpyDeviceToHost, op->stream));
    }
    return read_error(op);
  }
  return OC_OK;
}

// ---------------------------------------------------------------------------
// auxiliary entry points
// ---------------------------------------------------------------------------

static AuxArgs aux_args(oc_op *op) {
  AuxArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n_cells = op->n_cells; a.deg = op->d_deg; a.off = op->d_off; a.geo = op->d_geo;
  a.sd1 = op->d_sd[1]; a.sd2 = op->d_sd[2]; a.sdo1 = op->d_sdo[1]; a.sdo2 = op->d_sdo[2];
  const double cu = op->prm.threshold_wetdry;
  a.g = op->prm.g; a.cu4 = cu * cu * cu * cu;
  for (int k = 0; k < 8; ++k) a.vortex[k] = op->vortex[k];
  a.n_dofs = op->n_dofs;
  for (int k = 0; k < 5; ++k) a.n_sd[k] = op->sd_size[k];
  a.cell_rule = op->prm.cell_quadrature;
  a.err = op->d_err;
  return a;
}

extern "C" int32_t oc_bounds_checked(void) {
#ifdef OC_BOUNDS_CHECK
  return 1;
#else
  return 0;
#endif
}

extern "C" oc_status oc_bounds_selftest(oc_op *op) {
  if (!op) return OC_ERR_INVALID_ARG;
  OC_TRY(launch_bounds_selftest(op->d_err, op->stream));
  op->launches++;
  return read_error(op);
}

extern "C" oc_status oc_transport_speed(oc_op *op, const double *z, const double *q,
                                        int32_t memory, double *speed) {
  if (!op || !z || !q || !speed) return OC_ERR_INVALID_ARG;
  const size_t nz = op->n_dofs, nq = 2 * nz;
  const double *dz = z, *dq = q;
  if (memory == OC_MEM_HOST) {
    if (ensure(op, &op->st_rz, nz) || ensure(op, &op->st_rq, nq)) return OC_ERR_CUDA;
    OC_TRY(cudaMemcpyAsync(op->st_rz, z, nz * 8, cudaMemcpyHostToDevice, op->stream));
    OC_TRY(cudaMemcpyAsync(op->st_rq, q, nq * 8, cudaMemcpyHostToDevice, op->stream));
    dz = op->st_rz; dq = op->st_rq;
  }
  OC_TRY(cudaMemsetAsync(op->d_speed, 0, sizeof(unsigned long long), op->stream));
  {
    TimedScope ts(op, SCOPE_SPEED);
    OC_TRY(launch_transport_speed(aux_args(op), dz, dq, op->d_speed, nullptr, op->stream));
  }
  op->launches++;
  unsigned long long bits = 0;
  OC_TRY(cudaMemcpyAsync(&bits, op->d_speed, 8, cudaMemcpyDeviceToHost, op->stream));
  oc_status st = read_error(op);
  double v;
  std::memcpy(&v, &bits, 8);
  *speed = v;
  return st;
}

extern "C" oc_status oc_apply(oc_op *op, double time, const double *sz, const double *sq,
                              double *dz, double *dq, int32_t memory) {
  if (!op || !sz || !sq || !dz || !dq) return OC_ERR_INVALID_ARG;
  oc_status st = check_boundaries(op);
  if (st != OC_OK) return st;
  const size_t nz = op->n_dofs, nq = 2 * nz;
  const double *isz = sz, *isq = sq;
  double *odz = dz, *odq = dq;
  if (memory == OC_MEM_HOST) {
    if (ensure(op, &op->st_rz, nz) || ensure(op, &op->st_rq, nq) || ensure(op, &op->st_nz, nz) ||
        ensure(op, &op->st_nq, nq))
      return OC_ERR_CUDA;
    OC_TRY(cudaMemcpyAsync(op->st_rz, sz, nz * 8, cudaMemcpyHostToDevice, op->stream));
    OC_TRY(cudaMemcpyAsync(op->st_rq, sq, nq * 8, cudaMemcpyHostToDevice, op->stream));
    isz = op->st_rz; isq = op->st_rq; odz = op->st_nz; odq = op->st_nq;
  }
  StageArgs a;
  fill_common(op, a);
  StageDyn &dy = op->h_dyn[OC_MAXSTAGES];
  std::memset(&dy, 0, sizeof(dy));
  dy.time = time;
  stage_dyn_round(dy);
  OC_TRY(cudaMemcpyAsync(op->d_dyn + OC_MAXSTAGES, &dy, sizeof(dy), cudaMemcpyHostToDevice, op->stream));
  a.dyn = op->d_dyn + OC_MAXSTAGES;
  a.apply_mode = 1; a.n_stages = 1;
  a.rz = isz; a.rq = isq; a.un_z = isz; a.un_q = isq; a.out_z = odz; a.out_q = odq;
  // FP64 variant: apply() is the plain operator
  const int saved = op->prm.precision;
  st = launch_groups(op, a, saved == OC_PREC_MIXED ? 2 : 0);
  if (st != OC_OK) return st;
  if (memory == OC_MEM_HOST) {
    OC_TRY(cudaMemcpyAsync(dz, odz, nz * 8, cudaMemcpyDeviceToHost, op->stream));
    OC_TRY(cudaMemcpyAsync(dq, odq, nq * 8, cudaMemcpyDeviceToHost, op->stream));
  }
  return read_error(op);
}

extern "C" oc_status oc_velocity_field(oc_op *op, const double *z, const double *q, double *u,
                                       int32_t memory) {
  if (!op || !z || !q || !u) return OC_ERR_INVALID_ARG;
  const size_t nz = op->n_dofs, nq = 2 * nz;
  const double *dz = z, *dq = q;
  double *du = u;
  if (memory == OC_MEM_HOST) {
    if (ensure(op, &op->st_rz, nz) || ensure(op, &op->st_rq, nq) || ensure(op, &op->st_nq, nq))
      return OC_ERR_CUDA;
    OC_TRY(cudaMemcpyAsync(op->st_rz, z, nz * 8, cudaMemcpyHostToDevice, op->stream));
    OC_TRY(cudaMemcpyAsync(op->st_rq, q, nq * 8, cudaMemcpyHostToDevice, op->stream));
    dz = op->st_rz; dq = op->st_rq; du = op->st_nq;
  }
  OC_TRY(launch_velocity_field(aux_args(op), dz, dq, du, op->stream));
  op->launches++;
  if (memory == OC_MEM_HOST)
    OC_TRY(cudaMemcpyAsync(u, du, nq * 8, cudaMemcpyDeviceToHost, op->stream));
  return read_error(op);
}

// basis values and derivatives at QGauss(nq1d) for every degree, built once per nq1d:
// [B | D], each OC_MAXDEG * 8 * OC_MAXN doubles
static oc_status vorticity_tables(oc_op *op, int nq1d, const double **dB, const double **dD) {
  const size_t sz = OC_MAXDEG * 8 * OC_MAXN;
  if (!op->d_vtab[nq1d]) {
    std::vector<double> t(2 * sz, 0.0);
    double xq[16], wq[16], xn[16], wn[16];
    gauss_rule(nq1d, xq, wq);
    for (int p = 1; p <= OC_MAXDEG; ++p) {
      lobatto_rule(p + 1, xn, wn);
      for (int k = 0; k < nq1d; ++k)
        for (int i = 0; i <= p; ++i) {
          t[((p - 1) * 8 + k) * OC_MAXN + i] = lag(p + 1, xn, i, xq[k]);
          t[sz + ((p - 1) * 8 + k) * OC_MAXN + i] = lag_d(p + 1, xn, i, xq[k]);
        }
    }
    OC_TRY(alloc(op, (void **)&op->d_vtab[nq1d], 2 * sz * 8));
    OC_TRY(cudaMemcpy(op->d_vtab[nq1d], t.data(), 2 * sz * 8, cudaMemcpyHostToDevice));
  }
  *dB = op->d_vtab[nq1d];
  *dD = op->d_vtab[nq1d] + sz;
  return OC_OK;
}

extern "C" oc_status oc_vorticity_indicator(oc_op *op, const double *u, int32_t nq1d,
                                            float *ind, int32_t memory) {
  if (!op || !u || !ind || nq1d < 1 || nq1d > 8) return OC_ERR_INVALID_ARG;
  const size_t nq = 2 * op->n_dofs;
  const double *dB = nullptr, *dD = nullptr;
  oc_status vs = vorticity_tables(op, nq1d, &dB, &dD);
  if (vs != OC_OK) return vs;
  const double *du = u;
  float *dind = ind;
  float *tmp = nullptr;
  if (memory == OC_MEM_HOST) {
    if (ensure(op, &op->st_nq, nq)) return OC_ERR_CUDA;
    OC_TRY(cudaMemcpyAsync(op->st_nq, u, nq * 8, cudaMemcpyHostToDevice, op->stream));
    du = op->st_nq;
    OC_TRY(cudaMalloc((void **)&tmp, op->n_cells * sizeof(float)));
    dind = tmp;
  }
  OC_TRY(launch_vorticity(aux_args(op), du, nq1d, dB, dD, dind, op->stream));
  op->launches++;
  if (memory == OC_MEM_HOST)
    OC_TRY(cudaMemcpyAsync(ind, tmp, op->n_cells * sizeof(float), cudaMemcpyDeviceToHost, op->stream));
  oc_status st = read_error(op);
  if (tmp) cudaFree(tmp);
  return st;
}

extern "C" oc_status oc_errors_vortex(oc_op *op, double time, const double *z, const double *q,
                                      int32_t memory, double *errors) {
  if (!op || !z || !q || !errors) return OC_ERR_INVALID_ARG;
  const size_t nz = op->n_dofs, nq = 2 * nz;
  const double *dz = z, *dq = q;
  if (memory == OC_MEM_HOST) {
    if (ensure(op, &op->st_rz, nz) || ensure(op, &op->st_rq, nq)) return OC_ERR_CUDA;
    OC_TRY(cudaMemcpyAsync(op->st_rz, z, nz * 8, cudaMemcpyHostToDevice, op->stream));
    OC_TRY(cudaMemcpyAsync(op->st_rq, q, nq * 8, cudaMemcpyHostToDevice, op->stream));
    dz = op->st_rz; dq = op->st_rq;
  }
  if (ensure(op, &op->d_epart, 2 * (size_t)op->n_cells + 2)) return OC_ERR_CUDA;
  double *dout = op->d_epart + 2 * (size_t)op->n_cells;
  OC_TRY(launch_errors(aux_args(op), time, op->d_sd[0], op->d_sdo[0], dz, dq, op->d_epart, dout,
                       op->stream));
  op->launches += 2;
  OC_TRY(cudaMemcpyAsync(errors, dout, 2 * sizeof(double), cudaMemcpyDeviceToHost, op->stream));
  return read_error(op);
}

extern "C" oc_status oc_conservative_coarsening(oc_op *op, const uint8_t *mark, double *z,
                                                int32_t memory) {
  if (!op || !mark || !z) return OC_ERR_INVALID_ARG;
  const size_t nz = op->n_dofs, nc = op->n_cells;
  const unsigned char *dmark = mark;
  double *dz = z;
  unsigned char *tmark = nullptr;
  if (memory == OC_MEM_HOST) {
    if (ensure(op, &op->st_rz, nz)) return OC_ERR_CUDA;
    OC_TRY(cudaMalloc((void **)&tmark, nc));
    OC_TRY(cudaMemcpyAsync(tmark, mark, nc, cudaMemcpyHostToDevice, op->stream));
    OC_TRY(cudaMemcpyAsync(op->st_rz, z, nz * 8, cudaMemcpyHostToDevice, op->stream));
    dmark = tmark; dz = op->st_rz;
  }
  OC_TRY(launch_conservative_coarsening(aux_args(op), dmark, dz, op->stream));
  op->launches++;
  if (memory == OC_MEM_HOST)
    OC_TRY(cudaMemcpyAsync(z, dz, nz * 8, cudaMemcpyDeviceToHost, op->stream));
  oc_status st = read_error(op);
  if (tmark) cudaFree(tmark);
  return st;
}

extern "C" oc_status oc_indicator_features(oc_op *op, const double *z, const double *q,
                                           const int32_t *info, int32_t n_members, float thr,
                                           float *feat, float *flags, float *vort,
                                           int32_t memory) {
  if (!op || !z || !q || !info || !feat || n_members < 1) return OC_ERR_INVALID_ARG;
  const size_t nz = op->n_dofs, nq = 2 * nz, nc = op->n_cells;
  int pmax = 1;
  for (int p = 1; p <= OC_MAXDEG; ++p)
    if (op->group_n[p]) pmax = p;
  const double *dB = nullptr, *dD = nullptr;
  oc_status vs = vorticity_tables(op, pmax, &dB, &dD);  // QGauss(max degree), hpTuner.h:261
  if (vs != OC_OK) return vs;
  if (ensure(op, &op->d_ivel, nq)) return OC_ERR_CUDA;
  if (!op->d_ivort) OC_TRY(alloc(op, (void **)&op->d_ivort, nc * sizeof(float)));
  if (op->imax_n < n_members) {
    OC_TRY(alloc(op, (void **)&op->d_imax, n_members * sizeof(unsigned)));
    op->imax_n = n_members;
  }
  const double *dz = z, *dq = q;
  const int *dinfo = info;
  float *dfeat = feat, *dflags = flags, *dvort = vort;
  std::vector<void *> tmp;
  if (memory == OC_MEM_HOST) {
    void *p[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const size_t sz[6] = {nz * 8, nq * 8, nc * 6 * 4, nc * 12 * 4, nc * 4, nc * 4};
    for (int k = 0; k < 6; ++k) {
      if ((k == 4 && !flags) || (k == 5 && !vort)) continue;
      OC_TRY(cudaMalloc(&p[k], sz[k]));
      tmp.push_back(p[k]);
    }
    OC_TRY(cudaMemcpyAsync(p[0], z, sz[0], cudaMemcpyHostToDevice, op->stream));
    OC_TRY(cudaMemcpyAsync(p[1], q, sz[1], cudaMemcpyHostToDevice, op->stream));
    OC_TRY(cudaMemcpyAsync(p[2], info, sz[2], cudaMemcpyHostToDevice, op->stream));
    dz = (double *)p[0]; dq = (double *)p[1]; dinfo = (int *)p[2];
    dfeat = (float *)p[3]; dflags = (float *)p[4]; dvort = (float *)p[5];
  }
  const AuxArgs a = aux_args(op);
  OC_TRY(launch_velocity_field(a, dz, dq, op->d_ivel, op->stream));
  OC_TRY(launch_vorticity(a, op->d_ivel, pmax, dB, dD, op->d_ivort, op->stream));
  OC_TRY(launch_features(a, dz, dq, op->d_ivort, dinfo, n_members, op->d_imax, thr, dfeat,
                         dflags, dvort, op->stream));
  op->launches += 4;
  if (memory == OC_MEM_HOST) {
    OC_TRY(cudaMemcpyAsync(feat, dfeat, nc * 12 * 4, cudaMemcpyDeviceToHost, op->stream));
    if (flags) OC_TRY(cudaMemcpyAsync(flags, dflags, nc * 4, cudaMemcpyDeviceToHost, op->stream));
    if (vort) OC_TRY(cudaMemcpyAsync(vort, dvort, nc * 4, cudaMemcpyDeviceToHost, op->stream));
  }
  oc_status st = read_error(op);
  for (void *p : tmp) cudaFree(p);
  return st;
}

extern "C" oc_status oc_project_vortex(oc_op *op, double time, double *z, double *q,
                                       int32_t memory) {
  if (!op || !z || !q) return OC_ERR_INVALID_ARG;
  const size_t nz = op->n_dofs, nq = 2 * nz;
  double *dz = z, *dq = q;
  if (memory == OC_MEM_HOST) {
    if (ensure(op, &op->st_nz, nz) || ensure(op, &op->st_nq, nq)) return OC_ERR_CUDA;
    dz = op->st_nz; dq = op->st_nq;
  }
  OC_TRY(launch_project_vortex(aux_args(op), time, dz, dq, op->stream));
  op->launches++;
  if (memory == OC_MEM_HOST) {
    OC_TRY(cudaMemcpyAsync(z, dz, nz * 8, cudaMemcpyDeviceToHost, op->stream));
    OC_TRY(cudaMemcpyAsync(q, dq, nq * 8, cudaMemcpyDeviceToHost, op->stream));
  }
  return read_error(op);
}

extern "C" oc_status oc_set_timing(oc_op *op, int32_t on) {
  if (!op) return OC_ERR_INVALID_ARG;
  op->timing = on ? 1 : 0;
  return OC_OK;
}

extern "C" oc_status oc_timer_summary(oc_op *op, char *text, int64_t size) {
  if (!op || !text || size <= 0) return OC_ERR_INVALID_ARG;
  resolve_timers(op);
  std::string out;
  char line[256];
  for (const auto &sc : op->scopes) {
    std::snprintf(line, sizeof line, "%s\t%lld\t%.9g\t%.9g\n", sc.name, (long long)sc.calls,
                  sc.seconds, sc.calls ? sc.seconds / sc.calls : 0.0);
    out += line;
  }
  if ((int64_t)out.size() + 1 > size) return fail(op, OC_ERR_INVALID_ARG, "timer text buffer too small");
  std::memcpy(text, out.c_str(), out.size() + 1);
  return OC_OK;
}

extern "C" oc_status oc_set_cell_time_scale(oc_op *op, const double *scale) {
  if (!op) return OC_ERR_INVALID_ARG;
  if (!scale) {
    if (op->d_cscale) {
      OC_TRY(cudaStreamSynchronize(op->stream));
      for (void *p : {(void *)op->d_cscale, (void *)op->d_cscalef}) {
        cudaFree(p);
        op->bufs.erase(std::find(op->bufs.begin(), op->bufs.end(), p));
      }
      op->d_cscale = nullptr;
      op->d_cscalef = nullptr;
    }
  } else {
    std::vector<float> f(op->n_cells);
    for (int c = 0; c < op->n_cells; ++c) {
      if (!(scale[c] > 0.0) || !std::isfinite(scale[c]))
        return fail(op, OC_ERR_INVALID_ARG, "time scale of cell " + std::to_string(c) +
                                                " is not a positive finite number");
      f[c] = (float)scale[c];
    }
    if (!op->d_cscale) {
      OC_TRY(alloc(op, (void **)&op->d_cscale, op->n_cells * sizeof(double)));
      OC_TRY(alloc(op, (void **)&op->d_cscalef, op->n_cells * sizeof(float)));
    }
    OC_TRY(cudaStreamSynchronize(op->stream));
    OC_TRY(cudaMemcpy(op->d_cscale, scale, op->n_cells * sizeof(double), cudaMemcpyHostToDevice));
    OC_TRY(cudaMemcpy(op->d_cscalef, f.data(), op->n_cells * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (op->graph) {  // the captured step holds the old pointers
    cudaGraphExecDestroy(op->graph);
    op->graph = nullptr;
  }
  return OC_OK;
}

extern "C" oc_status oc_cell_transport_speed(oc_op *op, const double *z, const double *q,
                                             int32_t memory, double *speed) {
  if (!op || !z || !q || !speed) return OC_ERR_INVALID_ARG;
  const size_t nz = op->n_dofs, nq = 2 * nz;
  const double *dz = z, *dq = q;
  double *out = speed;
  if (memory == OC_MEM_HOST) {
    if (ensure(op, &op->st_rz, nz) || ensure(op, &op->st_rq, nq) ||
        ensure(op, &op->st_nz, std::max<size_t>(nz, op->n_cells)))
      return OC_ERR_CUDA;
    OC_TRY(cudaMemcpyAsync(op->st_rz, z, nz * 8, cudaMemcpyHostToDevice, op->stream));
    OC_TRY(cudaMemcpyAsync(op->st_rq, q, nq * 8, cudaMemcpyHostToDevice, op->stream));
    dz = op->st_rz; dq = op->st_rq; out = op->st_nz;
  }
  OC_TRY(cudaMemsetAsync(op->d_speed, 0, sizeof(unsigned long long), op->stream));
  OC_TRY(launch_transport_speed(aux_args(op), dz, dq, op->d_speed, out, op->stream));
  op->launches++;
  if (memory == OC_MEM_HOST)
    OC_TRY(cudaMemcpyAsync(speed, out, op->n_cells * 8, cudaMemcpyDeviceToHost, op->stream));
  return read_error(op);
}

// Handle data for oc_transport_speed_noalloc (oc_noalloc.cu): reads the handle only.
namespace oc {
bool noalloc_aux_args(const oc_op *op, AuxArgs *a, cudaStream_t *stream) {
  if (!op || !op->d_geo) return false;
  *a = aux_args(const_cast<oc_op *>(op));
  *stream = op->stream;
  return true;
}
void noalloc_set_error(oc_op *op, const std::string &msg) {
  if (op) op->err = msg;
}
}  // namespace oc
