/*
 * oceano_gpu.h -- C ABI of the GB300-native per-stage DG shallow-water operator.
 *
 * Drop-in for the two timed scopes of oceano's
 * SpaceDiscretization::OceanoOperator (lib/include/space_discretization/OceanDG.h):
 *   "rk_stage hydro - integrals L_h"      (OceanDG.h:1796, :1954)
 *   "rk_stage hydro - inv mass + vec upd"  (OceanDG.h:1829, :2009)
 * Plain pointers and sizes only; no exceptions cross this boundary.  Every call
 * returns an oc_status and sets a per-handle message readable with
 * oc_last_error().  One caller per handle (the reference runs one thread per
 * MPI rank, OceanDG.h:462-463); separate handles are independent.
 *
 * Vectors use deal.II's DoFHandler layout for FE_DGQ(p) on Gauss-Lobatto nodes:
 *   height    : cell-major, (p+1)^2 lexicographic nodal values per cell;
 *   discharge : cell-major, component-blocked FESystem(FE_DGQ(p),2) values per
 *               cell: [hu_0..hu_{n-1}, hv_0..hv_{n-1}], n = (p+1)^2;
 * in the cell order of oc_mesh_desc (offsets are the prefix sums of (p+1)^2).
 */
#ifndef OCEANO_GPU_H
#define OCEANO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  OC_OK = 0,
  OC_ERR_INVALID_ARG = 1,
  OC_ERR_UNKNOWN_BOUNDARY_ID = 2, /* OceanDG.h:1199-1203 AssertThrow */
  OC_ERR_NONFINITE = 3,
  OC_ERR_TIMEOUT = 4,
  OC_ERR_CUDA = 5,
  OC_ERR_UNSUPPORTED = 6,
  OC_ERR_NOMEM = 7,
  OC_ERR_BOUNDS = 8 /* bounds-checked build: an index read from a mesh table out of range */
} oc_status;

/* where the vector pointers of a call live */
enum { OC_MEM_HOST = 0, OC_MEM_DEVICE = 1 };

/* arithmetic of the operator */
enum {
  OC_PREC_FP64 = 0, /* everything in FP64: the plain form */
  OC_PREC_MIXED = 1 /* FP32 bulk (sum factorisation, fluxes, inverse masses), FP64 RK
                       accumulation and FP64 well-balanced differences */
};

/* boundary kinds of ICBC::BcBase (lib/include/icbc/IcbcBase.h:44-133) */
enum {
  OC_BC_NONE = 0,
  OC_BC_WALL = 1,
  OC_BC_SUPERCRITICAL_INFLOW = 2,
  OC_BC_SUPERCRITICAL_OUTFLOW = 3,
  OC_BC_HEIGHT_INFLOW = 4,
  OC_BC_DISCHARGE_INFLOW = 5,
  OC_BC_ABSORBING_OUTFLOW = 6
};
/* boundary data functions: constants, or the travelling vortex
 * (lib/include/icbc/Icbc_ShallowWaterVortex.h:139-226) */
enum { OC_FN_CONSTANT = 0, OC_FN_VORTEX = 1 };

/* Runge-Kutta schemes of lib/include/time_integrator/time_stepping.h */
enum {
  OC_ERK_FORWARD_EULER = 0,
  OC_ERK_SSP22 = 1,
  OC_ERK_SSP33 = 2,
  OC_ERK_RK4 = 3,
  OC_ERK_STAGE3_ORDER2 = 4,
  OC_ARK_STAGE3_ORDER2 = 5 /* Giraldo explicit + TR-BDF2 implicit friction */
};

typedef struct oc_op oc_op;

/*
 * Mesh in MatrixFree face-batch terms (what a deal.II adapter fills from
 * MatrixFree::get_face_info): cells with degree and the 4 vertices of an
 * affine cell (deal.II order v0=(0,0), v1=(1,0), v2=(0,1), v3=(1,1)); inner
 * faces first, then boundary faces (n_inner_face_batches /
 * n_boundary_face_batches, OceanDG.h:542, :558).  Face numbers: 0 x-, 1 x+,
 * 2 y-, 3 y+.  For a hanging face the minus (interior) cell is the finer one
 * and subface (0/1) is the half of the plus cell's face it covers; -1 marks a
 * conforming face.  Periodic faces are inner faces.
 */
typedef struct {
  int32_t n_cells;
  const int32_t *degree;      /* [n_cells], 1..4 */
  const double *vertices;     /* [n_cells*8] */
  int32_t n_inner_faces;
  int32_t n_boundary_faces;
  const int32_t *cell_m;      /* [n_inner + n_bnd] */
  const int32_t *cell_p;      /* [n_inner] */
  const int8_t *face_m;       /* [n_inner + n_bnd] */
  const int8_t *face_p;       /* [n_inner] */
  const int8_t *subface;      /* [n_inner] */
  const int8_t *orientation;  /* [n_inner] or NULL */
  const int32_t *boundary_id; /* [n_bnd], 0..15 */
} oc_mesh_desc;

/* Parameter names and defaults follow lib/include/io/ParameterReader.h */
typedef struct {
  double g;                    /* Physical constants/g = 9.81 */
  double threshold_wetdry;     /* Physical constants/Threshold_for_wetdry = 0.1 */
  double horizontal_viscosity; /* constant eddy viscosity = 0 */
  int32_t friction_model;      /* 0 none, 1 linear, 2 Manning (BottomFriction.h) */
  int32_t max_iteration_height;/* main.cc:226 = 15 */
  int32_t batch_width;         /* SIMD lanes of a cell batch for the zeta stop rule */
  int32_t precision;           /* OC_PREC_FP64 or OC_PREC_MIXED */
  double zeta_reference;       /* mixed form: FP32 free surface is stored as zeta - this */
  int32_t cell_quadrature;     /* Gauss points per direction of the cell integrals, boundary
                                  faces, cell/boundary static data and errors (the reference's
                                  n_points_1d, main.cc:216): OC_CELL_RULE_DEFAULT or
                                  OC_CELL_RULE_P1 */
} oc_params;

/* cell Gauss rules (oc_params.cell_quadrature) */
enum {
  OC_CELL_RULE_DEFAULT = 0, /* floor(1.5 p) + 1 points per direction (main.cc:216) */
  OC_CELL_RULE_P1 = 1       /* p + 1 points per direction (4x4 at p = 3) */
};

/* Replaces OceanoOperator::OceanoOperator + reinit + initialize_data_at_quadrature
 * (OceanDG.h:387-470, :497-569): uploads geometry and face tables. */
oc_status oc_create(const oc_mesh_desc *mesh, const oc_params *params, oc_op **out);
void oc_destroy(oc_op *op);
const char *oc_last_error(const oc_op *op);

/* Number of scalar DoFs of the height vector (discharge has twice as many);
 * replaces OceanoOperator::initialize_vector (OceanDG.h:243-245). */
int64_t oc_n_dofs(const oc_op *op);

/* ICBC::BcBase::set_*_boundary (IcbcBase.h:141-286).  values: 3 constants
 * (zeta, u, v; or zeta; or normal discharge in slot 1) for OC_FN_CONSTANT. */
oc_status oc_set_boundary(oc_op *op, int32_t boundary_id, int32_t kind, int32_t function,
                          const double *values);
/* vortex parameters: h0, u_inf, r0, Gamma, x0, y0 (Icbc_ShallowWaterVortex.h:56-61) */
oc_status oc_set_vortex(oc_op *op, const double *params6);

/*
 * Static problem data at quadrature points (OceanDG.h:497-569), host arrays in
 * the storage order of oc_quadrature_points; NULL means identically zero.
 *   cell0: Gauss n_q = floor(1.5p)+1 per direction, 5 values per point
 *          (zb, friction coefficient, wind x, wind y, Coriolis f)
 *   cell1: Gauss-Lobatto p+2, zb
 *   cell2: Gauss p+1, (zb, friction coefficient)
 *   face : inner faces, Gauss-Lobatto max(p-,p+)+2 points, (zb at x-1e-12n, zb at x+1e-12n)
 *   bnd  : boundary faces, Gauss n_q of the cell, zb
 */
oc_status oc_set_static_data(oc_op *op, const double *cell0, const double *cell1,
                             const double *cell2, const double *face, const double *bnd);
/* number of doubles of static array `which` (0 cell0, 1 cell1, 2 cell2, 3 face, 4 bnd) */
int64_t oc_static_data_size(const oc_op *op, int32_t which);
/* coordinates (x,y pairs) of the points of static array `which`; for faces two
 * points per quadrature point (shifted by -/+1e-12 along the minus normal) */
oc_status oc_quadrature_points(const oc_op *op, int32_t which, double *xy);

/*
 * One Runge-Kutta stage: OceanoOperator::perform_stage_hydro
 * (ERK OceanDG.h:183-196 / :1782-1912, ARK :197-208 / :1936-2119).
 *   factor_residual[stage+1]     : a_i[stage] or b_i, already times dt
 *   factor_tilde_residual        : NULL for explicit RK, else a~_i[stage] or b_i
 *   factor_matrix                : d~[stage]*dt (public member factor_matrix, :163)
 *   ri_height, ri_discharge      : current_ri[0], current_ri[1]
 *   ri_velocity                  : current_ri.back(); may be NULL when viscosity is 0
 *   ki_height[n_stages+1]        : vec_ki_height;  [stage+1] receives L_h zeta
 *   ki_discharge[n_stages+1]     : ERK: vec_ki_discharge, [stage+1] receives M^-1 L_h q
 *   ki_discharge[2*n_stages]     : ARK: [2s+1] explicit and [2s+2] stiff residuals
 *   ki_*[0] are scratch; their contents after the call are unspecified.
 *   solution_*, next_*           : as in the reference (last stage updates solution_*)
 * memory = OC_MEM_HOST copies vectors in and out; OC_MEM_DEVICE works in place.
 */
typedef struct {
  const double *ri_height;
  const double *ri_discharge;
  const double *ri_velocity;
  double *const *ki_height;
  int32_t n_ki_height;
  double *const *ki_discharge;
  int32_t n_ki_discharge;
  double *solution_height;
  double *solution_discharge;
  double *next_height;
  double *next_discharge;
} oc_stage_vectors;

oc_status oc_perform_stage_hydro(oc_op *op, uint32_t stage, uint32_t n_stages, double time,
                                 const double *factor_residual,
                                 const double *factor_tilde_residual, double factor_matrix,
                                 const oc_stage_vectors *vectors, int32_t memory);

/*
 * A whole time step: ExplicitRungeKuttaIntegrator::perform_time_step
 * (ExplicitRungeKuttaIntegrator.h:179-298) or AdditiveRungeKuttaIntegrator::
 * perform_time_step (AdditiveRungeKuttaIntegrator.h:206-339), with all stage
 * registers owned by the handle and the stage sequence replayed as a CUDA graph.
 * height/discharge are updated in place.  With OC_MEM_HOST they are copied in;
 * when both are page-locked (cudaHostAlloc / cudaHostRegister) the last stage
 * writes u^{n+1} into them directly, overlapping the transfer with the stage,
 * else they are copied out; on a mesh of one degree in the mixed form the copy
 * in then goes in three pieces, each chunk of stage 0 starting once its cells'
 * and their neighbours' DoFs have arrived.  The call returns when the host vectors hold u^{n+1}
 * (and reports device-side errors); with OC_MEM_DEVICE it returns once the step
 * is enqueued, and oc_synchronize reports its device-side errors.
 */
oc_status oc_perform_time_step(oc_op *op, int32_t scheme, double time, double dt,
                               double *height, double *discharge, int32_t memory);

/* OceanoOperator::compute_cell_transport_speed (OceanDG.h:2505-2580); the
 * result also carries a non-finite check (OC_ERR_NONFINITE). */
oc_status oc_transport_speed(oc_op *op, const double *height, const double *discharge,
                             int32_t memory, double *speed);

/* OceanoOperator::apply documented semantics (OceanDG.h:1658-1691):
 * dst = M^-1 L_h(t, src) with the exact Gauss(p+1) cell inverse for all three
 * variables (the reference's own apply() is dead code, OceanDG.h:1692-1727). */
oc_status oc_apply(oc_op *op, double time, const double *src_height,
                   const double *src_discharge, double *dst_height, double *dst_discharge,
                   int32_t memory);

/* OceanoOperator::evaluate_velocity_field (OceanDG.h:2599-2662) */
oc_status oc_velocity_field(oc_op *op, const double *height, const double *discharge,
                            double *velocity, int32_t memory);

/* hpTuner::estimate_error, vorticity indicator (lib/include/deal.II_oceano/hpTuner.h:247-305):
 * per cell max over QGauss(n_q_1d) points of |dv/dx - du/dy| of the velocity field */
oc_status oc_vorticity_indicator(oc_op *op, const double *velocity, int32_t n_q_1d,
                                 float *indicator, int32_t memory);

/* OceanoOperator::project_hydro (OceanDG.h:2241-2352) of the vortex exact solution
 * at time t (component 0 is zeta, components 1-2 velocity). */
oc_status oc_project_vortex(oc_op *op, double time, double *height, double *discharge,
                            int32_t memory);

/*
 * Transport-speed maximum without any device allocation.  No counterpart in
 * the reference: it serves callers that may not call cudaMalloc when they need
 * dt (hosts whose device memory belongs to a pool or arena they must not
 * bypass, real-time loops that forbid allocation after start-up, embedding
 * frameworks that account for every device byte).  height and discharge are
 * device vectors, speed is one device double written on the handle's stream
 * (NaN if a point speed is not finite, where oc_transport_speed returns
 * OC_ERR_NONFINITE); the call does not synchronise.  Scratch is a fixed device
 * array inside the library: at most 524,288 cells (else OC_ERR_UNSUPPORTED,
 * before any launch); calls that overlap on the GPU share it and race.  The
 * first call on a device sets it up (once per device, thread-safe) and should
 * come before any stream capture; a device reset after that call is not
 * supported.  Failures set oc_last_error; a CUDA error pending from earlier
 * work is reported (OC_ERR_CUDA) and not cleared.
 */
oc_status oc_transport_speed_noalloc(oc_op *op, const double *height, const double *discharge,
                                     double *speed);

/* Independent instances with their own step size in one launch (no reference
 * counterpart): oc_perform_time_step(dt) advances cell c by dt * scale[c]
 * (scale[c] > 0; the cells of one instance share it), so that the members of
 * an ensemble keep their own dt.  Boundary data are evaluated at the unscaled
 * time.  scale = NULL restores 1.  Explicit schemes only (the additive scheme
 * returns OC_ERR_UNSUPPORTED while scales are set); oc_perform_stage_hydro
 * ignores them. */
oc_status oc_set_cell_time_scale(oc_op *op, const double *scale);
/* compute_cell_transport_speed (OceanDG.h:2505-2580) per cell: speed[c] is the
 * maximum over the cell's Gauss-Lobatto (p+2)^2 points (the reference's value is
 * the maximum over all cells); host or device array per `memory`. */
oc_status oc_cell_transport_speed(oc_op *op, const double *height, const double *discharge,
                                  int32_t memory, double *speed);

/* Reference state of the mixed form (no reference counterpart; ignored by the
 * FP64 form): a constant depth h_ref = zeta_ref + zb_ref and discharge (qx, qy),
 * typically the undisturbed background of the run (h0, h0 u_inf).  The FP32
 * stage inputs hold q - q_ref and every flux is evaluated minus its value at
 * the reference state, which has no weak divergence: exact arithmetic is
 * unchanged, while FP32 rounding scales with the deviation.  The values are
 * rounded to FP32-representable numbers.  Default: depth 1, discharge 0. */
oc_status oc_set_reference_state(oc_op *op, double depth, double qx, double qy);

/* Launch configuration of the stage kernels (no reference counterpart: deal.II's
 * MatrixFree loops have no launch shape).  OC_LAUNCH_AUTO (default) times, at the
 * first oc_perform_time_step, one launch per degree group with 1, 2 or 4 warps
 * per block (the groups' launches run concurrently, one stream each) against one
 * launch over all groups (hp meshes) with 2 or 4, on a scratch copy of the
 * solution, and keeps the fastest.  The other modes fix the
 * launch shape and tune only the block size.  Setting a mode drops the tuned
 * configuration and the captured step graph. */
#define OC_LAUNCH_AUTO 0
#define OC_LAUNCH_PER_GROUP 1
#define OC_LAUNCH_ONE 2
oc_status oc_set_launch_mode(oc_op *op, int32_t mode);
/* out[0] one launch for all groups (0/1), out[1] its warps per block,
 * out[2..5] warps per block of the degree 1..4 groups, out[6] tuned (0/1) */
oc_status oc_launch_config(const oc_op *op, int32_t *out);

/* compute_errors_hydro (OceanDG.h:2380-2459) with the travelling vortex of
 * oc_set_vortex as the exact solution at `time`: errors[0] = L2 error of the
 * depth, errors[1] = L2 error of the discharge (both components), on the cell
 * Gauss rule, zb from the cell static data (0 without). errors is a host array. */
oc_status oc_errors_vortex(oc_op *op, double time, const double *height, const double *discharge,
                           int32_t memory, double *errors);
/* prepare_for_conservative_coarsening (OceanDG.h:2732-2778): on every cell with
 * mark[c] != 0 (degree p -> 0 in the next remesh) all nodal height values become the
 * average of zeta over the wet Gauss-Lobatto (p+2) points; cells with no wet point
 * are left unchanged.  height is updated in place. */
oc_status oc_conservative_coarsening(oc_op *op, const uint8_t *mark, double *height,
                                     int32_t memory);

/* ---- learned refinement indicator (no reference counterpart) -------------------
 * The reference refines where the vorticity indicator (hpTuner.h:247-305) exceeds
 * a fraction of its maximum (main.cc:749-765).  The functions below compute
 * per-cell features of the state on the GPU and train / evaluate a small BF16
 * multilayer perceptron that predicts those flags some steps ahead.
 *
 * oc_indicator_features: per cell c, from (zeta, q) and
 *   cell_info[6c + 0..3] = neighbour cell across faces 0..3 (-1 on the boundary;
 *                          on a coarse face with two fine neighbours, either),
 *   cell_info[6c + 4]    = refinement level, cell_info[6c + 5] = member index
 *                          (< n_members; the vorticity maximum is taken per member),
 * writes features[12c + 0..11] = cell means of zeta, hu, hv; L = log10(|w/max| + 1e-12);
 *   (L(face 1) - L(face 0)) / 2, (L(face 3) - L(face 2)) / 2 from the face neighbours;
 *   the four neighbours' L; level; degree (the threshold lies decades below the bulk
 *   of w/max, hence the log scale).  The vorticity is the reference indicator (max over QGauss(p_max)
 *   points of |dv/dx - du/dy|).  flags (may be NULL): 1 where w/max > threshold.
 *   vorticity (may be NULL): w/max per cell. */
oc_status oc_indicator_features(oc_op *op, const double *zeta, const double *q,
                                const int32_t *cell_info, int32_t n_members, float threshold,
                                float *features, float *flags, float *vorticity, int32_t memory);

#define OC_MLP_FEATURES 12
#define OC_MLP_HIDDEN 64
#define OC_MLP_PARAMS (64 * 12 + 64 + 64 * 64 + 64 + 64 + 1)
typedef struct oc_mlp oc_mlp;
/* seeded He-uniform initialisation; all array arguments of the oc_mlp_* calls
 * below are device pointers unless named host */
oc_status oc_mlp_create(uint64_t seed, oc_mlp **out);
void oc_mlp_destroy(oc_mlp *m);
const char *oc_mlp_last_error(const oc_mlp *m);
void *oc_mlp_stream(oc_mlp *m);
oc_status oc_mlp_synchronize(oc_mlp *m);
/* FP32 master parameters, host arrays of OC_MLP_PARAMS floats */
oc_status oc_mlp_get_params(oc_mlp *m, float *host_params);
oc_status oc_mlp_set_params(oc_mlp *m, const float *host_params);
/* input normalisation (mean[12], 1/std[12]), host arrays; fit from n feature rows */
oc_status oc_mlp_get_normalization(oc_mlp *m, float *host_mean_inv_std);
oc_status oc_mlp_set_normalization(oc_mlp *m, const float *host_mean_inv_std);
oc_status oc_mlp_fit_normalization(oc_mlp *m, const float *features, int64_t n);
/* logits of n feature rows */
oc_status oc_mlp_forward(oc_mlp *m, const float *features, int64_t n, float *logits);
/* mean weighted BCE-with-logits loss (host) and its gradient, kept in the handle
 * and copied to host_grad when not NULL */
oc_status oc_mlp_gradient(oc_mlp *m, const float *features, const float *labels, int64_t n,
                          float pos_weight, float *host_grad, double *host_loss);
/* one Adam step (beta 0.9, 0.999, eps 1e-8) with the handle's gradient */
oc_status oc_mlp_adam_step(oc_mlp *m, float lr);

/* GPU time by the reference's TimerOutput scopes (no reference counterpart in the
 * ABI: the reference times its own calls, OceanDG.h:1796, :1829, main.cc's
 * "rk time stepping total" and "compute transport speed"; here the two stage
 * scopes are one fused launch).  With timing on, the GPU work of each
 * oc_perform_stage_hydro, oc_perform_time_step and oc_transport_speed call is
 * bracketed by CUDA events on the handle's stream; every call also opens an NVTX
 * range of that name.  oc_timer_summary writes one line per scope,
 * "name<TAB>calls<TAB>total seconds<TAB>seconds per call", waiting for pending work. */
oc_status oc_set_timing(oc_op *op, int32_t on);
oc_status oc_timer_summary(oc_op *op, char *text, int64_t size);

/* Waits for the handle's stream, then reports and clears the device-side error
 * flags raised since the last check: OC_ERR_UNKNOWN_BOUNDARY_ID from a face
 * kernel, OC_ERR_NONFINITE when a time step or a last stage wrote a non-finite
 * u^{n+1}.  Calls on device vectors (OC_MEM_DEVICE) return without waiting, so
 * their device-side errors surface here (or at the next call on host vectors). */
oc_status oc_synchronize(oc_op *op);

/* Bounds-checked build.  A library compiled with OC_BOUNDS_CHECK range-checks
 * every index its kernels read from the mesh tables (cell ids and degrees, DoF
 * offsets, face records, boundary ids, static-data and face-pass offsets) where
 * it is loaded; an index out of range is replaced by 0 so that no access leaves
 * its array, and the next call that reads the device flags (oc_synchronize, or
 * any call on host vectors) returns OC_ERR_BOUNDS, with the site and the index
 * of the first failure in oc_last_error.  Without the macro the checks compile
 * to nothing.  oc_bounds_checked returns 1 in the bounds-checked build, else 0.
 * oc_bounds_selftest runs one device thread that checks an index outside its
 * range (no memory is accessed with it) and returns what the flags then report:
 * OC_ERR_BOUNDS ("bounds check failed: self-test index 5") in the
 * bounds-checked build, OC_OK otherwise. */
int32_t oc_bounds_checked(void);
oc_status oc_bounds_selftest(oc_op *op);
/* the stream the handle launches on */
void *oc_stream(oc_op *op);
/* kernels launched by this handle since creation (launch accounting) */
int64_t oc_launch_count(const oc_op *op);

#ifdef __cplusplus
}
#endif
#endif /* OCEANO_GPU_H */
