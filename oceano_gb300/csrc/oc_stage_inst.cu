// Instantiations of the fused stage kernel for one degree and one cell Gauss
// rule (compiled once per (degree, rule) with -DOC_DEGREE=p -DOC_CELL_RULE=r so
// that the units build in parallel).  Rule 0: floor(1.5 p) + 1 Gauss points per
// direction (main.cc:216); rule 1: p + 1.  The entry points of rule 1 carry the
// suffix _r1.  Each translation unit owns its copy of the constant-bank shape
// tables.
#include "oc_kernels.cuh"

#ifndef OC_DEGREE
#error "OC_DEGREE must be defined"
#endif
#ifndef OC_CELL_RULE
#define OC_CELL_RULE 0
#endif
#define OC_CAT2(a, b) a##b
#define OC_CAT(a, b) OC_CAT2(a, b)
#if OC_CELL_RULE == 1
#define OC_NAME(base) OC_CAT(OC_CAT(base, OC_DEGREE), _r1)
#else
#define OC_NAME(base) OC_CAT(base, OC_DEGREE)
#endif

namespace oc {

static const int kMaxWarpsPerBlock = 4;
static constexpr int kRule = OC_CELL_RULE;

template <typename R, typename KT, bool MIX, typename RIN, bool LEAN = false, bool CONF = false>
static cudaError_t configure_one() {
  constexpr int P = OC_DEGREE;
  const int smem = kMaxWarpsPerBlock * Dims<P, kRule>::template warp_bytes<R>();
  return cudaFuncSetAttribute(stage_kernel<P, R, KT, MIX, RIN, LEAN, kRule, CONF>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

template <typename R, typename KT, bool MIX, typename RIN, bool LEAN = false, bool CONF = false>
static cudaError_t launch_one(const StageArgs &a, int grid, int wpb, cudaStream_t st) {
  constexpr int P = OC_DEGREE;
  if (wpb > kMaxWarpsPerBlock) return cudaErrorInvalidValue;
  const int smem = wpb * Dims<P, kRule>::template warp_bytes<R>();
  return launch_programmatic(stage_kernel<P, R, KT, MIX, RIN, LEAN, kRule, CONF>, grid,
                             wpb * 32, smem, st, a);
}

// dynamic shared-memory opt-in, done once at set-up (outside any stream capture)
cudaError_t OC_NAME(configure_stage_p)() {
  cudaError_t e = configure_one<double, double, false, double>();
  if (e == cudaSuccess) e = configure_one<float, float, true, float>();
  if (e == cudaSuccess) e = configure_one<float, float, true, double>();
  if (e == cudaSuccess) e = configure_one<float, double, true, double>();
  if (e == cudaSuccess) e = configure_one<float, float, true, float, true>();
  if (e == cudaSuccess) e = configure_one<float, float, true, double, true>();
  if (e == cudaSuccess) e = configure_one<float, float, true, float, true, true>();
  if (e == cudaSuccess) e = configure_one<float, float, true, double, true, true>();
  return e;
}

// variant 0: FP64; 1: mixed time step with FP32 registers (FP64 stage input at
// stage 0, FP32 afterwards); 2: mixed reference-ABI stage (FP64 registers and
// vectors); 3: variant 1 compiled without static data, friction and ARK scheme
// (the lean kernel of workloads that use none of them); 4: variant 3 for a
// conforming mesh of this degree alone (no hanging face, standard orientation)
cudaError_t OC_NAME(launch_stage_p)(const StageArgs &a, int variant, int grid, int wpb,
                                    cudaStream_t st) {
  switch (variant) {
    case 0: return launch_one<double, double, false, double>(a, grid, wpb, st);
    case 1:
      return a.r_is_float ? launch_one<float, float, true, float>(a, grid, wpb, st)
                          : launch_one<float, float, true, double>(a, grid, wpb, st);
    case 2: return launch_one<float, double, true, double>(a, grid, wpb, st);
    case 3:
      return a.r_is_float ? launch_one<float, float, true, float, true>(a, grid, wpb, st)
                          : launch_one<float, float, true, double, true>(a, grid, wpb, st);
    case 4:
      return a.r_is_float ? launch_one<float, float, true, float, true, true>(a, grid, wpb, st)
                          : launch_one<float, float, true, double, true, true>(a, grid, wpb, st);
    default: return cudaErrorInvalidValue;
  }
}

int OC_NAME(stage_cells_per_warp_p)() { return Dims<OC_DEGREE, kRule>::CPW; }

cudaError_t OC_NAME(upload_tables_p)(const DegTables<double> *td, const DegTables<float> *tf) {
  cudaError_t e = cudaMemcpyToSymbol(c_tabd, td, sizeof(DegTables<double>) * OC_MAXDEG);
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_tabf, tf, sizeof(DegTables<float>) * OC_MAXDEG);
}

}  // namespace oc
