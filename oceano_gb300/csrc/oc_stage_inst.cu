// Instantiations of the fused stage kernel for one degree (compiled once per
// degree with -DOC_DEGREE=p so that the four degrees build in parallel).
// Each translation unit owns its copy of the constant-bank shape tables.
#include "oc_kernels.cuh"

#ifndef OC_DEGREE
#error "OC_DEGREE must be defined"
#endif
#define OC_CAT2(a, b) a##b
#define OC_CAT(a, b) OC_CAT2(a, b)

namespace oc {

static const int kMaxWarpsPerBlock = 4;

template <typename R, typename KT, bool MIX, typename RIN, bool LEAN = false>
static cudaError_t configure_one() {
  constexpr int P = OC_DEGREE;
  const int smem = kMaxWarpsPerBlock * Dims<P>::template warp_bytes<R>();
  return cudaFuncSetAttribute(stage_kernel<P, R, KT, MIX, RIN, LEAN>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

template <typename R, typename KT, bool MIX, typename RIN, bool LEAN = false>
static cudaError_t launch_one(const StageArgs &a, int grid, int wpb, cudaStream_t st) {
  constexpr int P = OC_DEGREE;
  if (wpb > kMaxWarpsPerBlock) return cudaErrorInvalidValue;
  const int smem = wpb * Dims<P>::template warp_bytes<R>();
  return launch_programmatic(stage_kernel<P, R, KT, MIX, RIN, LEAN>, grid, wpb * 32, smem, st,
                             a);
}

// dynamic shared-memory opt-in, done once at set-up (outside any stream capture)
cudaError_t OC_CAT(configure_stage_p, OC_DEGREE)() {
  cudaError_t e = configure_one<double, double, false, double>();
  if (e == cudaSuccess) e = configure_one<float, float, true, float>();
  if (e == cudaSuccess) e = configure_one<float, float, true, double>();
  if (e == cudaSuccess) e = configure_one<float, double, true, double>();
  if (e == cudaSuccess) e = configure_one<float, float, true, float, true>();
  if (e == cudaSuccess) e = configure_one<float, float, true, double, true>();
  return e;
}

// variant 0: FP64; 1: mixed time step with FP32 registers (FP64 stage input at
// stage 0, FP32 afterwards); 2: mixed reference-ABI stage (FP64 registers and
// vectors); 3: variant 1 compiled without static data, friction and ARK scheme
// (the lean kernel of workloads that use none of them)
cudaError_t OC_CAT(launch_stage_p, OC_DEGREE)(const StageArgs &a, int variant, int grid, int wpb,
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
    default: return cudaErrorInvalidValue;
  }
}

int OC_CAT(stage_cells_per_warp_p, OC_DEGREE)() { return Dims<OC_DEGREE>::CPW; }

cudaError_t OC_CAT(upload_tables_p, OC_DEGREE)(const DegTables<double> *td,
                                                const DegTables<float> *tf) {
  cudaError_t e = cudaMemcpyToSymbol(c_tabd, td, sizeof(DegTables<double>) * OC_MAXDEG);
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_tabf, tf, sizeof(DegTables<float>) * OC_MAXDEG);
}

}  // namespace oc
