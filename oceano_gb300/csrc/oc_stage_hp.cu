// One-launch stage over every degree group of an hp mesh (stage_kernel_hp),
// compiled once per kernel variant with -DOC_HP_VARIANT=v so that the variants
// build in parallel:
//   0: FP64 form; 1: mixed time step, FP32 stage input; 2: mixed time step,
//   FP64 stage input (stage 0).  The mixed variants also come as a lean kernel
//   (no static data, friction or ARK scheme).
// Each translation unit owns its copy of the constant-bank shape tables.
#include "oc_kernels.cuh"

#ifndef OC_HP_VARIANT
#error "OC_HP_VARIANT must be defined"
#endif
#define OC_CAT2(a, b) a##b
#define OC_CAT(a, b) OC_CAT2(a, b)

namespace oc {

#if OC_HP_VARIANT == 0
using HpR = double; using HpKT = double; using HpRIN = double;
static constexpr bool kHpMix = false;
#elif OC_HP_VARIANT == 1
using HpR = float; using HpKT = float; using HpRIN = float;
static constexpr bool kHpMix = true;
#else
using HpR = float; using HpKT = float; using HpRIN = double;
static constexpr bool kHpMix = true;
#endif

static const int kMaxWarpsPerBlock = 4;

// shared memory of one warp: the largest of the four degrees
static constexpr int hp_warp_bytes() {
  int m = Dims<1>::warp_bytes<HpR>();
  m = Dims<2>::warp_bytes<HpR>() > m ? Dims<2>::warp_bytes<HpR>() : m;
  m = Dims<3>::warp_bytes<HpR>() > m ? Dims<3>::warp_bytes<HpR>() : m;
  m = Dims<4>::warp_bytes<HpR>() > m ? Dims<4>::warp_bytes<HpR>() : m;
  return m;
}

cudaError_t OC_CAT(configure_stage_hp_v, OC_HP_VARIANT)() {
  cudaError_t e = cudaFuncSetAttribute(stage_kernel_hp<HpR, HpKT, kHpMix, HpRIN, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kMaxWarpsPerBlock * hp_warp_bytes());
  if (e == cudaSuccess && kHpMix)
    e = cudaFuncSetAttribute(stage_kernel_hp<HpR, HpKT, kHpMix, HpRIN, kHpMix>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kMaxWarpsPerBlock * hp_warp_bytes());
  return e;
}

cudaError_t OC_CAT(launch_stage_hp_v, OC_HP_VARIANT)(const StageArgs &a, int grid, int wpb,
                                                     bool lean, cudaStream_t st) {
  if (wpb > kMaxWarpsPerBlock) return cudaErrorInvalidValue;
  if (kHpMix && lean)
    return launch_programmatic(stage_kernel_hp<HpR, HpKT, kHpMix, HpRIN, kHpMix>, grid, wpb * 32,
                               wpb * hp_warp_bytes(), st, a);
  return launch_programmatic(stage_kernel_hp<HpR, HpKT, kHpMix, HpRIN, false>, grid, wpb * 32,
                             wpb * hp_warp_bytes(), st, a);
}

cudaError_t OC_CAT(upload_tables_hp_v, OC_HP_VARIANT)(const DegTables<double> *td,
                                                       const DegTables<float> *tf) {
  cudaError_t e = cudaMemcpyToSymbol(c_tabd, td, sizeof(DegTables<double>) * OC_MAXDEG);
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_tabf, tf, sizeof(DegTables<float>) * OC_MAXDEG);
}

}  // namespace oc
