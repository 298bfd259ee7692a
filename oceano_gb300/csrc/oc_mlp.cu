// Learned refinement indicator: a 12-64-64-1 multilayer perceptron with BF16
// weights and activations (FP32 accumulation, FP32 master weights), evaluated
// and trained on the GPU.  It predicts, from per-cell features of the state,
// whether the vorticity indicator (hpTuner.h:247-305 with the relative
// thresholds of main.cc:749-765) will flag the cell some steps ahead.
//
// Parameter vector (FP32, OC_MLP_PARAMS floats):
//   W1 [64][12] | b1 [64] | W2 [64][64] | b2 [64] | w3 [64] | b3
// Forward, per sample x (12 features):
//   xh = bf16((x - mean) * inv_std)
//   h1 = bf16(relu(b1 + W1 xh)),  h2 = bf16(relu(b2 + W2 h1)),  z = b3 + w3 . h2
// with W1, W2, w3 rounded to BF16.  Loss: mean over samples of the weighted
// binary cross-entropy with logits, weight pos_weight on positive labels.
// The gradient treats the BF16 roundings as identities (straight-through).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "oceano_gpu.h"

namespace {

constexpr int NF = OC_MLP_FEATURES, NH = OC_MLP_HIDDEN, NP = OC_MLP_PARAMS;
constexpr int OW1 = 0, OB1 = OW1 + NH * NF, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH,
              OB3 = OW3 + NH;
static_assert(OB3 + 1 == NP, "parameter layout");

constexpr int kGradBlocks = 304;   // persistent gradient grid (2 per SM)

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// ---------------------------------------------------------------------------
// Forward pass on the BF16 tensor cores (mma.sync m16n8k16, FP32 accumulation).
// One warp evaluates 16 samples per MMA row block: layer 1 is X [16 x 16] (12
// features, zero-padded) times W1^T [16 x 64] (8 MMAs), layer 2 is
// H1 [16 x 64] times W2^T [64 x 64] (4 k-steps x 8 n-tiles = 32 MMAs), layer 3
// a dot product with w3 reduced over the quad of lanes that share a row.  The
// accumulator fragment of layer 1 (rows g, g+8; columns 8j + 2t, +1 of n-tile
// j) is exactly the A fragment of layer 2 for k-tile j/2, so the activations
// never leave registers; the weights are held as B fragments in registers for
// the whole kernel.  Biases enter as the accumulators' initial values.
// (g = lane / 4, t = lane % 4, PTX ISA fragment layout of mma.m16n8k16.)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x (low half) = lo
  return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

constexpr int kMmaWarps = 4;

__global__ void __launch_bounds__(32 * kMmaWarps) mlp_forward_mma_kernel(
    const float *w, const float *norm, const float *feat, int64_t n, float *logit) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  // B fragments: layer 1 n-tile j: k = 2t, 2t+1 | 2t+8, 2t+9 (k >= 12: padding),
  // column n = 8j + g; layer 2 k-tile kk, n-tile j: k = 16kk + 2t (+1 | +8, +9)
  uint32_t B1[8][2], B2[4][8][2];
  float bias1[8][2], bias2[8][2], w3v[8][2];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float *r1 = w + OW1 + (8 * j + g) * NF;
    B1[j][0] = pack_bf16(r1[2 * t], r1[2 * t + 1]);
    B1[j][1] = t < 2 ? pack_bf16(r1[2 * t + 8], r1[2 * t + 9]) : 0u;
    const float *r2 = w + OW2 + (8 * j + g) * NH;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      B2[kk][j][0] = pack_bf16(r2[16 * kk + 2 * t], r2[16 * kk + 2 * t + 1]);
      B2[kk][j][1] = pack_bf16(r2[16 * kk + 2 * t + 8], r2[16 * kk + 2 * t + 9]);
    }
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int col = 8 * j + 2 * t + e;
      bias1[j][e] = w[OB1 + col];
      bias2[j][e] = w[OB2 + col];
      w3v[j][e] = bf(w[OW3 + col]);
    }
  }
  const float b3 = w[OB3];
  // normalisation of the four feature columns this lane holds
  const int fc[4] = {2 * t, 2 * t + 1, 2 * t + 8, 2 * t + 9};
  float mu[4], is[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    mu[e] = fc[e] < NF ? norm[fc[e]] : 0.f;
    is[e] = fc[e] < NF ? norm[NF + fc[e]] : 0.f;
  }
  const int64_t tiles = (n + 15) / 16;
  const int64_t warp0 = (int64_t)blockIdx.x * kMmaWarps + (threadIdx.x >> 5);
  const int64_t nwarps = (int64_t)gridDim.x * kMmaWarps;
  for (int64_t tile = warp0; tile < tiles; tile += nwarps) {
    const int64_t r0 = 16 * tile + g, r1 = r0 + 8;
    float x0[4], x1[4];  // rows r0, r1 at columns fc[]
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const bool col = fc[e] < NF;
      x0[e] = (col && r0 < n) ? bf((feat[r0 * NF + fc[e]] - mu[e]) * is[e]) : 0.f;
      x1[e] = (col && r1 < n) ? bf((feat[r1 * NF + fc[e]] - mu[e]) * is[e]) : 0.f;
    }
    const uint32_t a0 = pack_bf16(x0[0], x0[1]), a1 = pack_bf16(x1[0], x1[1]);
    const uint32_t a2 = pack_bf16(x0[2], x0[3]), a3 = pack_bf16(x1[2], x1[3]);
    // layer 1 -> A fragments of layer 2
    uint32_t H[4][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float c[4] = {bias1[j][0], bias1[j][1], bias1[j][0], bias1[j][1]};
      mma_bf16(c, a0, a1, a2, a3, B1[j][0], B1[j][1]);
      const uint32_t lo = pack_bf16(fmaxf(c[0], 0.f), fmaxf(c[1], 0.f));  // row g
      const uint32_t hi = pack_bf16(fmaxf(c[2], 0.f), fmaxf(c[3], 0.f));  // row g + 8
      H[j >> 1][(j & 1) * 2 + 0] = lo;
      H[j >> 1][(j & 1) * 2 + 1] = hi;
    }
    // layer 2 and the layer-3 dot products of rows g and g + 8
    float z0 = 0.f, z1 = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float c[4] = {bias2[j][0], bias2[j][1], bias2[j][0], bias2[j][1]};
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        mma_bf16(c, H[kk][0], H[kk][1], H[kk][2], H[kk][3], B2[kk][j][0], B2[kk][j][1]);
      z0 = fmaf(w3v[j][0], bf(fmaxf(c[0], 0.f)), z0);
      z0 = fmaf(w3v[j][1], bf(fmaxf(c[1], 0.f)), z0);
      z1 = fmaf(w3v[j][0], bf(fmaxf(c[2], 0.f)), z1);
      z1 = fmaf(w3v[j][1], bf(fmaxf(c[3], 0.f)), z1);
    }
    z0 += __shfl_xor_sync(0xffffffffu, z0, 1);
    z0 += __shfl_xor_sync(0xffffffffu, z0, 2);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 1);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 2);
    if (t == 0) {
      if (r0 < n) logit[r0] = b3 + z0;
      if (r1 < n) logit[r1] = b3 + z1;
    }
  }
}

// ---------------------------------------------------------------------------
// Gradient on the BF16 tensor cores (mma.sync m16n8k16, FP32 accumulation).
// A block of 4 warps takes 64 samples per tile.
// Phase 1, warp w on samples 16w .. 16w+15 of the tile: the forward pass as in
// mlp_forward_mma_kernel, the loss and dz = dL/dz, d2 = [h2 > 0] dz w3 and
// d1 = [h1 > 0] W2^T d2 (MMAs: d2 as A operand, W2 as B; the accumulator
// fragments of d2 are the A fragments, as in the forward pass).  The
// back-propagated signals enter every MMA as two BF16 terms, hi = bf16(d) and
// lo = bf16(d - hi), which keeps about 16 bits of their FP32 values; xh, h1
// and the BF16 weights are exact in BF16.  Phase 1 leaves xh, h1, d2 and d1
// transposed in shared memory ([column][sample], rows padded against bank
// conflicts).  Phase 2, warp w owning rows 16w .. 16w+15 of dW2 and of dW1:
// dW2 += d2^T h1 and dW1 += d1^T xh over the tile's 64 samples (4 k-steps of
// 16), accumulators in registers across the block's tiles.  Bias, w3 and b3
// sums come from phase 1's registers.  The block's partial gradient and loss go
// to part[block][NP + 1] (summed in a fixed order by mlp_reduce_kernel).
// ---------------------------------------------------------------------------
constexpr int kGradWarps = 4;
constexpr int kTile = 16 * kGradWarps;  // samples per block tile
constexpr int kTS = kTile + 8;          // row stride (BF16) of the transposed buffers

struct GradSmem {
  uint32_t B1[8][2][32];      // layer-1 B fragments (per lane)
  uint32_t B2[4][8][2][32];   // layer-2 B fragments: W2^T
  uint32_t BW2[4][8][2][32];  // back-propagation B fragments: W2
  __nv_bfloat16 xhT[16][kTS];  // [feature (12 + padding)][sample]
  __nv_bfloat16 h1T[NH][kTS];
  __nv_bfloat16 d2T[2][NH][kTS];  // hi, lo
  __nv_bfloat16 d1T[2][NH][kTS];
  float bias1[NH], bias2[NH], w3[NH];  // w3 rounded to BF16
  float colsum[kGradWarps][3][NH];  // per warp: d1, d2 and dz h2 column sums
  float b3sum[kGradWarps];
  double loss[kGradWarps];
};

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *p) {
  return *reinterpret_cast<const uint32_t *>(p);
}

// hi and lo BF16 terms of v (v ~= hi + lo)
__device__ __forceinline__ void split_bf16(float v, float &hi, float &lo) {
  hi = bf(v);
  lo = bf(v - hi);
}

__global__ void __launch_bounds__(32 * kGradWarps) mlp_grad_mma_kernel(
    const float *w, const float *norm, const float *feat, const float *label, int64_t n,
    float pos_weight, float inv_n, float *part) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GradSmem &S = *reinterpret_cast<GradSmem *>(smem_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
  // B fragments (the lane's entries), as in the forward kernel; BW2: B[k = j][n = k']
  // = W2[j][k'], rows j = 16kk + 2t (+1 | +8, +9), column k' = 8nk + g
  for (int idx = warp; idx < 8; idx += kGradWarps) {
    const int j = idx;
    const float *r1 = w + OW1 + (8 * j + g) * NF;
    S.B1[j][0][lane] = pack_bf16(r1[2 * t], r1[2 * t + 1]);
    S.B1[j][1][lane] = t < 2 ? pack_bf16(r1[2 * t + 8], r1[2 * t + 9]) : 0u;
    const float *r2 = w + OW2 + (8 * j + g) * NH;
    for (int kk = 0; kk < 4; ++kk) {
      S.B2[kk][j][0][lane] = pack_bf16(r2[16 * kk + 2 * t], r2[16 * kk + 2 * t + 1]);
      S.B2[kk][j][1][lane] = pack_bf16(r2[16 * kk + 2 * t + 8], r2[16 * kk + 2 * t + 9]);
      const float *c2 = w + OW2 + 8 * j + g;  // column 8j + g of W2, rows j'
      S.BW2[kk][j][0][lane] =
          pack_bf16(c2[(16 * kk + 2 * t) * NH], c2[(16 * kk + 2 * t + 1) * NH]);
      S.BW2[kk][j][1][lane] =
          pack_bf16(c2[(16 * kk + 2 * t + 8) * NH], c2[(16 * kk + 2 * t + 9) * NH]);
    }
  }
  for (int e = threadIdx.x; e < 4 * kTS; e += blockDim.x)  // feature rows 12..15 stay 0
    S.xhT[12 + e / kTS][e % kTS] = __float2bfloat16_rn(0.f);
  for (int c = threadIdx.x; c < NH; c += blockDim.x) {
    S.bias1[c] = w[OB1 + c];
    S.bias2[c] = w[OB2 + c];
    S.w3[c] = bf(w[OW3 + c]);
  }
  const float b3 = w[OB3];
  const int fc[4] = {2 * t, 2 * t + 1, 2 * t + 8, 2 * t + 9};
  float mu[4], is[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    mu[e] = fc[e] < NF ? norm[fc[e]] : 0.f;
    is[e] = fc[e] < NF ? norm[NF + fc[e]] : 0.f;
  }
  float acc2[8][4], acc1[2][4];  // dW2 rows 16w + g (+8) x 64; dW1 rows 16w + g (+8) x 16
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc2[j][e] = 0.f;
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc1[j][e] = 0.f;
  float sd1[8][2], sd2[8][2], sw3[8][2], sb3 = 0.f;  // column sums of rows g and g + 8
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int e = 0; e < 2; ++e) sd1[j][e] = sd2[j][e] = sw3[j][e] = 0.f;
  double loss = 0.0;
  __syncthreads();

  const int64_t tiles = (n + kTile - 1) / kTile;
  for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    // ---- phase 1: warp w, samples s0 = 16w + g and s1 = s0 + 8 of the tile
    const int s0 = 16 * warp + g, s1 = s0 + 8;
    const int64_t r0 = tile * kTile + s0, r1 = tile * kTile + s1;
    float x0[4], x1[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const bool col = fc[e] < NF;
      x0[e] = (col && r0 < n) ? bf((feat[r0 * NF + fc[e]] - mu[e]) * is[e]) : 0.f;
      x1[e] = (col && r1 < n) ? bf((feat[r1 * NF + fc[e]] - mu[e]) * is[e]) : 0.f;
      if (col) {
        S.xhT[fc[e]][s0] = __float2bfloat16_rn(x0[e]);
        S.xhT[fc[e]][s1] = __float2bfloat16_rn(x1[e]);
      }
    }
    const uint32_t a0 = pack_bf16(x0[0], x0[1]), a1 = pack_bf16(x1[0], x1[1]);
    const uint32_t a2 = pack_bf16(x0[2], x0[3]), a3 = pack_bf16(x1[2], x1[3]);
    uint32_t H[4][4];
    uint32_t m1 = 0u;  // h1 > 0: bit 4j + e (e: c0..c3 of n-tile j)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float ba = S.bias1[8 * j + 2 * t], bb = S.bias1[8 * j + 2 * t + 1];
      float c[4] = {ba, bb, ba, bb};
      mma_bf16(c, a0, a1, a2, a3, S.B1[j][0][lane], S.B1[j][1][lane]);
      float h[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        h[e] = bf(fmaxf(c[e], 0.f));
        m1 |= (h[e] > 0.f ? 1u : 0u) << (4 * j + e);
      }
      H[j >> 1][(j & 1) * 2 + 0] = pack_bf16(h[0], h[1]);
      H[j >> 1][(j & 1) * 2 + 1] = pack_bf16(h[2], h[3]);
      const int col = 8 * j + 2 * t;
      S.h1T[col][s0] = __float2bfloat16_rn(h[0]);
      S.h1T[col + 1][s0] = __float2bfloat16_rn(h[1]);
      S.h1T[col][s1] = __float2bfloat16_rn(h[2]);
      S.h1T[col + 1][s1] = __float2bfloat16_rn(h[3]);
    }
    float h2[8][4], z0 = 0.f, z1 = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float ba = S.bias2[8 * j + 2 * t], bb = S.bias2[8 * j + 2 * t + 1];
      float c[4] = {ba, bb, ba, bb};
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        mma_bf16(c, H[kk][0], H[kk][1], H[kk][2], H[kk][3], S.B2[kk][j][0][lane],
                 S.B2[kk][j][1][lane]);
#pragma unroll
      for (int e = 0; e < 4; ++e) h2[j][e] = bf(fmaxf(c[e], 0.f));
      const float wa = S.w3[8 * j + 2 * t], wb = S.w3[8 * j + 2 * t + 1];
      z0 = fmaf(wa, h2[j][0], z0);
      z0 = fmaf(wb, h2[j][1], z0);
      z1 = fmaf(wa, h2[j][2], z1);
      z1 = fmaf(wb, h2[j][3], z1);
    }
    z0 += __shfl_xor_sync(0xffffffffu, z0, 1);
    z0 += __shfl_xor_sync(0xffffffffu, z0, 2);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 1);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 2);
    z0 += b3;
    z1 += b3;
    // weighted BCE with logits: wt (softplus(z) - y z); dL/dz = wt (sigmoid(z) - y) / n
    float dz[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t r = h ? r1 : r0;
      const float z = h ? z1 : z0;
      const bool ok = r < n;
      const float y = ok ? label[r] : 0.f;
      const float wt = ok ? (y > 0.5f ? pos_weight : 1.f) : 0.f;
      if (t == 0) loss += (double)(wt * (fmaxf(z, 0.f) + log1pf(expf(-fabsf(z))) - y * z));
      dz[h] = wt * (1.f / (1.f + expf(-z)) - y) * inv_n;
    }
    if (t == 0) sb3 += dz[0] + dz[1];
    // d2 = [h2 > 0] dz w3 (accumulator layout), its A fragments (hi, lo) and its
    // transposed copy for phase 2
    uint32_t D2[2][4][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float hi[4], lo[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float d = h2[j][e] > 0.f ? dz[e >> 1] * S.w3[8 * j + 2 * t + (e & 1)] : 0.f;
        sd2[j][e & 1] += d;
        sw3[j][e & 1] += dz[e >> 1] * h2[j][e];
        split_bf16(d, hi[e], lo[e]);
      }
      D2[0][j >> 1][(j & 1) * 2 + 0] = pack_bf16(hi[0], hi[1]);
      D2[0][j >> 1][(j & 1) * 2 + 1] = pack_bf16(hi[2], hi[3]);
      D2[1][j >> 1][(j & 1) * 2 + 0] = pack_bf16(lo[0], lo[1]);
      D2[1][j >> 1][(j & 1) * 2 + 1] = pack_bf16(lo[2], lo[3]);
      const int col = 8 * j + 2 * t;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int cc = col + (e & 1), ss = (e >> 1) ? s1 : s0;
        S.d2T[0][cc][ss] = __float2bfloat16_rn(hi[e]);
        S.d2T[1][cc][ss] = __float2bfloat16_rn(lo[e]);
      }
    }
    // d1 = [h1 > 0] W2^T d2
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int p = 0; p < 2; ++p)
          mma_bf16(c, D2[p][kk][0], D2[p][kk][1], D2[p][kk][2], D2[p][kk][3],
                   S.BW2[kk][j][0][lane], S.BW2[kk][j][1][lane]);
      const int col = 8 * j + 2 * t;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float d = ((m1 >> (4 * j + e)) & 1u) ? c[e] : 0.f;
        sd1[j][e & 1] += d;
        float hi, lo;
        split_bf16(d, hi, lo);
        const int cc = col + (e & 1), ss = (e >> 1) ? s1 : s0;
        S.d1T[0][cc][ss] = __float2bfloat16_rn(hi);
        S.d1T[1][cc][ss] = __float2bfloat16_rn(lo);
      }
    }
    __syncthreads();
    // ---- phase 2: warp w owns rows 16w + g, 16w + g + 8 of dW2 (j) and dW1 (k)
    const int ra = 16 * warp + g, rb = ra + 8;
#pragma unroll
    for (int ks = 0; ks < kGradWarps; ++ks) {  // samples 16 ks .. 16 ks + 15
      const int sc = 16 * ks + 2 * t;
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const uint32_t e0 = ld_pair(&S.d2T[p][ra][sc]), e1 = ld_pair(&S.d2T[p][rb][sc]);
        const uint32_t e2 = ld_pair(&S.d2T[p][ra][sc + 8]), e3 = ld_pair(&S.d2T[p][rb][sc + 8]);
#pragma unroll
        for (int nk = 0; nk < 8; ++nk)
          mma_bf16(acc2[nk], e0, e1, e2, e3, ld_pair(&S.h1T[8 * nk + g][sc]),
                   ld_pair(&S.h1T[8 * nk + g][sc + 8]));
        const uint32_t f0 = ld_pair(&S.d1T[p][ra][sc]), f1 = ld_pair(&S.d1T[p][rb][sc]);
        const uint32_t f2 = ld_pair(&S.d1T[p][ra][sc + 8]), f3 = ld_pair(&S.d1T[p][rb][sc + 8]);
#pragma unroll
        for (int ni = 0; ni < 2; ++ni)
          mma_bf16(acc1[ni], f0, f1, f2, f3, ld_pair(&S.xhT[8 * ni + g][sc]),
                   ld_pair(&S.xhT[8 * ni + g][sc + 8]));
      }
    }
    __syncthreads();
  }
  // ---- block partial gradient: dW2, dW1 from the accumulators; column sums over
  // the lanes of equal t (shuffles across g), then over the warps in order
  float *out = part + (int64_t)blockIdx.x * (NP + 1);
  const int ra = 16 * warp + g, rb = ra + 8;
#pragma unroll
  for (int nk = 0; nk < 8; ++nk)
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      out[OW2 + ra * NH + 8 * nk + 2 * t + e] = acc2[nk][e];
      out[OW2 + rb * NH + 8 * nk + 2 * t + e] = acc2[nk][2 + e];
    }
#pragma unroll
  for (int ni = 0; ni < 2; ++ni)
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int i = 8 * ni + 2 * t + e;
      if (i < NF) {
        out[OW1 + ra * NF + i] = acc1[ni][e];
        out[OW1 + rb * NF + i] = acc1[ni][2 + e];
      }
    }
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      float v1 = sd1[j][e], v2 = sd2[j][e], v3 = sw3[j][e];
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) {
        v1 += __shfl_xor_sync(0xffffffffu, v1, o);
        v2 += __shfl_xor_sync(0xffffffffu, v2, o);
        v3 += __shfl_xor_sync(0xffffffffu, v3, o);
      }
      if (g == 0) {
        const int col = 8 * j + 2 * t + e;
        S.colsum[warp][0][col] = v1;
        S.colsum[warp][1][col] = v2;
        S.colsum[warp][2][col] = v3;
      }
    }
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    sb3 += __shfl_xor_sync(0xffffffffu, sb3, o);
    loss += __shfl_xor_sync(0xffffffffu, loss, o);
  }
  if (lane == 0) {
    S.b3sum[warp] = sb3;
    S.loss[warp] = loss;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < NH; c += blockDim.x) {
    float v1 = 0.f, v2 = 0.f, v3 = 0.f;
    for (int q = 0; q < kGradWarps; ++q) {
      v1 += S.colsum[q][0][c];
      v2 += S.colsum[q][1][c];
      v3 += S.colsum[q][2][c];
    }
    out[OB1 + c] = v1;
    out[OB2 + c] = v2;
    out[OW3 + c] = v3;
  }
  if (threadIdx.x == 0) {
    float vb = 0.f;
    double vl = 0.0;
    for (int q = 0; q < kGradWarps; ++q) {
      vb += S.b3sum[q];
      vl += S.loss[q];
    }
    out[OB3] = vb;
    out[NP] = (float)vl;
  }
}

__global__ void mlp_reduce_kernel(const float *part, int nb, float *grad, double *loss) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e > NP) return;
  double v = 0.0;
  for (int b = 0; b < nb; ++b) v += part[(int64_t)b * (NP + 1) + e];
  if (e < NP) grad[e] = (float)v;
  else *loss = v;
}

// Adam (Kingma & Ba 2015) on the FP32 master weights.
__global__ void mlp_adam_kernel(float *w, float *m, float *v, const float *g, float lr, float b1,
                                float b2, float eps, float c1, float c2) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= NP) return;
  const float gi = g[e];
  const float mi = b1 * m[e] + (1.f - b1) * gi;
  const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
  m[e] = mi;
  v[e] = vi;
  w[e] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// per-feature sum and sum of squares (normalisation statistics)
__global__ void mlp_stats_kernel(const float *feat, int64_t n, double *stats) {
  __shared__ double s[2 * NF];
  if (threadIdx.x < 2 * NF) s[threadIdx.x] = 0.0;
  __syncthreads();
  double a[NF], b[NF];
  for (int i = 0; i < NF; ++i) a[i] = b[i] = 0.0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    for (int i = 0; i < NF; ++i) {
      const double x = feat[c * NF + i];
      a[i] += x;
      b[i] += x * x;
    }
  for (int i = 0; i < NF; ++i) {
    atomicAdd(&s[i], a[i]);
    atomicAdd(&s[NF + i], b[i]);
  }
  __syncthreads();
  if (threadIdx.x < 2 * NF) atomicAdd(&stats[threadIdx.x], s[threadIdx.x]);
}

}  // namespace

struct oc_mlp {
  cudaStream_t stream = nullptr;
  float *d_w = nullptr, *d_m = nullptr, *d_v = nullptr, *d_g = nullptr, *d_part = nullptr,
        *d_norm = nullptr;
  double *d_loss = nullptr, *d_stats = nullptr;
  int64_t steps = 0;
  std::string err;
};

#define MLP_TRY(call)                                                         \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      m->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
      return OC_ERR_CUDA;                                                     \
    }                                                                         \
  } while (0)

static size_t grad_smem() { return sizeof(GradSmem); }

// splitmix64 (Steele, Lea, Flood 2014) for the seeded initialisation
static uint64_t splitmix64(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

extern "C" {

oc_status oc_mlp_create(uint64_t seed, oc_mlp **out) {
  if (!out) return OC_ERR_INVALID_ARG;
  oc_mlp *m = new oc_mlp();
  *out = m;
  MLP_TRY(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  MLP_TRY(cudaMalloc((void **)&m->d_w, NP * 4));
  MLP_TRY(cudaMalloc((void **)&m->d_m, NP * 4));
  MLP_TRY(cudaMalloc((void **)&m->d_v, NP * 4));
  MLP_TRY(cudaMalloc((void **)&m->d_g, NP * 4));
  MLP_TRY(cudaMalloc((void **)&m->d_norm, 2 * NF * 4));
  MLP_TRY(cudaMalloc((void **)&m->d_part, (size_t)kGradBlocks * (NP + 1) * 4));
  MLP_TRY(cudaMalloc((void **)&m->d_loss, 8));
  MLP_TRY(cudaMalloc((void **)&m->d_stats, 2 * NF * 8));
  MLP_TRY(cudaFuncSetAttribute(mlp_grad_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)grad_smem()));
  // He-uniform weights U(-sqrt(6/fan_in), +sqrt(6/fan_in)), zero biases
  std::vector<float> w(NP, 0.f);
  uint64_t st = seed;
  auto uni = [&](float lim) {
    const double u = (splitmix64(st) >> 11) * (1.0 / 9007199254740992.0);
    return (float)((2.0 * u - 1.0) * lim);
  };
  for (int i = 0; i < NH * NF; ++i) w[OW1 + i] = uni(std::sqrt(6.f / NF));
  for (int i = 0; i < NH * NH; ++i) w[OW2 + i] = uni(std::sqrt(6.f / NH));
  for (int i = 0; i < NH; ++i) w[OW3 + i] = uni(std::sqrt(6.f / NH));
  std::vector<float> norm(2 * NF, 0.f);
  for (int i = 0; i < NF; ++i) norm[NF + i] = 1.f;
  MLP_TRY(cudaMemcpy(m->d_w, w.data(), NP * 4, cudaMemcpyHostToDevice));
  MLP_TRY(cudaMemcpy(m->d_norm, norm.data(), 2 * NF * 4, cudaMemcpyHostToDevice));
  MLP_TRY(cudaMemset(m->d_m, 0, NP * 4));
  MLP_TRY(cudaMemset(m->d_v, 0, NP * 4));
  MLP_TRY(cudaMemset(m->d_g, 0, NP * 4));
  return OC_OK;
}

void oc_mlp_destroy(oc_mlp *m) {
  if (!m) return;
  if (m->stream) cudaStreamSynchronize(m->stream);
  for (void *p : {(void *)m->d_w, (void *)m->d_m, (void *)m->d_v, (void *)m->d_g,
                  (void *)m->d_part, (void *)m->d_norm, (void *)m->d_loss, (void *)m->d_stats})
    if (p) cudaFree(p);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

const char *oc_mlp_last_error(const oc_mlp *m) { return m ? m->err.c_str() : "null handle"; }
void *oc_mlp_stream(oc_mlp *m) { return m ? (void *)m->stream : nullptr; }

oc_status oc_mlp_get_params(oc_mlp *m, float *params) {
  if (!m || !params) return OC_ERR_INVALID_ARG;
  MLP_TRY(cudaMemcpyAsync(params, m->d_w, NP * 4, cudaMemcpyDeviceToHost, m->stream));
  MLP_TRY(cudaStreamSynchronize(m->stream));
  return OC_OK;
}

oc_status oc_mlp_set_params(oc_mlp *m, const float *params) {
  if (!m || !params) return OC_ERR_INVALID_ARG;
  MLP_TRY(cudaMemcpyAsync(m->d_w, params, NP * 4, cudaMemcpyHostToDevice, m->stream));
  MLP_TRY(cudaMemsetAsync(m->d_m, 0, NP * 4, m->stream));
  MLP_TRY(cudaMemsetAsync(m->d_v, 0, NP * 4, m->stream));
  MLP_TRY(cudaStreamSynchronize(m->stream));
  m->steps = 0;
  return OC_OK;
}

oc_status oc_mlp_get_normalization(oc_mlp *m, float *mean_inv_std) {
  if (!m || !mean_inv_std) return OC_ERR_INVALID_ARG;
  MLP_TRY(cudaMemcpyAsync(mean_inv_std, m->d_norm, 2 * NF * 4, cudaMemcpyDeviceToHost, m->stream));
  MLP_TRY(cudaStreamSynchronize(m->stream));
  return OC_OK;
}

oc_status oc_mlp_set_normalization(oc_mlp *m, const float *mean_inv_std) {
  if (!m || !mean_inv_std) return OC_ERR_INVALID_ARG;
  MLP_TRY(cudaMemcpyAsync(m->d_norm, mean_inv_std, 2 * NF * 4, cudaMemcpyHostToDevice, m->stream));
  MLP_TRY(cudaStreamSynchronize(m->stream));
  return OC_OK;
}

oc_status oc_mlp_fit_normalization(oc_mlp *m, const float *features, int64_t n) {
  if (!m || !features || n <= 0) return OC_ERR_INVALID_ARG;
  MLP_TRY(cudaMemsetAsync(m->d_stats, 0, 2 * NF * 8, m->stream));
  const int grid = (int)std::min<int64_t>(1216, (n + 255) / 256);
  mlp_stats_kernel<<<grid, 256, 0, m->stream>>>(features, n, m->d_stats);
  MLP_TRY(cudaGetLastError());
  double st[2 * NF];
  MLP_TRY(cudaMemcpyAsync(st, m->d_stats, sizeof(st), cudaMemcpyDeviceToHost, m->stream));
  MLP_TRY(cudaStreamSynchronize(m->stream));
  float norm[2 * NF];
  for (int i = 0; i < NF; ++i) {
    const double mu = st[i] / n, var = std::max(st[NF + i] / n - mu * mu, 0.0);
    norm[i] = (float)mu;
    norm[NF + i] = var > 1e-20 ? (float)(1.0 / std::sqrt(var)) : 1.f;
  }
  return oc_mlp_set_normalization(m, norm);
}

oc_status oc_mlp_forward(oc_mlp *m, const float *features, int64_t n, float *logits) {
  if (!m || !features || !logits || n < 0) return OC_ERR_INVALID_ARG;
  if (n == 0) return OC_OK;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t tiles = (n + 15) / 16;
  const int grid = (int)std::min<int64_t>((int64_t)sms * 8, (tiles + kMmaWarps - 1) / kMmaWarps);
  mlp_forward_mma_kernel<<<grid, 32 * kMmaWarps, 0, m->stream>>>(m->d_w, m->d_norm, features, n,
                                                                  logits);
  MLP_TRY(cudaGetLastError());
  return OC_OK;
}

oc_status oc_mlp_gradient(oc_mlp *m, const float *features, const float *labels, int64_t n,
                          float pos_weight, float *grad, double *loss) {
  if (!m || !features || !labels || n <= 0) return OC_ERR_INVALID_ARG;
  const int64_t tiles = (n + kTile - 1) / kTile;
  const int grid = (int)std::min<int64_t>(kGradBlocks, tiles);
  mlp_grad_mma_kernel<<<grid, 32 * kGradWarps, grad_smem(), m->stream>>>(
      m->d_w, m->d_norm, features, labels, n, pos_weight, (float)(1.0 / (double)n), m->d_part);
  MLP_TRY(cudaGetLastError());
  mlp_reduce_kernel<<<(NP + 1 + 255) / 256, 256, 0, m->stream>>>(m->d_part, grid, m->d_g,
                                                                  m->d_loss);
  MLP_TRY(cudaGetLastError());
  if (grad) MLP_TRY(cudaMemcpyAsync(grad, m->d_g, NP * 4, cudaMemcpyDeviceToHost, m->stream));
  if (loss) {
    double l = 0;
    MLP_TRY(cudaMemcpyAsync(&l, m->d_loss, 8, cudaMemcpyDeviceToHost, m->stream));
    MLP_TRY(cudaStreamSynchronize(m->stream));
    *loss = l / (double)n;
  } else if (grad) {
    MLP_TRY(cudaStreamSynchronize(m->stream));
  }
  return OC_OK;
}

oc_status oc_mlp_adam_step(oc_mlp *m, float lr) {
  if (!m || !(lr > 0.f)) return OC_ERR_INVALID_ARG;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  m->steps++;
  const float c1 = 1.f - std::pow(b1, (float)m->steps), c2 = 1.f - std::pow(b2, (float)m->steps);
  mlp_adam_kernel<<<(NP + 255) / 256, 256, 0, m->stream>>>(m->d_w, m->d_m, m->d_v, m->d_g, lr,
                                                           b1, b2, eps, c1, c2);
  MLP_TRY(cudaGetLastError());
  return OC_OK;
}

oc_status oc_mlp_synchronize(oc_mlp *m) {
  if (!m) return OC_ERR_INVALID_ARG;
  MLP_TRY(cudaStreamSynchronize(m->stream));
  return OC_OK;
}

}  // extern "C"
