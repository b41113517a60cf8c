// The learned relabelling proposal: a 3-layer perceptron (8 -> 64 -> 64 -> 1)
// that scores each landmark whose current label differs from its CV
// prediction, trained on snapshots of plain runs.  BF16 weights and
// activations, FP32 accumulation: scalar FMA chains in training (mlp.cu),
// tensor-pipe warp tiles in inference (mlp_logit_warp).  Used by the evolution kernel (evolve.cu)
// to pick which candidates a proposal relabels; every proposal is still
// accepted or rejected by the exact cross-validated accuracy.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace kgb {

constexpr int kMlpIn = 8;
constexpr int kMlpHidden = 64;
// parameter vector: W1 (in x hidden, row-major), b1, W2 (hidden x hidden), b2, w3 (hidden), b3
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpIn * kMlpHidden;
constexpr int kMlpW2 = kMlpB1 + kMlpHidden;
constexpr int kMlpB2 = kMlpW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpW3 = kMlpB2 + kMlpHidden;
constexpr int kMlpB3 = kMlpW3 + kMlpHidden;
constexpr int kMlpParams = kMlpB3 + 1;
constexpr int kMlpGradBlock = 32;  // rows per gradient block (static shared memory)

__device__ __forceinline__ float bf16_round(float v) {
  // round to the nearest bfloat16 (ties to even), kept in a float
  const unsigned u = __float_as_uint(v);
  if ((u & 0x7f800000u) == 0x7f800000u) return v;  // inf / nan unchanged
  const unsigned r = u + 0x7fffu + ((u >> 16) & 1u);
  return __uint_as_float(r & 0xffff0000u);
}

// ---------------------------------------------------------------------------
// Warp-tile inference on the tensor pipe (mma.sync, bf16 in, f32 accumulate).
// A warp scores 32 rows at once as two 16-row tiles: layer 1 is one
// m16n8k8 per 8 hidden units, layer 2 four m16n8k16 per 8 hidden units with
// layer 1's accumulators reused as A fragments, and the output layer a dot
// product per quad of lanes.  The network is packed once into fragment
// order ("frag", kMlpFragWords 32-bit words, see mlp_pack_params) so every
// B fragment is one coalesced load through L1.
// ---------------------------------------------------------------------------
constexpr int kMlpFragW1 = 0;                          // 8 n-tiles x 32 lanes x 1 word
constexpr int kMlpFragW2 = kMlpFragW1 + 8 * 32;        // (4 k-slices x 8 n-tiles) x 32 lanes x 2 words
constexpr int kMlpFragB1 = kMlpFragW2 + 32 * 32 * 2;   // 64 floats
constexpr int kMlpFragB2 = kMlpFragB1 + kMlpHidden;    // 64 floats
constexpr int kMlpFragW3 = kMlpFragB2 + kMlpHidden;    // 64 floats (bf16 values)
constexpr int kMlpFragB3 = kMlpFragW3 + kMlpHidden;    // 1 float
constexpr int kMlpFragWords = (kMlpFragB3 + 1 + 3) / 4 * 4;

// two floats as a bfloat16 pair (lo in the low half), each rounded like bf16_round
__device__ __forceinline__ uint32_t bf16_pack(float lo, float hi) {
  return (__float_as_uint(bf16_round(lo)) >> 16) | (__float_as_uint(bf16_round(hi)) & 0xffff0000u);
}

// the 8 features of a row as 4 bfloat16 pairs
__device__ __forceinline__ void mlp_pack_row(const float* x, uint32_t* w) {
#pragma unroll
  for (int k = 0; k < 4; ++k) w[k] = bf16_pack(x[2 * k], x[2 * k + 1]);
}

__device__ __forceinline__ void mma_bf16_k8(float* d, uint32_t a0, uint32_t a1, uint32_t b0) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(b0));
}

__device__ __forceinline__ void mma_bf16_k16(float* d, const uint32_t* a, uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// Logit of the row whose packed features (mlp_pack_row) lane l holds, for all
// 32 lanes of the warp (call with the whole warp converged).  Lanes without a
// row pass zeros and ignore the result; `rows` (warp-uniform) is how many of
// lanes 0..31 hold rows, so an empty second tile is skipped.
__device__ __forceinline__ float mlp_logit_warp(const uint32_t* __restrict__ frag, const uint32_t* fw, int rows) {
  const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
  const float* fb = reinterpret_cast<const float*>(frag);
  float mine = 0.0f;
#pragma unroll 1
  for (int t = 0; t < 2; ++t) {
    if (16 * t >= rows) break;
    // A fragment of the input tile: rows g, g + 8; features 2 tig, 2 tig + 1
    uint32_t a0, a1;
    {
      const int src0 = 16 * t + g, src1 = src0 + 8;
      const uint32_t p0 = __shfl_sync(0xffffffffu, fw[0], src0), p1 = __shfl_sync(0xffffffffu, fw[1], src0);
      const uint32_t p2 = __shfl_sync(0xffffffffu, fw[2], src0), p3 = __shfl_sync(0xffffffffu, fw[3], src0);
      const uint32_t q0 = __shfl_sync(0xffffffffu, fw[0], src1), q1 = __shfl_sync(0xffffffffu, fw[1], src1);
      const uint32_t q2 = __shfl_sync(0xffffffffu, fw[2], src1), q3 = __shfl_sync(0xffffffffu, fw[3], src1);
      a0 = tig == 0 ? p0 : tig == 1 ? p1 : tig == 2 ? p2 : p3;
      a1 = tig == 0 ? q0 : tig == 1 ? q1 : tig == 2 ? q2 : q3;
    }
    // layer 1 -> A fragments of layer 2 (k-slice s = hidden units 16 s .. 16 s + 15)
    uint32_t h[4][4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      float d0[4], d1[4];
      const float bl0 = __ldg(fb + kMlpFragB1 + 16 * s + 2 * tig), bh0 = __ldg(fb + kMlpFragB1 + 16 * s + 2 * tig + 1);
      const float bl1 = __ldg(fb + kMlpFragB1 + 16 * s + 8 + 2 * tig),
                  bh1 = __ldg(fb + kMlpFragB1 + 16 * s + 8 + 2 * tig + 1);
      d0[0] = bl0; d0[1] = bh0; d0[2] = bl0; d0[3] = bh0;
      d1[0] = bl1; d1[1] = bh1; d1[2] = bl1; d1[3] = bh1;
      mma_bf16_k8(d0, a0, a1, __ldg(frag + kMlpFragW1 + (2 * s) * 32 + lane));
      mma_bf16_k8(d1, a0, a1, __ldg(frag + kMlpFragW1 + (2 * s + 1) * 32 + lane));
      h[s][0] = bf16_pack(fmaxf(d0[0], 0.0f), fmaxf(d0[1], 0.0f));
      h[s][1] = bf16_pack(fmaxf(d0[2], 0.0f), fmaxf(d0[3], 0.0f));
      h[s][2] = bf16_pack(fmaxf(d1[0], 0.0f), fmaxf(d1[1], 0.0f));
      h[s][3] = bf16_pack(fmaxf(d1[2], 0.0f), fmaxf(d1[3], 0.0f));
    }
    // layer 2 per 8 hidden units, folded straight into the output dot product
    float zlo = 0.0f, zhi = 0.0f;  // rows g and g + 8
    const uint2* w2 = reinterpret_cast<const uint2*>(frag + kMlpFragW2);
#pragma unroll 1
    for (int j = 0; j < 8; ++j) {
      const float bl = __ldg(fb + kMlpFragB2 + 8 * j + 2 * tig), bh = __ldg(fb + kMlpFragB2 + 8 * j + 2 * tig + 1);
      float c[4] = {bl, bh, bl, bh};
#pragma unroll
      for (int s = 0; s < 4; ++s) mma_bf16_k16(c, h[s], __ldg(w2 + (s * 8 + j) * 32 + lane));
      const float wl = __ldg(fb + kMlpFragW3 + 8 * j + 2 * tig), wh = __ldg(fb + kMlpFragW3 + 8 * j + 2 * tig + 1);
      zlo = fmaf(bf16_round(fmaxf(c[0], 0.0f)), wl, zlo);
      zlo = fmaf(bf16_round(fmaxf(c[1], 0.0f)), wh, zlo);
      zhi = fmaf(bf16_round(fmaxf(c[2], 0.0f)), wl, zhi);
      zhi = fmaf(bf16_round(fmaxf(c[3], 0.0f)), wh, zhi);
    }
    zlo += __shfl_xor_sync(0xffffffffu, zlo, 1);
    zlo += __shfl_xor_sync(0xffffffffu, zlo, 2);
    zhi += __shfl_xor_sync(0xffffffffu, zhi, 1);
    zhi += __shfl_xor_sync(0xffffffffu, zhi, 2);
    // lane 16 t + r takes row r of this tile from quad r mod 8
    const int r = lane & 15;
    const float vlo = __shfl_sync(0xffffffffu, zlo, 4 * (r & 7));
    const float vhi = __shfl_sync(0xffffffffu, zhi, 4 * (r & 7));
    if ((lane >> 4) == t) mine = (r < 8 ? vlo : vhi) + __ldg(fb + kMlpFragB3);
  }
  return mine;
}

// Rounds a float parameter vector to bfloat16 weights (biases stay float).
int mlp_round_params(const float* master, float* rounded, cudaStream_t st);

// Packs rounded parameters (mlp_round_params) into fragment order for
// mlp_logit_warp: kMlpFragWords words.
int mlp_pack_params(const float* rounded, uint32_t* frag, cudaStream_t st);

// Mean binary cross-entropy gradient of a batch of n rows (rows idx[0..n)
// of feat / target) at `rounded` parameters: grad (kMlpParams floats) and
// the mean loss.  Deterministic: per-block partial sums reduced in order.
// partial holds ceil(n / kMlpGradBlock) x (kMlpParams + 1) floats.
int mlp_gradient(const float* rounded, const float* feat, const uint8_t* target, const int* idx, int n,
                 float* partial, float* grad, float* loss, cudaStream_t st);

// One Adam step on the master parameters (t = step number from 1).
int mlp_adam(float* master, float* m, float* v, const float* grad, float lr, int t, cudaStream_t st);

// Logits of n rows with the warp-tile path (packed parameters).
int mlp_predict(const uint32_t* frag, const float* feat, int n, float* out, cudaStream_t st);

}  // namespace kgb
