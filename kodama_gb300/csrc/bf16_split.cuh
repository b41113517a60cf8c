// bfloat16 hi + lo split of float rows for the mma.sync m16n8k16 fragments
// (knn_tc.cu, kmeans.cu): x = hi + lo + r with |r| <= 2^-16 |x|.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace kgb {

// Round to the nearest bfloat16 (ties to even); inf / nan kept.
__device__ __forceinline__ uint32_t bf16_bits(float v) {
  const uint32_t u = __float_as_uint(v);
  if ((u & 0x7f800000u) == 0x7f800000u) return u >> 16;
  return (u + 0x7fffu + ((u >> 16) & 1u)) >> 16;
}

// Position of coordinate k inside its 16-block: the four values a lane feeds
// to one m16n8k16 fragment (k = 2t, 2t+1, 2t+8, 2t+9) are contiguous at 4t.
__device__ __forceinline__ int perm16(int k) {
  const int kk = k & 15;
  return (k & ~15) | (4 * ((kk & 7) >> 1) + ((kk & 1) | ((kk >> 3) << 1)));
}

// Words per centroid / candidate row of a staged B operand: dp / 2 rounded so
// that rw = 8 (mod 16), which spreads the 8 rows x 4 lanes of a fragment load
// over distinct banks.
__host__ __device__ __forceinline__ int tc_row_words(int dp) {
  const int half = dp / 2;
  return (half % 16 == 8) ? half : half + 8;
}

}  // namespace kgb
