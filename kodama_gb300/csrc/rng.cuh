// Device random streams that reproduce the reference's host draws exactly.
//
// The reference draws every perturb/accept decision from std::mt19937_64
// seeded per run (core.cpp:1315, common.cpp:117) through libstdc++ 13
// algorithms.  This header restates, from the published algorithms, what those
// draws compute:
//   * MT19937-64 (Matsumoto & Nishimura 2000; n=312, m=156, r=31), seeding by
//     x[i] = f*(x[i-1] ^ (x[i-1] >> 62)) + i, outputs tempered per block;
//   * integer downscaling of one 64-bit output to [0, range) by Lemire's
//     nearly-divisionless method (Lemire 2019), which is what
//     std::uniform_int_distribution does for a full-width 64-bit engine: take
//     the high word of u*range, redraw only when the low word falls below
//     (2^64 - range) mod range;
//   * a double in [0,1) from one output: double(u) * 2^-64, clamped below 1
//     (std::generate_canonical<double,53> for a 64-bit engine);
//   * discrete draws: weights normalised by their running sum, cumulative sums
//     with the last forced to 1, first cumulative >= canonical draw; fewer than
//     two weights draw nothing and return 0.
//
// One CTA owns one stream.  The state lives in shared memory; a whole warp can
// regenerate a block of 312 outputs in parallel (mt64_refill_warp), and a
// single thread can draw scalars (mt64_next_serial) with a serial refill.
#pragma once

#include <stdint.h>

namespace kgb {

constexpr int kMtN = 312;
constexpr int kMtM = 156;
constexpr uint64_t kMtA = 0xB5026F5AA96619E9ull;
constexpr uint64_t kMtUpper = 0xFFFFFFFF80000000ull;
constexpr uint64_t kMtLower = 0x000000007FFFFFFFull;

struct Mt64State {
  uint64_t mt[kMtN];
  uint64_t out[kMtN];
  int pos;  // next unread entry of out; kMtN = exhausted
  int pad;
};

__device__ __forceinline__ uint64_t mt64_temper(uint64_t y) {
  y ^= (y >> 29) & 0x5555555555555555ull;
  y ^= (y << 17) & 0x71D67FFFEDA60000ull;
  y ^= (y << 37) & 0xFFF7EEE000000000ull;
  y ^= (y >> 43);
  return y;
}

__device__ __forceinline__ uint64_t mt64_mix(uint64_t cur, uint64_t next, uint64_t far) {
  const uint64_t y = (cur & kMtUpper) | (next & kMtLower);
  return far ^ (y >> 1) ^ ((y & 1ull) ? kMtA : 0ull);
}

// Serial seeding by one thread.
__device__ inline void mt64_seed(Mt64State& s, uint64_t seed) {
  s.mt[0] = seed;
  for (int i = 1; i < kMtN; ++i) {
    const uint64_t p = s.mt[i - 1];
    s.mt[i] = 6364136223846793005ull * (p ^ (p >> 62)) + static_cast<uint64_t>(i);
  }
  s.pos = kMtN;
}

// Regenerate the state block and its tempered outputs with one full warp.
// Must be called by all 32 lanes of one warp.
__device__ inline void mt64_refill_warp(Mt64State& s, int lane) {
  uint64_t v[5];
  // k in [0, 156): reads only not-yet-updated words
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    const int k = lane + 32 * t;
    if (k < kMtN - kMtM) v[t] = mt64_mix(s.mt[k], s.mt[k + 1], s.mt[k + kMtM]);
  }
  __syncwarp();
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    const int k = lane + 32 * t;
    if (k < kMtN - kMtM) s.mt[k] = v[t];
  }
  __syncwarp();
  // k in [156, 311]: far word already updated, next word not yet
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    const int k = kMtN - kMtM + lane + 32 * t;
    if (k < kMtN - 1) {
      v[t] = mt64_mix(s.mt[k], s.mt[k + 1], s.mt[k - (kMtN - kMtM)]);
    } else if (k == kMtN - 1) {
      v[t] = mt64_mix(s.mt[kMtN - 1], s.mt[0], s.mt[kMtM - 1]);
    }
  }
  __syncwarp();
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    const int k = kMtN - kMtM + lane + 32 * t;
    if (k < kMtN) s.mt[k] = v[t];
  }
  __syncwarp();
  for (int k = lane; k < kMtN; k += 32) s.out[k] = mt64_temper(s.mt[k]);
  if (lane == 0) s.pos = 0;
  __syncwarp();
}

// Serial regeneration (one thread).
__device__ inline void mt64_refill_serial(Mt64State& s) {
  int k = 0;
  for (; k < kMtN - kMtM; ++k) s.mt[k] = mt64_mix(s.mt[k], s.mt[k + 1], s.mt[k + kMtM]);
  for (; k < kMtN - 1; ++k) s.mt[k] = mt64_mix(s.mt[k], s.mt[k + 1], s.mt[k - (kMtN - kMtM)]);
  s.mt[kMtN - 1] = mt64_mix(s.mt[kMtN - 1], s.mt[0], s.mt[kMtM - 1]);
  for (k = 0; k < kMtN; ++k) s.out[k] = mt64_temper(s.mt[k]);
  s.pos = 0;
}

__device__ __forceinline__ uint64_t mt64_next_serial(Mt64State& s) {
  if (s.pos >= kMtN) mt64_refill_serial(s);
  return s.out[s.pos++];
}

// Lemire downscaling of engine outputs to [0, range), range >= 1.
__device__ inline uint64_t draw_below_serial(Mt64State& s, uint64_t range) {
  uint64_t u = mt64_next_serial(s);
  uint64_t lo = u * range;
  if (lo < range) {
    const uint64_t threshold = (0ull - range) % range;
    while (lo < threshold) {
      u = mt64_next_serial(s);
      lo = u * range;
    }
  }
  return __umul64hi(u, range);
}

// std::uniform_int_distribution<int>(a, b)(engine), a <= b.
__device__ inline int uniform_int_serial(Mt64State& s, int a, int b) {
  const uint64_t range = static_cast<uint64_t>(static_cast<int64_t>(b) - static_cast<int64_t>(a)) + 1ull;
  return static_cast<int>(static_cast<int64_t>(a) + static_cast<int64_t>(draw_below_serial(s, range)));
}

// std::generate_canonical<double, 53>(engine) for a 64-bit engine.
__device__ inline double canonical_serial(Mt64State& s) {
  const uint64_t u = mt64_next_serial(s);
  const double r = __dmul_rn(__ull2double_rn(u), 0x1p-64);
  return r >= 1.0 ? 0x1.fffffffffffffp-1 : r;
}

// std::discrete_distribution<int>(w, w+n)(engine).  cp is scratch of n doubles.
__device__ inline int discrete_serial(Mt64State& s, const double* w, int n, double* cp) {
  if (n < 2) return 0;
  double sum = 0.0;
  for (int i = 0; i < n; ++i) sum = __dadd_rn(sum, w[i]);
  double acc = 0.0;
  for (int i = 0; i < n; ++i) {
    const double p = __ddiv_rn(w[i], sum);
    acc = i == 0 ? p : __dadd_rn(acc, p);
    cp[i] = acc;
  }
  cp[n - 1] = 1.0;
  const double u = canonical_serial(s);
  // lower_bound with the standard halving probe sequence (the cumulative array
  // can be non-monotone in its last entry after rounding, so the probe order
  // must be the standard one, not any bisection).
  int first = 0, len = n;
  while (len > 0) {
    const int half = len >> 1;
    const int mid = first + half;
    if (cp[mid] < u) {
      first = mid + 1;
      len = len - half - 1;
    } else {
      len = half;
    }
  }
  return first;
}

}  // namespace kgb
