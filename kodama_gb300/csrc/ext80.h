// Software model of x86 80-bit extended precision (64-bit significand,
// round-to-nearest-even) for the few non-negative operations the reference
// performs in `long double`: the landmark quota allocation
// (kodama_matrix.cpp:856-944 quota_sample_landmarks) and the squared row
// norms of the cosine search matrix (core.cpp:182-188).
//
// The reference is built with g++ on x86-64, where `long double` is the x87
// 80-bit format; on aarch64 it is IEEE binary128, which would round the
// residual-quota comparisons differently.  This header reproduces the x86
// results on any host (and on the device: every function is host+device).
//
// Values are non-negative: v = m * 2^e with m normalised (bit 63 set) or m == 0.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define EXT80_HD __host__ __device__ __forceinline__
#else
#define EXT80_HD inline
#endif

struct Ext80 {
  uint64_t m;
  int e;
};

EXT80_HD int ext80_clz128(unsigned __int128 v) {
  const uint64_t hi = static_cast<uint64_t>(v >> 64);
  const uint64_t lo = static_cast<uint64_t>(v);
#if defined(__CUDA_ARCH__)
  if (hi) return __clzll(static_cast<long long>(hi));
  if (lo) return 64 + __clzll(static_cast<long long>(lo));
#else
  if (hi) return __builtin_clzll(hi);
  if (lo) return 64 + __builtin_clzll(lo);
#endif
  return 128;
}

// Round a 128-bit magnitude v * 2^e (plus a sticky flag for bits already
// shifted out below v) to a 64-bit significand, nearest-even.
EXT80_HD Ext80 ext80_round(unsigned __int128 v, int e, bool sticky) {
  if (v == 0) return Ext80{0, 0};
  const int lz = ext80_clz128(v);
  // place the leading one at bit 127
  v <<= lz;
  e -= lz;
  uint64_t hi = static_cast<uint64_t>(v >> 64);
  const uint64_t lo = static_cast<uint64_t>(v);
  const bool guard = (lo >> 63) & 1u;
  const bool rest = (lo & ~(1ull << 63)) != 0 || sticky;
  e += 64;
  if (guard && (rest || (hi & 1u))) {
    ++hi;
    if (hi == 0) {  // carried out of 64 bits
      hi = 1ull << 63;
      ++e;
    }
  }
  return Ext80{hi, e};
}

EXT80_HD Ext80 ext80_from_u64(uint64_t v) { return ext80_round(static_cast<unsigned __int128>(v), 0, false); }

// u * 2^-64, the value std::generate_canonical<long double, 64> yields for one
// 64-bit engine output (exact on x86).
EXT80_HD Ext80 ext80_canonical(uint64_t u) { return ext80_round(static_cast<unsigned __int128>(u), -64, false); }

EXT80_HD Ext80 ext80_div(Ext80 a, Ext80 b) {
  if (a.m == 0) return Ext80{0, 0};
  const unsigned __int128 num = static_cast<unsigned __int128>(a.m) << 64;
  const unsigned __int128 q = num / b.m;
  const unsigned __int128 r = num % b.m;
  // q has 64 or 65 significant bits; give the rounding two extra bits by
  // computing one more quotient bit from the remainder.
  const unsigned __int128 r2 = r << 1;
  const unsigned __int128 q_ext = (q << 1) | (r2 >= b.m ? 1u : 0u);
  const unsigned __int128 r_ext = r2 >= b.m ? r2 - b.m : r2;
  return ext80_round(q_ext, a.e - b.e - 64 - 1, r_ext != 0);
}

EXT80_HD Ext80 ext80_add(Ext80 a, Ext80 b) {
  if (a.m == 0) return b;
  if (b.m == 0) return a;
  if (a.e < b.e) { const Ext80 t = a; a = b; b = t; }
  // work with 62 spare low bits so the alignment shift keeps guard and sticky
  const int shift = a.e - b.e;
  unsigned __int128 va = static_cast<unsigned __int128>(a.m) << 62;
  unsigned __int128 vb = static_cast<unsigned __int128>(b.m) << 62;
  bool sticky = false;
  if (shift >= 126) {
    sticky = vb != 0;
    vb = 0;
  } else if (shift > 0) {
    const unsigned __int128 mask = (static_cast<unsigned __int128>(1) << shift) - 1;
    sticky = (vb & mask) != 0;
    vb >>= shift;
  }
  return ext80_round(va + vb, a.e - 62, sticky);
}

// a - b for a >= b >= 0.
EXT80_HD Ext80 ext80_sub(Ext80 a, Ext80 b) {
  if (b.m == 0) return a;
  const int shift = a.e - b.e;
  unsigned __int128 va = static_cast<unsigned __int128>(a.m) << 62;
  unsigned __int128 vb = static_cast<unsigned __int128>(b.m) << 62;
  bool sticky = false;
  if (shift >= 126) {
    sticky = vb != 0;
    vb = 0;
  } else if (shift > 0) {
    const unsigned __int128 mask = (static_cast<unsigned __int128>(1) << shift) - 1;
    sticky = (vb & mask) != 0;
    vb >>= shift;
  }
  if (sticky) {
    // a true borrow below the kept bits: subtract one more unit and keep the
    // remainder sticky (the exact difference lies strictly inside it).
    return ext80_round(va - vb - 1, a.e - 62, true);
  }
  return ext80_round(va - vb, a.e - 62, false);
}

EXT80_HD bool ext80_lt(Ext80 a, Ext80 b) {
  if (a.m == 0) return b.m != 0;
  if (b.m == 0) return false;
  if (a.e != b.e) return a.e < b.e;
  return a.m < b.m;
}

// floor(v) as an integer for 0 <= v < 2^31.
EXT80_HD int ext80_floor_int(Ext80 v) {
  if (v.m == 0) return 0;
  if (v.e >= 0) return static_cast<int>(v.m << v.e);
  if (v.e <= -64) return 0;
  return static_cast<int>(v.m >> (-v.e));
}

// The square of a finite float, exactly (at most 48 significant bits).
EXT80_HD Ext80 ext80_float_square(float v) {
#if defined(__CUDA_ARCH__)
  const uint32_t u = __float_as_uint(v) & 0x7fffffffu;
#else
  uint32_t u;
  __builtin_memcpy(&u, &v, sizeof(u));
  u &= 0x7fffffffu;
#endif
  const int be = static_cast<int>(u >> 23);
  uint64_t m = u & 0x7fffffu;
  int e = -149;
  if (be != 0) {
    m |= 0x800000u;
    e = be - 150;
  }
  return ext80_round(static_cast<unsigned __int128>(m * m), 2 * e, false);
}

// static_cast<double>(long double): nearest-even rounding of the 64-bit
// significand to 53 bits (values within the normal double range).
EXT80_HD double ext80_to_double(Ext80 a) {
  if (a.m == 0) return 0.0;
  uint64_t q = a.m >> 11;
  const uint64_t rem = a.m & 0x7ffu;
  int e = a.e + 11;
  if (rem > 0x400u || (rem == 0x400u && (q & 1u))) {
    ++q;
    if (q == (1ull << 53)) {
      q >>= 1;
      ++e;
    }
  }
  const uint64_t bits = (static_cast<uint64_t>(e + 52 + 1023) << 52) | (q & ((1ull << 52) - 1));
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(bits));
#else
  double out;
  __builtin_memcpy(&out, &bits, sizeof(out));
  return out;
#endif
}
