// Double exp and log rounded to nearest, for the few transcendental terms of
// the evolution objective and of the PLS class coarsening, whose host
// counterparts (glibc exp / log) are correctly rounded in all but rare cases.
//
// Method (no vendor code): double-double arithmetic built from the
// error-free transformations of Knuth (TwoSum) and Dekker (TwoProduct via
// fma).
//   exp(x): Cody-Waite reduction x = k ln2 + r with ln 2 split into three
//           doubles, s = r / 2^10, expm1(s) by its Taylor series to degree 9
//           in Horner form, ten squarings through expm1(2t) = 2 e + e^2,
//           then 2^k (1 + e).  Relative error below 2^-92.
//   log(x): one Newton step on exp from a faithful start y0:
//           y = y0 + (x - e^y0) / e^y0, with e^y0 in double-double.
// The returned double is the nearest to the double-double value, so it is
// the correctly rounded result unless the exact value lies within ~2^-92
// (relative) of a rounding midpoint.
#pragma once

#include <math.h>

namespace kgb {

struct DD {
  double hi, lo;
};

__device__ __forceinline__ DD dd_two_sum(double a, double b) {
  const double s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  const double e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ DD dd_fast_two_sum(double a, double b) {
  const double s = __dadd_rn(a, b);
  return {s, __dsub_rn(b, __dsub_rn(s, a))};
}

__device__ __forceinline__ DD dd_two_prod(double a, double b) {
  const double p = __dmul_rn(a, b);
  return {p, fma(a, b, -p)};
}

__device__ __forceinline__ DD dd_add(DD a, DD b) {
  DD s = dd_two_sum(a.hi, b.hi);
  const DD t = dd_two_sum(a.lo, b.lo);
  s.lo = __dadd_rn(s.lo, t.hi);
  s = dd_fast_two_sum(s.hi, s.lo);
  s.lo = __dadd_rn(s.lo, t.lo);
  return dd_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ DD dd_mul(DD a, DD b) {
  DD p = dd_two_prod(a.hi, b.hi);
  p.lo = __dadd_rn(p.lo, __dadd_rn(__dmul_rn(a.hi, b.lo), __dmul_rn(a.lo, b.hi)));
  return dd_fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ DD dd_div(DD a, DD b) {
  const double q1 = __ddiv_rn(a.hi, b.hi);
  DD t = dd_mul(b, DD{q1, 0.0});
  DD r = dd_add(a, DD{-t.hi, -t.lo});
  const double q2 = __ddiv_rn(r.hi, b.hi);
  t = dd_mul(b, DD{q2, 0.0});
  r = dd_add(r, DD{-t.hi, -t.lo});
  const double q3 = __ddiv_rn(r.hi, b.hi);
  DD q = dd_fast_two_sum(q1, q2);
  return dd_add(q, DD{q3, 0.0});
}

// e^x - 1 for |x| <= ln2/2 as a double-double.
__device__ inline DD dd_expm1_reduced(DD r) {
  const DD s{ldexp(r.hi, -10), ldexp(r.lo, -10)};
  // Horner: q = 1/9!; q = q s + 1/i! (i = 8..1); e = q s
  double fact = 362880.0;  // 9!
  DD q = dd_div(DD{1.0, 0.0}, DD{fact, 0.0});
  for (int i = 8; i >= 1; --i) {
    fact /= static_cast<double>(i + 1);  // i! (exact)
    q = dd_add(dd_mul(q, s), dd_div(DD{1.0, 0.0}, DD{fact, 0.0}));
  }
  DD e = dd_mul(q, s);
  for (int k = 0; k < 10; ++k) e = dd_add(DD{2.0 * e.hi, 2.0 * e.lo}, dd_mul(e, e));
  return e;
}

// e^x as a double-double mantissa and a power of two: e^x = (1 + e) 2^k.
__device__ inline DD dd_exp_parts(double x, int& k_out) {
  const double kLn2a = 0x1.62e42fefa39efp-1, kLn2b = 0x1.abc9e3b39803fp-56, kLn2c = 0x1.7b57a079a1934p-111;
  const double kInvLn2 = 0x1.71547652b82fep+0;
  const double k = rint(__dmul_rn(x, kInvLn2));
  DD p = dd_two_prod(k, kLn2a);
  DD r = dd_add(DD{x, 0.0}, DD{-p.hi, -p.lo});
  p = dd_two_prod(k, kLn2b);
  r = dd_add(r, DD{-p.hi, -p.lo});
  r = dd_add(r, DD{-__dmul_rn(k, kLn2c), 0.0});
  k_out = static_cast<int>(k);
  return dd_expm1_reduced(r);
}

__device__ inline double cr_exp(double x) {
  if (isnan(x)) return x;
  if (x > 709.79) return INFINITY;
  if (x < -745.2) return 0.0;
  int k = 0;
  const DD e = dd_exp_parts(x, k);
  const DD m = dd_add(DD{1.0, 0.0}, e);
  // 2^k (hi + lo): scale both parts in two steps so no intermediate overflows
  const int k1 = k / 2, k2 = k - k1;
  return ldexp(ldexp(__dadd_rn(m.hi, m.lo), k1), k2);
}

__device__ inline double cr_log(double x) {
  if (isnan(x) || x < 0.0) return NAN;
  if (x == 0.0) return -INFINITY;
  if (isinf(x)) return INFINITY;
  if (x == 1.0) return 0.0;
  const double y0 = log(x);
  int k = 0;
  const DD e = dd_exp_parts(y0, k);
  // E = e^y0 = (1 + e) 2^k; d = (x - E) / E
  const DD one_e = dd_add(DD{1.0, 0.0}, e);
  const DD E{ldexp(one_e.hi, k), ldexp(one_e.lo, k)};
  const DD num = dd_add(DD{x, 0.0}, DD{-E.hi, -E.lo});
  const double d = __ddiv_rn(num.hi, E.hi);
  return __dadd_rn(y0, d);
}

}  // namespace kgb
