// PLS-LDA on the device: the float32 SIMPLS + LDA path of the reference
// (plscv.cpp) restated operation for operation, so that predictions are
// bit-identical to PLSLDACV_CPU / PLSLDAPredict_CPU.
//
//   fold statistics   train_center_scale_float        plscv.cpp:669-698
//   standardisation   subset_scale_float              plscv.cpp:409-424
//   fold Gram         densef_gram                     plscv.cpp:436-447
//   cross-product     centered_label_crossprod_*      plscv.cpp:700-731
//   SIMPLS weights    fit_pls_components_from_crossprod_float  plscv.cpp:816-955
//   LDA               fit_predict_pls_lda_streamed_cpu_float   plscv.cpp:1544-1608
//                     fit_lda_from_score_statistics_float      plscv.cpp:1419-1487
//                     cholesky_solve_float                     plscv.cpp:1379-1412
//
// Every float accumulation of the reference is a sequential chain in a fixed
// order (rows ascending, features ascending, classes ascending); each chain
// runs in one thread (or one warp feeding one accumulator) in that order, and
// the parallelism is across chains: slices x features x classes x rows.
// Double accumulators of the reference (dot_float, mat_vec_float,
// t_mat_vec_float, power_norm2_float) sum exact float products; they are
// reproduced by an exact integer sum with a rounding-safety check, and by
// the sequential double sum only when that check cannot decide
// (warp_exact_dot below).  Built with --fmad=false: no multiply-add is fused
// unless written as one.
#include "pls.cuh"
#include "launch_count.cuh"

#include <float.h>
#include <math.h>

namespace kgb {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kEvalThreads = 512;
constexpr int kEvalWarps = kEvalThreads / 32;

// ---------------------------------------------------------------------------
// Preparation (label independent)
// ---------------------------------------------------------------------------

// train_center_scale_float: one thread per (slice, column).
__global__ void stats_kernel(PlsPrepArgs a) {
  const int s = blockIdx.x, r = s / a.F;
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  if (j >= a.p) return;
  const float* X = a.X + static_cast<size_t>(r) * a.L * a.p;
  const int b = a.train_off[s], e = a.train_off[s + 1], nt = e - b;
  const int* rows = a.train_idx;
  float m = 0.0f;
  if (a.center) {
    for (int t = b; t < e; t += 8) {
      float v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = t + q < e ? X[static_cast<size_t>(rows[t + q]) * a.p + j] : 0.0f;
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (t + q < e) m = __fadd_rn(m, v[q]);
    }
    const float inv = nt == 0 ? 0.0f : __fdiv_rn(1.0f, static_cast<float>(nt));
    m = __fmul_rn(m, inv);
  }
  float sd = 1.0f;
  if (a.scale) {
    float acc = 1.0f;  // the reference's scale vector starts at 1
    for (int t = b; t < e; t += 8) {
      float v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = t + q < e ? X[static_cast<size_t>(rows[t + q]) * a.p + j] : 0.0f;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        if (t + q < e) {
          const float d = __fsub_rn(v[q], m);
          acc = __fadd_rn(acc, __fmul_rn(d, d));
        }
      }
    }
    // std::max(1.0f, float(rows.size() - 1)) with size_t arithmetic
    const float den1 = static_cast<float>(static_cast<unsigned long long>(nt) - 1ull);
    const float den = 1.0f < den1 ? den1 : 1.0f;
    const float q = __fsqrt_rn(__fdiv_rn(acc, den));
    sd = (q > 0.0f && isfinite(q)) ? q : 1.0f;
  }
  a.mean[static_cast<size_t>(s) * a.p + j] = m;
  a.sdev[static_cast<size_t>(s) * a.p + j] = sd;
}

// subset_scale_float for every row of every slice (and, in predict mode, for
// the rows to predict).
__global__ void standardize_kernel(PlsPrepArgs a) {
  // blockIdx.y strides over slices (problems in predict mode), blockIdx.x over
  // rows, threads over columns: no index division per element
  const int S = a.problems * a.F, p = a.p;
  for (int s = blockIdx.y; s < S; s += gridDim.y) {
    const float* X = a.X + static_cast<size_t>(s / a.F) * a.L * p;
    float* Z = a.Z + static_cast<size_t>(s) * a.L * p;
    const float* mu = a.mean + static_cast<size_t>(s) * p;
    const float* sd = a.sdev + static_cast<size_t>(s) * p;
    for (int i = blockIdx.x; i < a.L; i += gridDim.x)
      for (int j = threadIdx.x; j < p; j += blockDim.x)
        Z[static_cast<size_t>(i) * p + j] = __fdiv_rn(__fsub_rn(X[static_cast<size_t>(i) * p + j], mu[j]), sd[j]);
  }
  if (a.Xv == nullptr) return;
  for (int r = blockIdx.y; r < a.problems; r += gridDim.y) {
    const size_t s = static_cast<size_t>(r) * a.F;
    const float* Xv = a.Xv + static_cast<size_t>(r) * a.NV * p;
    float* Zv = a.Zv + static_cast<size_t>(r) * a.NV * p;
    for (int i = blockIdx.x; i < a.NV; i += gridDim.x)
      for (int j = threadIdx.x; j < p; j += blockDim.x)
        Zv[static_cast<size_t>(i) * p + j] =
            __fdiv_rn(__fsub_rn(Xv[static_cast<size_t>(i) * p + j], a.mean[s * p + j]), a.sdev[s * p + j]);
  }
}

__device__ __forceinline__ int biased_exp1(float v) {
  return max(static_cast<int>((__float_as_uint(v) >> 23) & 0xffu), 1);
}

// Column sums of the standardised training rows in row order (the x_sum of
// the cross-product, label independent), and each column's largest biased
// exponent over those rows (the fixed-point bound of block_loading).
__global__ void xsum_kernel(PlsPrepArgs a) {
  const int s = blockIdx.x;
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  if (j >= a.p) return;
  const float* Zs = a.Z + static_cast<size_t>(s) * a.L * a.p;
  const int b = a.train_off[s], e = a.train_off[s + 1];
  float acc = 0.0f;
  int ze = 1;
  for (int t = b; t < e; t += 8) {
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = t + q < e ? Zs[static_cast<size_t>(a.train_idx[t + q]) * a.p + j] : 0.0f;
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (t + q < e) {
        acc = __fadd_rn(acc, v[q]);
        ze = max(ze, biased_exp1(v[q]));
      }
  }
  a.xsum[static_cast<size_t>(s) * a.p + j] = acc;
  a.zexp[static_cast<size_t>(s) * a.p + j] = ze;
}

// densef_gram: G(j, k) = sum over training rows (ascending) of z_j * z_k, one
// kGramT x kGramT tile of the lower triangle per CTA (blockIdx.y enumerates
// tiles), written to both triangles.  Each thread keeps a 4 x 4 block of
// entries, every one a float chain over the rows in ascending order; rows are
// staged kGramR at a time (padding rows and columns are never added).
constexpr int kGramT = 64;
constexpr int kGramR = 32;
__global__ void __launch_bounds__(256) gram_kernel(PlsPrepArgs a, const uint8_t* want) {
  const int s = blockIdx.x;
  if (!want[s]) return;
  int tile = blockIdx.y, jb = 0;
  while (tile > jb) {
    tile -= jb + 1;
    ++jb;
  }
  const int kb = tile;
  __shared__ __align__(16) float zj[kGramR][kGramT];
  __shared__ __align__(16) float zk[kGramR][kGramT];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const float* Zs = a.Z + static_cast<size_t>(s) * a.L * a.p;
  const int b = a.train_off[s], e = a.train_off[s + 1];
  float acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.0f;
  for (int t0 = b; t0 < e; t0 += kGramR) {
    for (int i = threadIdx.x; i < kGramR * kGramT; i += 256) {
      const int q = i / kGramT, c = i - q * kGramT;
      const int row = t0 + q < e ? a.train_idx[t0 + q] : -1;
      const int cj = jb * kGramT + c, ck = kb * kGramT + c;
      zj[q][c] = (row >= 0 && cj < a.p) ? Zs[static_cast<size_t>(row) * a.p + cj] : 0.0f;
      zk[q][c] = (row >= 0 && ck < a.p) ? Zs[static_cast<size_t>(row) * a.p + ck] : 0.0f;
    }
    __syncthreads();
    // rows of the tile past the last column hold no entry (warp-uniform: a
    // warp is two values of ty)
    const int cnt = jb * kGramT + ty * 4 < a.p ? min(kGramR, e - t0) : 0;
    for (int q = 0; q < cnt; ++q) {
      const float4 vj = *reinterpret_cast<const float4*>(&zj[q][ty * 4]);
      const float4 vk = *reinterpret_cast<const float4*>(&zk[q][tx * 4]);
      const float fj[4] = {vj.x, vj.y, vj.z, vj.w}, fk[4] = {vk.x, vk.y, vk.z, vk.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = __fadd_rn(acc[u][v], __fmul_rn(fj[u], fk[v]));
    }
    __syncthreads();
  }
  float* G = a.gram + static_cast<size_t>(s) * a.p * a.p;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int J = jb * kGramT + ty * 4 + u;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int K = kb * kGramT + tx * 4 + v;
      if (J < a.p && K < a.p && K <= J) {
        G[static_cast<size_t>(J) * a.p + K] = acc[u][v];
        G[static_cast<size_t>(K) * a.p + J] = acc[u][v];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Evaluation: one CTA per slice
// ---------------------------------------------------------------------------

constexpr int kMaxNC = 8;      // components per register pass over the rows
constexpr int kMaxComp = 64;   // components of a fit held per row (local array)
constexpr int kTile = 32 * 33; // per-warp transposing tile (floats)

struct EvalShared {
  int m, nt, stop, best, lab, fail;
  float rn, inv;
};

// ---------------------------------------------------------------------------
// float(sum_k double(a_k) * double(b_k)) summed sequentially in double, as the
// reference's dot_float / mat_vec_float / t_mat_vec_float / power_norm2_float
// do, without double arithmetic on the common path.
//
// Each product of two floats is exact in double, so the sequential sum S_seq
// differs from the exact sum S by at most n * 2^-53 * sum|t_k| (recursive
// summation of exact terms; 2^-52 is used below).  A warp forms S exactly as
// a 64-bit fixed-point integer from the 24-bit mantissas (terms below the
// fixed point truncated: at most n units of error), rounds it to float and
// checks that the rounding interval of that float contains S widened by both
// error bounds; then float(S_seq) is that float.  When the check cannot
// decide (S close to a rounding boundary, massive cancellation, non-finite
// or extreme values), lane 0 runs the sequential double sum.  The point:
// this GPU issues a dependent double FMA only every 64-152 cycles.
// ---------------------------------------------------------------------------

__device__ __forceinline__ int clog2i(int n) { return n <= 1 ? 0 : 32 - __clz(n - 1); }

__device__ __forceinline__ float warp_sum_ru(float v) {
  for (int o = 16; o > 0; o >>= 1) v = __fadd_ru(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

__device__ __forceinline__ long long warp_sum_i64(long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// The float nearest to V * 2^LSB, if S_seq provably rounds to it (see above).
__device__ __forceinline__ bool round_check(long long V, int LSB, float A, int n, float& out) {
  if (V == 0) {
    if (A == 0.0f) {
      out = 0.0f;
      return true;
    }
    return false;
  }
  const bool neg = V < 0;
  const unsigned long long mag = neg ? 0ull - static_cast<unsigned long long>(V) : static_cast<unsigned long long>(V);
  const int e = 63 - __clzll(static_cast<long long>(mag));
  const int shift = e - 23;
  if (shift <= 0) return false;
  const float bu = __fadd_ru(__fmul_ru(ldexpf(A, -52 - LSB), static_cast<float>(n)), static_cast<float>(n + 1));
  if (!(bu < 1e30f)) return false;
  const unsigned long long one = 1ull;
  unsigned long long m = mag >> shift;
  const unsigned long long rem = mag & ((one << shift) - 1ull), half = one << (shift - 1);
  const bool up = rem > half || (rem == half && (m & 1ull));
  unsigned long long dlo, dhi;
  if (!up) {
    if (rem == half) return false;
    dhi = half - rem;
    dlo = rem + (m == 0x800000ull ? (half >> 1) : half);
  } else {
    dlo = rem - half;
    dhi = ((one << shift) - rem) + half;
  }
  const float dmin = __ull2float_rz(dlo < dhi ? dlo : dhi);
  if (!(dmin > bu)) return false;
  if (up) ++m;
  int ex = shift + LSB;
  if (m == 0x1000000ull) {
    m >>= 1;
    ++ex;
  }
  if (ex + 23 > 126 || ex + 23 < -126) return false;
  const float fv = ldexpf(static_cast<float>(m), ex);
  out = neg ? -fv : fv;
  return true;
}

// First pass of an exact dot, one term: the largest product exponent (top),
// non-finite operands (bad) and an upward-rounded bound A of sum |x y|.
__device__ __forceinline__ void exact_scan_term(float x, float y, int& top, int& bad, float& A) {
  const unsigned ux = __float_as_uint(x), uy = __float_as_uint(y);
  const int ex = static_cast<int>((ux >> 23) & 0xffu), ey = static_cast<int>((uy >> 23) & 0xffu);
  bad |= (ex == 0xff) | (ey == 0xff);
  if ((ux << 1) != 0u && (uy << 1) != 0u) top = max(top, max(ex, 1) + max(ey, 1) - 252);
  A = __fadd_ru(A, __fmul_ru(fabsf(x), fabsf(y)));
}

// Second pass, one term: x y as a multiple of 2^LSB (truncated below it).
__device__ __forceinline__ long long exact_fixed_term(float x, float y, int LSB) {
  const unsigned ux = __float_as_uint(x), uy = __float_as_uint(y);
  const unsigned bx = (ux >> 23) & 0xffu, by = (uy >> 23) & 0xffu;
  const unsigned mx = (ux & 0x7fffffu) | (bx ? 0x800000u : 0u), my = (uy & 0x7fffffu) | (by ? 0x800000u : 0u);
  const unsigned long long P = static_cast<unsigned long long>(mx) * my;
  if (P == 0ull) return 0;
  const int E = (bx ? static_cast<int>(bx) - 150 : -149) + (by ? static_cast<int>(by) - 150 : -149);
  const int sh = E - LSB;
  unsigned long long v;
  if (sh >= 0) v = P << sh;
  else v = -sh >= 64 ? 0ull : P >> (-sh);
  return ((ux ^ uy) >> 31) ? -static_cast<long long>(v) : static_cast<long long>(v);
}

// Exact fixed-point sum over the warp; returns whether `out` is float(S_seq).
template <class Term>
__device__ bool warp_exact_dot(int n, Term term, int lane, float& out) {
  int top = -100000, bad = 0;
  float A = 0.0f;
  for (int k = lane; k < n; k += 32) {
    float x, y;
    term(k, x, y);
    exact_scan_term(x, y, top, bad, A);
  }
  bad = __reduce_or_sync(kFull, bad);
  top = __reduce_max_sync(kFull, top);
  if (bad) return false;
  A = warp_sum_ru(A);
  if (top == -100000) {  // every term is zero
    out = 0.0f;
    return true;
  }
  const int LSB = top + clog2i(n) - 62;
  long long acc = 0;
  for (int k = lane; k < n; k += 32) {
    float x, y;
    term(k, x, y);
    acc += exact_fixed_term(x, y, LSB);
  }
  acc = warp_sum_i64(acc);
  return round_check(acc, LSB, A, n, out);
}

// The reference's sequential double chains, acc = fma(x_k, y_k, acc) for k
// ascending, by a whole warp.  A product of two floats is exact in double,
// so fma(x, y, acc) is acc + x*y rounded once: the lanes form 32 products at a
// time, every lane adds them in order (the same chain in every lane) and the
// next 32 terms load meanwhile.  n can be a column over the training rows,
// where one lane's loop would wait on every load.
template <class Term>
__device__ double warp_fma_chain(int n, Term term, int lane) {
  double s = 0.0;
  float x = 0.0f, y = 0.0f;
  if (lane < n) term(lane, x, y);
  for (int k0 = 0; k0 < n; k0 += 32) {
    const double prod = __dmul_rn(static_cast<double>(x), static_cast<double>(y));
    x = 0.0f;
    y = 0.0f;
    if (k0 + 32 + lane < n) term(k0 + 32 + lane, x, y);
    const int cnt = min(32, n - k0);
    for (int q = 0; q < cnt; ++q) s = __dadd_rn(s, __shfl_sync(kFull, prod, q));
  }
  return s;
}

// acc = 0.0; acc += double(x_k) for k ascending, the same way.
template <class Term>
__device__ double warp_add_chain(int n, Term term, int lane) {
  double s = 0.0;
  float x = lane < n ? term(lane) : 0.0f;
  for (int k0 = 0; k0 < n; k0 += 32) {
    const double v = static_cast<double>(x);
    x = k0 + 32 + lane < n ? term(k0 + 32 + lane) : 0.0f;
    const int cnt = min(32, n - k0);
    for (int q = 0; q < cnt; ++q) s = __dadd_rn(s, __shfl_sync(kFull, v, q));
  }
  return s;
}

// Sequential double sum of n floats, S_seq (acc = 0.0; acc += double(x_k)
// in order).  All terms are multiples of 2^emin (the smallest ulp); when the
// sum of |x| stays below 2^(emin + 53), every partial sum is exact in double,
// so S_seq is the exact fixed-point sum.  Otherwise lane 0 runs the chain.
template <class Term>
__device__ double warp_seq_sum_double(int n, Term term, int lane) {
  int emin = 1 << 20, emax = -(1 << 20), bad = 0;
  float A = 0.0f;
  for (int k = lane; k < n; k += 32) {
    const float x = term(k);
    const unsigned ux = __float_as_uint(x);
    const int be = static_cast<int>((ux >> 23) & 0xffu);
    bad |= be == 0xff;
    if ((ux << 1) != 0u) {
      const int ue = be ? be - 150 : -149;
      emin = min(emin, ue);
      emax = max(emax, ue);
      A = __fadd_ru(A, fabsf(x));
    }
  }
  bad = __reduce_or_sync(kFull, bad);
  emin = __reduce_min_sync(kFull, emin);
  emax = __reduce_max_sync(kFull, emax);
  A = warp_sum_ru(A);
  bool exact = !bad;
  if (exact && emin == (1 << 20)) return 0.0;  // every term is zero
  if (exact) exact = emax - emin + 24 + clog2i(n) <= 62 && A < ldexpf(1.0f, min(emin + 53, 127));
  if (exact) {
    long long acc = 0;
    for (int k = lane; k < n; k += 32) {
      const float x = term(k);
      const unsigned ux = __float_as_uint(x);
      if ((ux << 1) == 0u) continue;
      const int be = static_cast<int>((ux >> 23) & 0xffu);
      const long long mant = static_cast<long long>((ux & 0x7fffffu) | (be ? 0x800000u : 0u));
      const long long v = mant << ((be ? be - 150 : -149) - emin);
      acc += (ux >> 31) ? -v : v;
    }
    acc = warp_sum_i64(acc);
    // |acc| < 2^53: exact in double; 2^emin is a normal double (emin >= -149)
    return __dmul_rn(__ll2double_rn(acc), __longlong_as_double(static_cast<long long>(emin + 1023) << 52));
  }
  return warp_add_chain(n, term, lane);
}

// dot_float / mat_vec_float / t_mat_vec_float element: float(S_seq).
template <class Term>
__device__ float warp_seq_dot(int n, Term term, int lane) {
  float out = 0.0f;
  if (!warp_exact_dot(n, term, lane, out)) out = __double2float_rn(warp_fma_chain(n, term, lane));
  return out;
}

__device__ __forceinline__ float power_norm2(double sum) {
  if (!isfinite(sum) || sum < 0.0) return INFINITY;
  if (sum <= static_cast<double>(FLT_MAX)) return __fsqrt_rn(__double2float_rn(sum));
  return __double2float_rn(__dsqrt_rn(sum));
}

// power_norm2_float of v[0..n) by one warp.
__device__ float warp_power_norm(const float* v, int n, int lane) {
  float out = 0.0f;
  auto t = [&](int k, float& x, float& y) {
    x = v[k];
    y = v[k];
  };
  if (warp_exact_dot(n, t, lane, out)) return __fsqrt_rn(out);
  return power_norm2(warp_fma_chain(n, t, lane));
}

// loading[j] = float(S_seq) of sum over training rows k (ascending) of
// double(Z[tix[k]][j]) * double(sc[k]), for every column j: t_mat_vec_float
// of the scores path (plscv.cpp:884).  A thread per column and row group, so
// the loads of a row are coalesced, and one pass over the rows: the fixed
// point of warp_exact_dot is placed from an upper bound of the largest
// product exponent, zexp[j] (the column's largest exponent, label
// independent) plus the scores' largest exponent, instead of the exact one
// (every term still fits: the bound only lowers the magnitudes).  The row
// indices and scores are staged in shared memory so the loads of Z issue
// back to back.  Partial sums of row groups combine exactly (integers), the
// partial bounds of sum |x y| rounding upward; the check and the sequential
// fallback are those of warp_exact_dot / warp_seq_dot.  `scratch` holds
// 4 * kEvalThreads + 2 * kLoadChunk words plus 8 bytes of alignment; every
// thread of the block calls this.
constexpr int kLoadChunk = 1024;
__device__ void block_loading(const float* __restrict__ Zs, int p, const int* __restrict__ tix, int nt,
                              const float* __restrict__ sc, const int* __restrict__ zexp, float* ld, float* scratch,
                              int lane, int warp) {
  long long* pacc = reinterpret_cast<long long*>((reinterpret_cast<uintptr_t>(scratch) + 7) & ~uintptr_t(7));
  float* pA = reinterpret_cast<float*>(pacc + kEvalThreads);
  int* pflag = reinterpret_cast<int*>(pA + kEvalThreads);  // bit 0: non-finite, bit 1: a nonzero term
  int* srow = pflag + kEvalThreads;
  float* ssc = reinterpret_cast<float*>(srow + kLoadChunk);
  int* flist = reinterpret_cast<int*>(pacc);  // undecided columns (after the partials are read)
  __shared__ int fcount, smax;
  const int t = threadIdx.x, lg = clog2i(nt);
  if (t == 0) smax = 1;
  __syncthreads();
  {
    int m = 1;
    for (int k = t; k < nt; k += kEvalThreads) m = max(m, biased_exp1(sc[k]));
    m = __reduce_max_sync(kFull, m);
    if (lane == 0) atomicMax(&smax, m);
  }
  __syncthreads();
  const int se = smax;
  for (int j0 = 0; j0 < p; j0 += kEvalThreads) {
    const int PB = min(p - j0, kEvalThreads), G = kEvalThreads / PB;
    const int g = t / PB, jj = t - g * PB, j = j0 + jj;
    const bool on = g < G;
    const int LSB = (on ? zexp[j] : 1) + se - 252 + lg - 62;
    long long acc = 0;
    float A = 0.0f;
    int bad = 0, nz = 0;
    for (int k0 = 0; k0 < nt; k0 += kLoadChunk) {
      const int cn = min(kLoadChunk, nt - k0);
      for (int i = t; i < cn; i += kEvalThreads) {
        srow[i] = tix[k0 + i];
        ssc[i] = sc[k0 + i];
      }
      __syncthreads();
      if (on) {
#pragma unroll 8
        for (int i = g; i < cn; i += G) {
          const float x = Zs[static_cast<size_t>(srow[i]) * p + j], y = ssc[i];
          const unsigned ux = __float_as_uint(x), uy = __float_as_uint(y);
          bad |= (((ux >> 23) & 0xffu) == 0xffu) | (((uy >> 23) & 0xffu) == 0xffu);
          nz |= ((ux << 1) != 0u) & ((uy << 1) != 0u);
          A = __fadd_ru(A, __fmul_ru(fabsf(x), fabsf(y)));
          acc += exact_fixed_term(x, y, LSB);
        }
      }
      __syncthreads();
    }
    if (on) {
      pacc[t] = acc;
      pA[t] = A;
      pflag[t] = bad | (nz << 1);
    }
    __syncthreads();
    float out = 0.0f;
    bool ok = false;
    if (t < PB) {
      int fl = pflag[t];
      for (int q = 1; q < G; ++q) {
        acc += pacc[t + q * PB];
        A = __fadd_ru(A, pA[t + q * PB]);
        fl |= pflag[t + q * PB];
      }
      if (!(fl & 1)) ok = (fl & 2) ? round_check(acc, LSB, A, nt, out) : (out = 0.0f, true);
    }
    if (t == 0) fcount = 0;
    __syncthreads();
    if (t < PB) {
      if (ok) ld[j] = out;
      else flist[atomicAdd(&fcount, 1)] = j;
    }
    __syncthreads();
    const int nf = fcount;
    for (int f = warp; f < nf; f += kEvalWarps) {
      const int jf = flist[f];
      const double s = warp_fma_chain(nt, [&](int k, float& x, float& y) {
        x = Zs[static_cast<size_t>(tix[k]) * p + jf];
        y = sc[k];
      }, lane);
      if (lane == 0) ld[jf] = __double2float_rn(s);
    }
    __syncthreads();
  }
}

// Scores of 32 rows (one per lane; row < 0 = none) for components
// q0 .. q0+nq-1 (nq <= kMaxNC): acc[q] = sum over features in order of
// z(row, j) * W(j, q0+q).  The rows come in through the warp's transposing
// tile with 128-byte loads.
__device__ __forceinline__ void warp_scores(const float* __restrict__ base, int p, int myrow, const float* W, int ldw,
                                            int q0, int nq, float* tile, int lane, float* acc) {
#pragma unroll
  for (int q = 0; q < kMaxNC; ++q) acc[q] = 0.0f;
  for (int j0 = 0; j0 < p; j0 += 32) {
    const int jl = j0 + lane;
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
      const int ri = __shfl_sync(kFull, myrow, i);
      tile[i * 33 + lane] = (ri >= 0 && jl < p) ? base[static_cast<size_t>(ri) * p + jl] : 0.0f;
    }
    __syncwarp();
    const int jn = min(32, p - j0);
    for (int jj = 0; jj < jn; ++jj) {
      const float v = tile[lane * 33 + jj];
      const float* wr = W + static_cast<size_t>(j0 + jj) * ldw + q0;
#pragma unroll
      for (int q = 0; q < kMaxNC; ++q)
        if (q < nq) acc[q] = __fadd_rn(acc[q], __fmul_rn(v, wr[q]));
    }
    __syncwarp();
  }
}

// Sequential float chain over positions b..e-1 of a row-major matrix
// (stride ld, column c) counting only the positions whose flag is set,
// warp-cooperative: each 32-position group is loaded D groups ahead, then
// every lane adds the group's values in position order.
template <int D>
__device__ float warp_masked_chain(const float* __restrict__ m, int ld, int c, const uint8_t* __restrict__ ok, int b,
                                   int e, int lane) {
  float acc = 0.0f;
  float v[D];
  bool f[D];
#pragma unroll
  for (int g = 0; g < D; ++g) {
    const int i = b + g * 32 + lane;
    v[g] = i < e ? m[static_cast<size_t>(i) * ld + c] : 0.0f;
    f[g] = i < e && ok[i] != 0;
  }
  for (int base = b; base < e; base += 32 * D) {
#pragma unroll
    for (int g = 0; g < D; ++g) {
      const int gb = base + g * 32;
      if (gb >= e) break;
      const unsigned msk = __ballot_sync(kFull, f[g]);
      const float cur = v[g];
      const int i = gb + D * 32 + lane;
      v[g] = i < e ? m[static_cast<size_t>(i) * ld + c] : 0.0f;
      f[g] = i < e && ok[i] != 0;
#pragma unroll 8
      for (int q = 0; q < 32; ++q) {
        const float t = __shfl_sync(kFull, cur, q);
        if ((msk >> q) & 1u) acc = __fadd_rn(acc, t);
      }
    }
  }
  return acc;
}

// Sequential float chain sum_i a_i * b_i over i = 0..n-1 (rows of a
// row-major matrix with stride ld, columns ca and cb), warp-cooperative like
// warp_chain; each 32-row group's operands are loaded D groups ahead of its
// products and adds, so nothing waits on a fresh load.
template <int D>
__device__ float warp_product_chain(const float* __restrict__ m, int n, int ld, int ca, int cb, int lane) {
  float acc = 0.0f;
  float va[D], vb[D];
#pragma unroll
  for (int g = 0; g < D; ++g) {
    const int i = g * 32 + lane;
    va[g] = i < n ? m[static_cast<size_t>(i) * ld + ca] : 0.0f;
    vb[g] = i < n ? m[static_cast<size_t>(i) * ld + cb] : 0.0f;
  }
  for (int base = 0; base < n; base += 32 * D) {
#pragma unroll
    for (int g = 0; g < D; ++g) {
      const int gb = base + g * 32;
      if (gb >= n) break;
      const float prod = __fmul_rn(va[g], vb[g]);
      const int i = gb + D * 32 + lane;
      va[g] = i < n ? m[static_cast<size_t>(i) * ld + ca] : 0.0f;
      vb[g] = i < n ? m[static_cast<size_t>(i) * ld + cb] : 0.0f;
      const int cnt = min(32, n - gb);
#pragma unroll 8
      for (int q = 0; q < 32; ++q) {
        const float t = __shfl_sync(kFull, prod, q);
        if (q < cnt) acc = __fadd_rn(acc, t);
      }
    }
  }
  return acc;
}

__global__ void __launch_bounds__(kEvalThreads, 2) eval_kernel(PlsEvalArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int s = blockIdx.x, r = s / a.F, f = s % a.F;
  const int p = a.p, L = a.L, C = a.C0max, NCm = a.requested, ldw = a.max_components;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  EvalShared& sh = *reinterpret_cast<EvalShared*>(smem);
  size_t off = 64;
  auto carve = [&](size_t bytes) {
    unsigned char* q = smem + off;
    off += (bytes + 15) / 16 * 16;
    return q;
  };
  int* cnt = reinterpret_cast<int*>(carve(sizeof(int) * C));
  int* klist = reinterpret_cast<int*>(carve(sizeof(int) * C));
  float* w = reinterpret_cast<float*>(carve(sizeof(float) * p));
  float* ld = reinterpret_cast<float*>(carve(sizeof(float) * p));
  float* pw = reinterpret_cast<float*>(carve(sizeof(float) * p));
  float* tv = reinterpret_cast<float*>(carve(sizeof(float) * C));
  float* Wsm = reinterpret_cast<float*>(carve(sizeof(float) * p * ldw));
  float* Vsm = reinterpret_cast<float*>(carve(sizeof(float) * p * ldw));
  float* cs = reinterpret_cast<float*>(carve(sizeof(float) * C * NCm));
  float* cp = reinterpret_cast<float*>(carve(sizeof(float) * NCm * NCm));
  float* pooled = reinterpret_cast<float*>(carve(sizeof(float) * NCm * NCm));
  float* Lc = reinterpret_cast<float*>(carve(sizeof(float) * NCm * NCm));
  float* sol = reinterpret_cast<float*>(carve(sizeof(float) * NCm * C));
  float* lin = reinterpret_cast<float*>(carve(sizeof(float) * C * NCm));
  float* cst = reinterpret_cast<float*>(carve(sizeof(float) * C));
  double* ssum = reinterpret_cast<double*>(carve(sizeof(double) * NCm));  // PLS-DA score sums
  // shared region: the cross-product (when it fits) and the score tiles,
  // which overlap it unless a slice of the launch computes scores during the
  // fit (no fold Gram)
  float* region = reinterpret_cast<float*>(carve(0));
  float* tiles = (a.s_in_smem && a.tiles_after_s) ? region + static_cast<size_t>(p) * C : region;

  const uint16_t* lab = a.labels + static_cast<size_t>(r) * L;
  const int* coff = a.class_off + static_cast<size_t>(r) * (C + 1);
  const uint16_t* crow = a.class_rows + static_cast<size_t>(r) * L;
  const uint8_t* fold = a.predict_mode ? nullptr : a.folds + static_cast<size_t>(r) * L;
  const float* Zs = a.Z + static_cast<size_t>(s) * L * p;
  const int tb = a.train_off[s], te = a.train_off[s + 1];
  const int nv = a.predict_mode ? a.NV : a.val_off[s + 1] - a.val_off[s];
  const int* vidx = a.predict_mode ? nullptr : a.val_idx + a.val_off[s];
  uint16_t* pred = a.pred + static_cast<size_t>(r) * (a.predict_mode ? a.NV : L);
  const float* vbase = a.predict_mode ? a.Zv + static_cast<size_t>(r) * a.NV * p : Zs;

  // --- fold classes: codes with training rows, ascending -------------------
  for (int c = threadIdx.x; c < C; c += kEvalThreads) cnt[c] = coff[c + 1] - coff[c];
  __syncthreads();
  if (!a.predict_mode)
    for (int v = threadIdx.x; v < nv; v += kEvalThreads) atomicSub(&cnt[lab[vidx[v]]], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = 0;
    for (int c = 0; c < C; ++c)
      if (cnt[c] > 0) klist[m++] = c;
    sh.m = m;
    sh.nt = te - tb;
    a.status[s] = 0;
  }
  // class-list position of every row, and whether that position trains the slice
  uint16_t* posof = a.pos + static_cast<size_t>(s) * L;
  uint8_t* posok = a.posok + static_cast<size_t>(s) * L;
  for (int i = threadIdx.x; i < L; i += kEvalThreads) {
    const int row = crow[i];
    posof[row] = static_cast<uint16_t>(i);
    posok[i] = (fold == nullptr || fold[row] != f) ? 1 : 0;
  }
  __syncthreads();
  const int m = sh.m, nt = sh.nt;
  if (m <= 1) {
    // one training class: it is every prediction (labels.front() without one)
    const int only = m == 1 ? klist[0] : lab[0];
    for (int v = threadIdx.x; v < nv; v += kEvalThreads)
      pred[a.predict_mode ? v : vidx[v]] = static_cast<uint16_t>(only);
    if (threadIdx.x == 0) a.eval_comp[s] = 1;
    return;
  }

  // --- label cross-product S (p x m), column k = fold class k -------------
  float* S = a.s_in_smem ? region : a.s_scr + static_cast<size_t>(s) * p * C;
  {
    const int JB = (p + 31) / 32;
    const float inv_n = nt > 0 ? __fdiv_rn(1.0f, static_cast<float>(nt)) : 0.0f;
    for (int it = warp; it < m * JB; it += kEvalWarps) {
      const int k = it / JB, j = (it % JB) * 32 + lane;
      const int code = klist[k];
      const int b = coff[code], e = coff[code + 1];
      float acc = 0.0f;
      for (int base = b; base < e; base += 32) {
        const int row = base + lane < e ? crow[base + lane] : -1;
        const bool ok = row >= 0 && (fold == nullptr || fold[row] != f);
        const unsigned msk = __ballot_sync(kFull, ok);
        float v[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int rq = __shfl_sync(kFull, row, q);
          v[q] = (((msk >> q) & 1u) && j < p) ? Zs[static_cast<size_t>(rq) * p + j] : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < 32; ++q)
          if ((msk >> q) & 1u) acc = __fadd_rn(acc, v[q]);
      }
      if (j < p) {
        const float y_mean = __fmul_rn(static_cast<float>(cnt[code]), inv_n);
        S[j + static_cast<size_t>(k) * p] =
            __fsub_rn(acc, __fmul_rn(y_mean, a.xsum[static_cast<size_t>(s) * p + j]));
      }
    }
  }
  __syncthreads();

  // --- SIMPLS weights ------------------------------------------------------
  const int maxr = min(min(a.max_components, p), max(1, nt - 1));
  const bool gram = a.gram != nullptr && a.use_gram[s];
  const float* G = gram ? a.gram + static_cast<size_t>(s) * p * p : nullptr;
  float* scv = a.sc + static_cast<size_t>(s) * L;
  const int* tix = a.train_idx + tb;
  int fitted = 0;
  for (int comp = 0; comp < maxr; ++comp) {
    for (int j = threadIdx.x; j < p; j += kEvalThreads) w[j] = comp == 0 ? a.w0[j] : pw[j];
    __syncthreads();
    // two power iterations (a second pass only for the strongest-column retry)
    for (int pass = 0; pass < 2; ++pass) {
      for (int it = 0; it < 2; ++it) {
        for (int c = warp; c < m; c += kEvalWarps) {
          const float* col = S + static_cast<size_t>(c) * p;
          const float v = warp_seq_dot(p, [&](int k, float& x, float& y) {
            x = col[k];
            y = w[k];
          }, lane);
          if (lane == 0) tv[c] = v;
        }
        __syncthreads();
        for (int j = warp; j < p; j += kEvalWarps) {
          const float v = warp_seq_dot(m, [&](int k, float& x, float& y) {
            x = S[j + static_cast<size_t>(k) * p];
            y = tv[k];
          }, lane);
          if (lane == 0) w[j] = v;
        }
        __syncthreads();
      }
      if (warp == 0) {
        const float rn = warp_power_norm(w, p, lane);
        if (lane == 0) {
          sh.rn = rn;
          sh.best = -1;
          if (pass == 0 && comp == 0 && !(isfinite(rn) && rn > 1.0e-10f)) {
            // retry on the response column with the largest norm (rare: double sums)
            double bn = 0.0;
            int best = -1;
            for (int k = 0; k < m; ++k) {
              double ns = 0.0;
              for (int j = 0; j < p; ++j) {
                const double v = static_cast<double>(S[j + static_cast<size_t>(k) * p]);
                ns = fma(v, v, ns);
              }
              if (isfinite(ns) && ns > bn) {
                bn = ns;
                best = k;
              }
            }
            if (best >= 0 && bn > 1.0e-20) sh.best = best;
          }
        }
      }
      __syncthreads();
      if (sh.best < 0) break;
      const int best = sh.best;
      for (int j = threadIdx.x; j < p; j += kEvalThreads) w[j] = S[j + static_cast<size_t>(best) * p];
      __syncthreads();
    }
    const float rn = sh.rn;
    if (!(isfinite(rn) && rn > 1.0e-10f)) break;
    for (int j = threadIdx.x; j < p; j += kEvalThreads) w[j] = __fdiv_rn(w[j], rn);
    __syncthreads();
    if (gram) {
      for (int i = warp; i < p; i += kEvalWarps) {
        const float* gi = G + static_cast<size_t>(i) * p;
        const float v = warp_seq_dot(p, [&](int k, float& x, float& y) {
          x = gi[k];
          y = w[k];
        }, lane);
        if (lane == 0) ld[i] = v;
      }
      __syncthreads();
      if (warp == 0) {
        const float sns = warp_seq_dot(p, [&](int k, float& x, float& y) {
          x = w[k];
          y = ld[k];
        }, lane);
        if (lane == 0) {
          sh.stop = !(isfinite(sns) && sns > 1.0e-20f);
          sh.inv = sh.stop ? 0.0f : __fdiv_rn(1.0f, __fsqrt_rn(sns));
        }
      }
      __syncthreads();
      if (sh.stop) break;
      const float inv = sh.inv;
      for (int j = threadIdx.x; j < p; j += kEvalThreads) {
        w[j] = __fmul_rn(w[j], inv);
        ld[j] = __fmul_rn(ld[j], inv);
      }
      __syncthreads();
    } else {
      // scores of the training rows, their norm, loading = X^T scores
      float* tile = tiles + warp * kTile;
      for (int b0 = warp * 32; b0 < nt; b0 += kEvalWarps * 32) {
        const int t = b0 + lane;
        const int row = t < nt ? tix[t] : -1;
        float acc[kMaxNC];
        warp_scores(Zs, p, row, w, 1, 0, 1, tile, lane, acc);
        if (t < nt) scv[t] = acc[0];
      }
      __syncthreads();
      if (warp == 0) {
        const float d = warp_seq_dot(nt, [&](int k, float& x, float& y) {
          x = scv[k];
          y = scv[k];
        }, lane);
        if (lane == 0) {
          const float sn = __fsqrt_rn(0.0f < d ? d : 0.0f);
          sh.stop = !(isfinite(sn) && sn > 1.0e-10f);
          sh.inv = sh.stop ? 0.0f : __fdiv_rn(1.0f, sn);
        }
      }
      __syncthreads();
      if (sh.stop) break;
      const float inv = sh.inv;
      for (int t = threadIdx.x; t < nt; t += kEvalThreads) scv[t] = __fmul_rn(scv[t], inv);
      for (int j = threadIdx.x; j < p; j += kEvalThreads) w[j] = __fmul_rn(w[j], inv);
      __syncthreads();
      block_loading(Zs, p, tix, nt, scv, a.zexp + static_cast<size_t>(s) * p, ld, tiles, lane, warp);
    }
    for (int j = threadIdx.x; j < p; j += kEvalThreads) pw[j] = w[j];
    // Gram-Schmidt against the previous loadings
    for (int q = 0; q < comp; ++q) {
      if (threadIdx.x == 0) {
        float proj = 0.0f;
        for (int j = 0; j < p; ++j) proj = __fadd_rn(proj, __fmul_rn(Vsm[static_cast<size_t>(j) * ldw + q], ld[j]));
        sh.inv = proj;
      }
      __syncthreads();
      const float proj = sh.inv;
      for (int j = threadIdx.x; j < p; j += kEvalThreads)
        ld[j] = __fsub_rn(ld[j], __fmul_rn(proj, Vsm[static_cast<size_t>(j) * ldw + q]));
      __syncthreads();
    }
    if (warp == 0) {
      const float d = warp_seq_dot(p, [&](int k, float& x, float& y) {
        x = ld[k];
        y = ld[k];
      }, lane);
      if (lane == 0) {
        const float ln = __fsqrt_rn(0.0f < d ? d : 0.0f);
        sh.stop = !(isfinite(ln) && ln > 1.0e-10f);
        sh.inv = ln;
      }
    }
    __syncthreads();
    if (sh.stop) break;
    const float ln = sh.inv;
    for (int j = threadIdx.x; j < p; j += kEvalThreads) {
      ld[j] = __fdiv_rn(ld[j], ln);
      Wsm[static_cast<size_t>(j) * ldw + comp] = w[j];
      Vsm[static_cast<size_t>(j) * ldw + comp] = ld[j];
    }
    __syncthreads();
    // deflate the cross-product
    for (int k = threadIdx.x; k < m; k += kEvalThreads) {
      float acc = 0.0f;
      const float* col = S + static_cast<size_t>(k) * p;
      for (int j = 0; j < p; ++j) acc = __fadd_rn(acc, __fmul_rn(ld[j], col[j]));
      tv[k] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < p * m; e += kEvalThreads) {
      const int j = e % p, k = e / p;
      S[e] = __fsub_rn(S[e], __fmul_rn(ld[j], tv[k]));
    }
    __syncthreads();
    fitted = comp + 1;
  }

  if (fitted < 1) {
    if (a.predict_mode) {
      if (threadIdx.x == 0) a.status[s] = 1;
      return;
    }
    // DegeneratePLSFit: the most frequent training class, smallest on ties
    if (threadIdx.x == 0) {
      int bl = klist[0], bc = -1;
      for (int k = 0; k < m; ++k) {
        if (cnt[klist[k]] > bc) {
          bc = cnt[klist[k]];
          bl = klist[k];
        }
      }
      sh.lab = bl;
      a.eval_comp[s] = 1;
    }
    __syncthreads();
    for (int v = threadIdx.x; v < nv; v += kEvalThreads)
      pred[a.predict_mode ? v : vidx[v]] = static_cast<uint16_t>(sh.lab);
    return;
  }

  // --- LDA on the first nc score columns -----------------------------------
  const int nc = a.predict_mode ? fitted : min(a.requested, fitted);
  float* Ts = a.T + static_cast<size_t>(s) * L * NCm;   // by class-list position: Ts[pos * nc + q]
  float* Tt = a.Tt + static_cast<size_t>(s) * L * NCm;  // by training position: Tt[t * nc + q]
  {
    float* tile = tiles + warp * kTile;
    for (int b0 = warp * 32; b0 < nt; b0 += kEvalWarps * 32) {
      const int t = b0 + lane;
      const int row = t < nt ? tix[t] : -1;
      for (int q0 = 0; q0 < nc; q0 += kMaxNC) {
        const int nq = min(kMaxNC, nc - q0);
        float acc[kMaxNC];
        warp_scores(Zs, p, row, Wsm, ldw, q0, nq, tile, lane, acc);
        if (row >= 0) {
          const size_t ps = static_cast<size_t>(posof[row]) * nc;
#pragma unroll
          for (int q = 0; q < kMaxNC; ++q) {
            if (q < nq) {
              Ts[ps + q0 + q] = acc[q];
              Tt[static_cast<size_t>(t) * nc + q0 + q] = acc[q];
            }
          }
        }
      }
    }
  }
  __syncthreads();
  // class sums (the training rows of each class in row order, i.e. the
  // flagged class-list positions in order): one warp per chain
  const int ncs = m * nc, ncp = nc * (nc + 1) / 2;
  for (int it = warp; it < ncs; it += kEvalWarps) {
    const int k = it / nc, q = it % nc;
    const int code = klist[k];
    const float acc = warp_masked_chain<2>(Ts, nc, q, posok, coff[code], coff[code + 1], lane);
    if (lane == 0) cs[k * nc + q] = acc;
  }
  if (a.da_mode) {
    // --- PLS-DA (the PLS_DA branch of run_plscv_host, plscv.cpp:2428-2443) ---
    // class means of the one-hot labels (label_means_float, plscv.cpp:1210)
    __syncthreads();
    const float inv_n = nt > 0 ? __fdiv_rn(1.0f, static_cast<float>(nt)) : 0.0f;
    for (int k = threadIdx.x; k < m; k += kEvalThreads) cst[k] = __fmul_rn(static_cast<float>(cnt[klist[k]]), inv_n);
    // regression_coefficients_centered_one_hot_float (plscv.cpp:1222-1265):
    // double score sums and double score cross-products over the training rows
    for (int q = warp; q < nc; q += kEvalWarps) {
      const double v = warp_seq_sum_double(nt, [&](int i) { return Tt[static_cast<size_t>(i) * nc + q]; }, lane);
      if (lane == 0) ssum[q] = v;
    }
    for (int it = warp; it < ncp; it += kEvalWarps) {
      int pr = it, rr = 0;
      while (pr > rr) {
        pr -= rr + 1;
        ++rr;
      }
      const int col = pr;
      const float v = warp_seq_dot(nt, [&](int i, float& x, float& y) {
        x = Tt[static_cast<size_t>(i) * nc + col];
        y = Tt[static_cast<size_t>(i) * nc + rr];
      }, lane);
      if (lane == 0) {
        pooled[rr * nc + col] = v;
        pooled[col * nc + rr] = v;
      }
    }
    __syncthreads();
    for (int it = threadIdx.x; it < nc * m; it += kEvalThreads) {
      const int q = it / m, k = it % m;
      sol[q * m + k] = __fsub_rn(cs[k * nc + q], __double2float_rn(__dmul_rn(ssum[q], static_cast<double>(cst[k]))));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      // solve_linear_float (plscv.cpp:1346-1377): Gauss-Jordan with partial
      // pivoting on lhs + 1e-9 I
      float* A = pooled;
      for (int i = 0; i < nc; ++i) A[i * nc + i] = __fadd_rn(A[i * nc + i], 1.0e-9f);
      for (int c = 0; c < nc; ++c) {
        int piv = c;
        float best = fabsf(A[c * nc + c]);
        for (int r2 = c + 1; r2 < nc; ++r2) {
          const float val = fabsf(A[r2 * nc + c]);
          if (val > best) {
            best = val;
            piv = r2;
          }
        }
        if (best < 1.0e-12f) continue;
        if (piv != c) {
          for (int j = 0; j < nc; ++j) {
            const float t = A[c * nc + j];
            A[c * nc + j] = A[piv * nc + j];
            A[piv * nc + j] = t;
          }
          for (int j = 0; j < m; ++j) {
            const float t = sol[c * m + j];
            sol[c * m + j] = sol[piv * m + j];
            sol[piv * m + j] = t;
          }
        }
        const float dv = A[c * nc + c];
        for (int j = c; j < nc; ++j) A[c * nc + j] = __fdiv_rn(A[c * nc + j], dv);
        for (int j = 0; j < m; ++j) sol[c * m + j] = __fdiv_rn(sol[c * m + j], dv);
        for (int r2 = 0; r2 < nc; ++r2) {
          if (r2 == c) continue;
          const float fct = A[r2 * nc + c];
          if (fct == 0.0f) continue;
          for (int j = c; j < nc; ++j) A[r2 * nc + j] = __fsub_rn(A[r2 * nc + j], __fmul_rn(fct, A[c * nc + j]));
          for (int j = 0; j < m; ++j) sol[r2 * m + j] = __fsub_rn(sol[r2 * m + j], __fmul_rn(fct, sol[c * m + j]));
        }
      }
      a.eval_comp[s] = nc;
    }
    __syncthreads();
    // predict_pls_da_labels_float (plscv.cpp:1267-1292): first maximum of
    // mean + scores x coefficients
    float* tile = tiles + warp * kTile;
    for (int b0 = warp * 32; b0 < nv; b0 += kEvalWarps * 32) {
      const int v = b0 + lane;
      const int row = v < nv ? (a.predict_mode ? v : vidx[v]) : -1;
      float sr[kMaxComp];
      for (int q0 = 0; q0 < nc; q0 += kMaxNC) {
        const int nq = min(kMaxNC, nc - q0);
        float acc[kMaxNC];
        warp_scores(vbase, p, row, Wsm, ldw, q0, nq, tile, lane, acc);
#pragma unroll
        for (int q = 0; q < kMaxNC; ++q)
          if (q < nq) sr[q0 + q] = acc[q];
      }
      if (row >= 0) {
        int best = 0;
        float bs = -INFINITY;
        for (int k = 0; k < m; ++k) {
          float sc = cst[k];
          for (int q = 0; q < nc; ++q) sc = __fadd_rn(sc, __fmul_rn(sr[q], sol[q * m + k]));
          if (sc > bs) {
            bs = sc;
            best = k;
          }
        }
        pred[row] = static_cast<uint16_t>(klist[best]);
      }
    }
    return;
  }
  // score cross-products (all training rows in order): one warp per chain
  for (int it = warp; it < ncp; it += kEvalWarps) {
    int pr = it, rr = 0;
    while (pr > rr) {
      pr -= rr + 1;
      ++rr;
    }
    const int col = pr;
    const float acc = warp_product_chain<4>(Tt, nt, nc, rr, col, lane);
    if (lane == 0) {
      cp[rr * nc + col] = acc;
      cp[col * nc + rr] = acc;
    }
  }
  __syncthreads();
  // fit_lda_from_score_statistics_float, parallel where the reference's loops
  // are independent of one another
  for (int it = threadIdx.x; it < m * nc; it += kEvalThreads) {
    const int k = it / nc, c = cnt[klist[k]];
    const float inv = c > 0 ? __fdiv_rn(1.0f, static_cast<float>(c)) : 0.0f;
    cs[it] = __fmul_rn(cs[it], inv);
  }
  __syncthreads();
  const float df = static_cast<float>(max(1, nt - m));
  for (int it = threadIdx.x; it < ncp; it += kEvalThreads) {
    int pr = it, rr = 0;
    while (pr > rr) {
      pr -= rr + 1;
      ++rr;
    }
    const int col = pr;
    float between = 0.0f;
    for (int k = 0; k < m; ++k)
      between = __fadd_rn(between, __fmul_rn(__fmul_rn(static_cast<float>(cnt[klist[k]]), cs[k * nc + rr]),
                                             cs[k * nc + col]));
    const float cv = __fdiv_rn(__fsub_rn(cp[rr * nc + col], between), df);
    pooled[rr * nc + col] = cv;
    pooled[col * nc + rr] = cv;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // the ridge grid and the Cholesky factor (independent of the right-hand sides)
    float trace = 0.0f;
    for (int rr = 0; rr < nc; ++rr) trace = __fadd_rn(trace, pooled[rr * nc + rr]);
    const float ridge_scale =
        (isfinite(trace) && trace > 0.0f) ? __fdiv_rn(trace, static_cast<float>(max(1, nc))) : 1.0f;
    const float grid[6] = {1e-8f, 1e-6f, 1e-5f, 1e-4f, 1e-3f, 1e-2f};
    bool ok = false;
    for (int g = 0; g < 6 && !ok; ++g) {
      const float lambda = __fmul_rn(grid[g], ridge_scale);
      ok = true;
      for (int row = 0; row < nc && ok; ++row) {
        for (int col = 0; col <= row && ok; ++col) {
          float v = pooled[row * nc + col];
          if (row == col) v = __fadd_rn(v, lambda);
          for (int q = 0; q < col; ++q) v = __fsub_rn(v, __fmul_rn(Lc[row * nc + q], Lc[col * nc + q]));
          if (row == col) {
            if (!isfinite(v) || v <= 0.0f) ok = false;
            else Lc[row * nc + col] = __fsqrt_rn(v);
          } else {
            const float dgl = Lc[col * nc + col];
            if (!isfinite(dgl) || dgl <= 0.0f) ok = false;
            else Lc[row * nc + col] = __fdiv_rn(v, dgl);
          }
        }
      }
    }
    sh.fail = ok ? 0 : 1;
    if (!ok) a.status[s] = 2;
    a.eval_comp[s] = nc;
  }
  __syncthreads();
  if (sh.fail) return;
  const float* lp = a.logprior + a.lp_off[s];
  for (int k = threadIdx.x; k < m; k += kEvalThreads) {
    // forward and backward substitution for the right-hand side of class k
    for (int row = 0; row < nc; ++row) {
      float v = cs[k * nc + row];
      for (int q = 0; q < row; ++q) v = __fsub_rn(v, __fmul_rn(Lc[row * nc + q], sol[q * m + k]));
      sol[row * m + k] = __fdiv_rn(v, Lc[row * nc + row]);
    }
    for (int row = nc - 1; row >= 0; --row) {
      float v = sol[row * m + k];
      for (int q = row + 1; q < nc; ++q) v = __fsub_rn(v, __fmul_rn(Lc[q * nc + row], sol[q * m + k]));
      sol[row * m + k] = __fdiv_rn(v, Lc[row * nc + row]);
    }
    float dot_mu = 0.0f;
    for (int q = 0; q < nc; ++q) {
      lin[k * nc + q] = sol[q * m + k];
      dot_mu = __fadd_rn(dot_mu, __fmul_rn(cs[k * nc + q], lin[k * nc + q]));
    }
    cst[k] = __fadd_rn(__fmul_rn(-0.5f, dot_mu), lp[cnt[klist[k]]]);
  }
  __syncthreads();
  // --- predictions ---------------------------------------------------------
  {
    float* tile = tiles + warp * kTile;
    for (int b0 = warp * 32; b0 < nv; b0 += kEvalWarps * 32) {
      const int v = b0 + lane;
      const int row = v < nv ? (a.predict_mode ? v : vidx[v]) : -1;
      float sr[kMaxComp];
      for (int q0 = 0; q0 < nc; q0 += kMaxNC) {
        const int nq = min(kMaxNC, nc - q0);
        float acc[kMaxNC];
        warp_scores(vbase, p, row, Wsm, ldw, q0, nq, tile, lane, acc);
#pragma unroll
        for (int q = 0; q < kMaxNC; ++q)
          if (q < nq) sr[q0 + q] = acc[q];
      }
      if (row >= 0) {
        int best = 0;
        float bs = -INFINITY;
        for (int k = 0; k < m; ++k) {
          float sc = cst[k];
          for (int q = 0; q < nc; ++q) sc = __fadd_rn(sc, __fmul_rn(sr[q], lin[k * nc + q]));
          if (sc > bs) {
            bs = sc;
            best = k;
          }
        }
        pred[row] = static_cast<uint16_t>(klist[best]);
      }
    }
  }
}

__global__ void gather_kernel(const float* __restrict__ x, int p, const int* __restrict__ rows, size_t nrows,
                              float* __restrict__ out) {
  const size_t total = nrows * p;
  for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t i = e / p;
    out[e] = x[static_cast<size_t>(rows[i]) * p + (e - i * p)];
  }
}

__global__ void assemble_kernel(int problems, int n, int L, int NV, const int* land, const int* test_rows,
                                const uint16_t* clbest, const uint16_t* proj, const int* c2l, int C0max, int* res) {
  const size_t per = static_cast<size_t>(L) + NV;
  const size_t total = static_cast<size_t>(problems) * per;
  for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t r = e / per, i = e - r * per;
    const int* map = c2l + r * C0max;
    if (i < static_cast<size_t>(L)) {
      res[r * n + land[r * L + i]] = map[clbest[r * L + i]];
    } else {
      const size_t t = i - L;
      res[r * n + test_rows[r * NV + t]] = map[proj[r * NV + t]];
    }
  }
}

}  // namespace

int pls_gather_rows(const float* x, int p, const int* rows, size_t nrows, float* out, cudaStream_t st) {
  gather_kernel<<<4 * 152, 256, 0, st>>>(x, p, rows, nrows, out);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int pls_assemble_result(int problems, int n, int L, int NV, const int* land, const int* test_rows,
                        const uint16_t* clbest, const uint16_t* proj, const int* code2label, int C0max, int* res,
                        cudaStream_t st) {
  assemble_kernel<<<2 * 152, 256, 0, st>>>(problems, n, L, NV, land, test_rows, clbest, proj, code2label, C0max,
                                           res);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int pls_prepare(const PlsPrepArgs& a, cudaStream_t st) {
  const int S = a.problems * a.F;
  dim3 g1(S, (a.p + 127) / 128);
  stats_kernel<<<g1, 128, 0, st>>>(a);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return static_cast<int>(e);
  {
    const int ys = std::max(1, std::min(S, 65535));
    const int xs = std::max(1, std::min(std::max(a.L, a.NV), std::max(1, 4096 / ys)));
    standardize_kernel<<<dim3(xs, ys), a.p <= 128 ? 128 : 256, 0, st>>>(a);
  }
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return static_cast<int>(e);
  xsum_kernel<<<g1, 128, 0, st>>>(a);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int pls_build_gram(const PlsPrepArgs& a, const uint8_t* want, cudaStream_t st) {
  const int S = a.problems * a.F;
  const int JB = (a.p + kGramT - 1) / kGramT;
  dim3 grid(S, JB * (JB + 1) / 2);
  gram_kernel<<<grid, 256, 0, st>>>(a, want);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

size_t pls_eval_smem(int p, int C0max, int requested, int max_components, bool s_in_smem, bool tiles_after_s) {
  auto al = [](size_t v) { return (v + 15) / 16 * 16; };
  const size_t C = static_cast<size_t>(C0max), N = static_cast<size_t>(requested);
  size_t b = 64;
  b += 2 * al(sizeof(int) * C);
  b += 3 * al(sizeof(float) * p) + al(sizeof(float) * C);
  b += 2 * al(sizeof(float) * p * max_components);
  b += al(sizeof(float) * C * N) + 3 * al(sizeof(float) * N * N) + al(sizeof(float) * N * C);
  b += al(sizeof(float) * C * N) + al(sizeof(float) * C) + al(sizeof(double) * N);
  const size_t cross = s_in_smem ? sizeof(float) * static_cast<size_t>(p) * C : 0;
  const size_t tiles = sizeof(float) * static_cast<size_t>(kEvalWarps) * kTile;
  b += tiles_after_s ? cross + tiles : (cross > tiles ? cross : tiles);
  return b;
}

int pls_evaluate(const PlsEvalArgs& a, cudaStream_t st) {
  const int S = a.problems * a.F;
  if (a.requested > kMaxComp || a.max_components > kMaxComp) return static_cast<int>(cudaErrorInvalidValue);
  const size_t smem =
      pls_eval_smem(a.p, a.C0max, a.requested, a.max_components, a.s_in_smem != 0, a.tiles_after_s != 0);
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
  }
  eval_kernel<<<S, kEvalThreads, smem, st>>>(a);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
