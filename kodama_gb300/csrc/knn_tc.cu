// Exact kNN graph through a tensor-core candidate search (knn.cuh).
//
// The canonical result (knn.cu: squared L2 as a float32 chain over the
// coordinates in order, each term separately rounded, ties by index) is
// found in three steps:
//
//  1. candidates: every row is split once into bfloat16 hi + lo parts
//     (x = hi + lo + r, |r| <= 2^-16 |x|); a warp computes the approximate
//     distances a = |q|^2 + |c|^2 - 2 (hi.hi + hi.lo + lo.hi) of 16 queries
//     to a 64-row candidate tile with mma.sync (bf16 in, f32 accumulate).
//     The candidate tiles are dealt to S segments (grid.y) in a scattered
//     order; per segment every query keeps the kp smallest approximate
//     distances of each half of its columns in two max-heaps, one per lane
//     (lanes r and r + 16 own query row r).  The lanes holding the
//     accumulator fragments flag the values below their heap's threshold and
//     publish per-row masks; each owner lane inserts only its flagged
//     values, so the 32 heaps of a warp fill side by side;
//  2. re-rank: one warp per query takes A_K, the K-th smallest approximate
//     distance over its heaps, computes the canonical distances of the
//     candidates with a <= A_K + 2 delta, and keeps the K smallest by
//     (distance, index);
//  3. certificate: every row left out of the heaps has a >= B, the smallest
//     final heap threshold.  A row of the true top K (ties by index
//     included) has e <= e_K <= A_K + delta, hence a <= A_K + 2 delta, so
//     B > A_K + 2 delta proves it was kept and re-ranked.  Rows whose
//     certificate fails are listed and recomputed by the brute-force kernels
//     (knn.cu).  delta bounds |a - e| for every row (below).
//
// Error bound (u = 2^-24): with D the true squared distance and e its
// canonical value, |e - D| <= (d + 4) u D <= 2 (d + 4) u (|q|^2 + |c|^2);
// the split drops hi.hi residuals of at most ~3.1 * 2^-16 sum|q_i c_i|, the
// f32 accumulation of 3 dp products adds at most 3 dp 2^-22 sum|q_i c_i|
// (tensor-core accumulation allowed two ulps per add), and
// sum|q_i c_i| <= (|q|^2 + |c|^2) / 2; the f32 norms and the final
// combination add (d + 8) u (|q|^2 + |c|^2).  So
// delta <= (|q|^2 + max |c|^2) * (1e-4 + 2e-6 dp), a safe over-estimate.
#include "knn.cuh"
#include "launch_count.cuh"

#include "bf16_split.cuh"

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace kgb {

namespace {

constexpr int kTcWarps = 4;            // warps per CTA, 16 queries each
constexpr int kTcQ = 16 * kTcWarps;    // queries per CTA
constexpr int kTcN = 64;               // candidates per tile
constexpr int kTcRegKs = 8;            // k-steps whose query fragments (hi and lo) sit in registers
constexpr int kTcMaxKs = 16;           // dp <= 256: above kTcRegKs the lo fragments come from shared memory
constexpr size_t kTcSmemLimit = 227 * 1024;
constexpr int kTileStride = kTcN + 8;  // floats per row of a warp's distance tile

__global__ void tc_prep_kernel(const float* __restrict__ x, int n, int d, int dp, uint16_t* __restrict__ xh,
                               uint16_t* __restrict__ xl, float* __restrict__ nrm, unsigned* __restrict__ nrm_max,
                               int* __restrict__ nonfinite) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float s = 0.0f;
  bool fin = true;
  for (int k = 0; k < dp; ++k) {
    const float v = k < d ? x[static_cast<size_t>(r) * d + k] : 0.0f;
    fin = fin && isfinite(v);
    const uint32_t hb = bf16_bits(v);
    const float h = __uint_as_float(hb << 16);
    const uint32_t lb = bf16_bits(__fsub_rn(v, h));
    const size_t o = static_cast<size_t>(r) * dp + perm16(k);
    xh[o] = static_cast<uint16_t>(hb);
    xl[o] = static_cast<uint16_t>(lb);
    s = __fadd_rn(s, __fmul_rn(v, v));
  }
  nrm[r] = s;
  if (fin) atomicMax(nrm_max, __float_as_uint(s));
  else atomicExch(nonfinite, 1);
}

__global__ void split_rows_kernel(const float* __restrict__ x, int n, int d, int dp, uint16_t* __restrict__ xh,
                                  uint16_t* __restrict__ xl) {
  const size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<size_t>(n) * dp) return;
  const int r = static_cast<int>(e / dp), k = static_cast<int>(e % dp);
  const float v = k < d ? x[static_cast<size_t>(r) * d + k] : 0.0f;
  const uint32_t hb = bf16_bits(v);
  const uint32_t lb = bf16_bits(__fsub_rn(v, __uint_as_float(hb << 16)));
  const size_t o = static_cast<size_t>(r) * dp + perm16(k);
  xh[o] = static_cast<uint16_t>(hb);
  xl[o] = static_cast<uint16_t>(lb);
}

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

struct TcArgs {
  const uint16_t* xh;   // n x dp, permuted 16-blocks
  const uint16_t* xl;
  const float* nrm;     // n
  int n, dp, kp, segs;
  int row_words;        // 32-bit words per candidate row in shared memory (= 8 mod 16)
  int* cand;            // n x segs x 2 x kp candidate rows (-1 = none)
  float* cand_a;        // their approximate distances
  float* bound;         // n x segs: the smaller final heap threshold (+inf = nothing excluded)
};

constexpr int kMaxPer = 8;   // re-rank candidates per lane (segs x 2 x kp <= 256)

// Shared memory: 2 x (hi, lo) candidate tiles, 2 x tile norms, per warp a
// 16 x kTileStride distance tile, 16 x 4 flag masks, 32 thresholds and 32
// lane-interleaved max-heaps of kp (distance, row) entries; above kTcRegKs
// k-steps also the warp's 16 lo query rows (row stride row_words, the
// candidate tiles' conflict-free stride).
size_t tc_smem_bytes(int row_words, int kp, int dp) {
  const size_t lo_rows = dp > 16 * kTcRegKs ? kTcWarps * 16 * static_cast<size_t>(row_words) * 4 : 0;
  return 2 * 2 * static_cast<size_t>(kTcN) * row_words * 4 + 2 * kTcN * 4 +
         kTcWarps * (16 * kTileStride * 4 + 64 * 4 + 32 * 4 + 32 * static_cast<size_t>(kp) * 8) + lo_rows;
}

// KS: k-steps of 16 coordinates in the query fragments (dp <= 16 KS).  Up to
// kTcRegKs every thread keeps its 2 KS 16-byte chunks of a candidate tile
// (kTcN x dp / 8 / 128) in registers; above it the chunks are recomputed per
// tile and the lo query fragments are read from shared memory per k-step.
template <int KS>
__global__ void __launch_bounds__(32 * kTcWarps, 2) tc_candidates_kernel(TcArgs A) {
  constexpr bool kLoShared = KS > kTcRegKs;
  constexpr int kMaxLoads = kLoShared ? 1 : 2 * KS;
  constexpr int kRegLo = kLoShared ? 1 : KS;
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
  const int n = A.n, dp = A.dp, kp = A.kp, rw = A.row_words, ksn = dp >> 4;
  const int seg = blockIdx.y, segs = A.segs;
  uint32_t* cbuf = reinterpret_cast<uint32_t*>(smem);  // [buf][hi/lo][kTcN][rw]
  float* cnb = reinterpret_cast<float*>(cbuf + 2 * 2 * kTcN * rw);  // [buf][kTcN]
  float* dt = cnb + 2 * kTcN + warp * (16 * kTileStride + 64 + 32 + 32 * kp * 2);  // [16][kTileStride]
  unsigned* fmask = reinterpret_cast<unsigned*>(dt + 16 * kTileStride);            // [16][4]
  float* htau = reinterpret_cast<float*>(fmask + 64);                              // [32] per heap
  float* hv = htau + 32;                                                           // [kp][32]
  int* hj = reinterpret_cast<int*>(hv + 32 * kp);                                  // [kp][32]
  htau[lane] = INFINITY;

  const int q0 = blockIdx.x * kTcQ + warp * 16;
  // the warp's 16 lo query rows in shared memory (only above kTcRegKs)
  uint32_t* qlo = reinterpret_cast<uint32_t*>(cnb + 2 * kTcN + kTcWarps * (16 * kTileStride + 64 + 32 + 32 * kp * 2)) +
                  warp * 16 * rw;
  if (kLoShared) {
    const int hw = dp >> 1;  // 32-bit words per row
    const uint32_t* src = reinterpret_cast<const uint32_t*>(A.xl);
    for (int w = lane; w < 16 * hw; w += 32) {
      const int rr = w / hw, c = w - rr * hw;
      qlo[rr * rw + c] = src[static_cast<size_t>(min(q0 + rr, n - 1)) * hw + c];
    }
    __syncwarp();
  }
  // query fragments: rows g and g + 8 of the warp's 16 queries
  uint32_t ah[KS][4], al[kRegLo][4];
  {
    const int ra = min(q0 + g, n - 1), rb = min(q0 + g + 8, n - 1);
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
      uint2 pa = make_uint2(0u, 0u), pb = pa, qa = pa, qb = pa;
      if (ks < ksn) {
        pa = *reinterpret_cast<const uint2*>(A.xh + static_cast<size_t>(ra) * dp + ks * 16 + 4 * tig);
        pb = *reinterpret_cast<const uint2*>(A.xh + static_cast<size_t>(rb) * dp + ks * 16 + 4 * tig);
        if (!kLoShared) {
          qa = *reinterpret_cast<const uint2*>(A.xl + static_cast<size_t>(ra) * dp + ks * 16 + 4 * tig);
          qb = *reinterpret_cast<const uint2*>(A.xl + static_cast<size_t>(rb) * dp + ks * 16 + 4 * tig);
        }
      }
      ah[ks][0] = pa.x; ah[ks][2] = pa.y; ah[ks][1] = pb.x; ah[ks][3] = pb.y;
      if (!kLoShared) {
        al[ks][0] = qa.x; al[ks][2] = qa.y; al[ks][1] = qb.x; al[ks][3] = qb.y;
      }
    }
  }
  const int qa_row = q0 + g, qb_row = q0 + g + 8;
  const float nq_g = A.nrm[min(qa_row, n - 1)], nq_g8 = A.nrm[min(qb_row, n - 1)];
  // the heap this lane owns: query row r, the columns of quad lanes 2 h, 2 h + 1
  const int r = lane & 15, h = lane >> 4, myq = q0 + r;
  // the heaps whose thresholds this lane's fragment values are filtered by
  const int heap_a = g + 16 * (tig >> 1), heap_b = heap_a + 8;
  int cnt = 0;
  float tau = INFINITY;

  // this thread's 16-byte chunks of a tile (the same every tile): smem word
  // offset of the hi chunk and element offset inside the tile's rows
  const int chunks = dp >> 3;
  int ld_smem[kMaxLoads], ld_row[kMaxLoads], ld_col[kMaxLoads], nld = 0;
#pragma unroll
  for (int t = 0; t < kMaxLoads; ++t) {
    const int e = threadIdx.x + t * 32 * kTcWarps;
    ld_row[t] = 0;
    ld_col[t] = 0;
    ld_smem[t] = 0;
    if (!kLoShared && e < kTcN * chunks) {
      const int c = e / chunks, ch = e - c * chunks;
      ld_row[t] = c;
      ld_col[t] = ch * 8;
      ld_smem[t] = c * rw + ch * 4;
      nld = t + 1;
    }
  }
  __syncwarp();

  // scattered tile order: the tile at step k is (first + k * stride) mod ntiles,
  // stride coprime to ntiles (1000003 is a prime above any tile count); this
  // segment takes the steps seg, seg + segs, ...
  const int ntiles = (n + kTcN - 1) / kTcN;
  const int stride = static_cast<int>(1000003ull % static_cast<unsigned long long>(ntiles));
  const int jump = static_cast<int>((static_cast<unsigned long long>(stride) * segs) % ntiles);
  const int first = static_cast<int>((static_cast<unsigned long long>(blockIdx.x) * 7919ull +
                                      static_cast<unsigned long long>(seg) * stride) % ntiles);
  const int nsteps = ntiles > seg ? (ntiles - seg + segs - 1) / segs : 0;

  auto load_tile = [&](int buf, int tile) {
    const int base = tile * kTcN;
    uint32_t* dh = cbuf + (buf * 2 + 0) * kTcN * rw;
    uint32_t* dl = cbuf + (buf * 2 + 1) * kTcN * rw;
    if (kLoShared) {
      for (int e = threadIdx.x; e < kTcN * chunks; e += 32 * kTcWarps) {
        const int c = e / chunks, ch = e - c * chunks;
        const int so = c * rw + ch * 4;
        if (base + c < n) {
          const size_t src = static_cast<size_t>(base + c) * dp + ch * 8;
          cp_async16(dh + so, A.xh + src);
          cp_async16(dl + so, A.xl + src);
        } else {
          *reinterpret_cast<uint4*>(dh + so) = make_uint4(0u, 0u, 0u, 0u);
          *reinterpret_cast<uint4*>(dl + so) = make_uint4(0u, 0u, 0u, 0u);
        }
      }
    }
#pragma unroll
    for (int t = 0; t < kMaxLoads; ++t) {
      if (!kLoShared && t < nld) {
        const int row = base + ld_row[t];
        if (row < n) {
          const size_t src = static_cast<size_t>(row) * dp + ld_col[t];
          cp_async16(dh + ld_smem[t], A.xh + src);
          cp_async16(dl + ld_smem[t], A.xl + src);
        } else {
          *reinterpret_cast<uint4*>(dh + ld_smem[t]) = make_uint4(0u, 0u, 0u, 0u);
          *reinterpret_cast<uint4*>(dl + ld_smem[t]) = make_uint4(0u, 0u, 0u, 0u);
        }
      }
    }
    for (int c = threadIdx.x; c < kTcN; c += 32 * kTcWarps) cnb[buf * kTcN + c] = base + c < n ? A.nrm[base + c] : 0.0f;
    cp_async_commit();
  };

  int tile = first;
  if (nsteps > 0) load_tile(0, tile);
  for (int step = 0; step < nsteps; ++step) {
    const int buf = step & 1;
    const int t0 = tile * kTcN;
    int next = tile + jump;
    if (next >= ntiles) next -= ntiles;
    if (step + 1 < nsteps) {
      load_tile(buf ^ 1, next);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const uint32_t* th = cbuf + (buf * 2 + 0) * kTcN * rw;
    const uint32_t* tl = cbuf + (buf * 2 + 1) * kTcN * rw;
    const float* cn = cnb + buf * kTcN;
    // only the last tile and the tiles holding this warp's queries need the
    // column checks (past the end, the query itself)
    const bool edge = t0 + kTcN > n || (t0 < q0 + 16 && q0 < t0 + kTcN) || q0 + 16 > n;
    const float tau_a = htau[heap_a], tau_b = htau[heap_b];
    unsigned fa = 0u, fb = 0u;  // bit 2 nt + c: column nt * 8 + 2 tig + c of rows g / g + 8
    // eight independent accumulator chains (one per n-tile) hide the mma latency
    float accs[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) accs[nt][0] = accs[nt][1] = accs[nt][2] = accs[nt][3] = 0.0f;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
      if (ks < ksn) {
        uint32_t lo[4];
        if (kLoShared) {
          const uint2 la = *reinterpret_cast<const uint2*>(qlo + g * rw + ks * 8 + 2 * tig);
          const uint2 lb = *reinterpret_cast<const uint2*>(qlo + (g + 8) * rw + ks * 8 + 2 * tig);
          lo[0] = la.x; lo[2] = la.y; lo[1] = lb.x; lo[3] = lb.y;
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i) lo[i] = al[kLoShared ? 0 : ks][i];
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const int off = (nt * 8 + g) * rw + ks * 8 + 2 * tig;
          const uint2 bh = *reinterpret_cast<const uint2*>(th + off);
          const uint2 bl = *reinterpret_cast<const uint2*>(tl + off);
          mma16816(accs[nt], ah[ks], bh);
          mma16816(accs[nt], ah[ks], bl);
          mma16816(accs[nt], lo, bh);
        }
      }
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const float* acc = accs[nt];
      const int col = nt * 8 + 2 * tig;
      const float c0 = cn[col], c1 = cn[col + 1];
      const float v0 = nq_g + c0 - 2.0f * acc[0], v1 = nq_g + c1 - 2.0f * acc[1];
      const float v2 = nq_g8 + c0 - 2.0f * acc[2], v3 = nq_g8 + c1 - 2.0f * acc[3];
      bool f0 = v0 < tau_a, f1 = v1 < tau_a, f2 = v2 < tau_b, f3 = v3 < tau_b;
      if (edge) {
        const int j0 = t0 + col, j1 = j0 + 1;
        f0 = f0 && j0 < n && j0 != qa_row && qa_row < n;
        f1 = f1 && j1 < n && j1 != qa_row && qa_row < n;
        f2 = f2 && j0 < n && j0 != qb_row && qb_row < n;
        f3 = f3 && j1 < n && j1 != qb_row && qb_row < n;
      }
      fa |= (static_cast<unsigned>(f0) | (static_cast<unsigned>(f1) << 1)) << (2 * nt);
      fb |= (static_cast<unsigned>(f2) | (static_cast<unsigned>(f3) << 1)) << (2 * nt);
      if (f0 | f1) *reinterpret_cast<float2*>(dt + g * kTileStride + col) = make_float2(v0, v1);
      if (f2 | f3) *reinterpret_cast<float2*>(dt + (g + 8) * kTileStride + col) = make_float2(v2, v3);
    }
    fmask[g * 4 + tig] = fa;
    fmask[(g + 8) * 4 + tig] = fb;
    __syncwarp();
    // the owner of each heap inserts its flagged values: 16 bits per quad lane,
    // quad lanes 2 h and 2 h + 1 feed heap (r, h)
    unsigned m = fmask[r * 4 + 2 * h] | (fmask[r * 4 + 2 * h + 1] << 16);
    while (m != 0u) {
      const int b = __ffs(m) - 1;
      m &= m - 1u;
      const int qt = 2 * h + (b >> 4), bb = b & 15;
      const int col = (bb >> 1) * 8 + 2 * qt + (bb & 1);
      const float v = dt[r * kTileStride + col];
      if (!(v < tau)) continue;
      const int j = t0 + col;
      if (cnt < kp) {
        // push: sift up
        int c = cnt++;
        while (c > 0) {
          const int p = (c - 1) >> 1;
          const float pv = hv[p * 32 + lane];
          if (!(pv < v)) break;
          hv[c * 32 + lane] = pv;
          hj[c * 32 + lane] = hj[p * 32 + lane];
          c = p;
        }
        hv[c * 32 + lane] = v;
        hj[c * 32 + lane] = j;
        if (cnt == kp) tau = hv[lane];
      } else {
        // replace the maximum: sift down
        int c = 0;
        for (;;) {
          const int l = 2 * c + 1;
          if (l >= kp) break;
          int big = l;
          float bv = hv[l * 32 + lane];
          if (l + 1 < kp) {
            const float rv = hv[(l + 1) * 32 + lane];
            if (rv > bv) {
              big = l + 1;
              bv = rv;
            }
          }
          if (!(bv > v)) break;
          hv[c * 32 + lane] = bv;
          hj[c * 32 + lane] = hj[big * 32 + lane];
          c = big;
        }
        hv[c * 32 + lane] = v;
        hj[c * 32 + lane] = j;
        tau = hv[lane];
      }
    }
    htau[lane] = tau;
    tile = next;
    __syncthreads();
  }
  // heaps out; the bound is the smaller final threshold of the row's two heaps
  const float mine = cnt == kp ? tau : INFINITY;
  const float other = __shfl_xor_sync(0xffffffffu, mine, 16);
  if (myq < n) {
    const size_t base = ((static_cast<size_t>(myq) * segs + seg) * 2 + h) * kp;
    for (int e = 0; e < kp; ++e) {
      A.cand[base + e] = e < cnt ? hj[e * 32 + lane] : -1;
      A.cand_a[base + e] = e < cnt ? hv[e * 32 + lane] : INFINITY;
    }
    if (h == 0) A.bound[static_cast<size_t>(myq) * segs + seg] = fminf(mine, other);
  }
}

// order-preserving image of a float as an unsigned
__device__ __forceinline__ unsigned ord_float(float v) {
  const unsigned u = __float_as_uint(v);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// One warp per query: A_K (the K-th smallest approximate distance of its
// m = segs x 2 x kp candidates), canonical distances of the candidates with
// a <= A_K + 2 delta, the K smallest of those by (distance, index), and the
// certificate B > A_K + 2 delta (every row goes to the fallback list when the
// data hold a non-finite value).
__global__ void tc_rerank_kernel(const float* __restrict__ x, int n, int d, int K, int m, int segs,
                                 const int* __restrict__ cand, const float* __restrict__ cand_a,
                                 const float* __restrict__ bound, const float* __restrict__ nrm,
                                 const unsigned* __restrict__ nrm_max, const int* __restrict__ nonfinite,
                                 float crel, int* __restrict__ idx, float* __restrict__ dist,
                                 int* __restrict__ fb_rows, int* __restrict__ fb_count) {
  const int lane = threadIdx.x & 31;
  const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= n) return;
  if (*nonfinite) {
    if (lane == 0) fb_rows[atomicAdd(fb_count, 1)] = q;
    return;
  }
  float av[kMaxPer];
  int jv[kMaxPer];
  unsigned long long key[kMaxPer];
#pragma unroll
  for (int t = 0; t < kMaxPer; ++t) {
    const int e = lane + 32 * t;
    av[t] = INFINITY;
    jv[t] = -1;
    if (e < m) {
      const int j = cand[static_cast<size_t>(q) * m + e];
      if (j >= 0) {
        jv[t] = j;
        av[t] = cand_a[static_cast<size_t>(q) * m + e];
      }
    }
  }
  float thr = INFINITY;
  {
    // A_K: the approximate distance of the K-th smallest (a, row) key
    unsigned long long k2[kMaxPer];
#pragma unroll
    for (int t = 0; t < kMaxPer; ++t)
      k2[t] = jv[t] >= 0 ? (static_cast<unsigned long long>(ord_float(av[t])) << 32) | static_cast<unsigned>(jv[t])
                         : ~0ull;
    unsigned long long kth = ~0ull;
    for (int o = 0; o < K; ++o) {
      unsigned long long best = k2[0];
#pragma unroll
      for (int t = 1; t < kMaxPer; ++t) best = k2[t] < best ? k2[t] : best;
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, s);
        best = other < best ? other : best;
      }
      kth = best;
      if (best == ~0ull) break;
#pragma unroll
      for (int t = 0; t < kMaxPer; ++t)
        if (k2[t] == best) k2[t] = ~0ull;
    }
    if (kth != ~0ull) {
      const unsigned o = static_cast<unsigned>(kth >> 32);
      thr = __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
    }
  }
  const float delta = (nrm[q] + __uint_as_float(*nrm_max)) * crel;
  const float limit = thr + 2.0f * delta;
  const float* xq = x + static_cast<size_t>(q) * d;
  // canonical distances of the candidates within the limit
#pragma unroll
  for (int t = 0; t < kMaxPer; ++t) {
    key[t] = ~0ull;
    if (jv[t] >= 0 && av[t] <= limit) {
      const float* xj = x + static_cast<size_t>(jv[t]) * d;
      float a = 0.0f;
      for (int k = 0; k < d; ++k) {
        const float diff = __fsub_rn(xq[k], xj[k]);
        a = __fadd_rn(a, __fmul_rn(diff, diff));
      }
      // canonical distances are >= 0: their bit patterns order like the values
      key[t] = (static_cast<unsigned long long>(__float_as_uint(a)) << 32) | static_cast<unsigned>(jv[t]);
    }
  }
  for (int o = 0; o < K; ++o) {
    unsigned long long best = key[0];
#pragma unroll
    for (int t = 1; t < kMaxPer; ++t) best = key[t] < best ? key[t] : best;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, s);
      best = other < best ? other : best;
    }
#pragma unroll
    for (int t = 0; t < kMaxPer; ++t)
      if (key[t] == best) key[t] = ~0ull;
    if (lane == 0) {
      const size_t out = static_cast<size_t>(q) * K + o;
      if (best == ~0ull) {
        idx[out] = -1;
        dist[out] = INFINITY;
      } else {
        idx[out] = static_cast<int>(best & 0xffffffffu);
        dist[out] = __fsqrt_rn(__uint_as_float(static_cast<unsigned>(best >> 32)));
      }
    }
  }
  if (lane == 0) {
    float B = INFINITY;
    for (int s = 0; s < segs; ++s) B = fminf(B, bound[static_cast<size_t>(q) * segs + s]);
    if (!(B > limit)) fb_rows[atomicAdd(fb_count, 1)] = q;
  }
}

}  // namespace

// Segments and heap size: the K nearest rows spread over segs x 2 heaps,
// each heap holding about twice its expected share plus a margin.
void tc_shape(int K, int* segs, int* kp) {
  *segs = K <= 40 ? 8 : 4;
  const int share = (K + 2 * *segs - 1) / (2 * *segs);
  int k = (2 * share + 8 + 7) / 8 * 8;
  k = k < 16 ? 16 : k;
  const int cap = kMaxPer * 32 / (2 * *segs);
  *kp = k > cap ? cap : k;
}

int bf16_split_rows(const float* x, int n, int d, int dp, uint16_t* xh, uint16_t* xl, cudaStream_t st) {
  const size_t total = static_cast<size_t>(n) * dp;
  if (total == 0) return 0;
  split_rows_kernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, st>>>(x, n, d, dp, xh, xl);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

bool knn_tc_supported(int n, int d, int K) {
  int segs = 0, kp = 0;
  tc_shape(K, &segs, &kp);
  if (!(d >= 1 && d <= 16 * kTcMaxKs && K >= 1 && K <= 96 && n > 2 * kp + kTcN)) return false;
  const int dp = (d + 15) / 16 * 16, half = dp / 2;
  const int rw = (half % 16 == 8) ? half : half + 8;
  return tc_smem_bytes(rw, kp, dp) <= kTcSmemLimit;
}

namespace {

struct TcLayout {
  int dp, kp, segs, rw;
  size_t o_xh, o_xl, o_nrm, o_flags, o_cand, o_canda, o_bound, o_fb, o_brute, total;
};

TcLayout tc_layout(int n, int d, int K, int segments) {
  TcLayout L{};
  L.dp = (d + 15) / 16 * 16;
  tc_shape(K, &L.segs, &L.kp);
  const int half = L.dp / 2;
  L.rw = (half % 16 == 8) ? half : half + 8;
  const size_t m = static_cast<size_t>(L.segs) * 2 * L.kp;
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  size_t o = 0;
  L.o_xh = o; o = al(o + static_cast<size_t>(n) * L.dp * 2);
  L.o_xl = o; o = al(o + static_cast<size_t>(n) * L.dp * 2);
  L.o_nrm = o; o = al(o + static_cast<size_t>(n) * 4);
  L.o_flags = o; o = al(o + 16);  // nrm_max, nonfinite, fb_count
  L.o_cand = o; o = al(o + static_cast<size_t>(n) * m * 4);
  L.o_canda = o; o = al(o + static_cast<size_t>(n) * m * 4);
  L.o_bound = o; o = al(o + static_cast<size_t>(n) * L.segs * 4);
  L.o_fb = o; o = al(o + static_cast<size_t>(n) * 4);
  L.o_brute = o; o = al(o + knn_bruteforce_scratch(n, K, segments));
  L.total = o;
  return L;
}

}  // namespace

size_t knn_tc_scratch(int n, int d, int K, int segments) { return tc_layout(n, d, K, segments).total; }

int knn_tc_graph(const float* x, int n, int d, int K, int segments, void* scratch, int* idx, float* dist,
                 cudaStream_t st) {
  const TcLayout L = tc_layout(n, d, K, segments);
  unsigned char* b = static_cast<unsigned char*>(scratch);
  uint16_t* xh = reinterpret_cast<uint16_t*>(b + L.o_xh);
  uint16_t* xl = reinterpret_cast<uint16_t*>(b + L.o_xl);
  float* nrm = reinterpret_cast<float*>(b + L.o_nrm);
  unsigned* flags = reinterpret_cast<unsigned*>(b + L.o_flags);  // [0] nrm_max bits, [1] nonfinite, [2] fallback count
  int* cand = reinterpret_cast<int*>(b + L.o_cand);
  float* cand_a = reinterpret_cast<float*>(b + L.o_canda);
  float* bound = reinterpret_cast<float*>(b + L.o_bound);
  int* fb = reinterpret_cast<int*>(b + L.o_fb);
  cudaError_t e = cudaMemsetAsync(flags, 0, 16, st);
  if (e != cudaSuccess) return static_cast<int>(e);
  tc_prep_kernel<<<(n + 127) / 128, 128, 0, st>>>(x, n, d, L.dp, xh, xl, nrm, flags,
                                                 reinterpret_cast<int*>(flags + 1));
  TcArgs A{};
  A.xh = xh;
  A.xl = xl;
  A.nrm = nrm;
  A.n = n;
  A.dp = L.dp;
  A.kp = L.kp;
  A.segs = L.segs;
  A.row_words = L.rw;
  A.cand = cand;
  A.cand_a = cand_a;
  A.bound = bound;
  const size_t smem = tc_smem_bytes(L.rw, L.kp, L.dp);
  const dim3 grid((n + kTcQ - 1) / kTcQ, L.segs);
  if (L.dp <= 64) {
    e = cudaFuncSetAttribute(tc_candidates_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
    tc_candidates_kernel<4><<<grid, 32 * kTcWarps, smem, st>>>(A);
  } else if (L.dp <= 16 * kTcRegKs) {
    e = cudaFuncSetAttribute(tc_candidates_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
    tc_candidates_kernel<8><<<grid, 32 * kTcWarps, smem, st>>>(A);
  } else {
    e = cudaFuncSetAttribute(tc_candidates_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
    tc_candidates_kernel<16><<<grid, 32 * kTcWarps, smem, st>>>(A);
  }
  const float crel = 1e-4f + 2e-6f * static_cast<float>(L.dp);
  tc_rerank_kernel<<<(n + 3) / 4, 128, 0, st>>>(x, n, d, K, L.segs * 2 * L.kp, L.segs, cand, cand_a, bound, nrm,
                                                 flags, reinterpret_cast<const int*>(flags + 1), crel, idx, dist, fb,
                                                 reinterpret_cast<int*>(flags + 2));
  count_launch(3);
  e = cudaGetLastError();
  if (e != cudaSuccess) return static_cast<int>(e);
  return knn_bruteforce_rows(x, n, d, K, segments, fb, reinterpret_cast<const int*>(flags + 2), b + L.o_brute, idx,
                             dist, st);
}

int knn_tc_fallback_count(const void* scratch, int n, int d, int K, int segments, int* out, cudaStream_t st) {
  const TcLayout L = tc_layout(n, d, K, segments);
  const unsigned char* b = static_cast<const unsigned char*>(scratch);
  return static_cast<int>(cudaMemcpyAsync(out, b + L.o_flags + 8, sizeof(int), cudaMemcpyDeviceToHost, st));
}

}  // namespace kgb
