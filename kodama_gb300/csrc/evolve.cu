// Persistent label-evolution kernel: every problem (KODAMA.matrix run, or
// CoreKNNGraph call) runs all of its Tcycle perturb / vote / score / accept
// steps inside one CTA, in one launch, with the labels resident in shared
// memory and the fold-filtered neighbour table streamed from HBM/L2.
//
// It restates maximize_core (core.cpp:1269-1549) with the precomputed-kNN
// predictor predict_precomputed_knn (core.cpp:784-914) and the training-fold
// fallbacks (core.cpp:274-309):
//   proposal size   sample_proposal_group_count  core.cpp:1228-1254
//   group shuffle   std::shuffle of the group ids core.cpp:1363-1365
//   relabel         prediction-guided draw        core.cpp:1384-1419
//   absorption      propose_many_to_one_absorption core.cpp:1110-1226
//   score           core_objective_score          core.cpp:916-972
//   accept          greedy / annealed              core.cpp:1471-1508
// Labels are carried as 16-bit codes: the rank of the label among the sorted
// distinct initial labels, so every label comparison of the reference (ties to
// the smaller label, ordered maps) is a code comparison.
//
// Exactness: all double arithmetic uses explicit round-to-nearest intrinsics
// (no contraction), random draws follow rng.cuh, and the unordered_map
// iteration order that fixes the summation order of the diversity term is
// reproduced (reverse first-insertion order, bucket runs on collisions).
#include "evolve.cuh"
#include "launch_count.cuh"
#include "rng.cuh"
#include "crmath.cuh"
#include "mlp.cuh"

#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

namespace kgb {

namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kRowArrays = 8;  // cl, cur, curpred, pred/perm, J, list, 2 x (32-bit scratch)

struct Fixed {
  Mt64State rng;
  uint64_t mt_alt[kMtN];  // the engine state's second buffer (produce_outputs_group)
  int first_reject;
  int i0;
  int ns;
  int red_i[kWarps];
  int flag;
  int nc;          // distinct labels of the proposal
  int changed_cnt;  // dirty_rows_block: rows whose label changed
  int dirty_cnt;    // dirty_rows_block: rows listed for the vote
  int moves_sel;
  int n_empty;
  int selected_target;
  int rev_total;   // this problem's reverse-neighbour entries (rev_off[L])
  double acc;
  double score;
  int accept;
  int improves;
  // this problem's groups and fixed flags (bind_groups)
  const int* goff;
  const int* gmem;
  const int* fxd;
  int G;
  // learned proposal: candidate count and radix-select state
  int sel_count;
  int sel_digit;
  int sel_need;
  int sel_hist[256];
};

struct Smem {
  Fixed* f;
  uint16_t* cl;      // proposal
  uint16_t* cur;     // current state (evolutionary) or best state (greedy)
  uint16_t* curpred; // CV predictions of cur
  uint16_t* pred;    // CV predictions of the proposal
  uint16_t* perm;    // shuffled group ids (first ns positions; aliases pred during the shuffle)
  uint16_t* jarr;    // swap target of every shuffle step
  uint16_t* list;    // shuffle steps bucketed by swap target
  int* scratch32;    // per-position counts / bucket offsets
  int* trans;        // class x prediction counts (shared or global)
  uint64_t* raw;     // engine outputs of one shuffle (global scratch)
  int* cnt;          // per code: count in proposal
  int* firstpos;     // per code: first row
  int* movable;      // per code: non-fixed rows
  int* order;        // per code: unordered_map iteration order / scratch
  int* bt;           // per code: absorption target (-1 none)
  int* aux;          // per code: scratch counts
  double* bsur;      // per code: absorption surplus
  double* weight;    // per code: per-target weight / discrete weights
  double* cp;        // discrete cumulative scratch
};

__device__ __forceinline__ size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

__device__ int block_sum(int v, Fixed& f) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = __reduce_add_sync(kFull, v);
  if (lane == 0) f.red_i[warp] = v;
  __syncthreads();
  int t = 0;
  if (threadIdx.x < 32) {
    t = f.red_i[threadIdx.x];
    t = __reduce_add_sync(kFull, t);
  }
  __syncthreads();
  if (threadIdx.x == 0) f.red_i[0] = t;
  __syncthreads();
  const int out = f.red_i[0];
  __syncthreads();
  return out;
}

// ---------------------------------------------------------------------------
// Group shuffle (std::shuffle of iota(G) with a 64-bit engine).  For an engine
// range wider than G^2 the draws come two at a time: one downscaled draw over
// (i+1)*(i+2) gives the swap targets of positions i and i+1 (quotient and
// remainder by i+2); an even G first swaps position 1 with a draw over {0,1}.
//
// Only the groups at positions [0, ns) are used, so the permutation is not
// materialised serially.  Step i (swap of positions i and J[i] <= i) moves
// group i, which is still at position i, to J[i].  Hence the final occupant of
// position q is the last step i > q with J[i] == q if there is one; otherwise
// it is whatever step q pulled into position q, i.e. the occupant of position
// J[q] just before step q (q itself when J[q] == q; 0 for position 0).  The
// CTA computes all J[i] in parallel from the engine blocks, buckets the steps
// by target, and walks each wanted position down this chain.
// ---------------------------------------------------------------------------
// Exclusive prefix sum of a[0..n) in place (block-wide).
__device__ void block_exclusive_scan(int* a, int n, Fixed& f) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int chunk = (n + kThreads - 1) / kThreads;
  const int b = threadIdx.x * chunk, e = min(n, b + chunk);
  int local = 0;
  for (int i = b; i < e; ++i) local += a[i];
  int incl = local;
  for (int off = 1; off < 32; off <<= 1) {
    const int v = __shfl_up_sync(kFull, incl, off);
    if (lane >= off) incl += v;
  }
  if (lane == 31) f.red_i[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = f.red_i[lane];
    for (int off = 1; off < 32; off <<= 1) {
      const int v = __shfl_up_sync(kFull, w, off);
      if (lane >= off) w += v;
    }
    f.red_i[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  int run = (warp > 0 ? f.red_i[warp - 1] : 0) + incl - local;
  for (int i = b; i < e; ++i) {
    const int v = a[i];
    a[i] = run;
    run += v;
  }
  __syncthreads();
}

// Engine producer group: the first 160 threads (warps 0-4) synchronised by
// named barrier 1.
constexpr int kProducerThreads = 160;
__device__ __forceinline__ void producer_sync() { asm volatile("bar.sync 1, 160;" ::: "memory"); }

// Copy the next `count` engine outputs into raw[start..] (producer group).
// The outputs left in g.out are copied first; every whole block of 312 that
// follows is regenerated with its tempered words written straight into raw
// (g.out is only refreshed for the last block, whose tail later draws read).
// A regeneration reads the old state words from one buffer and writes the new
// ones to the other (g.mt and alt in turn), so one barrier separates
// regenerations: thread t < 156 forms word t from old words t, t + 1, t + 156
// and then word t + 156 from old words t + 156, t + 157 and its own new word t
// (word 311 takes the new word 0, which thread 155 forms again itself).
__device__ void produce_outputs_group(Mt64State& g, uint64_t* alt, uint64_t* raw, int start, int count, int t) {
  const int pos0 = g.pos;
  const int lead = min(kMtN - pos0, count);
  for (int i = t; i < lead; i += kProducerThreads) raw[start + i] = g.out[pos0 + i];
  int done = lead;
  int pos = pos0 + lead;
  uint64_t* cur = g.mt;
  uint64_t* nxt = alt;
  while (done < count) {
    const int take = min(kMtN, count - done);
    if (t < kMtN - kMtM) {
      const int h = t + kMtM;
      const uint64_t lo = mt64_mix(cur[t], cur[t + 1], cur[h]);
      const uint64_t hi = h < kMtN - 1 ? mt64_mix(cur[h], cur[h + 1], lo)
                                       : mt64_mix(cur[h], mt64_mix(cur[0], cur[1], cur[kMtM]), lo);
      nxt[t] = lo;
      nxt[h] = hi;
      const uint64_t tl = mt64_temper(lo), th = mt64_temper(hi);
      if (t < take) raw[start + done + t] = tl;
      if (h < take) raw[start + done + h] = th;
      if (take < kMtN) {
        g.out[t] = tl;
        g.out[h] = th;
      }
    }
    // the next regeneration reads what this one wrote and overwrites what it read
    producer_sync();
    uint64_t* const tmp = cur;
    cur = nxt;
    nxt = tmp;
    done += take;
    pos = take;
  }
  if (cur != g.mt) {
    for (int k = t; k < kMtN; k += kProducerThreads) g.mt[k] = cur[k];
  }
  if (t == 0) g.pos = pos;
  producer_sync();
}

// Swap targets J[i] of every step of the shuffle of G groups.  The producer
// group streams the engine outputs the pair draws consume into `raw`; the whole CTA then
// downscales them in parallel.  A rejected draw (Lemire resampling, about one
// in 2^64/G^2) shifts every later pair by one output: the pairs from the
// rejection on are redone with the next output appended.
__device__ void shuffle_targets_block(Fixed& f, uint16_t* J, int G, uint64_t* raw) {
  if (threadIdx.x == 0) {
    f.i0 = 1;
    if (G >= 2 && (G & 1) == 0) {
      J[1] = static_cast<uint16_t>(draw_below_serial(f.rng, 2));
      f.i0 = 2;
    }
  }
  __syncthreads();
  const int i0 = f.i0;
  const int npairs = (G - i0) >> 1;
  if (npairs <= 0) return;
  if (threadIdx.x < kProducerThreads) produce_outputs_group(f.rng, f.mt_alt, raw, 0, npairs, threadIdx.x);
  __syncthreads();
  int from = 0, shift = 0;
  for (;;) {
    if (threadIdx.x == 0) f.first_reject = npairs;
    __syncthreads();
    for (int p = from + threadIdx.x; p < npairs; p += kThreads) {
      const uint64_t b0 = static_cast<uint64_t>(i0 + 2 * p) + 1ull;
      const uint64_t b1 = b0 + 1ull;
      const uint64_t range = b0 * b1;
      const uint64_t u = raw[p + shift];
      const uint64_t lo = u * range;
      if (lo < range && lo < (0ull - range) % range) {
        atomicMin(&f.first_reject, p);
      } else {
        // x < (G-1)*G < 2^32 for G <= 65535: 32-bit quotient and remainder
        const uint32_t x = static_cast<uint32_t>(__umul64hi(u, range));
        const uint32_t d1 = static_cast<uint32_t>(b1);
        const uint32_t qv = x / d1;
        J[i0 + 2 * p] = static_cast<uint16_t>(qv);
        J[i0 + 2 * p + 1] = static_cast<uint16_t>(x - qv * d1);
      }
    }
    __syncthreads();
    const int r = f.first_reject;
    if (r >= npairs) break;
    // the output at r + shift was rejected: pairs r.. use one output later
    if (threadIdx.x < kProducerThreads) produce_outputs_group(f.rng, f.mt_alt, raw, npairs + shift, 1, threadIdx.x);
    ++shift;
    from = r;
    __syncthreads();
  }
}

// Bucket the steps by swap target, for the targets below lim (the used
// positions [0, ns)): afterwards cnt[q] is the end of bucket q in `list` and
// the start of bucket q+1.  A group only moves to higher positions (a later
// step targeting its position p sits at a position above p), so walks that
// decide membership of [0, lim) never need a bucket at or above lim.
__device__ void bucket_steps_block(const Smem& s, int G, int lim) {
  const uint16_t* J = s.jarr;
  int* cnt = s.scratch32;
  uint16_t* list = s.list;
  for (int q = threadIdx.x; q < lim; q += kThreads) cnt[q] = 0;
  __syncthreads();
  for (int st = 1 + threadIdx.x; st < G; st += kThreads)
    if (J[st] < lim) atomicAdd(&cnt[J[st]], 1);
  __syncthreads();
  block_exclusive_scan(cnt, lim, *s.f);
  for (int st = 1 + threadIdx.x; st < G; st += kThreads) {
    if (J[st] >= lim) continue;
    const int slot = atomicAdd(&cnt[J[st]], 1);
    list[slot] = static_cast<uint16_t>(st);
  }
  __syncthreads();
}

// Group at final position p: last step > q targeting q, else what step q
// pulled into q (see above).
__device__ int occupant_of(const Smem& s, int G, int p) {
  const uint16_t* J = s.jarr;
  const int* cnt = s.scratch32;
  int q = p, t = G - 1;
  for (;;) {
    const int b = q > 0 ? cnt[q - 1] : 0, e = cnt[q];
    int best = -1;
    for (int k = b; k < e; ++k) {
      const int st = s.list[k];
      if (st > q && st <= t && st > best) best = st;
    }
    if (best >= 0) return best;
    if (q == 0) return 0;
    const int jq = J[q];
    if (jq == q) return q;
    t = q - 1;
    q = jq;
  }
}

// Final position of group e: it lands on J[e] at step e (group 0 starts at
// 0), then every later step targeting its position moves it to that step's
// own position.  Positions only grow, so once the position reaches lim (the
// buckets' limit) the walk stops and returns that position, which is enough
// for a `< lim` test.
__device__ int final_position_of(const Smem& s, int e, int lim) {
  const int* cnt = s.scratch32;
  int pos = e == 0 ? 0 : s.jarr[e];
  int time = e;
  for (;;) {
    if (pos >= lim) return pos;
    const int b = pos > 0 ? cnt[pos - 1] : 0, en = cnt[pos];
    int next = 0x7fffffff;
    for (int k = b; k < en; ++k) {
      const int st = s.list[k];
      if (st > time && st < next) next = st;
    }
    if (next == 0x7fffffff) return pos;
    pos = next;
    time = next;
  }
}

// ---------------------------------------------------------------------------
// Tie-break of a vote among the labels reaching the top count `maxc`
// (`tied`: one lane per such label).  The larger double score sum wins, then
// the smaller code.  With |s| = mant * 2^ex, if the non-zero magnitudes of the
// row span at most 24 binades every sequential double partial sum of <= 32 of
// them is exact, so when all scores share a sign (-(d*d) <= 0 for squared L2,
// inner products >= 0 among near neighbours) exact integer sums of the
// magnitudes order the tied labels exactly as the reference's double sums do
// (smaller magnitude first for non-positive scores, larger for non-negative);
// otherwise the double sums are formed in neighbour order.
// ---------------------------------------------------------------------------
__device__ __noinline__ int vote_tiebreak(int code, unsigned tied, const float* scrow, int w, int lane) {
  const float my = lane < w ? scrow[lane] : 0.0f;
  const uint32_t bits = __float_as_uint(my);
  const uint32_t ef = (bits >> 23) & 0xffu;
  const uint32_t mant = ef ? ((bits & 0x7fffffu) | 0x800000u) : (bits & 0x7fffffu);
  const int ex = ef ? static_cast<int>(ef) - 150 : -149;
  const bool live = code >= 0 && mant != 0u;
  const bool bad = code >= 0 && ef == 0xffu;
  const int emin = __reduce_min_sync(kFull, live ? ex : 0x7fffffff);
  const int emax = __reduce_max_sync(kFull, live ? ex : -0x7fffffff);
  const bool any_neg = __any_sync(kFull, live && (bits >> 31) != 0u);
  const bool any_pos = __any_sync(kFull, live && (bits >> 31) == 0u);
  const bool exact_ok = !__any_sync(kFull, bad) && !(any_neg && any_pos) &&
                        (emin == 0x7fffffff || emax - emin <= 24);
  uint32_t p0 = 0, p1 = 0, p2 = 0;
  if (exact_ok && live) {
    const uint64_t contrib = static_cast<uint64_t>(mant) << (ex - emin);
    p0 = static_cast<uint32_t>(contrib & 0x1fffffu);
    p1 = static_cast<uint32_t>((contrib >> 21) & 0x1fffffu);
    p2 = static_cast<uint32_t>(contrib >> 42);
  }
  uint64_t bmag = any_pos ? 0ull : ~0ull;
  double bsum = -INFINITY;
  int bc = 0x7fffffff;
  unsigned rem = tied;
  while (rem) {
    const int ld = __ffs(rem) - 1;
    rem &= rem - 1;
    const int v = __shfl_sync(kFull, code, ld);
    const bool in = code == v;
    if (exact_ok) {
      const uint64_t s0 = __reduce_add_sync(kFull, in ? p0 : 0u);
      const uint64_t s1 = __reduce_add_sync(kFull, in ? p1 : 0u);
      const uint64_t s2 = __reduce_add_sync(kFull, in ? p2 : 0u);
      const uint64_t mag = s0 + (s1 << 21) + (s2 << 42);
      if ((any_pos ? mag > bmag : mag < bmag) || (mag == bmag && v < bc)) {
        bmag = mag;
        bc = v;
      }
    } else {
      const unsigned msk = __ballot_sync(kFull, in);
      double sum = 0.0;
      for (int t = 0; t < w; ++t) {
        const float st = __shfl_sync(kFull, my, t);
        if ((msk >> t) & 1u) sum = __dadd_rn(sum, static_cast<double>(st));
      }
      if (sum > bsum || (sum == bsum && v < bc)) {
        bsum = sum;
        bc = v;
      }
    }
  }
  return bc;
}

// Fold votes of R rows by one warp (lane j holds neighbour slot j of every
// row).  Lanes holding the same label find each other with __match_any_sync,
// so a label's count is a popcount; winner: largest count, then (tie-break)
// largest double score sum, then the smallest code.  The R rows' steps are
// interleaved so their latencies overlap.  out[q] = -1 for a row without
// valid neighbours.
template <int R>
__device__ __forceinline__ void vote_rows_match(const uint16_t* lab, const uint16_t* id, const float* const* sc, int w,
                                                int lane, int* out) {
  int c[R], cnt[R], mx[R], best[R];
  unsigned m[R], tied[R];
#pragma unroll
  for (int q = 0; q < R; ++q) c[q] = id[q] != kNoRow ? static_cast<int>(lab[id[q]]) : -1;
#pragma unroll
  for (int q = 0; q < R; ++q) m[q] = __match_any_sync(kFull, c[q]);
#pragma unroll
  for (int q = 0; q < R; ++q) cnt[q] = c[q] >= 0 ? __popc(m[q]) : 0;
#pragma unroll
  for (int q = 0; q < R; ++q) mx[q] = __reduce_max_sync(kFull, cnt[q]);
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const bool top = c[q] >= 0 && cnt[q] == mx[q];
    best[q] = static_cast<int>(__reduce_min_sync(kFull, top ? static_cast<unsigned>(c[q]) : 0xffffffffu));
    // one lane (the lowest) per label reaching the top count
    tied[q] = __ballot_sync(kFull, top && (__ffs(m[q]) - 1) == lane);
  }
#pragma unroll
  for (int q = 0; q < R; ++q)
    out[q] = mx[q] == 0 ? -1 : (__popc(tied[q]) == 1 ? best[q] : vote_tiebreak(c[q], tied[q], sc[q], w, lane));
}

// Rows with no out-of-fold neighbour take the majority label of their
// training folds (ties to the smaller code); kept out of line, as it is rare.
__device__ __noinline__ void vote_empty_rows(const EvolveParams& P, const Smem& s, int prob, const uint16_t* lab,
                                             uint16_t* out, int C0) {
  const int L = P.L, w = P.w;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint16_t* nbp = P.nb + static_cast<size_t>(prob) * L * w;
  // per-fold training majority (codes in [0, C0)).  The fold x code counts
  // sit in s.scratch32 (L ints, free during the vote) when they fit, else in
  // global memory.
  const int F = P.F;
  const bool in_smem = static_cast<long long>(F) * C0 <= L;
  int* fc = in_smem ? s.scratch32 : P.foldcnt + static_cast<size_t>(prob) * F * P.C0max;
  const int stride = in_smem ? C0 : P.C0max;
  for (int i = threadIdx.x; i < F * stride; i += kThreads) fc[i] = 0;
  for (int c = threadIdx.x; c < C0; c += kThreads) s.aux[c] = 0;
  __syncthreads();
  const uint8_t* fo = P.folds + static_cast<size_t>(prob) * L;
  for (int r = threadIdx.x; r < L; r += kThreads) {
    atomicAdd(&fc[fo[r] * stride + lab[r]], 1);
    atomicAdd(&s.aux[lab[r]], 1);
  }
  __syncthreads();
  // one warp per fold, its lanes over the codes: the largest training count,
  // ties to the smaller code (the reference scans the codes in ascending
  // order keeping strict improvements)
  for (int fo_i = warp; fo_i < F; fo_i += kWarps) {
    int bl = 0x7fffffff, bcount = -1;
    for (int c = lane; c < C0; c += 32) {
      const int cnt = s.aux[c] - fc[fo_i * stride + c];
      if (cnt > bcount) {
        bl = c;
        bcount = cnt;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const int oc = __shfl_xor_sync(kFull, bcount, o), ol = __shfl_xor_sync(kFull, bl, o);
      if (oc > bcount || (oc == bcount && ol < bl)) {
        bcount = oc;
        bl = ol;
      }
    }
    if (lane == 0) s.order[fo_i] = bl;  // order[] is free here; F <= C0max guaranteed by host
  }
  __syncthreads();
  for (int r = threadIdx.x; r < L; r += kThreads) {
    if (nbp[static_cast<size_t>(r) * w] == kNoRow) out[r] = static_cast<uint16_t>(s.order[fo[r]]);
  }
}

// Rows per warp batch of the vote (a multiple of kVoteRows): the batch loop
// is unrolled, so this also sets how many copies of the vote code the kernel
// carries.
constexpr int kVoteBatch = 8;
constexpr int kVoteRows = 4;

// Vote rows into `out`: every row (rows == nullptr) or the nrows rows listed
// in `rows` (the caller has filled the others).  Rows with no out-of-fold
// neighbour take the majority label of their training folds (ties to the
// smaller label).  Neighbour ids are fetched 8 rows at a time per warp so the
// memory latency is paid once per batch; scores only for tied rows.
__device__ void vote_block(const EvolveParams& P, const Smem& s, int prob, const uint16_t* lab,
                           uint16_t* out, int C0, bool has_empty, const uint16_t* rows = nullptr,
                           int nrows = -1) {
  const int L = P.L, w = P.w;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint16_t* nbp = P.nb + static_cast<size_t>(prob) * L * w;
  const float* scp = P.sc + static_cast<size_t>(prob) * L * w;
  const int count = rows ? nrows : L;
  constexpr int kB = kVoteBatch;
  for (int i0 = warp * kB; i0 < count; i0 += kWarps * kB) {
    uint16_t ids[kB];
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      const int i = i0 + u;
      const int r = i < count ? (rows ? static_cast<int>(rows[i]) : i) : 0;
      ids[u] = (i < count && lane < w) ? nbp[static_cast<size_t>(r) * w + lane] : kNoRow;
    }
#pragma unroll
    for (int u = 0; u < kB; u += kVoteRows) {
      const int i = i0 + u;
      if (i >= count) break;
      int rr[kVoteRows], best[kVoteRows];
      uint16_t id[kVoteRows];
      const float* sc[kVoteRows];
#pragma unroll
      for (int q = 0; q < kVoteRows; ++q) {
        const bool in = i + q < count;
        rr[q] = in ? (rows ? static_cast<int>(rows[i + q]) : i + q) : -1;
        id[q] = in ? ids[u + q] : kNoRow;
        sc[q] = scp + static_cast<size_t>(in ? rr[q] : 0) * w;
      }
      vote_rows_match<kVoteRows>(lab, id, sc, w, lane, best);
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < kVoteRows; ++q)
          if (rr[q] >= 0 && best[q] >= 0) out[rr[q]] = static_cast<uint16_t>(best[q]);
      }
    }
  }
  if (has_empty) vote_empty_rows(P, s, prob, lab, out, C0);
  __syncthreads();
}

// Rows whose vote may differ from the current state's: reverse neighbours of
// the rows whose label changed.  Lists them in s.jarr (free after the
// relabel) and returns how many, or returns -1 when so many rows changed that
// a full vote is cheaper; either way s.pred starts as a copy of s.curpred.
//   pass: each warp takes a contiguous range of rows, copies their
//     predictions, clears their flags and appends its changed rows'
//     reverse-list bounds to s.list (one shared-counter atomic per warp step
//     that has any);
//   gather: each warp takes four changed rows at a time, its lanes reading 32
//     reverse entries of each per step (all four rows' loads in flight); the
//     lane that sets a row's flag first (atomicOr on the flag's word) appends
//     the row to the list.
// The list is in no particular order: every listed row is voted on its own.
__device__ int dirty_rows_block(const EvolveParams& P, const Smem& s, int prob) {
  Fixed& f = *s.f;
  const int L = P.L;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  uint8_t* flag = reinterpret_cast<uint8_t*>(s.scratch32);
  unsigned* flagw = reinterpret_cast<unsigned*>(s.scratch32);
  int* bounds = reinterpret_cast<int*>(s.list);  // 2 ints per changed row, room for L / 4 rows
  uint16_t* dirty = s.jarr;
  const int cap = L / 4;
  const int* roff = P.rev_off + static_cast<size_t>(prob) * (L + 1);
  const uint16_t* ridx = P.rev_idx + static_cast<size_t>(prob) * L * P.w;
  if (threadIdx.x == 0) {
    f.changed_cnt = 0;
    f.dirty_cnt = 0;
  }
  __syncthreads();
  const int chunk = ((L + kWarps - 1) / kWarps + 31) / 32 * 32;
  const int beg = min(L, warp * chunk), end = min(L, beg + chunk);
  for (int b = beg; b < end; b += 32) {
    const int r = b + lane;
    bool ch = false;
    if (r < end) {
      s.pred[r] = s.curpred[r];
      flag[r] = 0;
      ch = s.cl[r] != s.cur[r];
    }
    const unsigned bm = __ballot_sync(kFull, ch);
    if (bm != 0u) {
      int slot0 = 0;
      if (lane == 0) slot0 = atomicAdd(&f.changed_cnt, __popc(bm));
      slot0 = __shfl_sync(kFull, slot0, 0);
      const int slot = slot0 + __popc(bm & below);
      if (ch && slot < cap) {
        bounds[2 * slot] = roff[r];
        bounds[2 * slot + 1] = roff[r + 1];
      }
    }
  }
  __syncthreads();
  const int changed = f.changed_cnt;
  // changed * mean in-degree reverse entries mark about L (1 - exp(-e / L))
  // distinct rows for e entries; the gather costs little next to a vote, so
  // the full vote is kept for e > 3 L (about 95% of the rows dirty), and for
  // more changed rows than the bounds' room
  if (static_cast<long long>(changed) * f.rev_total > 3ll * L * L || changed > cap) return -1;
  for (int i0 = 4 * warp; i0 < changed; i0 += 4 * kWarps) {
    int b[4], e[4];
    int span = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = i0 + q;
      b[q] = i < changed ? bounds[2 * i] : 0;
      e[q] = i < changed ? bounds[2 * i + 1] : 0;
      span = max(span, e[q] - b[q]);
    }
    for (int k0 = 0; k0 < span; k0 += 32) {
      uint16_t v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k = b[q] + k0 + lane;
        v[q] = k < e[q] ? ridx[k] : kNoRow;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        bool first = false;
        if (v[q] != kNoRow) {
          const unsigned bit = 1u << (8 * (v[q] & 3u));
          first = (atomicOr(&flagw[v[q] >> 2], bit) & bit) == 0u;
        }
        const unsigned fm = __ballot_sync(kFull, first);
        if (fm != 0u) {
          int slot0 = 0;
          if (lane == 0) slot0 = atomicAdd(&f.dirty_cnt, __popc(fm));
          slot0 = __shfl_sync(kFull, slot0, 0);
          if (first) dirty[slot0 + __popc(fm & below)] = v[q];
        }
      }
    }
  }
  __syncthreads();
  return f.dirty_cnt;
}

// Count labels of `lab` per code, first positions and distinct count.
// have_cnt: s.cnt already holds the counts of `lab` (absorption_block counted
// the same labels and left them unchanged).  A thread's rows come in
// increasing order and a first position only decreases, so a row at or past
// the current first position of its code needs no atomicMin: the plain read
// filters nearly all of them after the first rows of each code.
// pred != nullptr: *ok also receives the count of rows with lab == pred
// (both totals from one block reduction: ok + 2^16 nc, L and C0 < 2^15).
__device__ int label_census(const EvolveParams& P, const Smem& s, const uint16_t* lab, int C0,
                            bool have_cnt = false, const uint16_t* pred = nullptr, int* ok = nullptr) {
  for (int c = threadIdx.x; c < C0; c += kThreads) {
    if (!have_cnt) s.cnt[c] = 0;
    s.firstpos[c] = 0x7fffffff;
  }
  __syncthreads();
  volatile int* fp = s.firstpos;
  int hits = 0;
  for (int r = threadIdx.x; r < P.L; r += kThreads) {
    const int code = lab[r];
    if (pred != nullptr) hits += code == pred[r];
    if (!have_cnt) atomicAdd(&s.cnt[code], 1);
    if (r < fp[code]) atomicMin(&s.firstpos[code], r);
  }
  __syncthreads();
  int local = 0;
  for (int c = threadIdx.x; c < C0; c += kThreads) local += s.cnt[c] > 0;
  if (pred == nullptr) return block_sum(local, *s.f);
  const int packed = block_sum(hits + (local << 16), *s.f);
  *ok = packed & 0xffff;
  return packed >> 16;
}

// s.order[0..nc) = the codes of the census in the iteration order of
// std::unordered_map<int,int> after reserve(L) and insertion in row order.
__device__ __noinline__ void map_order(const EvolveParams& P, const Smem& s, int prob, int C0) {
  const bool nocollide = P.nocollide[prob] != 0;
  if (nocollide) {
    // every key has its own bucket: each new key goes to the list front, so
    // a key's rank counts the keys first seen after it (one warp per key)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = warp; c < C0; c += kWarps) {
      if (s.cnt[c] == 0) continue;
      int rank = 0;
      const int fp = s.firstpos[c];
      for (int c2 = lane; c2 < C0; c2 += 32) rank += (s.cnt[c2] > 0 && s.firstpos[c2] > fp);
      rank = __reduce_add_sync(kFull, rank);
      if (lane == 0) s.order[rank] = c;
    }
    __syncthreads();
  } else if (threadIdx.x == 0) {
    // keys in insertion order, then simulate bucket-run insertion
    int* ins = s.bt;   // scratch
    int k = 0;
    for (int c = 0; c < C0; ++c) if (s.cnt[c] > 0) ins[k++] = c;
    for (int a = 1; a < k; ++a) {  // insertion sort by first position
      const int v = ins[a];
      int b = a - 1;
      while (b >= 0 && s.firstpos[ins[b]] > s.firstpos[v]) {
        ins[b + 1] = ins[b];
        --b;
      }
      ins[b + 1] = v;
    }
    const int* c2l = P.code2label + static_cast<size_t>(prob) * P.C0max;
    int* list = s.order;  // list[0..len) in iteration order
    int len = 0;
    for (int a = 0; a < k; ++a) {
      const int code = ins[a];
      const uint64_t bkt = static_cast<uint64_t>(static_cast<int64_t>(c2l[code])) % P.bucket_count;
      int at = -1;
      for (int q = 0; q < len; ++q) {
        const uint64_t bq = static_cast<uint64_t>(static_cast<int64_t>(c2l[list[q]])) % P.bucket_count;
        if (bq == bkt) {
          at = q;
          break;
        }
      }
      if (at < 0) at = 0;
      for (int q = len; q > at; --q) list[q] = list[q - 1];
      list[at] = code;
      ++len;
    }
  }
  __syncthreads();
}

// core_objective_score for the kNN classifier; census must be current.
__device__ double objective(const EvolveParams& P, const Smem& s, int prob, double acc, int nc, int C0) {
  const bool use_div = P.guarded && P.pol_diversity;
  const bool reject1 = P.guarded && P.pol_reject1;
  if (!use_div && !reject1) return acc;
  if (reject1 && nc == 1) return -INFINITY;
  if (!use_div) return acc;
  map_order(P, s, prob, C0);
  if (threadIdx.x < 32) {
    // psq[c] = (c/L)*(c/L) rounded as the reference rounds each step; the
    // warp loads the terms, lane 0 adds them in iteration order
    for (int q = threadIdx.x; q < nc; q += 32) s.cp[q] = P.psq[s.cnt[s.order[q]]];
    __syncwarp();
    if (threadIdx.x == 0) {
      double same = 0.0;
      for (int q = 0; q < nc; ++q) same = __dadd_rn(same, s.cp[q]);
      const double diff = __dsub_rn(1.0, same);
      const double dlp = (0.0 < diff) ? diff : 0.0;
      s.f->score = __dmul_rn(acc, __dsqrt_rn(dlp));
    }
  }
  __syncthreads();
  const double out = s.f->score;
  __syncthreads();
  return out;
}

// propose_many_to_one_absorption on s.cl given proposal predictions pp.
// Returns 1 if the labels changed.
__device__ int absorption_block(const EvolveParams& P, const Smem& s, int prob, const uint16_t* pp, int C0) {
  Fixed& f = *s.f;
  int* tr = s.trans;
  const int C = P.C0max;
  for (int i = threadIdx.x; i < C0 * C; i += kThreads) tr[i] = 0;
  for (int c = threadIdx.x; c < C0; c += kThreads) {
    s.cnt[c] = 0;
    s.movable[c] = 0;
    s.bt[c] = -1;
  }
  __syncthreads();
  // one atomic per row into the table: with the table in shared memory the
  // class sizes are its row sums; with it in global memory a second,
  // shared-memory atomic per row counts them.  Without fixed rows every row
  // is movable.
  const bool any_fixed = s.f->fxd != nullptr;
  const bool count_rows = !P.smem_trans;
  for (int r = threadIdx.x; r < P.L; r += kThreads) {
    const int a = s.cl[r];
    atomicAdd(&tr[a * C + pp[r]], 1);
    if (count_rows) atomicAdd(&s.cnt[a], 1);
    if (any_fixed && s.f->fxd[r] != 1) atomicAdd(&s.movable[a], 1);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int local = 0;
  if (count_rows) {
    for (int c = threadIdx.x; c < C0; c += kThreads) {
      if (!any_fixed) s.movable[c] = s.cnt[c];
      local += s.cnt[c] > 0;
    }
  } else {
    // class sizes: one warp per class, its lanes over the predictions
    for (int c = warp; c < C0; c += kWarps) {
      int sz = 0;
      for (int q = lane; q < C0; q += 32) sz += tr[c * C + q];
      sz = __reduce_add_sync(kFull, sz);
      if (lane == 0) {
        s.cnt[c] = sz;
        if (!any_fixed) s.movable[c] = sz;
        local += sz > 0;
      }
    }
  }
  const int nc = block_sum(local, f);  // its barriers also publish the sizes
  if (nc <= 2) return 0;
  const double n = static_cast<double>(P.L);
  const double nmax = (1.0 < n) ? n : 1.0;  // std::max(1.0, n)
  // one warp per source, its lanes over the destinations.  The reference
  // scans the destinations in ascending order keeping the best by
  // (surplus, count, destination size, smaller destination), starting from
  // (0, 0, source size, source): that is the lexicographic maximum of those
  // keys, found here by a warp reduction.
  for (int src = warp; src < C0; src += kWarps) {
    const int ssize = s.cnt[src];
    if (ssize == 0 || s.movable[src] <= 0) continue;
    const int* row = tr + src * C;
    const int stay = row[src];
    // exact surplus x n = cnt*n - ssize*dsize; only the candidates at the
    // exact maximum can win the double comparison chain (double rounding is
    // far below the 1/n spacing of distinct exact surpluses)
    long long kmax = -0x7fffffffffffffffll;
#pragma unroll 4
    for (int dst = lane; dst < C0; dst += 32) {
      const int cntd = row[dst];
      const int dsize = s.cnt[dst];
      if (dst == src || cntd == 0 || dsize == 0) continue;
      const long long kx = static_cast<long long>(cntd) * P.L - static_cast<long long>(ssize) * dsize;
      if (kx > kmax) kmax = kx;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long other = __shfl_xor_sync(kFull, kmax, o);
      if (other > kmax) kmax = other;
    }
    int bt = src, bcount = 0, bsize = ssize;
    double bsur = 0.0;
    bool cand = false;
#pragma unroll 4
    for (int dst = lane; dst < C0; dst += 32) {
      const int cntd = row[dst];
      const int dsize = s.cnt[dst];
      if (dst == src || cntd == 0 || dsize == 0) continue;
      if (static_cast<long long>(cntd) * P.L - static_cast<long long>(ssize) * dsize != kmax) continue;
      cand = true;
      const double expected = __ddiv_rn(__dmul_rn(static_cast<double>(ssize), static_cast<double>(dsize)), nmax);
      const double sur = __dsub_rn(static_cast<double>(cntd), expected);
      if (sur > bsur || (sur == bsur && cntd > bcount) || (sur == bsur && cntd == bcount && dsize > bsize) ||
          (sur == bsur && cntd == bcount && dsize == bsize && dst < bt)) {
        bt = dst;
        bsize = dsize;
        bcount = cntd;
        bsur = sur;
      }
    }
    const unsigned cands = __ballot_sync(kFull, cand);
    if (cands == 0u) continue;
    if ((cands & (cands - 1u)) == 0u) {
      // one lane holds every candidate: its best is the warp's
      const int ld = __ffs(cands) - 1;
      bt = __shfl_sync(kFull, bt, ld);
      bcount = __shfl_sync(kFull, bcount, ld);
      bsur = __shfl_sync(kFull, bsur, ld);
    } else {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double osur = __shfl_xor_sync(kFull, bsur, o);
      const int ocount = __shfl_xor_sync(kFull, bcount, o);
      const int osize = __shfl_xor_sync(kFull, bsize, o);
      const int obt = __shfl_xor_sync(kFull, bt, o);
      if (osur > bsur || (osur == bsur && ocount > bcount) || (osur == bsur && ocount == bcount && osize > bsize) ||
          (osur == bsur && ocount == bcount && osize == bsize && obt < bt)) {
        bt = obt;
        bsize = osize;
        bcount = ocount;
        bsur = osur;
      }
    }
    }
    if (lane == 0 && !(bt == src || bsur <= 0.0 || bcount <= stay)) {
      s.bt[src] = bt;
      s.bsur[src] = bsur;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // per-target weights accumulated in ascending source order
    for (int c = 0; c < C0; ++c) {
      s.aux[c] = 0;
      s.weight[c] = 0.0;
    }
    for (int src = 0; src < C0; ++src) {
      const int t = s.bt[src];
      if (t < 0) continue;
      s.weight[t] = __dadd_rn(s.weight[t], s.bsur[src]);
      s.aux[t] += 1;
    }
    int nmulti = 0, nsingle = 0;
    for (int t = 0; t < C0; ++t) {
      if (s.aux[t] > 1) ++nmulti;
      else if (s.aux[t] == 1) ++nsingle;
    }
    int sel = -1;
    if (nmulti + nsingle > 0) {
      const int want_multi = nmulti > 0;
      int k = 0;
      for (int t = 0; t < C0; ++t) {
        if (s.aux[t] == 0 || (s.aux[t] > 1) != (want_multi != 0)) continue;
        s.order[k] = t;
        s.cp[C0 + k] = s.weight[t] > DBL_MIN ? s.weight[t] : DBL_MIN;  // std::max(weight, DBL_MIN)
        ++k;
      }
      const int pick = discrete_serial(f.rng, s.cp + C0, k, s.cp);
      sel = s.order[pick];
    }
    f.selected_target = sel;
  }
  __syncthreads();
  const int sel = f.selected_target;
  if (sel < 0) return 0;
  // sizes after remapping every non-fixed row of the selected sources
  if (threadIdx.x == 0) {
    int moved = 0;
    int after = 0;
    for (int c = 0; c < C0; ++c) {
      int size = s.cnt[c];
      if (s.bt[c] == sel && c != sel) {
        moved += s.movable[c];
        size -= s.movable[c];
      }
      s.aux[c] = size;
    }
    s.aux[sel] += moved;
    for (int c = 0; c < C0; ++c) after += s.aux[c] > 0;
    f.flag = (moved > 0 && after > 1 && after < nc) ? 1 : 0;
  }
  __syncthreads();
  const int apply = f.flag;
  if (apply) {
    for (int r = threadIdx.x; r < P.L; r += kThreads) {
      const int a = s.cl[r];
      if (s.f->fxd != nullptr && s.f->fxd[r] == 1) continue;
      if (a != sel && s.bt[a] == sel) s.cl[r] = static_cast<uint16_t>(sel);
    }
  }
  __syncthreads();
  return apply;
}

// Relabel of sampled groups when draws are needed (groups of several rows, or
// no prediction guidance).  Thread 0, in shuffled order.
__device__ __noinline__ void relabel_serial(const EvolveParams& P, const Smem& s, const uint16_t* pp, int ns, int C0) {
  Fixed& f = *s.f;
  int* hist = s.aux;
  for (int c = 0; c < C0; ++c) hist[c] = 0;
  int nemp = 0;
  if (!P.pol_guidance) {
    // empirical distribution of the labels at the start of the cycle
    for (int r = 0; r < P.L; ++r) hist[s.cl[r]]++;
    for (int c = 0; c < C0; ++c) {
      if (hist[c] > 0) {
        s.order[nemp] = c;
        s.weight[nemp] = static_cast<double>(hist[c]);
        ++nemp;
      }
      hist[c] = 0;
    }
  }
  for (int q = 0; q < ns; ++q) {
    const int g = s.perm[q];
    const int beg = s.f->goff[g], end = s.f->goff[g + 1];
    int neligible = 0;
    for (int a = beg; a < end; ++a) neligible += (s.f->fxd == nullptr || s.f->fxd[s.f->gmem[a]] != 1);
    if (neligible == 0) continue;
    int rep;
    if (P.pol_guidance) {
      // candidate labels: predictions of the eligible members, ascending, with counts
      int k = 0;
      for (int a = beg; a < end; ++a) {
        const int row = s.f->gmem[a];
        if (s.f->fxd != nullptr && s.f->fxd[row] == 1) continue;
        const int c = pp[row];
        if (hist[c]++ == 0) s.bt[k++] = c;
      }
      for (int a = 1; a < k; ++a) {
        const int v = s.bt[a];
        int b = a - 1;
        while (b >= 0 && s.bt[b] > v) {
          s.bt[b + 1] = s.bt[b];
          --b;
        }
        s.bt[b + 1] = v;
      }
      for (int a = 0; a < k; ++a) {
        s.cp[C0 + a] = static_cast<double>(hist[s.bt[a]]);
        hist[s.bt[a]] = 0;
      }
      rep = s.bt[discrete_serial(f.rng, s.cp + C0, k, s.cp)];
    } else {
      if (nemp == 0) continue;
      rep = s.order[discrete_serial(f.rng, s.weight, nemp, s.cp)];
    }
    for (int a = beg; a < end; ++a) {
      const int row = s.f->gmem[a];
      if (s.f->fxd != nullptr && s.f->fxd[row] == 1) continue;
      s.cl[row] = static_cast<uint16_t>(rep);
    }
  }
}

// ---------------------------------------------------------------------------
// Learned relabelling proposal (mlp.cuh)
// ---------------------------------------------------------------------------

// Features of `row` in the current state (s.cur / s.curpred), census of
// s.cur in `cnt_cur`: among the row's fold-filtered neighbours, the fractions
// sharing its label, holding its prediction as label, predicting its
// prediction and whose label equals their prediction; the sizes of its label
// and prediction classes; the run's progress; the fraction of valid
// neighbours.
__device__ void proposal_features(const EvolveParams& P, const Smem& s, int prob, int row, const int* cnt_cur,
                                  float progress, float* f) {
  const uint16_t* nbr = P.nb + (static_cast<size_t>(prob) * P.L + row) * P.w;
  const int c = s.cur[row], q = s.curpred[row];
  int nv = 0, same_cur = 0, same_pred = 0, pred_pred = 0, stable = 0;
  for (int j = 0; j < P.w; ++j) {
    const int id = nbr[j];
    if (id == kNoRow) break;
    ++nv;
    const int lc = s.cur[id], lp = s.curpred[id];
    same_cur += lc == c;
    same_pred += lc == q;
    pred_pred += lp == q;
    stable += lc == lp;
  }
  const float inv = nv > 0 ? 1.0f / static_cast<float>(nv) : 0.0f;
  const float invL = 1.0f / static_cast<float>(P.L);
  f[0] = same_cur * inv;
  f[1] = same_pred * inv;
  f[2] = pred_pred * inv;
  f[3] = stable * inv;
  f[4] = cnt_cur[c] * invL;
  f[5] = cnt_cur[q] * invL;
  f[6] = progress;
  f[7] = static_cast<float>(nv) / static_cast<float>(P.w);
}

// Census of s.cur into s.aux (per code).
__device__ void census_cur(const EvolveParams& P, const Smem& s, int C0) {
  for (int c = threadIdx.x; c < C0; c += kThreads) s.aux[c] = 0;
  __syncthreads();
  for (int r = threadIdx.x; r < P.L; r += kThreads) atomicAdd(&s.aux[s.cur[r]], 1);
  __syncthreads();
}

// Gumbel(0, 1) noise of (run seed, cycle, row): a splitmix64 hash of the
// three (Steele, Lea and Flood, "Fast splittable pseudorandom number
// generators", 2014) mapped to u in (0, 1), then -log(-log u).
__device__ __forceinline__ float gumbel_noise(uint64_t seed, int cycle, int row) {
  uint64_t z = seed + 0x9e3779b97f4a7c15ull * (static_cast<uint64_t>(cycle) * 65536ull + static_cast<uint64_t>(row) + 1ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  const float u = (static_cast<float>(z >> 40) + 0.5f) * (1.0f / 16777216.0f);
  return -__logf(-__logf(u));
}

// Relabels to their prediction `take` of the candidates (label != prediction,
// not fixed).  The candidates are compacted into keys whose low 16 bits are
// 65535 - row; each warp scores 32 of them on the tensor pipe
// (mlp_logit_warp) and puts the top 16 bits of the order-preserving image of
// the score (plus Gumbel noise unless P.mlp_greedy: sampling without
// replacement from the network's softmax over the candidates) above the row,
// so all keys are distinct and ties go to the smaller row.  The take-th
// largest key is found by a 4-pass radix select with 8-bit digits.
__device__ __noinline__ void learned_flip(const EvolveParams& P, const Smem& s, int prob, int cycle, int take, int C0) {
  Fixed& f = *s.f;
  if (take <= 0) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  census_cur(P, s, C0);
  unsigned* key = reinterpret_cast<unsigned*>(s.scratch32);
  if (threadIdx.x == 0) f.sel_count = 0;
  __syncthreads();
  for (int base = warp * 32; base < P.L; base += kThreads) {
    const int r = base + lane;
    const bool c = r < P.L && s.cur[r] != s.curpred[r] && (s.f->fxd == nullptr || s.f->fxd[r] != 1);
    const unsigned b = __ballot_sync(kFull, c);
    int at = 0;
    if (lane == 0 && b != 0u) at = atomicAdd(&f.sel_count, __popc(b));
    at = __shfl_sync(kFull, at, 0);
    if (c) key[at + __popc(b & ((1u << lane) - 1u))] = 0xffffu - static_cast<unsigned>(r);
  }
  __syncthreads();
  const int count = f.sel_count;
  if (take >= count) {
    for (int i = threadIdx.x; i < count; i += kThreads) {
      const int r = 0xffff - static_cast<int>(key[i] & 0xffffu);
      s.cl[r] = s.curpred[r];
    }
    __syncthreads();
    return;
  }
  const float progress = static_cast<float>(cycle) / static_cast<float>(P.T > 0 ? P.T : 1);
  const uint64_t seed = P.seeds[prob];
  for (int base = warp * 32; base < count; base += kThreads) {
    const int i = base + lane;
    uint32_t fw[4] = {0u, 0u, 0u, 0u};
    int r = -1;
    if (i < count) {
      r = 0xffff - static_cast<int>(key[i] & 0xffffu);
      float x[kMlpIn];
      proposal_features(P, s, prob, r, s.aux, progress, x);
      mlp_pack_row(x, fw);
    }
    float z = mlp_logit_warp(P.mlp, fw, min(32, count - base));
    if (i < count) {
      if (!P.mlp_greedy) z += gumbel_noise(seed, cycle, r);
      const unsigned u = __float_as_uint(z);
      const unsigned ord = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
      key[i] = (ord & 0xffff0000u) | (0xffffu - static_cast<unsigned>(r));
    }
  }
  __syncthreads();
  unsigned prefix = 0u;
  int need = take;
  for (int pass = 3; pass >= 0; --pass) {
    const int shift = 8 * pass;
    const unsigned hmask = pass == 3 ? 0u : (0xffffffffu << (shift + 8));
    for (int b = threadIdx.x; b < 256; b += kThreads) f.sel_hist[b] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < count; i += kThreads) {
      const unsigned k = key[i];
      if ((k & hmask) == prefix) atomicAdd(&f.sel_hist[(k >> shift) & 255u], 1);
    }
    __syncthreads();
    if (warp == 0) {
      // lane l holds digits 8 l .. 8 l + 7; find the largest digit whose
      // count of keys at or above it reaches `need`
      int c[8], tot = 0;
#pragma unroll
      for (int d = 0; d < 8; ++d) {
        c[d] = f.sel_hist[8 * lane + d];
        tot += c[d];
      }
      int suf = tot;  // keys in lanes >= this lane
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_down_sync(kFull, suf, o);
        if (lane + o < 32) suf += v;
      }
      const unsigned ball = __ballot_sync(kFull, suf >= need);
      if (lane == 31 - __clz(ball)) {
        int above = suf - tot, d = 7;
        while (d > 0 && above + c[d] < need) above += c[d--];
        f.sel_digit = 8 * lane + d;
        f.sel_need = need - above;
      }
    }
    __syncthreads();
    prefix |= static_cast<unsigned>(f.sel_digit) << shift;
    need = f.sel_need;
    __syncthreads();
  }
  for (int i = threadIdx.x; i < count; i += kThreads) {
    if (key[i] >= prefix) {
      const int r = 0xffff - static_cast<int>(key[i] & 0xffffu);
      s.cl[r] = s.curpred[r];
    }
  }
  __syncthreads();
}

// Training snapshot of the current state: features of every row and its
// label / prediction codes.
__device__ __noinline__ void snapshot_state(const EvolveParams& P, const Smem& s, int prob, int cycle, int C0) {
  census_cur(P, s, C0);
  const float progress = static_cast<float>(cycle) / static_cast<float>(P.T > 0 ? P.T : 1);
  for (int r = threadIdx.x; r < P.L; r += kThreads) {
    const size_t o = static_cast<size_t>(prob) * P.L + r;
    float x[kMlpIn];
    proposal_features(P, s, prob, r, s.aux, progress, x);
    for (int i = 0; i < kMlpIn; ++i) P.snap_feat[o * kMlpIn + i] = x[i];
    P.snap_cur[o] = s.cur[r];
    P.snap_pred[o] = s.curpred[r];
  }
  __syncthreads();
}

// Points the CTA at problem prob's groups and fixed flags: shared by all
// problems, or one block per problem (per_problem_groups: goff stride L + 1,
// gmem and fixed stride L, group count gcount[prob]).
__device__ __noinline__ void bind_groups(const EvolveParams& P, const Smem& s, int prob) {
  if (threadIdx.x == 0) {
    const bool per = P.per_problem_groups != 0;
    s.f->goff = P.goff + (per ? static_cast<size_t>(prob) * (P.L + 1) : 0);
    s.f->gmem = P.gmem + (per ? static_cast<size_t>(prob) * P.L : 0);
    s.f->fxd = P.fixed == nullptr ? nullptr : P.fixed + (per ? static_cast<size_t>(prob) * P.L : 0);
    s.f->G = per ? P.gcount[prob] : P.G;
  }
  __syncthreads();
}

__device__ void evolve_problem(const EvolveParams& P, const Smem& s, int prob) {
  Fixed& f = *s.f;
  bind_groups(P, s, prob);
  const int L = P.L, T = P.T, G = f.G;
  const int C0 = P.ncodes[prob];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint16_t* init = P.init + static_cast<size_t>(prob) * L;
  uint16_t* gbest = P.clbest + static_cast<size_t>(prob) * L;
  uint16_t* gbestpred = P.cvpredbest + static_cast<size_t>(prob) * L;
  double* vacc = P.vect_acc + static_cast<size_t>(prob) * T;
  double* vscore = P.vect_score + static_cast<size_t>(prob) * T;
  int* psize = P.proposal_size + static_cast<size_t>(prob) * T;
  int* act = P.active + static_cast<size_t>(prob) * T;
  uint8_t* fl = P.flags + static_cast<size_t>(prob) * T * 3;
  const uint16_t* nbp = P.nb + static_cast<size_t>(prob) * L * P.w;

  if (threadIdx.x == 0) {
    mt64_seed(f.rng, P.seeds[prob]);
    f.rev_total = P.rev_off[static_cast<size_t>(prob) * (L + 1) + L];
  }
  int local_empty = 0;
  for (int r = threadIdx.x; r < L; r += kThreads) {
    s.cur[r] = init[r];
    local_empty += nbp[static_cast<size_t>(r) * P.w] == kNoRow;
  }
  __syncthreads();
  const bool has_empty = block_sum(local_empty, f) > 0;

  // initial evaluation
  vote_block(P, s, prob, s.cur, s.curpred, C0, has_empty);
  int ok = 0;
  for (int r = threadIdx.x; r < L; r += kThreads) {
    ok += s.cur[r] == s.curpred[r];
    gbest[r] = s.cur[r];
    gbestpred[r] = s.curpred[r];
  }
  ok = block_sum(ok, f);
  const double n = static_cast<double>(L);
  double accbest = __ddiv_rn(static_cast<double>(ok), n);
  int nc_cur = label_census(P, s, s.cur, C0);
  double scorebest = objective(P, s, prob, accbest, nc_cur, C0);
  double cur_acc = accbest, cur_score = scorebest;
  int nc_best = nc_cur;
  int proposals = 0, best_updates = 0, accepts = 0, st_att = 0, st_acc = 0, rejections = 0,
      absorb_moves = 0, tr_att = 0, tr_acc = 0, success = 0;

  for (int cycle = 0; cycle < T; ++cycle) {
    if (P.snap_feat != nullptr && cycle == P.snap_cycle) snapshot_state(P, s, prob, cycle, C0);
    // proposal = current (evolutionary) or best (greedy) state; s.cur holds
    // it.  Thread 0 draws the proposal size before its share of the copy.
    {
      if (threadIdx.x == 0) {
        int ns;
        if (G <= 1) {
          ns = G > 0 ? G : 0;
        } else if (!(P.adaptive && P.pol_adaptive) || T <= 1) {
          ns = uniform_int_serial(f.rng, 1, G);
        } else {
          double progress = __ddiv_rn(static_cast<double>(cycle + 1), static_cast<double>(T + 1));
          progress = progress < 0.0 ? 0.0 : (progress > 1.0 ? 1.0 : progress);
          const double smooth = __dmul_rn(__dmul_rn(progress, progress), __dsub_rn(3.0, __dmul_rn(2.0, progress)));
          double temp = __dsub_rn(1.0, smooth);
          temp = temp < 0.0 ? 0.0 : (temp > 1.0 ? 1.0 : temp);
          const int mc = 1 + static_cast<int>(floor(__dmul_rn(static_cast<double>(G - 1), temp)));
          ns = uniform_int_serial(f.rng, 1, mc > 1 ? mc : 1);
        }
        f.ns = ns;
      }
      for (int r = threadIdx.x; r < L; r += kThreads) s.cl[r] = s.cur[r];
    }
    __syncthreads();
    shuffle_targets_block(f, s.jarr, G, s.raw);
    const int ns = f.ns;
    if (threadIdx.x == 0) psize[cycle] = ns;
    if (ns > 0) {
      bucket_steps_block(s, G, ns);
      if (P.singleton && P.pol_guidance && P.mlp != nullptr) {
        // learned proposal: as many relabellings as the plain draw would make,
        // given to the candidates the network scores highest
        int take = 0;
        for (int g = threadIdx.x; g < G; g += kThreads) {
          const int row = s.f->gmem[g];
          if (s.curpred[row] == s.cur[row]) continue;
          if (s.f->fxd != nullptr && s.f->fxd[row] == 1) continue;
          take += final_position_of(s, g, ns) < ns;
        }
        take = block_sum(take, f);
        learned_flip(P, s, prob, cycle, take, C0);
      } else if (P.singleton && P.pol_guidance) {
        // Each sampled group takes its own CV prediction; only groups whose
        // prediction differs from their label can change, so walk just those
        // forward to their final shuffled position.
        for (int g = threadIdx.x; g < G; g += kThreads) {
          const int row = s.f->gmem[g];
          if (s.curpred[row] == s.cur[row]) continue;
          if (s.f->fxd != nullptr && s.f->fxd[row] == 1) continue;
          if (final_position_of(s, g, ns) < ns) s.cl[row] = s.curpred[row];
        }
      } else {
        for (int p = threadIdx.x; p < ns; p += kThreads) s.perm[p] = static_cast<uint16_t>(occupant_of(s, G, p));
        __syncthreads();
        if (threadIdx.x == 0) relabel_serial(P, s, s.curpred, ns, C0);
      }
    }
    __syncthreads();

    int absorbed = 0;
    bool cnt_of_cl = false;  // s.cnt holds the counts of s.cl
    if (P.pol_transition && P.absorption) {
      ++tr_att;
      absorbed = absorption_block(P, s, prob, s.curpred, C0);
      absorb_moves += absorbed;
      cnt_of_cl = absorbed == 0;
    }

    {
      const int nd = dirty_rows_block(P, s, prob);  // s.pred = s.curpred on return
      if (nd < 0) {
        vote_block(P, s, prob, s.cl, s.pred, C0, has_empty);
      } else {
        vote_block(P, s, prob, s.cl, s.pred, C0, has_empty, s.jarr, nd);
      }
    }
    const int nc = L < 32768 && C0 < 32768 ? label_census(P, s, s.cl, C0, cnt_of_cl, s.pred, &ok)
                                           : label_census(P, s, s.cl, C0, cnt_of_cl);
    if (L >= 32768 || C0 >= 32768) {
      ok = 0;
      for (int r = threadIdx.x; r < L; r += kThreads) ok += s.cl[r] == s.pred[r];
      ok = block_sum(ok, f);
    }
    const double acc = __ddiv_rn(static_cast<double>(ok), n);
    const double score = objective(P, s, prob, acc, nc, C0);
    ++proposals;

    const bool improves = score > scorebest;
    bool accepted = improves, improving = improves, stoch = false;
    if (P.evolutionary) {
      if (threadIdx.x == 0) {
        const double cooling = __dsub_rn(1.0, __ddiv_rn(static_cast<double>(cycle + 1),
                                                        static_cast<double>(T > 1 ? T : 1)));
        const double one_minus = __dsub_rn(1.0, cur_acc);
        const double clipped = (0.0 < one_minus) ? one_minus : 0.0;
        const double t0 = __dmul_rn(__dmul_rn(0.10, clipped), cooling);
        const double temperature = (1.0e-9 < t0) ? t0 : 1.0e-9;
        int acc_cur = score >= cur_score;
        int impr = acc_cur;
        int st = 0;
        if (!acc_cur && P.pol_stochastic && temperature > 1.0e-9) {
          st = 2;  // attempted
          const double u = canonical_serial(f.rng);
          acc_cur = u < exp(__ddiv_rn(__dsub_rn(score, cur_score), temperature));
          if (acc_cur) st = 3;
        }
        f.accept = acc_cur | (impr << 1) | (st << 2);
      }
      __syncthreads();
      const int code = f.accept;
      accepted = code & 1;
      improving = (code >> 1) & 1;
      const int st = code >> 2;
      if (st >= 2) ++st_att;
      stoch = st == 3;
    }
    __syncthreads();
    if (improves) {
      for (int r = threadIdx.x; r < L; r += kThreads) {
        gbest[r] = s.cl[r];
        gbestpred[r] = s.pred[r];
      }
      accbest = acc;
      scorebest = score;
      ++best_updates;
      nc_best = nc;
    }
    const bool take = P.evolutionary ? accepted : improves;
    if (take) {
      for (int r = threadIdx.x; r < L; r += kThreads) {
        s.cur[r] = s.cl[r];
        s.curpred[r] = s.pred[r];
      }
    }
    if (P.evolutionary) {
      if (accepted) {
        cur_acc = acc;
        cur_score = score;
        nc_cur = nc;
        ++accepts;
        if (stoch) ++st_acc;
      } else {
        ++rejections;
      }
    }
    if (accepted && absorbed) ++tr_acc;
    if (threadIdx.x == 0) {
      fl[3 * cycle + 0] = accepted ? 1 : 0;
      fl[3 * cycle + 1] = (accepted && improving) ? 1 : 0;
      fl[3 * cycle + 2] = stoch ? 1 : 0;
      act[cycle] = P.evolutionary ? nc_cur : nc_best;
      vacc[cycle] = accbest;
      vscore[cycle] = scorebest;
    }
    if (acc == 1.0 && isfinite(score)) success = 1;
    __syncthreads();
  }

  if (threadIdx.x == 0) {
    int* c = P.counters + static_cast<size_t>(prob) * 16;
    c[0] = T;
    c[1] = proposals;
    c[2] = best_updates;
    c[3] = accepts;
    c[4] = st_att;
    c[5] = st_acc;
    c[6] = rejections;
    c[7] = 0;
    c[8] = absorb_moves;
    c[9] = tr_att;
    c[10] = tr_acc;
    c[11] = tr_att;
    c[12] = tr_acc;
    c[13] = proposals + 1;
    c[14] = success;
    c[15] = 0;
    P.best[2 * prob] = accbest;
    P.best[2 * prob + 1] = scorebest;
    P.status[prob] = 0;
  }
  __syncthreads();
}

__device__ Smem carve_smem(const EvolveParams& P, unsigned char* smem_raw) {
  Smem s;
  size_t off = 0;
  s.f = reinterpret_cast<Fixed*>(smem_raw);
  off = align_up(sizeof(Fixed), 16);
  const int C = P.C0max;
  s.cnt = reinterpret_cast<int*>(smem_raw + off); off += align_up(sizeof(int) * C, 16);
  s.firstpos = reinterpret_cast<int*>(smem_raw + off); off += align_up(sizeof(int) * C, 16);
  s.movable = reinterpret_cast<int*>(smem_raw + off); off += align_up(sizeof(int) * C, 16);
  s.order = reinterpret_cast<int*>(smem_raw + off); off += align_up(sizeof(int) * (C + 1), 16);
  s.bt = reinterpret_cast<int*>(smem_raw + off); off += align_up(sizeof(int) * C, 16);
  s.aux = reinterpret_cast<int*>(smem_raw + off); off += align_up(sizeof(int) * C, 16);
  s.bsur = reinterpret_cast<double*>(smem_raw + off); off += align_up(sizeof(double) * C, 16);
  s.weight = reinterpret_cast<double*>(smem_raw + off); off += align_up(sizeof(double) * C, 16);
  s.cp = reinterpret_cast<double*>(smem_raw + off); off += align_up(sizeof(double) * 2 * C, 16);
  const size_t Lp = align_up(static_cast<size_t>(P.L), 8);
  s.raw = P.raw_scratch + static_cast<size_t>(blockIdx.x) * (P.L / 2 + 64);
  if (P.smem_trans) {
    s.trans = reinterpret_cast<int*>(smem_raw + off);
    off += align_up(sizeof(int) * static_cast<size_t>(C) * C, 16);
  } else {
    s.trans = nullptr;
  }
  uint16_t* rows = P.smem_rows ? reinterpret_cast<uint16_t*>(smem_raw + off)
                               : P.rows_scratch + static_cast<size_t>(blockIdx.x) * kRowArrays * Lp;
  s.cl = rows;
  s.cur = rows + Lp;
  s.curpred = rows + 2 * Lp;
  s.pred = rows + 3 * Lp;
  s.perm = s.pred;
  s.jarr = rows + 4 * Lp;
  s.list = rows + 5 * Lp;
  s.scratch32 = reinterpret_cast<int*>(rows + 6 * Lp);  // 2 * Lp u16 = Lp ints
  return s;
}

__global__ void __launch_bounds__(kThreads, 1) evolve_kernel(EvolveParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem s = carve_smem(P, smem_raw);
  const int C = P.C0max;
  for (int prob = blockIdx.x; prob < P.problems; prob += gridDim.x) {
    if (!P.smem_trans) s.trans = P.trans + static_cast<size_t>(prob) * C * C;
    evolve_problem(P, s, prob);
  }
}

// ===========================================================================
// PLS-LDA evolution: maximize_core (core.cpp:1269-1549) with PLSLDACV as the
// predictor.  The predictor runs as separate launches over all problems and
// folds (pls.cu), so each cycle is split in two: this kernel accepts the
// previous proposal (its CV predictions are in Q.pred) and builds the next
// one, keeping the engine, the current state and the counters in global
// memory between launches.  PLS adds to the kNN cycle:
//   propose_auto_class_coarsening   core.cpp:995-1108
//   the fragmentation penalty       core.cpp:954-968
// ===========================================================================

// Serial std::shuffle of a[0..n) with the libstdc++ 64-bit-engine algorithm
// (pair draws, see shuffle_targets_block); a holds (a0, a1) int pairs and a
// double key, swapped together.
__device__ void shuffle_triples_serial(Mt64State& g, int* a0, int* a1, double* key, int n) {
  auto swap3 = [&](int i, int j) {
    const int t0 = a0[i], t1 = a1[i];
    const double tk = key[i];
    a0[i] = a0[j];
    a1[i] = a1[j];
    key[i] = key[j];
    a0[j] = t0;
    a1[j] = t1;
    key[j] = tk;
  };
  if (n <= 1) return;
  int i = 1;
  if ((n & 1) == 0) {
    swap3(1, static_cast<int>(draw_below_serial(g, 2)));
    i = 2;
  }
  while (i < n) {
    const uint64_t b0 = static_cast<uint64_t>(i) + 1ull, b1 = b0 + 1ull;
    const uint64_t x = draw_below_serial(g, b0 * b1);
    swap3(i, static_cast<int>(x / b1));
    swap3(i + 1, static_cast<int>(x % b1));
    i += 2;
  }
}

// Class sizes, movable sizes and class x prediction counts of s.cl against pp
// (build_class_transition_stats, core.cpp:980-993).  Returns the class count.
__device__ int transition_stats(const EvolveParams& P, const Smem& s, const uint16_t* pp, int C0) {
  int* tr = s.trans;
  const int C = P.C0max;
  for (int i = threadIdx.x; i < C0 * C; i += kThreads) tr[i] = 0;
  for (int c = threadIdx.x; c < C0; c += kThreads) {
    s.cnt[c] = 0;
    s.movable[c] = 0;
  }
  __syncthreads();
  // one atomic per row: the class sizes are the rows of the class x
  // prediction table, and without fixed rows every row is movable
  const bool any_fixed = s.f->fxd != nullptr;
  for (int r = threadIdx.x; r < P.L; r += kThreads) {
    const int a = s.cl[r];
    atomicAdd(&tr[a * C + pp[r]], 1);
    if (any_fixed && s.f->fxd[r] != 1) atomicAdd(&s.movable[a], 1);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < C0; c += kThreads) {
    int sz = 0;
    for (int q = 0; q < C0; ++q) sz += tr[c * C + q];
    s.cnt[c] = sz;
    if (!any_fixed) s.movable[c] = sz;
  }
  __syncthreads();
  int local = 0;
  for (int c = threadIdx.x; c < C0; c += kThreads) local += s.cnt[c] > 0;
  return block_sum(local, *s.f);
}

// propose_auto_class_coarsening on s.cl.  plogp[k] = (k/L) * log(k/L) as the
// reference rounds it.  One thread per source class computes its transition
// entropy, its destination and its candidate score; the transition entropy
// is formed as log(s) - sum_c c log(c) / s from host tables of k log k and
// log k: it only feeds ceil(temperature * redundant), which an ulp-level
// difference cannot move unless that product lies within an ulp of an
// integer.  Returns 1 if the labels changed.
__device__ int coarsening_block(const EvolvePlsParams& Q, const Smem& s, int prob, const uint16_t* pp, int C0) {
  const EvolveParams& P = Q.base;
  Fixed& f = *s.f;
  const int nc = transition_stats(P, s, pp, C0);
  if (nc <= 2) return 0;
  const int C = P.C0max;
  double* te_of = s.bsur;     // per source: transition entropy
  int* dst_of = s.bt;         // per source: destination, -1 = not a candidate
  double* score_of = s.cp;    // per source: candidate score
  for (int src = threadIdx.x; src < C0; src += kThreads) {
    const int ssize = s.cnt[src];
    dst_of[src] = -1;
    te_of[src] = 0.0;
    if (ssize == 0 || s.movable[src] <= 0) continue;
    const int* row = s.trans + src * C;
    int dbest = src, dsize = ssize, bcount = 0;
    double clc = 0.0;
    for (int dst = 0; dst < C0; ++dst) {
      const int cntd = row[dst];
      if (cntd == 0) continue;
      clc = __dadd_rn(clc, Q.klogk[cntd]);
      const int sz = s.cnt[dst];
      if (dst != src && sz > 0 &&
          (cntd > bcount || (cntd == bcount && sz > dsize) || (cntd == bcount && sz == dsize && dst < dbest))) {
        dbest = dst;
        dsize = sz;
        bcount = cntd;
      }
    }
    te_of[src] = __dsub_rn(Q.logk[ssize], __ddiv_rn(clc, static_cast<double>(ssize)));
    if (dbest == src || bcount == 0) continue;
    const double stay = __ddiv_rn(static_cast<double>(row[src]), static_cast<double>(ssize));
    dst_of[src] = dbest;
    score_of[src] =
        __dmul_rn(__ddiv_rn(1.0, __dsqrt_rn(static_cast<double>(s.movable[src]))), __dsub_rn(1.0, stay));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double n = static_cast<double>(P.L);
    double ce = 0.0;
    for (int c = 0; c < C0; ++c)
      if (s.cnt[c] > 0) ce = __dsub_rn(ce, Q.plogp[s.cnt[c]]);
    const double keff = cr_exp(ce);
    const double lr = cr_log(__ddiv_rn(static_cast<double>(nc), 1.0 < keff ? keff : 1.0));
    const double frag = 0.0 < lr ? lr : 0.0;
    double wte = 0.0;
    int K = 0;
    int* csrc = s.order;   // candidates in ascending source order: source, destination, score
    int* cdst = s.firstpos;
    double* cscore = s.weight;
    for (int src = 0; src < C0; ++src) {
      if (s.cnt[src] == 0 || s.movable[src] <= 0) continue;
      wte = __dadd_rn(wte, __dmul_rn(__ddiv_rn(static_cast<double>(s.cnt[src]), n), te_of[src]));
      if (dst_of[src] < 0) continue;
      csrc[K] = src;
      cdst[K] = dst_of[src];
      cscore[K] = score_of[src];
      ++K;
    }
    int budget = 0;
    if (K > 0) {
      const double temperature = __ddiv_rn(frag, __dadd_rn(__dadd_rn(frag, wte), 1.0));
      const double rd = __dsub_rn(static_cast<double>(nc), keff);
      const double redundant = 0.0 < rd ? rd : 0.0;
      budget = static_cast<int>(ceil(__dmul_rn(temperature, redundant)));
      if (budget < 1 && frag > 0.0) budget = 1;
      budget = min(budget, nc - 2);
    }
    int merged = 0;
    if (K > 0 && budget > 0) {
      shuffle_triples_serial(f.rng, csrc, cdst, cscore, K);
      for (int a = 1; a < K; ++a) {  // stable sort by score, descending
        const int v0 = csrc[a], v1 = cdst[a];
        const double vk = cscore[a];
        int b = a - 1;
        while (b >= 0 && vk > cscore[b]) {
          csrc[b + 1] = csrc[b];
          cdst[b + 1] = cdst[b];
          cscore[b + 1] = cscore[b];
          --b;
        }
        csrc[b + 1] = v0;
        cdst[b + 1] = v1;
        cscore[b + 1] = vk;
      }
      int* remap = s.aux;
      for (int c = 0; c < C0; ++c) remap[c] = c;
      for (int q = 0; q < K && merged < budget; ++q) {
        const int src = csrc[q];
        if (remap[src] != src) continue;
        int d = cdst[q];
        while (remap[d] != d) d = remap[d];
        if (d == src) continue;
        remap[src] = d;
        ++merged;
      }
    }
    f.flag = merged;
  }
  __syncthreads();
  if (f.flag == 0) return 0;
  int changed = 0;
  const int* remap = s.aux;
  for (int r = threadIdx.x; r < P.L; r += kThreads) {
    if (s.f->fxd != nullptr && s.f->fxd[r] == 1) continue;
    const int a = s.cl[r];
    int d = a;
    while (remap[d] != d) d = remap[d];
    if (d != a) {
      s.cl[r] = static_cast<uint16_t>(d);
      changed = 1;
    }
  }
  return block_sum(changed, f) > 0 ? 1 : 0;
}

// core_objective_score with the PLS fragmentation penalty; census current.
__device__ double objective_pls(const EvolvePlsParams& Q, const Smem& s, int prob, double acc, int nc, int C0) {
  const EvolveParams& P = Q.base;
  const bool use_div = P.guarded && P.pol_diversity;
  const bool use_frag = Q.coarsening && Q.pol_frag;
  const bool reject1 = P.guarded && P.pol_reject1;
  if (!use_div && !use_frag && !reject1) return acc;
  if (reject1 && nc == 1) return -INFINITY;
  if (!use_div && !(use_frag && nc > 1)) return acc;
  map_order(P, s, prob, C0);
  if (threadIdx.x == 0) {
    double score = acc;
    if (use_div) {
      double same = 0.0;
      for (int q = 0; q < nc; ++q) same = __dadd_rn(same, P.psq[s.cnt[s.order[q]]]);
      const double diff = __dsub_rn(1.0, same);
      score = __dmul_rn(score, __dsqrt_rn(0.0 < diff ? diff : 0.0));
    }
    if (use_frag && nc > 1) {
      double entropy = 0.0;
      for (int q = 0; q < nc; ++q) entropy = __dsub_rn(entropy, Q.plogp[s.cnt[s.order[q]]]);
      const double mse = P.L > 1 ? Q.logn : 0.0;
      double code_cost = 0.0;
      if (mse > 0.0) {
        const double v = __ddiv_rn(entropy, mse);
        code_cost = v < 0.0 ? 0.0 : (1.0 < v ? 1.0 : v);
      }
      const double keff = cr_exp(entropy);
      const double lr = cr_log(__ddiv_rn(static_cast<double>(nc), 1.0 < keff ? keff : 1.0));
      const double frag = 0.0 < lr ? lr : 0.0;
      const double frag_cost = __ddiv_rn(frag, __dadd_rn(1.0, frag));
      const double pc = code_cost < frag_cost ? frag_cost : code_cost;
      score = __dsub_rn(score, __dmul_rn(__dsub_rn(1.0, acc), pc));
    }
    s.f->score = score;
  }
  __syncthreads();
  const double out = s.f->score;
  __syncthreads();
  return out;
}

// Rows of s.cl grouped by code, ascending rows within a code, for the
// cross-product chains of the PLS predictor: one warp per code.
__device__ void class_lists(const EvolvePlsParams& Q, const Smem& s, int prob, int C0) {
  const int L = Q.base.L, C = Q.base.C0max;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int c = threadIdx.x; c < C0; c += kThreads) s.cnt[c] = 0;
  __syncthreads();
  for (int r = threadIdx.x; r < L; r += kThreads) atomicAdd(&s.cnt[s.cl[r]], 1);
  __syncthreads();
  int* coff = Q.class_off + static_cast<size_t>(prob) * (C + 1);
  if (threadIdx.x == 0) {
    int run = 0;
    for (int c = 0; c < C; ++c) {
      coff[c] = run;
      s.aux[c] = run;
      run += c < C0 ? s.cnt[c] : 0;
    }
    coff[C] = run;
  }
  __syncthreads();
  uint16_t* rows = Q.class_rows + static_cast<size_t>(prob) * L;
  for (int c = warp; c < C0; c += kWarps) {
    if (s.cnt[c] == 0) continue;
    int pos = s.aux[c];
    for (int base = 0; base < L; base += 32) {
      const int r = base + lane;
      const bool hit = r < L && s.cl[r] == c;
      const unsigned m = __ballot_sync(kFull, hit);
      if (hit) rows[pos + __popc(m & ((1u << lane) - 1u))] = static_cast<uint16_t>(r);
      pos += __popc(m);
    }
  }
  __syncthreads();
}

__device__ void pls_propose(const EvolvePlsParams& Q, const Smem& s, int prob, int cycle, PlsRunState& st, int C0) {
  const EvolveParams& P = Q.base;
  Fixed& f = *s.f;
  const int L = P.L, T = P.T, G = f.G;
  for (int r = threadIdx.x; r < L; r += kThreads) s.cl[r] = s.cur[r];
  __syncthreads();
  if (threadIdx.x == 0) {
    int ns;
    if (G <= 1) {
      ns = G > 0 ? G : 0;
    } else if (!(P.adaptive && P.pol_adaptive) || T <= 1) {
      ns = uniform_int_serial(f.rng, 1, G);
    } else {
      double progress = __ddiv_rn(static_cast<double>(cycle + 1), static_cast<double>(T + 1));
      progress = progress < 0.0 ? 0.0 : (progress > 1.0 ? 1.0 : progress);
      const double smooth = __dmul_rn(__dmul_rn(progress, progress), __dsub_rn(3.0, __dmul_rn(2.0, progress)));
      double temp = __dsub_rn(1.0, smooth);
      temp = temp < 0.0 ? 0.0 : (temp > 1.0 ? 1.0 : temp);
      const int mc = 1 + static_cast<int>(floor(__dmul_rn(static_cast<double>(G - 1), temp)));
      ns = uniform_int_serial(f.rng, 1, mc > 1 ? mc : 1);
    }
    f.ns = ns;
    P.proposal_size[static_cast<size_t>(prob) * T + cycle] = ns;
  }
  __syncthreads();
  shuffle_targets_block(f, s.jarr, G, s.raw);
  const int ns = f.ns;
  if (ns > 0) {
    bucket_steps_block(s, G, ns);
    if (P.singleton && P.pol_guidance) {
      for (int g = threadIdx.x; g < G; g += kThreads) {
        const int row = s.f->gmem[g];
        if (s.curpred[row] == s.cur[row]) continue;
        if (s.f->fxd != nullptr && s.f->fxd[row] == 1) continue;
        if (final_position_of(s, g, ns) < ns) s.cl[row] = s.curpred[row];
      }
    } else {
      for (int q = threadIdx.x; q < ns; q += kThreads) s.perm[q] = static_cast<uint16_t>(occupant_of(s, G, q));
      __syncthreads();
      if (threadIdx.x == 0) relabel_serial(P, s, s.curpred, ns, C0);
    }
  }
  __syncthreads();
  const bool attempt_co = P.pol_transition && Q.coarsening && Q.pol_coarsen;
  const bool attempt_ab = P.pol_transition && P.absorption;
  int coarsened = 0, absorbed = 0;
  if (attempt_co) coarsened = coarsening_block(Q, s, prob, s.curpred, C0);
  if (attempt_ab) absorbed = absorption_block(P, s, prob, s.curpred, C0);
  if (threadIdx.x == 0) {
    if (attempt_co || attempt_ab) ++st.tr_att;
    if (attempt_co) {
      ++st.co_att;
      st.co_moves += coarsened;
    }
    if (attempt_ab) {
      ++st.m1_att;
      st.absorb_moves += absorbed;
    }
    st.coarsened = coarsened;
    st.absorbed = absorbed;
  }
  __syncthreads();
  class_lists(Q, s, prob, C0);
}

__device__ void pls_step(const EvolvePlsParams& Q, const Smem& s, int prob) {
  const EvolveParams& P = Q.base;
  Fixed& f = *s.f;
  bind_groups(P, s, prob);
  const int L = P.L, T = P.T;
  const int C0 = P.ncodes[prob];
  const size_t ro = static_cast<size_t>(prob) * L;
  PlsRunState& gst = Q.state[prob];
  __shared__ PlsRunState st;
  if (Q.phase == 0) {
    if (threadIdx.x == 0) {
      mt64_seed(f.rng, P.seeds[prob]);
      st = PlsRunState{};
    }
    for (int r = threadIdx.x; r < L; r += kThreads) {
      s.cl[r] = P.init[ro + r];
      Q.cl[ro + r] = s.cl[r];
    }
    __syncthreads();
    class_lists(Q, s, prob, C0);
  } else {
    const int cycle = Q.cycle;  // proposal `cycle - 1` was evaluated (cycle 0: the initial labels)
    const Mt64State& g = Q.rng[prob];
    for (int i = threadIdx.x; i < kMtN; i += kThreads) {
      f.rng.mt[i] = g.mt[i];
      f.rng.out[i] = g.out[i];
    }
    if (threadIdx.x == 0) {
      f.rng.pos = g.pos;
      st = gst;
    }
    for (int r = threadIdx.x; r < L; r += kThreads) {
      s.cl[r] = Q.cl[ro + r];
      s.pred[r] = Q.pred[ro + r];
      if (cycle > 0) {
        s.cur[r] = Q.cur[ro + r];
        s.curpred[r] = Q.curpred[ro + r];
      }
    }
    __syncthreads();
    uint16_t* gbest = P.clbest + ro;
    uint16_t* gbestpred = P.cvpredbest + ro;
    int ok = 0;
    for (int r = threadIdx.x; r < L; r += kThreads) ok += s.cl[r] == s.pred[r];
    ok = block_sum(ok, f);
    const double acc = __ddiv_rn(static_cast<double>(ok), static_cast<double>(L));
    const int nc = label_census(P, s, s.cl, C0);
    const double score = objective_pls(Q, s, prob, acc, nc, C0);
    if (cycle == 0) {
      for (int r = threadIdx.x; r < L; r += kThreads) {
        s.cur[r] = s.cl[r];
        s.curpred[r] = s.pred[r];
        gbest[r] = s.cl[r];
        gbestpred[r] = s.pred[r];
      }
      if (threadIdx.x == 0) {
        st.accbest = st.cur_acc = acc;
        st.scorebest = st.cur_score = score;
        st.nc_cur = st.nc_best = nc;
      }
    } else {
      const int c = cycle - 1;
      if (threadIdx.x == 0) {
        ++st.proposals;
        const bool improves = score > st.scorebest;
        int accepted = improves, improving = improves, stoch = 0;
        if (P.evolutionary) {
          const double cooling = __dsub_rn(1.0, __ddiv_rn(static_cast<double>(c + 1), static_cast<double>(T > 1 ? T : 1)));
          const double one_minus = __dsub_rn(1.0, st.cur_acc);
          const double clipped = (0.0 < one_minus) ? one_minus : 0.0;
          const double t0 = __dmul_rn(__dmul_rn(0.10, clipped), cooling);
          const double temperature = (1.0e-9 < t0) ? t0 : 1.0e-9;
          int acc_cur = score >= st.cur_score;
          improving = acc_cur;
          if (!acc_cur && P.pol_stochastic && temperature > 1.0e-9) {
            ++st.st_att;
            const double u = canonical_serial(f.rng);
            acc_cur = u < exp(__ddiv_rn(__dsub_rn(score, st.cur_score), temperature));
            stoch = acc_cur;
          }
          accepted = acc_cur;
        }
        f.accept = accepted | (improves << 1) | (stoch << 2) | (improving << 3);
        if (improves) {
          st.accbest = acc;
          st.scorebest = score;
          ++st.best_updates;
          st.nc_best = nc;
        }
        if (P.evolutionary) {
          if (accepted) {
            st.cur_acc = acc;
            st.cur_score = score;
            st.nc_cur = nc;
            ++st.accepts;
            if (stoch) ++st.st_acc;
          } else {
            ++st.rejections;
          }
        }
        if (accepted && (st.coarsened || st.absorbed)) {
          ++st.tr_acc;
          if (st.coarsened) ++st.co_acc;
          if (st.absorbed) ++st.m1_acc;
        }
        uint8_t* fl = P.flags + (static_cast<size_t>(prob) * T + c) * 3;
        fl[0] = accepted ? 1 : 0;
        fl[1] = (accepted && improving) ? 1 : 0;
        fl[2] = stoch ? 1 : 0;
        P.active[static_cast<size_t>(prob) * T + c] = P.evolutionary ? st.nc_cur : st.nc_best;
        P.vect_acc[static_cast<size_t>(prob) * T + c] = st.accbest;
        P.vect_score[static_cast<size_t>(prob) * T + c] = st.scorebest;
        if (acc == 1.0 && isfinite(score)) st.success = 1;
      }
      __syncthreads();
      const int code = f.accept;
      const bool improves = (code >> 1) & 1;
      const bool take = P.evolutionary ? (code & 1) : improves;
      if (improves) {
        for (int r = threadIdx.x; r < L; r += kThreads) {
          gbest[r] = s.cl[r];
          gbestpred[r] = s.pred[r];
        }
      }
      if (take) {
        for (int r = threadIdx.x; r < L; r += kThreads) {
          s.cur[r] = s.cl[r];
          s.curpred[r] = s.pred[r];
        }
      }
      __syncthreads();
    }
    if (cycle == T) {
      // the rows of the best labels by code, for the projection
      __syncthreads();
      for (int r = threadIdx.x; r < L; r += kThreads) s.cl[r] = gbest[r];
      __syncthreads();
      class_lists(Q, s, prob, C0);
    }
    if (cycle < T) {
      pls_propose(Q, s, prob, cycle, st, C0);
      for (int r = threadIdx.x; r < L; r += kThreads) Q.cl[ro + r] = s.cl[r];
    } else if (threadIdx.x == 0) {
      int* c = P.counters + static_cast<size_t>(prob) * 18;
      c[0] = T;
      c[1] = st.proposals;
      c[2] = st.best_updates;
      c[3] = st.accepts;
      c[4] = st.st_att;
      c[5] = st.st_acc;
      c[6] = st.rejections;
      c[7] = st.co_moves;
      c[8] = st.absorb_moves;
      c[9] = st.tr_att;
      c[10] = st.tr_acc;
      c[11] = st.m1_att;
      c[12] = st.m1_acc;
      c[13] = st.proposals + 1;
      c[14] = st.success;
      c[15] = 0;
      c[16] = st.co_att;
      c[17] = st.co_acc;
      P.best[2 * prob] = st.accbest;
      P.best[2 * prob + 1] = st.scorebest;
      P.status[prob] = 0;
    }
    for (int r = threadIdx.x; r < L; r += kThreads) {
      Q.cur[ro + r] = s.cur[r];
      Q.curpred[ro + r] = s.curpred[r];
    }
  }
  __syncthreads();
  Mt64State& g = Q.rng[prob];
  for (int i = threadIdx.x; i < kMtN; i += kThreads) {
    g.mt[i] = f.rng.mt[i];
    g.out[i] = f.rng.out[i];
  }
  if (threadIdx.x == 0) {
    g.pos = f.rng.pos;
    gst = st;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kThreads, 1) evolve_pls_kernel(EvolvePlsParams Q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem s = carve_smem(Q.base, smem_raw);
  const int C = Q.base.C0max;
  for (int prob = blockIdx.x; prob < Q.base.problems; prob += gridDim.x) {
    if (!Q.base.smem_trans) s.trans = Q.base.trans + static_cast<size_t>(prob) * C * C;
    pls_step(Q, s, prob);
  }
}

}  // namespace

size_t evolve_smem_bytes(int L, int C0max, bool rows_in_smem, bool trans_in_smem) {
  auto al = [](size_t v) { return (v + 15) / 16 * 16; };
  size_t b = al(sizeof(Fixed));
  b += 6 * al(sizeof(int) * C0max) + al(sizeof(int) * (C0max + 1));
  b += 2 * al(sizeof(double) * C0max) + al(sizeof(double) * 2 * C0max);
  if (trans_in_smem) b += al(sizeof(int) * static_cast<size_t>(C0max) * C0max);
  if (rows_in_smem) b += kRowArrays * ((static_cast<size_t>(L) + 7) / 8 * 8) * sizeof(uint16_t);
  return b;
}

int evolve_pls_launch(const EvolvePlsParams& q, int grid, size_t smem, void* stream) {
  cudaError_t e = cudaFuncSetAttribute(evolve_pls_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return static_cast<int>(e);
  evolve_pls_kernel<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(q);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int evolve_launch(const EvolveParams& p, int grid, size_t smem, void* stream) {
  cudaError_t e = cudaFuncSetAttribute(evolve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return static_cast<int>(e);
  evolve_kernel<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(p);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
