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

#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

namespace kgb {

namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr unsigned kFull = 0xffffffffu;

struct Fixed {
  Mt64State rng;
  uint16_t jbuf[2 * kMtN];
  int first_reject;
  int ns;
  int red_i[kWarps];
  int flag;
  int nc;          // distinct labels of the proposal
  int changed_cnt;
  int moves_sel;
  int n_empty;
  int selected_target;
  double acc;
  double score;
  int accept;
  int improves;
};

struct Smem {
  Fixed* f;
  uint16_t* cl;      // proposal
  uint16_t* cur;     // current state (evolutionary) or best state (greedy)
  uint16_t* curpred; // CV predictions of cur
  uint16_t* pred;    // CV predictions of the proposal
  uint16_t* perm;    // shuffled group ids
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
// Group shuffle (std::shuffle of iota(G) with a 64-bit engine): for an engine
// range wider than G^2 the draws come two at a time, one downscaled draw over
// (i+1)*(i+2) giving the swap targets of positions i and i+1 (quotient and
// remainder by i+2); an even G first swaps position 1 with a draw over {0,1}.
// Positions >= i are untouched before step i, so each swap is "place i at j
// and move the old occupant of j to i".  Warp 0 computes the targets of up to
// 312 pairs in parallel from one engine block; lane 0 applies them in order.
// ---------------------------------------------------------------------------
__device__ void shuffle_groups_warp(Fixed& f, uint16_t* perm, int G, int lane) {
  int i = 1;
  if (G >= 2 && (G & 1) == 0) {
    if (lane == 0) {
      const int j = static_cast<int>(draw_below_serial(f.rng, 2));
      const uint16_t t = perm[j];
      perm[1] = t;
      perm[j] = 1;
    }
    i = 2;
  }
  __syncwarp();
  while (i < G) {
    if (f.rng.pos >= kMtN) mt64_refill_warp(f.rng, lane);
    const int pos = f.rng.pos;
    const int np = min(kMtN - pos, (G - i) >> 1);
    if (lane == 0) f.first_reject = np;
    __syncwarp();
    for (int p = lane; p < np; p += 32) {
      const uint64_t b0 = static_cast<uint64_t>(i + 2 * p) + 1ull;
      const uint64_t b1 = b0 + 1ull;
      const uint64_t range = b0 * b1;
      const uint64_t u = f.rng.out[pos + p];
      const uint64_t lo = u * range;
      bool rej = false;
      if (lo < range) {
        const uint64_t thr = (0ull - range) % range;
        rej = lo < thr;
      }
      if (rej) {
        atomicMin(&f.first_reject, p);
      } else {
        const uint64_t x = __umul64hi(u, range);
        f.jbuf[2 * p] = static_cast<uint16_t>(x / b1);
        f.jbuf[2 * p + 1] = static_cast<uint16_t>(x % b1);
      }
    }
    __syncwarp();
    const int r = f.first_reject;
    if (lane == 0) {
      for (int p = 0; p < r; ++p) {
        const int a = i + 2 * p;
        int j = f.jbuf[2 * p];
        uint16_t t = perm[j];
        perm[a] = t;
        perm[j] = static_cast<uint16_t>(a);
        j = f.jbuf[2 * p + 1];
        t = perm[j];
        perm[a + 1] = t;
        perm[j] = static_cast<uint16_t>(a + 1);
      }
      f.rng.pos = pos + r + (r < np ? 1 : 0);
    }
    i += 2 * r;
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Fold vote: one warp per row, one lane per neighbour slot.  Winner: largest
// count, then largest double score sum (neighbour order), then smallest code.
// Rows with no out-of-fold neighbour take the majority label of their
// training folds (ties to the smaller label).
// ---------------------------------------------------------------------------
__device__ void vote_block(const EvolveParams& P, const Smem& s, int prob, const uint16_t* lab,
                           uint16_t* out, int C0, bool has_empty) {
  const int L = P.L, w = P.w;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint16_t* nbp = P.nb + static_cast<size_t>(prob) * L * w;
  const float* scp = P.sc + static_cast<size_t>(prob) * L * w;
  for (int r = warp; r < L; r += kWarps) {
    const uint16_t id = lane < w ? nbp[static_cast<size_t>(r) * w + lane] : kNoRow;
    const int code = id != kNoRow ? static_cast<int>(lab[id]) : -1;
    const unsigned valid = __ballot_sync(kFull, code >= 0);
    if (valid == 0u) continue;  // empty row, fallback below
    const unsigned m = __match_any_sync(kFull, code);
    const int cnt = code >= 0 ? __popc(m) : 0;
    const int maxc = __reduce_max_sync(kFull, cnt);
    const bool leader = code >= 0 && cnt == maxc && (__ffs(m) - 1) == lane;
    const unsigned leaders = __ballot_sync(kFull, leader);
    int best;
    if (__popc(leaders) == 1) {
      best = __shfl_sync(kFull, code, __ffs(leaders) - 1);
    } else {
      const float my = lane < w ? scp[static_cast<size_t>(r) * w + lane] : 0.0f;
      double sum = 0.0;
      for (int t = 0; t < w; ++t) {
        const float st = __shfl_sync(kFull, my, t);
        if (leader && ((m >> t) & 1u)) sum = __dadd_rn(sum, static_cast<double>(st));
      }
      double bs = sum;
      int bc = leader ? code : 0x7fffffff;
      int bv = leader ? 1 : 0;
      for (int off = 16; off > 0; off >>= 1) {
        const double os = __shfl_xor_sync(kFull, bs, off);
        const int oc = __shfl_xor_sync(kFull, bc, off);
        const int ov = __shfl_xor_sync(kFull, bv, off);
        if (ov && (!bv || os > bs || (os == bs && oc < bc))) {
          bs = os;
          bc = oc;
          bv = 1;
        }
      }
      best = bc;
    }
    if (lane == 0) out[r] = static_cast<uint16_t>(best);
  }
  if (has_empty) {
    // per-fold training majority (codes in [0, C0))
    int* fc = P.foldcnt + static_cast<size_t>(prob) * P.F * P.C0max;
    for (int i = threadIdx.x; i < P.F * P.C0max; i += kThreads) fc[i] = 0;
    for (int c = threadIdx.x; c < C0; c += kThreads) s.aux[c] = 0;
    __syncthreads();
    const uint8_t* fo = P.folds + static_cast<size_t>(prob) * L;
    for (int r = threadIdx.x; r < L; r += kThreads) {
      atomicAdd(&fc[fo[r] * P.C0max + lab[r]], 1);
      atomicAdd(&s.aux[lab[r]], 1);
    }
    __syncthreads();
    for (int fo_i = threadIdx.x; fo_i < P.F; fo_i += kThreads) {
      int bl = 0, bcount = -1;
      for (int c = 0; c < C0; ++c) {
        const int count = s.aux[c] - fc[fo_i * P.C0max + c];
        if (count > bcount) {  // ascending codes: ties keep the smaller label
          bl = c;
          bcount = count;
        }
      }
      s.order[fo_i] = bl;  // order[] is free here; F <= C0max guaranteed by host
    }
    __syncthreads();
    for (int r = threadIdx.x; r < L; r += kThreads) {
      if (nbp[static_cast<size_t>(r) * w] == kNoRow) out[r] = static_cast<uint16_t>(s.order[fo[r]]);
    }
  }
  __syncthreads();
}

// Count labels of `lab` per code, first positions and distinct count.
__device__ int label_census(const EvolveParams& P, const Smem& s, const uint16_t* lab, int C0) {
  for (int c = threadIdx.x; c < C0; c += kThreads) {
    s.cnt[c] = 0;
    s.firstpos[c] = 0x7fffffff;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < P.L; r += kThreads) {
    atomicAdd(&s.cnt[lab[r]], 1);
    atomicMin(&s.firstpos[lab[r]], r);
  }
  __syncthreads();
  int local = 0;
  for (int c = threadIdx.x; c < C0; c += kThreads) local += s.cnt[c] > 0;
  return block_sum(local, *s.f);
}

// core_objective_score for the kNN classifier; census must be current.
__device__ double objective(const EvolveParams& P, const Smem& s, int prob, double acc, int nc, int C0) {
  const bool use_div = P.guarded && P.pol_diversity;
  const bool reject1 = P.guarded && P.pol_reject1;
  if (!use_div && !reject1) return acc;
  if (reject1 && nc == 1) return -INFINITY;
  if (!use_div) return acc;
  // iteration order of std::unordered_map<int,int> after reserve(L) and
  // insertion in row order
  const bool nocollide = P.nocollide[prob] != 0;
  if (nocollide) {
    // every key has its own bucket: each new key goes to the list front
    for (int c = threadIdx.x; c < C0; c += kThreads) {
      if (s.cnt[c] == 0) continue;
      int rank = 0;
      const int fp = s.firstpos[c];
      for (int c2 = 0; c2 < C0; ++c2) rank += (s.cnt[c2] > 0 && s.firstpos[c2] > fp);
      s.order[rank] = c;
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
  if (threadIdx.x == 0) {
    const double n = static_cast<double>(P.L);
    double same = 0.0;
    for (int q = 0; q < nc; ++q) {
      const double p = __ddiv_rn(static_cast<double>(s.cnt[s.order[q]]), n);
      same = __dadd_rn(same, __dmul_rn(p, p));
    }
    const double diff = __dsub_rn(1.0, same);
    const double dlp = (0.0 < diff) ? diff : 0.0;
    s.f->score = __dmul_rn(acc, __dsqrt_rn(dlp));
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
  int* tr = P.trans + static_cast<size_t>(prob) * P.C0max * P.C0max;
  const int C = P.C0max;
  for (int i = threadIdx.x; i < C0 * C; i += kThreads) tr[(i / C) * C + (i % C)] = 0;
  for (int c = threadIdx.x; c < C0; c += kThreads) {
    s.cnt[c] = 0;
    s.movable[c] = 0;
    s.bt[c] = -1;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < P.L; r += kThreads) {
    const int a = s.cl[r];
    atomicAdd(&s.cnt[a], 1);
    atomicAdd(&tr[a * C + pp[r]], 1);
    if (P.fixed == nullptr || P.fixed[r] != 1) atomicAdd(&s.movable[a], 1);
  }
  __syncthreads();
  int local = 0;
  for (int c = threadIdx.x; c < C0; c += kThreads) local += s.cnt[c] > 0;
  const int nc = block_sum(local, f);
  if (nc <= 2) return 0;
  const double n = static_cast<double>(P.L);
  const double nmax = (1.0 < n) ? n : 1.0;  // std::max(1.0, n)
  for (int src = threadIdx.x; src < C0; src += kThreads) {
    const int ssize = s.cnt[src];
    if (ssize == 0 || s.movable[src] <= 0) continue;
    const int* row = tr + src * C;
    const int stay = row[src];
    int bt = src, bcount = 0, bsize = ssize;
    double bsur = 0.0;
    for (int dst = 0; dst < C0; ++dst) {
      const int cntd = row[dst];
      if (dst == src || cntd == 0) continue;
      const int dsize = s.cnt[dst];
      if (dsize == 0) continue;
      const double expected = __ddiv_rn(__dmul_rn(static_cast<double>(ssize), static_cast<double>(dsize)), nmax);
      const double sur = __dsub_rn(static_cast<double>(cntd), expected);
      if (sur > bsur || (sur == bsur && cntd > bcount) ||
          (sur == bsur && cntd == bcount && dsize > bsize) ||
          (sur == bsur && cntd == bcount && dsize == bsize && dst < bt)) {
        bt = dst;
        bsize = dsize;
        bcount = cntd;
        bsur = sur;
      }
    }
    if (bt == src || bsur <= 0.0 || bcount <= stay) continue;
    s.bt[src] = bt;
    s.bsur[src] = bsur;
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
      if (P.fixed != nullptr && P.fixed[r] == 1) continue;
      if (a != sel && s.bt[a] == sel) s.cl[r] = static_cast<uint16_t>(sel);
    }
  }
  __syncthreads();
  return apply;
}

// Relabel of sampled groups when draws are needed (groups of several rows, or
// no prediction guidance).  Thread 0, in shuffled order.
__device__ void relabel_serial(const EvolveParams& P, const Smem& s, const uint16_t* pp, int ns, int C0) {
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
    const int beg = P.goff[g], end = P.goff[g + 1];
    int neligible = 0;
    for (int a = beg; a < end; ++a) neligible += (P.fixed == nullptr || P.fixed[P.gmem[a]] != 1);
    if (neligible == 0) continue;
    int rep;
    if (P.pol_guidance) {
      // candidate labels: predictions of the eligible members, ascending, with counts
      int k = 0;
      for (int a = beg; a < end; ++a) {
        const int row = P.gmem[a];
        if (P.fixed != nullptr && P.fixed[row] == 1) continue;
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
      const int row = P.gmem[a];
      if (P.fixed != nullptr && P.fixed[row] == 1) continue;
      s.cl[row] = static_cast<uint16_t>(rep);
    }
  }
}

__device__ void evolve_problem(const EvolveParams& P, const Smem& s, int prob) {
  Fixed& f = *s.f;
  const int L = P.L, T = P.T, G = P.G;
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

  if (threadIdx.x == 0) mt64_seed(f.rng, P.seeds[prob]);
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
    // proposal = current (evolutionary) or best (greedy) state; s.cur holds it
    for (int r = threadIdx.x; r < L; r += kThreads) s.cl[r] = s.cur[r];
    for (int g = threadIdx.x; g < G; g += kThreads) s.perm[g] = static_cast<uint16_t>(g);
    __syncthreads();
    if (warp == 0) {
      if (lane == 0) {
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
      __syncwarp();
      shuffle_groups_warp(f, s.perm, G, lane);
    }
    __syncthreads();
    const int ns = f.ns;
    psize[cycle] = ns;  // every thread writes the same value
    if (P.singleton && P.pol_guidance) {
      for (int q = threadIdx.x; q < ns; q += kThreads) {
        const int row = P.gmem[s.perm[q]];
        if (P.fixed != nullptr && P.fixed[row] == 1) continue;
        s.cl[row] = s.curpred[row];
      }
    } else if (threadIdx.x == 0) {
      relabel_serial(P, s, s.curpred, ns, C0);
    }
    __syncthreads();

    int absorbed = 0;
    if (P.pol_transition && P.absorption) {
      ++tr_att;
      absorbed = absorption_block(P, s, prob, s.curpred, C0);
      absorb_moves += absorbed;
    }

    vote_block(P, s, prob, s.cl, s.pred, C0, has_empty);
    ok = 0;
    for (int r = threadIdx.x; r < L; r += kThreads) ok += s.cl[r] == s.pred[r];
    ok = block_sum(ok, f);
    const double acc = __ddiv_rn(static_cast<double>(ok), n);
    const int nc = label_census(P, s, s.cl, C0);
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

__global__ void __launch_bounds__(kThreads, 1) evolve_kernel(EvolveParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
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
  for (int prob = blockIdx.x; prob < P.problems; prob += gridDim.x) {
    uint16_t* rows;
    if (P.smem_rows) {
      rows = reinterpret_cast<uint16_t*>(smem_raw + off);
    } else {
      rows = P.rows_scratch + static_cast<size_t>(blockIdx.x) * 5 * Lp;
    }
    s.cl = rows;
    s.cur = rows + Lp;
    s.curpred = rows + 2 * Lp;
    s.pred = rows + 3 * Lp;
    s.perm = rows + 4 * Lp;
    evolve_problem(P, s, prob);
  }
}

}  // namespace

size_t evolve_smem_bytes(int L, int C0max, bool rows_in_smem) {
  auto al = [](size_t v) { return (v + 15) / 16 * 16; };
  size_t b = al(sizeof(Fixed));
  b += 6 * al(sizeof(int) * C0max) + al(sizeof(int) * (C0max + 1));
  b += 2 * al(sizeof(double) * C0max) + al(sizeof(double) * 2 * C0max);
  if (rows_in_smem) b += 5 * ((static_cast<size_t>(L) + 7) / 8 * 8) * sizeof(uint16_t);
  return b;
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
