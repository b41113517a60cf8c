// Per-run landmark planning on the device.
//
//   strata_kernel (one CTA): index_strata (kodama_matrix.cpp:806-854): the
//     rows of every atlas cluster in ascending row order (counting sort, the
//     stable scatter done by one warp with __match_any_sync ranks), and the
//     run-independent parts of the quota allocation
//     (kodama_matrix.cpp:880-903): floor of target*count/n and its fractional
//     part, both in x86 extended precision (ext80.h).
//   plan_runs_kernel (one CTA per run): the run's std::mt19937_64 stream
//     (seed + run, one output discarded), the shuffle of the non-empty strata,
//     the systematic residual allocation, std::sample inside each stratum
//     (selection sampling with two positions per draw), then the init k-means
//     seed; the selected rows are compacted in ascending order by the whole
//     CTA, and the first init_k entries of the FAISS-compatible permutation
//     (std::mt19937 seeded (draw & 0x7fffffff) + 1, swaps r <-> r + u % (L-r),
//     kodama_matrix.cpp:535-564) give the initial centroid rows.
//
// The serial parts restate the libstdc++ 13 algorithms the reference calls:
// std::shuffle and std::sample draw two positions per engine call when the
// engine range allows it (uniform integer in [0, b0*b1) split as x / b1,
// x % b1), and uniform_int_distribution downscales one 64-bit output by
// Lemire's method (rng.cuh).
#include "ext80.h"
#include "launch_count.cuh"
#include "plan.cuh"
#include "rng.cuh"

namespace kgb {
namespace {

constexpr int kPlanThreads = 256;
constexpr int kSharedStrata = 8192;  // cursor/histogram in shared memory up to this many strata
constexpr int kRounded = 0x40000000;  // marks a stratum of the shuffled order that took a residual slot

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

struct PlanScratch {
  int* counts;    // strata
  int* offsets;   // strata + 1
  int* cursor;    // strata
  int* rows;      // n
  int* base;      // strata
  Ext80* frac;    // strata
  int* assigned;  // 1
  int* order;     // runs x strata
  int* quota;     // runs x strata
  uint8_t* flags; // runs x n
  int* perm;      // runs x target
};

PlanScratch carve(const PlanArgs& a) {
  PlanScratch s{};
  char* p = static_cast<char*>(a.scratch);
  auto take = [&](size_t bytes) {
    char* q = p;
    p += align256(bytes);
    return q;
  };
  const size_t S = static_cast<size_t>(a.strata), R = static_cast<size_t>(a.runs);
  s.counts = reinterpret_cast<int*>(take(sizeof(int) * S));
  s.offsets = reinterpret_cast<int*>(take(sizeof(int) * (S + 1)));
  s.cursor = reinterpret_cast<int*>(take(sizeof(int) * S));
  s.rows = reinterpret_cast<int*>(take(sizeof(int) * a.n));
  s.base = reinterpret_cast<int*>(take(sizeof(int) * S));
  s.frac = reinterpret_cast<Ext80*>(take(sizeof(Ext80) * S));
  s.assigned = reinterpret_cast<int*>(take(sizeof(int)));
  s.order = reinterpret_cast<int*>(take(sizeof(int) * S * R));
  s.quota = reinterpret_cast<int*>(take(sizeof(int) * S * R));
  s.flags = reinterpret_cast<uint8_t*>(take(static_cast<size_t>(a.n) * R));
  s.perm = reinterpret_cast<int*>(take(sizeof(int) * static_cast<size_t>(a.target) * R));
  return s;
}

__global__ void __launch_bounds__(1024) strata_kernel(PlanArgs a, PlanScratch s) {
  __shared__ int sh_count[kSharedStrata];
  __shared__ int bad;
  __shared__ unsigned long long asum;
  const int tid = threadIdx.x;
  const bool in_shared = a.strata <= kSharedStrata;
  int* count = in_shared ? sh_count : s.counts;
  if (tid == 0) {
    bad = 0;
    asum = 0;
  }
  for (int t = tid; t < a.strata; t += blockDim.x) count[t] = 0;
  __syncthreads();
  for (int r = tid; r < a.n; r += blockDim.x) {
    const int l = a.atlas[r];
    if (l < 1 || l > a.strata) {
      bad = 1;
      continue;
    }
    atomicAdd(&count[l - 1], 1);
  }
  __syncthreads();
  if (bad) {
    if (tid == 0) atomicExch(a.status, 1);
    return;
  }
  // exclusive scan of the counts (one warp); the cursor starts at the offsets
  if (tid < 32) {
    int carry = 0;
    for (int b = 0; b < a.strata; b += 32) {
      const int t = b + tid;
      const int c = t < a.strata ? count[t] : 0;
      int v = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (tid >= o) v += y;
      }
      if (t < a.strata) s.offsets[t] = carry + v - c;
      carry += __shfl_sync(0xffffffffu, v, 31);
    }
    if (tid == 0) s.offsets[a.strata] = carry;
  }
  __syncthreads();
  for (int t = tid; t < a.strata; t += blockDim.x) count[t] = s.offsets[t];  // count becomes the cursor
  __syncthreads();
  // stable scatter: rows of one stratum keep ascending order (one warp; the
  // labels of eight 32-row steps are loaded ahead of their step)
  if (tid < 32) {
    for (int b0 = 0; b0 < a.n; b0 += 8 * 32) {
      int lv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int r = b0 + 32 * u + tid;
        lv[u] = r < a.n ? a.atlas[r] - 1 : -1;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int r = b0 + 32 * u + tid;
        const bool valid = r < a.n;
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (valid) {
          const int l = lv[u];
          const unsigned m = __match_any_sync(act, l);
          const int leader = __ffs(m) - 1;
          const int rank = __popc(m & ((1u << tid) - 1u));
          int pos = 0;
          if (tid == leader) {
            pos = count[l];
            count[l] = pos + __popc(m);
          }
          pos = __shfl_sync(act, pos, leader);
          s.rows[pos + rank] = r;
        }
        __syncwarp();
      }
    }
  }
  // quota parts (run-independent)
  const Ext80 total = ext80_from_u64(static_cast<uint64_t>(a.n));
  unsigned long long local = 0;
  for (int t = tid; t < a.strata; t += blockDim.x) {
    const int c = s.offsets[t + 1] - s.offsets[t];
    int base = 0;
    Ext80 frac{0, 0};
    if (c > 0) {
      const Ext80 expected =
          ext80_div(ext80_from_u64(static_cast<uint64_t>(a.target) * static_cast<uint64_t>(c)), total);
      base = min(c, ext80_floor_int(expected));
      frac = ext80_sub(expected, ext80_from_u64(static_cast<uint64_t>(base)));
    }
    s.base[t] = base;
    s.frac[t] = frac;
    local += static_cast<unsigned long long>(base);
  }
  atomicAdd(&asum, local);
  __syncthreads();
  if (tid == 0) *s.assigned = static_cast<int>(asum);
}

// x / b and x % b: 32-bit division when both fit.
__device__ __forceinline__ void divmod_u64(uint64_t x, uint64_t b, uint64_t& q, uint64_t& r) {
  if (x <= 0xffffffffull) {
    const uint32_t x32 = static_cast<uint32_t>(x), b32 = static_cast<uint32_t>(b);
    const uint32_t q32 = x32 / b32;
    q = q32;
    r = x32 - q32 * b32;
  } else {
    q = x / b;
    r = x % b;
  }
}

// std::shuffle of a[0..n) (random-access, 64-bit engine): one swap with a
// {0,1} draw first when n is even, then pairs from one draw each.
__device__ void shuffle_serial(int* a, int n, Mt64State& rng) {
  if (n <= 0) return;
  int i = 1;
  if ((n % 2) == 0) {
    const int j = static_cast<int>(draw_below_serial(rng, 2));
    const int t = a[i];
    a[i] = a[j];
    a[j] = t;
    ++i;
  }
  while (i != n) {
    const uint64_t r = static_cast<uint64_t>(i) + 1;
    uint64_t p1, p2;
    divmod_u64(draw_below_serial(rng, r * (r + 1)), r + 1, p1, p2);
    int t = a[i];
    a[i] = a[p1];
    a[p1] = t;
    ++i;
    t = a[i];
    a[i] = a[p2];
    a[p2] = t;
    ++i;
  }
}

// Lemire draw in [0, range) by a whole warp in lockstep (every lane computes
// the same value; the warp regenerates the state block when it runs out).
__device__ uint64_t draw_below_warp(Mt64State& rng, uint64_t range, int lane) {
  for (;;) {
    if (rng.pos >= kMtN) mt64_refill_warp(rng, lane);
    const uint64_t u = rng.out[rng.pos];
    __syncwarp();
    if (lane == 0) rng.pos += 1;
    __syncwarp();
    const uint64_t lo = u * range;
    if (lo >= range || lo >= (0ull - range) % range) return __umul64hi(u, range);
  }
}

// Shared state of one std::sample call run by the whole CTA.
struct __align__(16) SampleShared {
  uint32_t p1[kMtN];  // the two acceptance positions of each step of a batch
  uint32_t p2[kMtN];
  uint16_t sel[kMtN]; // the walk's decisions: bit 0 the first row of a step, bit 8 the second
  long long uns, nq;  // rows not yet visited, rows still wanted
  int i, taken;       // next row of the stratum, rows taken so far
  int rej;            // first step of the batch whose draw Lemire's method rejects
  int visited;        // rows the batch's walk visited
  int redraw;         // the rejected step is next and is drawn one output at a time
};

// std::sample of q rows out of the size rows starting at position first of
// the strata row list (forward population): selection sampling, two
// acceptance positions per draw while two or more rows remain.  The whole CTA
// in batches: a step's range depends only on how many rows remain, so the
// threads draw the acceptance positions of up to the rest of the engine's
// output block at once (one output per step); thread 0 then walks the
// acceptance recursion over them in order -- a compare and a decrement per
// row, the decisions stored as bytes -- and the CTA flags the taken rows.  A
// draw that Lemire's method would reject (probability about range / 2^64)
// ends the batch; warp 0 redraws that step one output at a time, as it does
// the single draws once fewer than two rows remain.  Called by every thread;
// the count of rows taken is returned to thread 0.
__device__ int sample_cta(int first, int size, int q, const int* __restrict__ rows, uint8_t* __restrict__ flags,
                          Mt64State& rng, SampleShared& ss, int tid) {
  if (size <= 0) return 0;
  const int lane = tid & 31;
  if (tid == 0) {
    ss.uns = size;
    ss.nq = q < size ? q : size;
    ss.i = 0;
    ss.taken = 0;
  }
  __syncthreads();
  long long uns = 0, nq = 0;
  for (;;) {
    uns = ss.uns;
    nq = ss.nq;
    const int pos0 = rng.pos, i0 = ss.i;
    __syncthreads();  // every thread has read the state before it changes
    if (nq == 0 || uns < 2) break;
    if (pos0 >= kMtN) {
      if (tid < 32) mt64_refill_warp(rng, lane);
      __syncthreads();
    }
    const int pos = pos0 >= kMtN ? 0 : pos0;
    const long long steps_left = uns / 2;
    const int batch = static_cast<int>(kMtN - pos < steps_left ? kMtN - pos : steps_left);
    if (tid == 0) ss.rej = batch;
    __syncthreads();
    for (int j = tid; j < batch; j += kPlanThreads) {
      const long long ul = uns - 2LL * j;
      const uint64_t b1 = static_cast<uint64_t>(ul - 1);
      const uint64_t range = static_cast<uint64_t>(ul) * b1;
      const uint64_t u = rng.out[pos + j];
      const uint64_t lo = u * range;
      if (lo < range && lo < (0ull - range) % range) atomicMin(&ss.rej, j);
      uint64_t p1, p2;
      divmod_u64(__umul64hi(u, range), b1, p1, p2);
      ss.p1[j] = static_cast<uint32_t>(p1);
      ss.p2[j] = static_cast<uint32_t>(p2);
    }
    __syncthreads();
    if (tid == 0) {
      // nq <= size < 2^31: 32-bit counters; after a step that ends the sample
      // (nn == 0) nothing more is taken, and the step's second row counts as
      // visited only if the first did not end it
      const int usable = ss.rej;
      uint32_t nn = static_cast<uint32_t>(nq), n1 = nn;
      int l = 0;
      bool done = false;
      // eight steps per pass without branches: once nn reaches 0 every later
      // compare fails and nn stays 0, so the pass runs to its end and the
      // step that ended the sample (and its n1) is picked out afterwards;
      // p1, p2 and sel start 16-byte aligned
      for (; l + 8 <= usable; l += 8) {
        const uint4 P0 = *reinterpret_cast<const uint4*>(ss.p1 + l);
        const uint4 P1 = *reinterpret_cast<const uint4*>(ss.p1 + l + 4);
        const uint4 Q0 = *reinterpret_cast<const uint4*>(ss.p2 + l);
        const uint4 Q1 = *reinterpret_cast<const uint4*>(ss.p2 + l + 4);
        const uint32_t a1[8] = {P0.x, P0.y, P0.z, P0.w, P1.x, P1.y, P1.z, P1.w};
        const uint32_t a2[8] = {Q0.x, Q0.y, Q0.z, Q0.w, Q1.x, Q1.y, Q1.z, Q1.w};
        uint32_t sel[8];
        int stop = 8;
        uint32_t stop_n1 = 0;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const uint32_t before = nn;
          const uint32_t t1 = a1[e] < nn ? 1u : 0u;
          const uint32_t m1 = nn - t1;
          const uint32_t t2 = a2[e] < m1 ? 1u : 0u;
          nn = m1 - t2;
          sel[e] = t1 | (t2 << 8);
          const bool hit = before != 0 && nn == 0;
          stop = hit ? e : stop;
          stop_n1 = hit ? m1 : stop_n1;
        }
        *reinterpret_cast<uint4*>(ss.sel + l) =
            make_uint4(sel[0] | (sel[1] << 16), sel[2] | (sel[3] << 16), sel[4] | (sel[5] << 16), sel[6] | (sel[7] << 16));
        if (nn == 0) {
          l += stop;  // the step that ended the sample
          n1 = stop_n1;
          done = true;
          break;
        }
      }
      for (; l < usable && !done; ++l) {
        const uint32_t a1 = ss.p1[l], a2 = ss.p2[l];
        const uint32_t t1 = a1 < nn ? 1u : 0u;
        n1 = nn - t1;
        const uint32_t t2 = a2 < n1 ? 1u : 0u;
        nn = n1 - t2;
        ss.sel[l] = static_cast<uint16_t>(t1 | (t2 << 8));
        if (nn == 0) {
          done = true;
          break;
        }
      }
      const int steps = done ? l + 1 : usable;
      const int visited = done ? 2 * l + 1 + (n1 != 0 ? 1 : 0) : 2 * usable;
      rng.pos = pos + steps;
      ss.uns = uns - visited;
      ss.nq = nn;
      ss.i = i0 + visited;
      ss.taken += static_cast<int>(nq - static_cast<long long>(nn));
      ss.visited = visited;
      ss.redraw = !done && usable < batch;
    }
    __syncthreads();
    for (int k = tid; k < ss.visited; k += kPlanThreads)
      if ((ss.sel[k >> 1] >> (8 * (k & 1))) & 1u) flags[rows[first + i0 + k]] = 1;
    if (ss.redraw) {
      // the rejected step, drawn one output at a time by warp 0
      if (tid < 32) {
        long long un = ss.uns, nn = ss.nq;
        int i = ss.i, taken = ss.taken;
        const uint64_t b1 = static_cast<uint64_t>(un - 1);
        uint64_t a1, a2;
        divmod_u64(draw_below_warp(rng, static_cast<uint64_t>(un) * b1, lane), b1, a1, a2);
        --un;
        if (static_cast<long long>(a1) < nn) {
          if (tid == 0) flags[rows[first + i]] = 1;
          --nn;
          ++taken;
        }
        ++i;
        if (nn != 0) {
          --un;
          if (static_cast<long long>(a2) < nn) {
            if (tid == 0) flags[rows[first + i]] = 1;
            --nn;
            ++taken;
          }
          ++i;
        }
        __syncwarp();
        if (tid == 0) {
          ss.uns = un;
          ss.nq = nn;
          ss.i = i;
          ss.taken = taken;
        }
      }
    }
    __syncthreads();
  }
  if (nq != 0) {
    // fewer than two rows left: one draw per row (warp 0)
    if (tid < 32) {
      long long un = uns, nn = nq;
      int i = ss.i, taken = ss.taken;
      for (; nn != 0; ++i) {
        --un;
        if (static_cast<long long>(draw_below_warp(rng, static_cast<uint64_t>(un) + 1, lane)) < nn) {
          if (tid == 0) flags[rows[first + i]] = 1;
          --nn;
          ++taken;
        }
      }
      __syncwarp();
      if (tid == 0) ss.taken = taken;
    }
    __syncthreads();
  }
  return tid == 0 ? ss.taken : 0;
}

// std::mt19937 (Matsumoto & Nishimura 1998: n=624, m=397), serial.
struct Mt32State {
  uint32_t mt[624];
  int pos;
};

__device__ void mt32_seed(Mt32State& s, uint32_t seed) {
  s.mt[0] = seed;
  for (int i = 1; i < 624; ++i) s.mt[i] = 1812433253u * (s.mt[i - 1] ^ (s.mt[i - 1] >> 30)) + static_cast<uint32_t>(i);
  s.pos = 624;
}

__device__ uint32_t mt32_next(Mt32State& s) {
  if (s.pos >= 624) {
    for (int i = 0; i < 624; ++i) {
      const uint32_t y = (s.mt[i] & 0x80000000u) | (s.mt[i + 1 < 624 ? i + 1 : 0] & 0x7fffffffu);
      s.mt[i] = s.mt[i + 397 < 624 ? i + 397 : i + 397 - 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    s.pos = 0;
  }
  uint32_t y = s.mt[s.pos++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

__global__ void __launch_bounds__(kPlanThreads) plan_runs_kernel(PlanArgs a, PlanScratch s) {
  __shared__ Mt64State rng;
  __shared__ Mt32State rng32;
  __shared__ SampleShared ss;
  __shared__ int sh_bad, sh_total;
  __shared__ uint32_t sh_kseed;
  __shared__ int sh_warp[kPlanThreads / 32];
  const int run = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  uint8_t* flags = s.flags + static_cast<size_t>(run) * a.n;
  int* quota = s.quota + static_cast<size_t>(run) * a.strata;
  int* order = s.order + static_cast<size_t>(run) * a.strata;
  for (int r = tid; r < a.n; r += kPlanThreads) flags[r] = 0;
  for (int t = tid; t < a.strata; t += kPlanThreads) quota[t] = s.base[t];
  __syncthreads();
  {
    if (tid == 0) {
      int bad = 0;
      mt64_seed(rng, a.seed + static_cast<uint64_t>(a.first_run + run));
      (void)mt64_next_serial(rng);
      int S = 0;
      for (int t = 0; t < a.strata; ++t)
        if (s.offsets[t + 1] > s.offsets[t]) order[S++] = t;
      shuffle_serial(order, S, rng);
      const int residual = a.target - *s.assigned;
      if (residual > 0) {
        const Ext80 offset = ext80_canonical(mt64_next_serial(rng));
        Ext80 cumulative{0, 0};
        int selected = 0;
        for (int i = 0; i < S; ++i) {
          const int t = order[i];
          cumulative = ext80_add(cumulative, s.frac[t]);
          const Ext80 next = ext80_add(offset, ext80_from_u64(static_cast<uint64_t>(selected)));
          if (selected < residual && ext80_lt(next, cumulative)) {
            ++quota[t];
            order[i] = t | kRounded;
            ++selected;
          }
        }
        while (selected < residual) {
          int best = -1, besti = -1;
          Ext80 bestv{0, 0};
          for (int i = 0; i < S; ++i) {
            const int t = order[i];
            if (t & kRounded) continue;
            if (best < 0 || ext80_lt(bestv, s.frac[t])) {
              bestv = s.frac[t];
              best = t;
              besti = i;
            }
          }
          if (best < 0) {
            bad = 2;
            break;
          }
          ++quota[best];
          order[besti] = best | kRounded;
          ++selected;
        }
      }
      sh_bad = bad;
    }
    __syncthreads();
    if (sh_bad == 0) {
      int total = 0;
      for (int t = 0; t < a.strata; ++t) {
        const int q = quota[t];
        if (q <= 0) continue;
        total += sample_cta(s.offsets[t], s.offsets[t + 1] - s.offsets[t], q, s.rows, flags, rng, ss, tid);
      }
      if (tid == 0 && total != a.target) sh_bad = 3;
    }
    __syncthreads();
    if (tid == 0) {
      sh_kseed = static_cast<uint32_t>((mt64_next_serial(rng) & 0x7fffffffull) + 1ull);
      sh_total = 0;
    }
  }
  __syncthreads();
  if (sh_bad) {
    if (tid == 0) atomicExch(a.status, sh_bad);
    return;
  }
  // ascending compaction of the selected rows (and of the others)
  int* land = a.land + static_cast<size_t>(run) * a.target;
  int* nonland = a.nonland == nullptr ? nullptr : a.nonland + static_cast<size_t>(run) * (a.n - a.target);
  for (int b = 0; b < a.n; b += kPlanThreads) {
    const int r = b + tid;
    const int f = r < a.n ? flags[r] : 0;
    const unsigned bal = __ballot_sync(0xffffffffu, f != 0);
    if (lane == 0) sh_warp[warp] = __popc(bal);
    __syncthreads();
    int pos = sh_total;
    for (int i = 0; i < warp; ++i) pos += sh_warp[i];
    pos += __popc(bal & ((1u << lane) - 1u));
    if (r < a.n) {
      if (f) {
        land[pos] = r;
      } else if (nonland != nullptr) {
        nonland[r - pos] = r;
      }
    }
    __syncthreads();
    if (tid == 0) {
      int t = 0;
      for (int i = 0; i < kPlanThreads / 32; ++i) t += sh_warp[i];
      sh_total += t;
    }
    __syncthreads();
  }
  // initial centroid rows: head of the permutation of 0..L-1
  const int L = a.target;
  const int k = max(1, min(a.init_k, L));
  int* perm = s.perm + static_cast<size_t>(run) * L;
  for (int i = tid; i < L; i += kPlanThreads) perm[i] = i;
  __syncthreads();
  if (tid == 0) {
    mt32_seed(rng32, sh_kseed);
    const int steps = min(k, L - 1);
    for (int r = 0; r < steps; ++r) {
      const uint32_t u = mt32_next(rng32);
      const int other = r + static_cast<int>(u % static_cast<uint32_t>(L - r));
      const int t = perm[r];
      perm[r] = perm[other];
      perm[other] = t;
    }
    int* out = a.init_rows + static_cast<size_t>(run) * a.init_k;
    for (int r = 0; r < k; ++r) out[r] = perm[r];
  }
}

// FNV-1a over each run's landmark rows (hash_integer_vector,
// kodama_matrix.cpp:1689-1699).
__global__ void land_hash_kernel(const int* __restrict__ land, int runs, int L, uint64_t* __restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= runs) return;
  const int* v = land + static_cast<size_t>(r) * L;
  uint64_t h = 1469598103934665603ull;
  for (int i = 0; i < L; ++i) {
    const uint32_t b = static_cast<uint32_t>(v[i]);
#pragma unroll
    for (int sft = 0; sft < 32; sft += 8) {
      h ^= static_cast<uint8_t>((b >> sft) & 0xffu);
      h *= 1099511628211ull;
    }
  }
  out[r] = h;
}

}  // namespace

size_t plan_scratch_bytes(int n, int strata, int target, int runs) {
  const size_t S = static_cast<size_t>(strata), R = static_cast<size_t>(runs);
  return align256(sizeof(int) * S) * 3 + align256(sizeof(int) * (S + 1)) + align256(sizeof(int) * n) +
         align256(sizeof(Ext80) * S) + align256(sizeof(int)) + align256(sizeof(int) * S * R) * 2 +
         align256(static_cast<size_t>(n) * R) + align256(sizeof(int) * static_cast<size_t>(target) * R);
}

int plan_landmarks(const PlanArgs& a, cudaStream_t st) {
  if (a.n < 1 || a.strata < 1 || a.target < 1 || a.target > a.n || a.runs < 1 || a.init_k < 1 ||
      a.init_k > a.target)
    return static_cast<int>(cudaErrorInvalidValue);
  const PlanScratch s = carve(a);
  strata_kernel<<<1, 1024, 0, st>>>(a, s);
  count_launch();
  plan_runs_kernel<<<a.runs, kPlanThreads, 0, st>>>(a, s);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

int plan_land_hash(const PlanArgs& a, cudaStream_t st) {
  land_hash_kernel<<<(a.runs + 127) / 128, 128, 0, st>>>(a.land, a.runs, a.target, a.land_hash);
  count_launch();
  return static_cast<int>(cudaGetLastError());
}

}  // namespace kgb
