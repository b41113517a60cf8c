// KODAMA.matrix label-evolution hot path: CPU restatement (the oracle).
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path in
// kodama_gb300/csrc.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline load it (through oracle/oracle.py); the product never does.
//
// It restates, step for step, the reference's CPU algorithm for the path,
// written as plain single-threaded-per-run C++17 over flat arrays.  Parity is
// pinned against the reference itself (oracle/_ref, built from the reference
// sources by oracle/build_ref.sh) by tests/test_oracle_pins.py and by the
// committed fixtures in tests/golden.
//
// Random streams: the reference draws through libstdc++'s std::mt19937_64 /
// std::mt19937 and its <random>/<algorithm> algorithms (uniform_int_distribution,
// shuffle, discrete_distribution, sample, generate_canonical).  The oracle calls
// the same libstdc++ (GCC 13) templates, so its streams are the reference's by
// construction on both x86-64 and aarch64 hosts.  Two host-dependent pieces of
// the reference are restated explicitly so that this file gives the x86-64
// answers everywhere:
//   * dot_float32 (kodama_matrix.cpp:91-122) uses 4x4 SSE accumulators without
//     FMA on x86-64 (FMA NEON on aarch64): dot_x86_order() below;
//   * quota_sample_landmarks (kodama_matrix.cpp:856-944) rounds in x87 80-bit
//     long double: ext80.h.
// Build with -ffp-contract=off so no multiply-add is fused.

#include "../kodama_gb300/csrc/ext80.h"
#include "pls_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <limits>
#include <map>
#include <numeric>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace orc {

thread_local std::string g_error;

// ---------------------------------------------------------------------------
// float32 dot product in the x86-64 SSE order of dot_float32
// (kodama_matrix.cpp:91-122): 16 partial sums p[l] over i = l (mod 16) for the
// leading multiple of 16, combined as ((p0+p4)+(p8+p12)) per lane l<4, then
// lane0+lane1+lane2+lane3, then the tail added sequentially.
// ---------------------------------------------------------------------------
float dot_x86_order(const float* a, const float* b, int n) {
  // Four 4-lane accumulators (GCC generic vectors: SSE on x86-64, NEON on
  // aarch64, no intrinsics); lane l of accumulator j holds p[4j + l].  With
  // -ffp-contract=off the multiply and the add stay separately rounded.
  typedef float v4f __attribute__((vector_size(16)));
  v4f s0 = {0, 0, 0, 0}, s1 = s0, s2 = s0, s3 = s0;
  int i = 0;
  for (; i + 15 < n; i += 16) {
    v4f a0, a1, a2, a3, b0, b1, b2, b3;
    std::memcpy(&a0, a + i, 16);
    std::memcpy(&a1, a + i + 4, 16);
    std::memcpy(&a2, a + i + 8, 16);
    std::memcpy(&a3, a + i + 12, 16);
    std::memcpy(&b0, b + i, 16);
    std::memcpy(&b1, b + i + 4, 16);
    std::memcpy(&b2, b + i + 8, 16);
    std::memcpy(&b3, b + i + 12, 16);
    const v4f m0 = a0 * b0, m1 = a1 * b1, m2 = a2 * b2, m3 = a3 * b3;
    s0 = s0 + m0;
    s1 = s1 + m1;
    s2 = s2 + m2;
    s3 = s3 + m3;
  }
  const v4f l01 = s0 + s1, l23 = s2 + s3;
  const v4f lane = l01 + l23;
  float sum = lane[0] + lane[1];
  sum = sum + lane[2];
  sum = sum + lane[3];
  for (; i < n; ++i) {
    const float prod = a[i] * b[i];
    sum = sum + prod;
  }
  return sum;
}

// ---------------------------------------------------------------------------
// Canonical exact kNN (the graph the GPU builder must reproduce): squared
// Euclidean distance accumulated in float32, coordinate order, no FMA; rank by
// (distance, index); self excluded; output distance = sqrtf(d2).
// Replaces the reference's approximate HNSW (native_knn.cpp:125) so that the
// raw-data path is deterministic; output convention native_knn.cpp:1157.
// ---------------------------------------------------------------------------
inline float sqdist_canonical(const float* a, const float* b, int d) {
  float acc = 0.0f;
  for (int k = 0; k < d; ++k) {
    const float diff = a[k] - b[k];
    const float sq = diff * diff;
    acc = acc + sq;
  }
  return acc;
}

// rows == nullptr: every row i writes output row i; else the nrows listed
// query rows write output rows 0..nrows-1.
void exact_knn(const float* x, int n, int d, int K, int* idx, float* dist, int threads,
               const int* rows = nullptr, int nrows = 0) {
  const int nq = rows ? nrows : n;
  auto work = [&](int t) {
    std::vector<std::pair<float, int>> row(static_cast<size_t>(n));
    for (int q = t; q < nq; q += threads) {
      const int i = rows ? rows[q] : q;
      int m = 0;
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        row[m++] = {sqdist_canonical(x + static_cast<size_t>(i) * d, x + static_cast<size_t>(j) * d, d), j};
      }
      const int take = std::min(K, m);
      std::partial_sort(row.begin(), row.begin() + take, row.begin() + m);
      for (int c = 0; c < K; ++c) {
        if (c < take) {
          idx[static_cast<size_t>(q) * K + c] = row[c].second;
          dist[static_cast<size_t>(q) * K + c] = std::sqrt(row[c].first);
        } else {
          idx[static_cast<size_t>(q) * K + c] = -1;
          dist[static_cast<size_t>(q) * K + c] = std::numeric_limits<float>::infinity();
        }
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) pool.emplace_back(work, t);
  for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------
// k-means (kodama_matrix.cpp:664-799 kmeans_labels, CPU branch), with the
// FAISS-compatible permutation (:535-564), the float Fenwick donor tree
// (:566-603) and empty-cluster splitting (:605-662).
// ---------------------------------------------------------------------------
struct Mt32Source {
  std::mt19937 g;
  explicit Mt32Source(uint64_t seed) : g(static_cast<uint32_t>(seed)) {}
  int integer(int maximum) { return static_cast<int>(g() % static_cast<uint32_t>(maximum)); }
  float uniform() { return static_cast<float>(g()) / static_cast<float>(std::mt19937::max()); }
};

// Only the first `needed` entries of the permutation are ever read.
std::vector<int> permutation_head(int rows, uint64_t seed, int needed) {
  std::vector<int> perm(static_cast<size_t>(rows));
  std::iota(perm.begin(), perm.end(), 0);
  Mt32Source src(seed);
  const int steps = std::min(needed, rows - 1);
  for (int r = 0; r < steps; ++r) {
    const int other = r + src.integer(rows - r);
    std::swap(perm[r], perm[other]);
  }
  perm.resize(static_cast<size_t>(std::min(needed, rows)));
  return perm;
}

struct FenwickF {
  std::vector<float> tree, vals;
  explicit FenwickF(const std::vector<float>& v) : tree(v.size() + 1, 0.0f), vals(v.size(), 0.0f) {
    for (size_t i = 0; i < v.size(); ++i) set(i, v[i]);
  }
  void set(size_t i, float value) {
    const float delta = value - vals[i];
    vals[i] = value;
    for (size_t j = i + 1; j < tree.size(); j += j & (~j + 1)) tree[j] = tree[j] + delta;
  }
  float total() const {
    float s = 0.0f;
    for (size_t j = vals.size(); j > 0; j -= j & (~j + 1)) s = s + tree[j];
    return s;
  }
  int select(float target) const {
    size_t pos = 0;
    float prefix = 0.0f;
    size_t step = 1;
    while ((step << 1) < tree.size()) step <<= 1;
    for (; step > 0; step >>= 1) {
      const size_t nxt = pos + step;
      if (nxt < tree.size() && prefix + tree[nxt] <= target) {
        pos = nxt;
        prefix = prefix + tree[nxt];
      }
    }
    return pos < vals.size() ? static_cast<int>(pos) : -1;
  }
};

void split_empty_clusters(int rows, int dims, int k, std::vector<float>& sizes, std::vector<float>& cent) {
  if (rows <= k) return;
  const float eps = 1.0f / 1024.0f;
  Mt32Source src(1234u);
  std::vector<float> w(static_cast<size_t>(k));
  for (int c = 0; c < k; ++c) w[c] = std::max(0.0f, sizes[c] - 1.0f);
  FenwickF tree(w);
  for (int e = 0; e < k; ++e) {
    if (sizes[e] != 0.0f) continue;
    const float total = tree.total();
    int donor = total > 0.0f ? tree.select(src.uniform() * total) : -1;
    if (donor < 0) {
      donor = 0;
      for (int c = 1; c < k; ++c) if (sizes[c] > sizes[donor]) donor = c;
    }
    float* ec = cent.data() + static_cast<size_t>(e) * dims;
    float* dc = cent.data() + static_cast<size_t>(donor) * dims;
    std::copy_n(dc, dims, ec);
    for (int j = 0; j < dims; ++j) {
      if ((j & 1) == 0) {
        ec[j] *= 1.0f + eps;
        dc[j] *= 1.0f - eps;
      } else {
        ec[j] *= 1.0f - eps;
        dc[j] *= 1.0f + eps;
      }
    }
    sizes[e] = sizes[donor] / 2.0f;
    sizes[donor] -= sizes[e];
    tree.set(static_cast<size_t>(e), std::max(0.0f, sizes[e] - 1.0f));
    tree.set(static_cast<size_t>(donor), std::max(0.0f, sizes[donor] - 1.0f));
  }
}

// Returns labels 1..k for the n rows of x (row-major n x p).
std::vector<int> kmeans_labels(const float* x, int n, int p, int k, std::mt19937_64& rng, int max_iter = 10,
                              int threads = 1) {
  k = std::max(1, std::min(k, n));
  const uint64_t kseed = rng() & 0x7fffffffULL;
  const std::vector<int> order = permutation_head(n, kseed + 1u, k);
  std::vector<float> cent(static_cast<size_t>(k) * p);
  for (int c = 0; c < k; ++c) std::copy_n(x + static_cast<size_t>(order[c]) * p, p, cent.data() + static_cast<size_t>(c) * p);
  std::vector<int> assign(static_cast<size_t>(n), -1);
  std::vector<float> pnorm(static_cast<size_t>(n)), cnorm(static_cast<size_t>(k)), sizes(static_cast<size_t>(k));
  for (int r = 0; r < n; ++r) pnorm[r] = dot_x86_order(x + static_cast<size_t>(r) * p, x + static_cast<size_t>(r) * p, p);
  // Rows are independent: with threads > 1 they are split into contiguous
  // blocks, as the reference's OpenMP static schedule does (:735-758).
  auto assign_rows = [&](int r0, int r1) {
    int changed = 0;
    for (int r = r0; r < r1; ++r) {
      int best = 0;
      float bestd = std::numeric_limits<float>::infinity();
      const float* pt = x + static_cast<size_t>(r) * p;
      for (int c = 0; c < k; ++c) {
        const float dt = dot_x86_order(pt, cent.data() + static_cast<size_t>(c) * p, p);
        const float twice = 2.0f * dt;
        const float dd = (pnorm[r] + cnorm[c]) - twice;
        if (dd < bestd || (dd == bestd && c < best)) {
          bestd = dd;
          best = c;
        }
      }
      if (assign[r] != best) {
        assign[r] = best;
        ++changed;
      }
    }
    return changed;
  };
  auto assign_step = [&]() {
    for (int c = 0; c < k; ++c) cnorm[c] = dot_x86_order(cent.data() + static_cast<size_t>(c) * p, cent.data() + static_cast<size_t>(c) * p, p);
    const int nt = std::max(1, std::min(threads, n / 256));
    if (nt == 1) return assign_rows(0, n);
    std::atomic<int> changed{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) {
      const int r0 = static_cast<int>(static_cast<long long>(n) * t / nt);
      const int r1 = static_cast<int>(static_cast<long long>(n) * (t + 1) / nt);
      pool.emplace_back([&, r0, r1]() { changed.fetch_add(assign_rows(r0, r1)); });
    }
    for (auto& th : pool) th.join();
    return changed.load();
  };
  for (int it = 0; it < std::max(1, max_iter); ++it) {
    const int changed = assign_step();
    std::fill(cent.begin(), cent.end(), 0.0f);
    std::fill(sizes.begin(), sizes.end(), 0.0f);
    for (int r = 0; r < n; ++r) {
      const int c = assign[r];
      sizes[c] += 1.0f;
      float* ct = cent.data() + static_cast<size_t>(c) * p;
      const float* pt = x + static_cast<size_t>(r) * p;
      for (int j = 0; j < p; ++j) ct[j] = ct[j] + pt[j];
    }
    for (int c = 0; c < k; ++c) {
      const float s = sizes[c];
      if (s == 0.0f) continue;
      const float inv = 1.0f / s;
      float* ct = cent.data() + static_cast<size_t>(c) * p;
      for (int j = 0; j < p; ++j) ct[j] = ct[j] * inv;
    }
    split_empty_clusters(n, p, k, sizes, cent);
    if (changed == 0) break;
  }
  assign_step();
  std::vector<int> labels(static_cast<size_t>(n));
  for (int r = 0; r < n; ++r) labels[r] = assign[r] + 1;
  return labels;
}

// ---------------------------------------------------------------------------
// Landmark strata (kodama_matrix.cpp:806-828 index_strata) and quota sampling
// (:856-944 quota_sample_landmarks, preserve_strata_order = false).
// ---------------------------------------------------------------------------
struct Strata {
  std::vector<int> offsets, rows;
};

Strata index_strata(const std::vector<int>& labels, int strata) {
  Strata s;
  s.offsets.assign(static_cast<size_t>(strata) + 1, 0);
  s.rows.resize(labels.size());
  for (int l : labels) ++s.offsets[static_cast<size_t>(l)];
  for (int t = 1; t <= strata; ++t) s.offsets[t] += s.offsets[t - 1];
  std::vector<int> cur = s.offsets;
  for (size_t r = 0; r < labels.size(); ++r) s.rows[static_cast<size_t>(cur[labels[r] - 1]++)] = static_cast<int>(r);
  return s;
}

std::vector<int> quota_sample(const Strata& st, int target, std::mt19937_64& rng) {
  const int samples = static_cast<int>(st.rows.size());
  target = std::max(1, std::min(target, samples));
  const int strata = static_cast<int>(st.offsets.size()) - 1;
  std::vector<int> quota(static_cast<size_t>(strata), 0);
  std::vector<Ext80> frac(static_cast<size_t>(strata), Ext80{0, 0});
  std::vector<int> order;
  int assigned = 0;
  const Ext80 samples_x = ext80_from_u64(static_cast<uint64_t>(samples));
  for (int s = 0; s < strata; ++s) {
    const int count = st.offsets[s + 1] - st.offsets[s];
    if (count <= 0) continue;
    order.push_back(s);
    const Ext80 expected = ext80_div(
      ext80_from_u64(static_cast<uint64_t>(target) * static_cast<uint64_t>(count)), samples_x);
    const int base = std::min(count, ext80_floor_int(expected));
    quota[s] = base;
    frac[s] = ext80_sub(expected, ext80_from_u64(static_cast<uint64_t>(base)));
    assigned += base;
  }
  std::shuffle(order.begin(), order.end(), rng);
  const int residual = target - assigned;
  if (residual > 0) {
    const Ext80 offset = ext80_canonical(rng());
    Ext80 cumulative{0, 0};
    int selected = 0;
    std::vector<char> up(static_cast<size_t>(strata), 0);
    for (int s : order) {
      cumulative = ext80_add(cumulative, frac[s]);
      const Ext80 next = ext80_add(offset, ext80_from_u64(static_cast<uint64_t>(selected)));
      if (selected < residual && ext80_lt(next, cumulative)) {
        ++quota[s];
        up[s] = 1;
        ++selected;
      }
    }
    while (selected < residual) {
      int best = -1;
      Ext80 bestv{0, 0};
      for (int s : order) {
        if (up[s]) continue;
        if (best < 0 || ext80_lt(bestv, frac[s])) {
          bestv = frac[s];
          best = s;
        }
      }
      if (best < 0) throw std::runtime_error("Unable to complete the landmark quota allocation.");
      ++quota[best];
      up[best] = 1;
      ++selected;
    }
  }
  std::vector<int> out;
  out.reserve(static_cast<size_t>(target));
  for (int s = 0; s < strata; ++s) {
    const int take = quota[s];
    if (take <= 0) continue;
    std::sample(st.rows.begin() + st.offsets[s], st.rows.begin() + st.offsets[s + 1],
                std::back_inserter(out), take, rng);
  }
  if (static_cast<int>(out.size()) != target) throw std::runtime_error("Landmark quota allocation produced the wrong sample size.");
  std::sort(out.begin(), out.end());
  return out;
}

// ---------------------------------------------------------------------------
// Folds (common.cpp:108-214 make_folds).
// ---------------------------------------------------------------------------
std::vector<int> make_folds(const std::vector<int>& labels, const std::vector<int>& constrain,
                            int folds, bool stratified, uint64_t seed) {
  if (folds < 2) throw std::invalid_argument("Number of folds must be at least 2.");
  const int n = static_cast<int>(labels.size());
  std::mt19937_64 rng(seed);
  std::vector<int> out(static_cast<size_t>(n), 0);
  if (constrain.empty()) {
    if (stratified) {
      std::map<int, std::vector<int>> by_label;
      for (int i = 0; i < n; ++i) by_label[labels[i]].push_back(i);
      std::vector<int> load(static_cast<size_t>(folds));
      for (auto& kv : by_label) {
        std::shuffle(kv.second.begin(), kv.second.end(), rng);
        std::fill(load.begin(), load.end(), 0);
        for (int idx : kv.second) {
          const int f = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
          out[idx] = f;
          load[f] += 1;
        }
      }
    } else {
      std::vector<int> order(static_cast<size_t>(n));
      std::iota(order.begin(), order.end(), 0);
      std::shuffle(order.begin(), order.end(), rng);
      for (size_t i = 0; i < order.size(); ++i) out[order[i]] = static_cast<int>(i % static_cast<size_t>(folds));
    }
    return out;
  }
  // constrained: one fold per group, groups in ascending constrain value
  std::map<int, std::vector<int>> members;
  for (int i = 0; i < n; ++i) members[constrain[i]].push_back(i);
  std::vector<int> glabel, gsize;
  for (const auto& kv : members) {
    std::map<int, int> counts;
    for (int idx : kv.second) counts[labels[idx]]++;
    int bl = counts.begin()->first, bc = counts.begin()->second;
    for (const auto& lc : counts) if (lc.second > bc) { bl = lc.first; bc = lc.second; }
    glabel.push_back(bl);
    gsize.push_back(static_cast<int>(kv.second.size()));
  }
  const size_t G = glabel.size();
  std::vector<int> gfold(G, 0);
  if (stratified) {
    std::map<int, std::vector<size_t>> by_label;
    for (size_t g = 0; g < G; ++g) by_label[glabel[g]].push_back(g);
    std::vector<int> load(static_cast<size_t>(folds));
    for (auto& kv : by_label) {
      std::shuffle(kv.second.begin(), kv.second.end(), rng);
      std::fill(load.begin(), load.end(), 0);
      for (size_t g : kv.second) {
        const int f = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
        gfold[g] = f;
        load[f] += gsize[g];
      }
    }
  } else {
    std::vector<size_t> order(G);
    std::iota(order.begin(), order.end(), 0);
    std::shuffle(order.begin(), order.end(), rng);
    for (size_t i = 0; i < G; ++i) gfold[order[i]] = static_cast<int>(i % static_cast<size_t>(folds));
  }
  size_t g = 0;
  for (const auto& kv : members) {
    for (int idx : kv.second) out[idx] = gfold[g];
    ++g;
  }
  return out;
}

// ---------------------------------------------------------------------------
// Fold-filtered neighbour table (core.cpp:586-692 normalize_graph_indices +
// precompute_knn_cv_graph): per row the first k' = max(1,min(k,K)) valid,
// non-self, out-of-fold, finite neighbours with score -(d*d) (Euclidean).
// ---------------------------------------------------------------------------
struct VoteTable {
  int samples = 0, width = 0;
  std::vector<int> nb;      // samples x width, -1 = empty
  std::vector<float> score; // samples x width
  std::vector<int> folds;
};

VoteTable build_vote_table(const int* gidx, const float* gdist, int samples, int gk, int index_base,
                           const std::vector<int>& folds, int k, bool euclidean) {
  int mn = std::numeric_limits<int>::max(), mx = std::numeric_limits<int>::min();
  const size_t total = static_cast<size_t>(samples) * gk;
  for (size_t i = 0; i < total; ++i) {
    if (gidx[i] < 0) continue;
    mn = std::min(mn, gidx[i]);
    mx = std::max(mx, gidx[i]);
  }
  const bool one_based = index_base == 1 || (index_base < 0 && mn >= 1 && mx <= samples);
  VoteTable t;
  t.samples = samples;
  t.width = std::max(1, std::min(k, gk));
  t.folds = folds;
  t.nb.assign(static_cast<size_t>(samples) * t.width, -1);
  t.score.assign(static_cast<size_t>(samples) * t.width, -std::numeric_limits<float>::infinity());
  for (int r = 0; r < samples; ++r) {
    int col = 0;
    for (int j = 0; j < gk && col < t.width; ++j) {
      const size_t off = static_cast<size_t>(r) * gk + j;
      int id = gidx[off];
      if (one_based && id > 0) --id;
      if (id < 0 || id >= samples || id == r) continue;
      const float raw = gdist[off];
      const float dd = std::isfinite(raw) && raw >= 0.0f ? raw : std::numeric_limits<float>::infinity();
      if (folds[id] == folds[r]) continue;
      if (!std::isfinite(dd)) continue;
      const float dc = std::max(0.0f, dd);
      t.nb[static_cast<size_t>(r) * t.width + col] = id;
      // precompute_knn_cv_graph (core.cpp:672-677)
      t.score[static_cast<size_t>(r) * t.width + col] = euclidean ? -(dc * dc) : 1.0f - dc;
      ++col;
    }
  }
  return t;
}

// Fold vote (core.cpp:784-914 predict_precomputed_knn + :274-309 training-fold
// fallbacks).  Labels are compared by value; ties: count, then score sum
// (double, neighbour order), then smaller label.
// `uniq` is the label universe (sorted): the initial labels' distinct values,
// rebuilt from the current labels only if one of them is unseen
// (core.cpp:392-420 initialize_knn_label_map, :795-808).
// Buffers reused across the evaluations of one run (the reference keeps the
// same kind of scratch, KNNPredictionScratch).  `lut` maps a label value v in
// [lut_lo, lut_lo + lut.size()) to its code in `uniq` (-1: not in `uniq`).
struct VoteScratch {
  std::vector<int> lut, code, cnt, touched, all, fold_counts, fallback;
  std::vector<double> ssum;
  std::vector<char> empty, fold_present;
  int lut_lo = 0;
  bool lut_ok = false;
};

void vote_lookup(VoteScratch& s, const std::vector<int>& uniq) {
  s.lut_ok = false;
  if (uniq.empty()) return;
  const long long span = static_cast<long long>(uniq.back()) - uniq.front() + 1;
  if (span > (1LL << 22)) return;  // sparse label values: binary search instead
  s.lut_lo = uniq.front();
  s.lut.assign(static_cast<size_t>(span), -1);
  for (size_t c = 0; c < uniq.size(); ++c) s.lut[static_cast<size_t>(uniq[c] - s.lut_lo)] = static_cast<int>(c);
  s.lut_ok = true;
}

inline int vote_code(const VoteScratch& s, const std::vector<int>& uniq, int v) {
  if (s.lut_ok) {
    const long long o = static_cast<long long>(v) - s.lut_lo;
    return o < 0 || o >= static_cast<long long>(s.lut.size()) ? -1 : s.lut[static_cast<size_t>(o)];
  }
  const auto it = std::lower_bound(uniq.begin(), uniq.end(), v);
  return it == uniq.end() || *it != v ? -1 : static_cast<int>(it - uniq.begin());
}

std::vector<int> vote_predict(const VoteTable& t, const std::vector<int>& labels, std::vector<int>& uniq, int folds_n,
                              VoteScratch& s) {
  const int n = t.samples;
  std::vector<int> pred(static_cast<size_t>(n), 0);
  if (!s.lut_ok && s.lut.empty()) vote_lookup(s, uniq);
  s.code.resize(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) {
    const int c = vote_code(s, uniq, labels[i]);
    if (c < 0) {
      // an unseen label: the universe is rebuilt from the current labels
      uniq = labels;
      std::sort(uniq.begin(), uniq.end());
      uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
      vote_lookup(s, uniq);
      for (int j = 0; j < n; ++j) s.code[j] = vote_code(s, uniq, labels[j]);
      break;
    }
    s.code[i] = c;
  }
  const int C = static_cast<int>(uniq.size());
  s.cnt.assign(static_cast<size_t>(C), 0);
  s.ssum.assign(static_cast<size_t>(C), 0.0);
  s.empty.assign(static_cast<size_t>(n), 0);
  const int* code = s.code.data();
  int* cnt = s.cnt.data();
  double* ssum = s.ssum.data();
  std::vector<int>& touched = s.touched;
  for (int r = 0; r < n; ++r) {
    touched.clear();
    const int* nbr = t.nb.data() + static_cast<size_t>(r) * t.width;
    const float* sc = t.score.data() + static_cast<size_t>(r) * t.width;
    for (int j = 0; j < t.width; ++j) {
      const int nb = nbr[j];
      if (nb < 0) continue;
      const int c = code[nb];
      if (cnt[c] == 0) touched.push_back(c);
      cnt[c]++;
      ssum[c] += static_cast<double>(sc[j]);
    }
    if (touched.empty()) {
      s.empty[r] = 1;
      continue;
    }
    int bl = 0, bc = -1;
    double bs = -std::numeric_limits<double>::infinity();
    for (int c : touched) {
      const int lab = uniq[c];
      if (cnt[c] > bc || (cnt[c] == bc && ssum[c] > bs) || (cnt[c] == bc && ssum[c] == bs && lab < bl)) {
        bl = lab;
        bc = cnt[c];
        bs = ssum[c];
      }
      cnt[c] = 0;
      ssum[c] = 0.0;
    }
    pred[r] = bl;
  }
  // training-fold majority for rows without any out-of-fold neighbour
  s.all.assign(static_cast<size_t>(C), 0);
  s.fold_counts.assign(static_cast<size_t>(folds_n) * C, 0);
  s.fold_present.assign(static_cast<size_t>(folds_n), 0);
  s.fallback.assign(static_cast<size_t>(folds_n), 0);
  for (int i = 0; i < n; ++i) {
    s.all[code[i]]++;
    s.fold_counts[static_cast<size_t>(t.folds[i]) * C + code[i]]++;
    s.fold_present[t.folds[i]] = 1;
  }
  for (int f = 0; f < folds_n; ++f) {
    if (!s.fold_present[f]) continue;
    int bl = C ? uniq[0] : 0, bc = -1;
    for (int c = 0; c < C; ++c) {
      const int count = s.all[c] - s.fold_counts[static_cast<size_t>(f) * C + c];
      if (count > bc || (count == bc && uniq[c] < bl)) {
        bl = uniq[c];
        bc = count;
      }
    }
    s.fallback[f] = bl;
  }
  for (int r = 0; r < n; ++r) if (s.empty[r]) pred[r] = s.fallback[t.folds[r]];
  return pred;
}

// ---------------------------------------------------------------------------
// Objective (core.cpp:916-972 core_objective_score), kNN classifier.
// ---------------------------------------------------------------------------
struct Policy {
  bool prediction_guidance = true, adaptive_proposal_size = true, transition_proposal = true,
       stochastic_acceptance = true, diversity_multiplier = true, pls_transition_coarsening = true,
       pls_fragmentation_penalty = true, reject_single_class = true;
};

// core_objective_score (core.cpp:916-972).  `fragmentation` is
// auto_class_coarsening with the PLS-LDA classifier.
double objective(const std::vector<int>& labels, double acc, bool guarded, const Policy& pol,
                 bool fragmentation = false) {
  const bool use_div = guarded && pol.diversity_multiplier;
  const bool use_frag = fragmentation && pol.pls_fragmentation_penalty;
  const bool reject1 = guarded && pol.reject_single_class;
  if (!use_div && !use_frag && !reject1) return acc;
  if (labels.empty()) return acc;
  std::unordered_map<int, int> counts;
  counts.reserve(labels.size());
  for (int l : labels) counts[l]++;
  const int nc = static_cast<int>(counts.size());
  if (nc < 1) return acc;
  if (reject1 && nc == 1) return -std::numeric_limits<double>::infinity();
  const double n = static_cast<double>(labels.size());
  double score = acc;
  if (use_div) {
    double same = 0.0;
    for (const auto& kv : counts) {
      const double p = static_cast<double>(kv.second) / n;
      same += p * p;
    }
    score *= std::sqrt(std::max(0.0, 1.0 - same));
  }
  if (use_frag && nc > 1) {
    double entropy = 0.0;
    for (const auto& kv : counts) {
      const double p = static_cast<double>(kv.second) / n;
      if (p > 0.0) entropy -= p * std::log(p);
    }
    const double max_entropy = n > 1.0 ? std::log(n) : 0.0;
    const double code_cost = max_entropy > 0.0 ? std::clamp(entropy / max_entropy, 0.0, 1.0) : 0.0;
    const double keff = std::exp(entropy);
    const double frag = std::max(0.0, std::log(static_cast<double>(nc) / std::max(1.0, keff)));
    const double frag_cost = frag / (1.0 + frag);
    score -= (1.0 - acc) * std::max(code_cost, frag_cost);
  }
  return score;
}

// propose_auto_class_coarsening (core.cpp:995-1108) over the transition
// statistics of build_class_transition_stats (:980-993).
bool coarsening(std::vector<int>& labels, const std::vector<int>& prev, const std::vector<int>& fixed,
                std::mt19937_64& rng) {
  std::map<int, int> sizes, movable;
  std::map<int, std::map<int, int>> trans;
  for (size_t i = 0; i < labels.size(); ++i) {
    ++sizes[labels[i]];
    ++trans[labels[i]][prev[i]];
    if (fixed[i] != 1) ++movable[labels[i]];
  }
  const int nc = static_cast<int>(sizes.size());
  if (nc <= 2) return false;
  const double n = static_cast<double>(labels.size());
  double class_entropy = 0.0;
  for (const auto& kv : sizes) {
    const double p = static_cast<double>(kv.second) / n;
    if (p > 0.0) class_entropy -= p * std::log(p);
  }
  const double keff = std::exp(class_entropy);
  const double frag = std::max(0.0, std::log(static_cast<double>(nc) / std::max(1.0, keff)));
  double wte = 0.0;
  struct Cand { int source, destination; double score; };
  std::vector<Cand> cands;
  for (const auto& kv : sizes) {
    const int src = kv.first, ssize = kv.second;
    const auto mv = movable.find(src);
    const int mov = mv == movable.end() ? 0 : mv->second;
    if (mov <= 0) continue;
    int dst_best = src, dsize = ssize, bcount = 0;
    double te = 0.0;
    const auto& row = trans.at(src);
    for (const auto& dst : row) {
      const double p = static_cast<double>(dst.second) / static_cast<double>(ssize);
      if (p > 0.0) te -= p * std::log(p);
      const auto cs = sizes.find(dst.first);
      if (dst.first != src && cs != sizes.end() &&
          (dst.second > bcount || (dst.second == bcount && cs->second > dsize) ||
           (dst.second == bcount && cs->second == dsize && dst.first < dst_best))) {
        dst_best = dst.first;
        dsize = cs->second;
        bcount = dst.second;
      }
    }
    wte += (static_cast<double>(ssize) / n) * te;
    if (dst_best == src || bcount == 0) continue;
    const double stay = static_cast<double>(row.count(src) ? row.at(src) : 0) / static_cast<double>(ssize);
    cands.push_back(Cand{src, dst_best, (1.0 / std::sqrt(static_cast<double>(mov))) * (1.0 - stay)});
  }
  if (cands.empty()) return false;
  const double temperature = frag / (frag + wte + 1.0);
  const double redundant = std::max(0.0, static_cast<double>(nc) - keff);
  int budget = static_cast<int>(std::ceil(temperature * redundant));
  if (budget < 1 && frag > 0.0) budget = 1;
  budget = std::min(budget, nc - 2);
  if (budget <= 0) return false;
  std::shuffle(cands.begin(), cands.end(), rng);
  std::stable_sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) { return a.score > b.score; });
  std::map<int, int> remap;
  for (const auto& kv : sizes) remap[kv.first] = kv.first;
  int merged = 0;
  for (const Cand& c : cands) {
    if (merged >= budget) break;
    if (remap[c.source] != c.source) continue;
    int d = c.destination;
    while (remap[d] != d) d = remap[d];
    if (d == c.source) continue;
    remap[c.source] = d;
    ++merged;
  }
  if (merged == 0) return false;
  bool changed = false;
  for (size_t i = 0; i < labels.size(); ++i) {
    if (fixed[i] == 1) continue;
    int d = labels[i];
    while (remap[d] != d) d = remap[d];
    if (d != labels[i]) {
      labels[i] = d;
      changed = true;
    }
  }
  return changed;
}

// Many-to-one absorption (core.cpp:980-993 build_class_transition_stats,
// :1110-1226 propose_many_to_one_absorption).
bool absorption_map(std::vector<int>& labels, const std::vector<int>& prev, const std::vector<int>& fixed,
                    std::mt19937_64& rng) {
  std::map<int, int> sizes, movable;
  std::map<int, std::map<int, int>> trans;
  for (size_t i = 0; i < labels.size(); ++i) {
    ++sizes[labels[i]];
    ++trans[labels[i]][prev[i]];
    if (fixed[i] != 1) ++movable[labels[i]];
  }
  const int nc = static_cast<int>(sizes.size());
  if (nc <= 2) return false;
  const double n = static_cast<double>(labels.size());
  struct Src { int source; double surplus; };
  struct Tgt { int target = 0; double weight = 0.0; std::vector<Src> sources; };
  std::map<int, Tgt> by_target;
  for (const auto& kv : sizes) {
    const int src = kv.first, ssize = kv.second;
    const auto mv = movable.find(src);
    if (mv == movable.end() || mv->second <= 0) continue;
    const auto& row = trans.at(src);
    const int stay = row.count(src) ? row.at(src) : 0;
    int bt = src, bcount = 0, bsize = ssize;
    double bsur = 0.0;
    for (const auto& dst : row) {
      if (dst.first == src) continue;
      const auto ds = sizes.find(dst.first);
      if (ds == sizes.end()) continue;
      const double expected = static_cast<double>(ssize) * static_cast<double>(ds->second) / std::max(1.0, n);
      const double sur = static_cast<double>(dst.second) - expected;
      if (sur > bsur || (sur == bsur && dst.second > bcount) ||
          (sur == bsur && dst.second == bcount && ds->second > bsize) ||
          (sur == bsur && dst.second == bcount && ds->second == bsize && dst.first < bt)) {
        bt = dst.first;
        bsize = ds->second;
        bcount = dst.second;
        bsur = sur;
      }
    }
    if (bt == src || bsur <= 0.0 || bcount <= stay) continue;
    Tgt& t = by_target[bt];
    t.target = bt;
    t.weight += bsur;
    t.sources.push_back(Src{src, bsur});
  }
  if (by_target.empty()) return false;
  std::vector<Tgt> multi, single;
  for (auto& kv : by_target) {
    std::sort(kv.second.sources.begin(), kv.second.sources.end(), [](const Src& a, const Src& b) {
      if (a.surplus != b.surplus) return a.surplus > b.surplus;
      return a.source < b.source;
    });
    (kv.second.sources.size() > 1 ? multi : single).push_back(std::move(kv.second));
  }
  std::vector<Tgt>& moves = multi.empty() ? single : multi;
  if (moves.empty()) return false;
  std::vector<double> w;
  for (const Tgt& t : moves) w.push_back(std::max(t.weight, std::numeric_limits<double>::min()));
  std::discrete_distribution<int> pick(w.begin(), w.end());
  const Tgt& sel = moves[static_cast<size_t>(pick(rng))];
  std::unordered_map<int, int> remap;
  for (const Src& s : sel.sources) if (s.source != sel.target) remap[s.source] = sel.target;
  if (remap.empty()) return false;
  std::vector<int> prop = labels;
  bool changed = false;
  for (size_t i = 0; i < prop.size(); ++i) {
    if (fixed[i] == 1) continue;
    const auto it = remap.find(prop[i]);
    if (it == remap.end()) continue;
    prop[i] = it->second;
    changed = true;
  }
  if (!changed) return false;
  std::vector<int> u = prop;
  std::sort(u.begin(), u.end());
  const int after = static_cast<int>(std::unique(u.begin(), u.end()) - u.begin());
  if (after <= 1 || after >= nc) return false;
  labels.swap(prop);
  return true;
}

// The same proposal over dense codes: label and prediction values are ranked
// in ascending order, which is the order the std::map statistics iterate in,
// so every comparison, every sum and the one discrete draw are the map form's.
// Falls back to absorption_map for sparse values or many classes.
bool absorption(std::vector<int>& labels, const std::vector<int>& prev, const std::vector<int>& fixed,
                std::mt19937_64& rng) {
  const size_t n_rows = labels.size();
  if (n_rows == 0) return false;
  int lo = labels[0], hi = labels[0];
  for (size_t i = 0; i < n_rows; ++i) {
    lo = std::min(lo, std::min(labels[i], prev[i]));
    hi = std::max(hi, std::max(labels[i], prev[i]));
  }
  const long long span = static_cast<long long>(hi) - lo + 1;
  if (span > (1LL << 20)) return absorption_map(labels, prev, fixed, rng);
  thread_local std::vector<int> lut, vals, sizes, movable, trans, remap;
  thread_local std::vector<char> seen;
  lut.assign(static_cast<size_t>(span), -1);
  for (size_t i = 0; i < n_rows; ++i) {
    lut[static_cast<size_t>(labels[i] - lo)] = 0;
    lut[static_cast<size_t>(prev[i] - lo)] = 0;
  }
  vals.clear();
  for (long long v = 0; v < span; ++v)
    if (lut[static_cast<size_t>(v)] == 0) {
      lut[static_cast<size_t>(v)] = static_cast<int>(vals.size());
      vals.push_back(static_cast<int>(v + lo));
    }
  const int C = static_cast<int>(vals.size());
  if (C > 2048) return absorption_map(labels, prev, fixed, rng);
  sizes.assign(static_cast<size_t>(C), 0);
  movable.assign(static_cast<size_t>(C), 0);
  trans.assign(static_cast<size_t>(C) * C, 0);
  for (size_t i = 0; i < n_rows; ++i) {
    const int a = lut[static_cast<size_t>(labels[i] - lo)];
    const int b = lut[static_cast<size_t>(prev[i] - lo)];
    ++sizes[a];
    ++trans[static_cast<size_t>(a) * C + b];
    if (fixed[i] != 1) ++movable[a];
  }
  int nc = 0;
  for (int a = 0; a < C; ++a) nc += sizes[a] > 0;
  if (nc <= 2) return false;
  const double n = static_cast<double>(n_rows);
  struct Src { int source; double surplus; };
  struct Tgt { int target = 0; double weight = 0.0; std::vector<Src> sources; };
  std::map<int, Tgt> by_target;
  for (int a = 0; a < C; ++a) {
    if (sizes[a] == 0 || movable[a] <= 0) continue;
    const int src = vals[a], ssize = sizes[a];
    const int* row = trans.data() + static_cast<size_t>(a) * C;
    const int stay = row[a];
    int bt = src, bcount = 0, bsize = ssize;
    double bsur = 0.0;
    for (int b = 0; b < C; ++b) {
      if (row[b] == 0 || b == a || sizes[b] == 0) continue;
      const double expected = static_cast<double>(ssize) * static_cast<double>(sizes[b]) / std::max(1.0, n);
      const double sur = static_cast<double>(row[b]) - expected;
      const int dv = vals[b];
      if (sur > bsur || (sur == bsur && row[b] > bcount) ||
          (sur == bsur && row[b] == bcount && sizes[b] > bsize) ||
          (sur == bsur && row[b] == bcount && sizes[b] == bsize && dv < bt)) {
        bt = dv;
        bsize = sizes[b];
        bcount = row[b];
        bsur = sur;
      }
    }
    if (bt == src || bsur <= 0.0 || bcount <= stay) continue;
    Tgt& t = by_target[bt];
    t.target = bt;
    t.weight += bsur;
    t.sources.push_back(Src{src, bsur});
  }
  if (by_target.empty()) return false;
  std::vector<Tgt> multi, single;
  for (auto& kv : by_target) {
    std::sort(kv.second.sources.begin(), kv.second.sources.end(), [](const Src& x, const Src& y) {
      if (x.surplus != y.surplus) return x.surplus > y.surplus;
      return x.source < y.source;
    });
    (kv.second.sources.size() > 1 ? multi : single).push_back(std::move(kv.second));
  }
  std::vector<Tgt>& moves = multi.empty() ? single : multi;
  if (moves.empty()) return false;
  std::vector<double> w;
  for (const Tgt& t : moves) w.push_back(std::max(t.weight, std::numeric_limits<double>::min()));
  std::discrete_distribution<int> pick(w.begin(), w.end());
  const Tgt& sel = moves[static_cast<size_t>(pick(rng))];
  remap.assign(static_cast<size_t>(C), -1);
  bool any = false;
  for (const Src& x : sel.sources)
    if (x.source != sel.target) {
      remap[static_cast<size_t>(lut[static_cast<size_t>(x.source - lo)])] = lut[static_cast<size_t>(sel.target - lo)];
      any = true;
    }
  if (!any) return false;
  bool changed = false;
  seen.assign(static_cast<size_t>(C), 0);
  thread_local std::vector<int> prop;
  prop.resize(n_rows);
  for (size_t i = 0; i < n_rows; ++i) {
    int a = lut[static_cast<size_t>(labels[i] - lo)];
    if (fixed[i] != 1 && remap[static_cast<size_t>(a)] >= 0) {
      a = remap[static_cast<size_t>(a)];
      changed = true;
    }
    prop[i] = a;
    seen[static_cast<size_t>(a)] = 1;
  }
  if (!changed) return false;
  int after = 0;
  for (int a = 0; a < C; ++a) after += seen[a];
  if (after <= 1 || after >= nc) return false;
  for (size_t i = 0; i < n_rows; ++i) labels[i] = vals[static_cast<size_t>(prop[i])];
  return true;
}

// Number of distinct values (a value-range bitmap; a sort for sparse values).
int count_distinct(const std::vector<int>& v) {
  if (v.empty()) return 0;
  const auto mm = std::minmax_element(v.begin(), v.end());
  const long long span = static_cast<long long>(*mm.second) - *mm.first + 1;
  if (span > (1LL << 22)) {
    std::vector<int> u = v;
    std::sort(u.begin(), u.end());
    return static_cast<int>(std::unique(u.begin(), u.end()) - u.begin());
  }
  thread_local std::vector<char> bits;
  bits.assign(static_cast<size_t>(span), 0);
  int d = 0;
  for (int x : v) {
    char& b = bits[static_cast<size_t>(x - *mm.first)];
    d += b == 0;
    b = 1;
  }
  return d;
}

int proposal_count(int G, int cycle, int cycles, bool adaptive, std::mt19937_64& rng) {
  if (G <= 1) return std::max(0, G);
  if (!adaptive || cycles <= 1) {
    std::uniform_int_distribution<int> d(1, G);
    return d(rng);
  }
  const double progress = std::clamp(static_cast<double>(cycle + 1) / static_cast<double>(cycles + 1), 0.0, 1.0);
  const double smooth = progress * progress * (3.0 - 2.0 * progress);
  const double temp = std::clamp(1.0 - smooth, 0.0, 1.0);
  const int mx = std::max(1, 1 + static_cast<int>(std::floor(static_cast<double>(G - 1) * temp)));
  std::uniform_int_distribution<int> d(1, mx);
  return d(rng);
}

// DistanceMetric values (kodama.hpp:27-31)
constexpr int kMetricCosine = 0, kMetricInner = 1, kMetricEuclidean = 2;

struct CoreOpts {
  int cycles = 100, k = 30, folds = 10;
  int metric = 2;  // knn.metric of the graph vote: 2 Euclidean (score -(d*d)), else 1 - d
  bool stratified = true, evolutionary = false, guarded = false, absorption = false, adaptive = true;
  bool coarsening = false;  // auto_class_coarsening (PLS-LDA classifier)
  uint64_t seed = 1, cv_seed = 1;
  Policy policy;
};

struct CoreOut {
  std::vector<int> clbest, cvpredbest, folds;
  std::vector<double> vect_acc, vect_score;
  std::vector<int> proposal_size, active_classes;
  std::vector<unsigned char> accepted, improving, temperature;
  double accbest = 0.0, scorebest = 0.0;
  // cycles_completed, proposals_evaluated, best_state_updates, current_state_accepts,
  // stochastic attempts / accepts, rejections, coarsening_moves, absorption_moves,
  // transition attempted / accepted, many_to_one attempted / accepted, cv_evaluations,
  // success, pls_coarsening_attempted, pls_coarsening_accepted
  int counters[18] = {0};
};

// maximize_core (core.cpp:1269-1549) for any predictor labels -> CV predictions.
template <class Predict>
CoreOut core_run(int samples, const std::vector<int>& init, const std::vector<int>& constrain,
                 const std::vector<int>& fixed_in, const CoreOpts& o, Predict&& predict) {
  CoreOut r;
  const int T = o.cycles;
  std::vector<int> fixed = fixed_in.empty() ? std::vector<int>(static_cast<size_t>(samples), 0) : fixed_in;
  r.vect_acc.assign(T, -1.0);
  r.vect_score.assign(T, -1.0);
  r.proposal_size.assign(T, 0);
  r.active_classes.assign(T, 0);
  r.accepted.assign(T, 0);
  r.improving.assign(T, 0);
  r.temperature.assign(T, 0);
  // groups: singletons without a constraint, else ascending constrain values
  const bool singleton = constrain.empty();
  std::vector<std::vector<int>> members;
  if (!singleton) {
    std::map<int, std::vector<int>> m;
    for (int i = 0; i < samples; ++i) m[constrain[i]].push_back(i);
    for (auto& kv : m) members.push_back(kv.second);
  }
  const int G = singleton ? samples : static_cast<int>(members.size());
  auto accuracy = [&](const std::vector<int>& a, const std::vector<int>& b) {
    size_t ok = 0;
    for (size_t i = 0; i < a.size(); ++i) ok += a[i] == b[i];
    return static_cast<double>(ok) / static_cast<double>(a.size());
  };
  auto distinct = [](const std::vector<int>& v) { return count_distinct(v); };
  std::mt19937_64 rng(o.seed);
  r.clbest = init;
  r.cvpredbest = predict(r.clbest);
  int cv_evals = 1, proposals = 0, best_updates = 0, accepts = 0, st_attempts = 0, st_accepts = 0,
      rejections = 0, absorb_moves = 0, tr_attempted = 0, tr_accepted = 0, m1_att = 0, m1_acc = 0,
      co_moves = 0, co_att = 0, co_acc = 0;
  bool success = false;
  r.accbest = accuracy(r.clbest, r.cvpredbest);
  r.scorebest = objective(r.clbest, r.accbest, o.guarded, o.policy, o.coarsening);
  std::vector<int> cur = r.clbest, curpred = r.cvpredbest;
  double cur_acc = r.accbest, cur_score = r.scorebest;
  std::vector<int> groups(static_cast<size_t>(G));
  for (int cycle = 0; cycle < T; ++cycle) {
    std::vector<int> cl = o.evolutionary ? cur : r.clbest;
    const std::vector<int>& pp = o.evolutionary ? curpred : r.cvpredbest;
    if (G > 0) {
      const int ns = proposal_count(G, cycle, T, o.adaptive && o.policy.adaptive_proposal_size, rng);
      r.proposal_size[cycle] = ns;
      std::iota(groups.begin(), groups.end(), 0);
      std::shuffle(groups.begin(), groups.end(), rng);
      std::vector<int> emp_l, emp_c;
      if (!o.policy.prediction_guidance) {
        emp_l = cl;
        std::sort(emp_l.begin(), emp_l.end());
        for (size_t i = 0; i < emp_l.size();) {
          size_t j = i + 1;
          while (j < emp_l.size() && emp_l[j] == emp_l[i]) ++j;
          emp_c.push_back(static_cast<int>(j - i));
          i = j;
        }
        emp_l.erase(std::unique(emp_l.begin(), emp_l.end()), emp_l.end());
      }
      std::vector<int> eligible, cand_l, cand_c;
      for (int s = 0; s < ns; ++s) {
        const int g = groups[s];
        eligible.clear();
        if (singleton) {
          if (fixed[g] != 1) eligible.push_back(g);
        } else {
          for (int idx : members[g]) if (fixed[idx] != 1) eligible.push_back(idx);
        }
        if (eligible.empty()) continue;
        cand_l.clear();
        cand_c.clear();
        if (o.policy.prediction_guidance) {
          for (int idx : eligible) cand_l.push_back(pp[idx]);
          std::sort(cand_l.begin(), cand_l.end());
          for (size_t i = 0; i < cand_l.size();) {
            size_t j = i + 1;
            while (j < cand_l.size() && cand_l[j] == cand_l[i]) ++j;
            cand_c.push_back(static_cast<int>(j - i));
            i = j;
          }
          cand_l.erase(std::unique(cand_l.begin(), cand_l.end()), cand_l.end());
        } else {
          cand_l = emp_l;
          cand_c = emp_c;
        }
        if (cand_l.empty()) continue;
        std::discrete_distribution<int> dist(cand_c.begin(), cand_c.end());
        const int rep = cand_l[static_cast<size_t>(dist(rng))];
        for (int idx : eligible) cl[idx] = rep;
      }
    }
    bool absorbed = false, coarsened = false;
    const bool attempt_co = o.policy.transition_proposal && o.coarsening && o.policy.pls_transition_coarsening;
    const bool attempt = o.policy.transition_proposal && o.absorption;
    if (attempt_co || attempt) ++tr_attempted;
    if (attempt_co) {
      ++co_att;
      coarsened = coarsening(cl, pp, fixed, rng);
      if (coarsened) ++co_moves;
    }
    if (attempt) {
      ++m1_att;
      absorbed = absorption(cl, pp, fixed, rng);
      if (absorbed) ++absorb_moves;
    }
    const std::vector<int> pred = predict(cl);
    ++cv_evals;
    ++proposals;
    const double acc = accuracy(cl, pred);
    const double score = objective(cl, acc, o.guarded, o.policy, o.coarsening);
    const bool improves = score > r.scorebest;
    if (improves) {
      r.cvpredbest = pred;
      r.clbest = cl;
      r.accbest = acc;
      r.scorebest = score;
      ++best_updates;
    }
    bool accepted = improves, improving = improves, stoch = false;
    if (o.evolutionary) {
      const double cooling = 1.0 - static_cast<double>(cycle + 1) / static_cast<double>(std::max(1, T));
      const double temp = std::max(1.0e-9, 0.10 * std::max(0.0, 1.0 - cur_acc) * cooling);
      bool acc_cur = score >= cur_score;
      improving = acc_cur;
      if (!acc_cur && o.policy.stochastic_acceptance && temp > 1.0e-9) {
        ++st_attempts;
        std::uniform_real_distribution<double> u(0.0, 1.0);
        acc_cur = u(rng) < std::exp((score - cur_score) / temp);
        stoch = acc_cur;
      }
      if (acc_cur) {
        cur = cl;
        curpred = pred;
        cur_acc = acc;
        cur_score = score;
        ++accepts;
        if (stoch) ++st_accepts;
      } else {
        ++rejections;
      }
      accepted = acc_cur;
    }
    r.accepted[cycle] = accepted ? 1 : 0;
    r.improving[cycle] = accepted && improving ? 1 : 0;
    r.temperature[cycle] = stoch ? 1 : 0;
    if (accepted && (coarsened || absorbed)) {
      ++tr_accepted;
      if (coarsened) ++co_acc;
      if (absorbed) ++m1_acc;
    }
    r.active_classes[cycle] = distinct(o.evolutionary ? cur : r.clbest);
    r.vect_acc[cycle] = r.accbest;
    r.vect_score[cycle] = r.scorebest;
    if (acc == 1.0 && std::isfinite(score)) success = true;
  }
  const int c[18] = {T, proposals, best_updates, accepts, st_attempts, st_accepts, rejections, co_moves,
                     absorb_moves, tr_attempted, tr_accepted, m1_att, m1_acc, cv_evals, success ? 1 : 0, 0,
                     co_att, co_acc};
  std::memcpy(r.counters, c, sizeof(c));
  return r;
}

// CoreKNNGraph_CPU: maximize_core with the kNN graph predictor
// (core_knn_graph_backend, core.cpp:1574-1620).
CoreOut core_knn_graph(const int* gidx, const float* gdist, int samples, int gk, int index_base,
                       const std::vector<int>& init, const std::vector<int>& constrain,
                       const std::vector<int>& fixed_in, const CoreOpts& o) {
  const std::vector<int> folds = make_folds(init, constrain, o.folds, o.stratified, o.cv_seed);
  const VoteTable table = build_vote_table(gidx, gdist, samples, gk, index_base, folds, o.k,
                                           o.metric == kMetricEuclidean);
  int nfold = 0;
  for (int f : folds) nfold = std::max(nfold, f + 1);
  std::vector<int> universe = init;
  std::sort(universe.begin(), universe.end());
  universe.erase(std::unique(universe.begin(), universe.end()), universe.end());
  VoteScratch scratch;
  CoreOut r = core_run(samples, init, constrain, fixed_in, o, [&](const std::vector<int>& labels) {
    return vote_predict(table, labels, universe, nfold, scratch);
  });
  r.folds = folds;
  return r;
}

// ---------------------------------------------------------------------------
// Raw-data fold-wise kNN: KNNCV_CUDA (knncv.cpp:421-488) and CoreKNN_CUDA
// (core.cpp:1782-1808 via precompute_knn_cv_cuda :695-782) with the exact
// search.  The reference's exact CUDA search (native_cuda_backend.hpp:165) has
// no source in the checkout and its CPU paths use approximate HNSW, so the
// exact search is defined here as on the device: the canonical distance below,
// neighbours ranked by (distance, row).
// ---------------------------------------------------------------------------

// Rows as searched (make_search_matrix): cosine rows multiplied in double by
// 1 / ||row|| (when finite and positive) and rounded to float; other metrics
// unchanged.  mode 0 sums the squares sequentially in double
// (knncv.cpp:85-108); mode 1 is core.cpp:166-195's long double sum in the x86
// 80-bit format (ext80.h: exact float squares, 64-bit significand sums)
// rounded to double; mode 2 is that sum with the row scaled in float
// (kodama_matrix.cpp:155-167, the global graph of KODAMA.matrix).
std::vector<float> search_matrix(const float* x, int n, int d, int metric, int mode) {
  std::vector<float> out(x, x + static_cast<size_t>(n) * d);
  if (metric != kMetricCosine) return out;
  for (int r = 0; r < n; ++r) {
    const float* row = x + static_cast<size_t>(r) * d;
    double ss;
    if (mode == 0) {
      ss = 0.0;
      for (int j = 0; j < d; ++j) ss += static_cast<double>(row[j]) * static_cast<double>(row[j]);
    } else {
      Ext80 acc{0, 0};
      bool finite = true;
      for (int j = 0; j < d; ++j) {
        finite = finite && std::isfinite(row[j]);
        acc = ext80_add(acc, ext80_float_square(row[j]));
      }
      ss = finite ? ext80_to_double(acc) : std::numeric_limits<double>::infinity();
    }
    const double nrm = std::sqrt(ss);
    if (mode == 2) {
      // normalize_rows_for_cosine (kodama_matrix.cpp:155-167): the float row
      // times the float rounding of 1 / norm; zero or non-finite norms skip
      if (!(nrm > 0.0) || !std::isfinite(nrm)) continue;
      const float scale = static_cast<float>(1.0 / nrm);
      for (int j = 0; j < d; ++j) out[static_cast<size_t>(r) * d + j] = row[j] * scale;
      continue;
    }
    const double scale = nrm > 0.0 && std::isfinite(nrm) ? 1.0 / nrm : 1.0;
    for (int j = 0; j < d; ++j)
      out[static_cast<size_t>(r) * d + j] = static_cast<float>(static_cast<double>(row[j]) * scale);
  }
  return out;
}

// Canonical internal distance: squared L2 as a float chain of separately
// rounded (a - b)^2 terms in coordinate order; for the inner product and
// cosine, minus the float chain of the a * b products (the internal
// representation of native_knn.cpp:40-95, score = -distance, :1153).
float canon_distance(const float* a, const float* b, int d, bool inner) {
  float acc = 0.0f;
  if (inner) {
    for (int j = 0; j < d; ++j) acc = acc + a[j] * b[j];
    return -acc;
  }
  for (int j = 0; j < d; ++j) {
    const float diff = a[j] - b[j];
    acc = acc + diff * diff;
  }
  return acc;
}

// The exact global graph under a metric (kgb_knn_graph_metric): cosine on the
// rows of search_matrix mode 2, ranked by (canon_distance, row), self
// excluded; reported distance native_knn_output_distance
// (native_knn.cpp:1157-1164): max(0, 1 + v) for cosine, 1 + v for the inner
// product.  The Euclidean graph is exact_knn.
void exact_knn_metric(const float* x, int n, int d, int K, int metric, int* idx, float* dist, int threads) {
  if (metric == kMetricEuclidean) {
    exact_knn(x, n, d, K, idx, dist, threads);
    return;
  }
  const std::vector<float> xs = search_matrix(x, n, d, metric, 2);
  auto work = [&](int t) {
    std::vector<std::pair<float, int>> row(static_cast<size_t>(n));
    for (int i = t; i < n; i += threads) {
      int m = 0;
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        row[m++] = {canon_distance(xs.data() + static_cast<size_t>(i) * d, xs.data() + static_cast<size_t>(j) * d, d,
                                   true), j};
      }
      const int take = std::min(K, m);
      std::partial_sort(row.begin(), row.begin() + take, row.begin() + m);
      for (int c = 0; c < K; ++c) {
        const size_t o = static_cast<size_t>(i) * K + c;
        if (c < take) {
          idx[o] = row[c].second;
          const float v = 1.0f + row[c].first;
          dist[o] = metric == kMetricCosine ? std::max(0.0f, v) : v;
        } else {
          idx[o] = -1;
          dist[o] = std::numeric_limits<float>::infinity();
        }
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) pool.emplace_back(work, t);
  for (auto& th : pool) th.join();
}

// Every fold must keep training rows (knncv.cpp:142, core.cpp:705).
void check_training_rows(const std::vector<int>& folds) {
  std::map<int, int> size;
  for (int f : folds) size[f]++;
  for (const auto& kv : size)
    if (kv.second == static_cast<int>(folds.size())) throw std::runtime_error("KNN fold has no training samples.");
}

// For each row its k nearest rows of the other folds by (distance, row), as a
// vote table with score = -distance.  Fewer than k candidates leave -1 slots
// (k = min(k, training rows) per fold).
VoteTable fold_knn_table(const std::vector<float>& xs, int n, int d, bool inner, const std::vector<int>& folds, int k) {
  VoteTable t;
  t.samples = n;
  t.width = std::max(1, k);
  t.folds = folds;
  t.nb.assign(static_cast<size_t>(n) * t.width, -1);
  t.score.assign(static_cast<size_t>(n) * t.width, -std::numeric_limits<float>::infinity());
  std::vector<std::pair<float, int>> cand;
  for (int r = 0; r < n; ++r) {
    cand.clear();
    for (int j = 0; j < n; ++j) {
      if (folds[j] == folds[r]) continue;
      cand.emplace_back(canon_distance(&xs[static_cast<size_t>(r) * d], &xs[static_cast<size_t>(j) * d], d, inner), j);
    }
    const int m = std::min<int>(t.width, static_cast<int>(cand.size()));
    std::partial_sort(cand.begin(), cand.begin() + m, cand.end(), [](const auto& a, const auto& b) {
      return a.first < b.first || (a.first == b.first && a.second < b.second);
    });
    for (int c = 0; c < m; ++c) {
      t.nb[static_cast<size_t>(r) * t.width + c] = cand[c].second;
      t.score[static_cast<size_t>(r) * t.width + c] = -cand[c].first;
    }
  }
  return t;
}

// majority_vote (knncv.cpp:111-131) of every row over its table row: per label
// the count and the double sum of the scores in neighbour order; the largest
// count, then the larger sum, then the smaller label.
std::vector<int> majority_votes(const VoteTable& t, const std::vector<int>& labels) {
  std::vector<int> pred(static_cast<size_t>(t.samples), 0);
  for (int r = 0; r < t.samples; ++r) {
    std::map<int, std::pair<int, double>> votes;
    for (int j = 0; j < t.width; ++j) {
      const int nb = t.nb[static_cast<size_t>(r) * t.width + j];
      if (nb < 0) continue;
      auto& v = votes[labels[nb]];
      v.first += 1;
      v.second += static_cast<double>(t.score[static_cast<size_t>(r) * t.width + j]);
    }
    if (votes.empty()) continue;
    int bl = votes.begin()->first, bc = votes.begin()->second.first;
    double bs = votes.begin()->second.second;
    for (const auto& kv : votes) {
      if (kv.second.first > bc || (kv.second.first == bc && kv.second.second > bs) ||
          (kv.second.first == bc && kv.second.second == bs && kv.first < bl)) {
        bl = kv.first;
        bc = kv.second.first;
        bs = kv.second.second;
      }
    }
    pred[r] = bl;
  }
  return pred;
}

// KNNCV with the exact search: predictions and fold assignments.
std::vector<int> knncv(const float* x, int n, int d, const std::vector<int>& labels, const std::vector<int>& constrain,
                       int k, int nfolds, bool stratified, int metric, uint64_t cv_seed, std::vector<int>& folds) {
  if (k < 1) throw std::invalid_argument("KNNOptions::k must be positive.");
  folds = make_folds(labels, constrain, nfolds, stratified, cv_seed);
  check_training_rows(folds);
  const std::vector<float> xs = search_matrix(x, n, d, metric, 0);
  const VoteTable t = fold_knn_table(xs, n, d, metric != kMetricEuclidean, folds, k);
  return majority_votes(t, labels);
}

// CoreKNN with the exact search: maximize_core over the fold-wise tables.
CoreOut core_knn(const float* x, int n, int d, const std::vector<int>& init, const std::vector<int>& constrain,
                 const std::vector<int>& fixed_in, const CoreOpts& o, int metric) {
  if (o.k < 1) throw std::invalid_argument("KNNOptions::k must be positive.");
  const std::vector<int> folds = make_folds(init, constrain, o.folds, o.stratified, o.cv_seed);
  check_training_rows(folds);
  const std::vector<float> xs = search_matrix(x, n, d, metric, 1);
  const VoteTable table = fold_knn_table(xs, n, d, metric != kMetricEuclidean, folds, o.k);
  int nfold = 0;
  for (int f : folds) nfold = std::max(nfold, f + 1);
  std::vector<int> universe = init;
  std::sort(universe.begin(), universe.end());
  universe.erase(std::unique(universe.begin(), universe.end()), universe.end());
  VoteScratch scratch;
  CoreOut r = core_run(n, init, constrain, fixed_in, o, [&](const std::vector<int>& labels) {
    return vote_predict(table, labels, universe, nfold, scratch);
  });
  r.folds = folds;
  return r;
}

// CorePLSLDA_CPU (core.cpp:1626-1646): maximize_core with PLSLDACV_CPU as the
// predictor under a fresh data epoch.  Non-stratified folds use the fold cache
// of plscv.cpp:593-667: the first evaluation computes loadings through the
// scores, later ones through the fold Gram (built on the second evaluation).
CoreOut core_plslda(const float* x, int samples, int p, const std::vector<int>& init,
                    const std::vector<int>& constrain, const std::vector<int>& fixed_in, const CoreOpts& o,
                    const PLSOpts& po) {
  PLSFoldCache cache;
  bool have_cache = false;
  CoreOut r = core_run(samples, init, constrain, fixed_in, o, [&](const std::vector<int>& labels) {
    if (po.stratified) return plsldacv(x, samples, p, labels, constrain, po).predicted;
    if (!have_cache) {
      cache = pls_fold_cache(x, samples, p, make_folds(labels, constrain, po.folds, false, po.cv_seed), po);
      have_cache = true;
      return plsldacv_on_cache(cache, samples, p, labels, po, false).predicted;
    }
    if (!cache.gram_built) pls_build_grams(cache, p);
    return plsldacv_on_cache(cache, samples, p, labels, po, true).predicted;
  });
  r.folds = make_folds(init, constrain, po.folds, po.stratified, po.cv_seed);
  return r;
}

// ---------------------------------------------------------------------------
// KODAMA.matrix, graph-input semantics (kodama_matrix.cpp:3324-4051
// run_kodama_matrix with a caller graph; run_iteration :2870-3322).
// ---------------------------------------------------------------------------
uint64_t fnv_hash(const std::vector<int>& v) {
  uint64_t h = 1469598103934665603ull;
  for (int x : v) {
    const uint32_t b = static_cast<uint32_t>(x);
    for (int s = 0; s < 32; s += 8) {
      h ^= static_cast<uint8_t>((b >> s) & 0xffu);
      h *= 1099511628211ull;
    }
  }
  return h;
}

struct MatrixOpts {
  int runs, cycles, landmarks, splitting, graph_neighbors, folds, knn_k, threads, materialize,
      classifier, components, apply_dissim, first_run, metric;
};

int majority_of(const std::vector<int>& v) {
  std::map<int, int> c;
  for (int x : v) c[x] += 1;
  int bl = c.begin()->first, bc = c.begin()->second;
  for (const auto& kv : c) if (kv.second > bc || (kv.second == bc && kv.first < bl)) { bl = kv.first; bc = kv.second; }
  return bl;
}

// Grouping helpers of the semi-supervised KODAMA.matrix (kodama_matrix.cpp):
// normalize_constrain :183-201 (ids 1.. by first appearance; none = each row
// its own group), factor_subset :988-1001 (the same over a row subset) and
// constrained_majority :1003-1011 (every row takes its group's majority label,
// ties to the smaller label).
std::vector<int> first_appearance_ids(const int* values, const std::vector<int>& rows) {
  std::map<int, int> ids;
  std::vector<int> out(rows.size(), 0);
  for (size_t i = 0; i < rows.size(); ++i) {
    auto it = ids.find(values[rows[i]]);
    if (it == ids.end()) it = ids.emplace(values[rows[i]], static_cast<int>(ids.size()) + 1).first;
    out[i] = it->second;
  }
  return out;
}

std::vector<int> constrained_majority(const std::vector<int>& labels, const std::vector<int>& groups) {
  std::map<int, std::vector<int>> by;
  for (size_t i = 0; i < labels.size(); ++i) by[groups[i]].push_back(labels[i]);
  std::map<int, int> lab;
  for (const auto& kv : by) lab[kv.first] = majority_of(kv.second);
  std::vector<int> out(labels.size());
  for (size_t i = 0; i < labels.size(); ++i) out[i] = lab[groups[i]];
  return out;
}

void dissimilarity(int* idx, float* dist, int samples, int K, const int* res, int runs, bool in1, bool out1) {
  std::vector<int> by(static_cast<size_t>(samples) * runs);
  for (int s = 0; s < samples; ++s)
    for (int r = 0; r < runs; ++r) by[static_cast<size_t>(s) * runs + r] = res[static_cast<size_t>(r) * samples + s];
  std::vector<std::pair<float, int>> row(static_cast<size_t>(K));
  for (int i = 0; i < samples; ++i) {
    for (int j = 0; j < K; ++j) {
      const size_t off = static_cast<size_t>(i) * K + j;
      const int stored = idx[off];
      const int nb = stored >= 0 && in1 ? stored - 1 : stored;
      float d = dist[off];
      if (nb < 0 || nb >= samples || !std::isfinite(d)) {
        row[j] = {std::numeric_limits<float>::infinity(), stored};
        continue;
      }
      int same = 0, valid = 0;
      const int* a = by.data() + static_cast<size_t>(i) * runs;
      const int* b = by.data() + static_cast<size_t>(nb) * runs;
      for (int r = 0; r < runs; ++r) {
        const int pv = a[r] != 0 && b[r] != 0;
        valid += pv;
        same += pv && a[r] == b[r];
      }
      if (same == 0 || valid == 0) {
        d = std::numeric_limits<float>::infinity();
      } else {
        const double agr = static_cast<double>(same) / static_cast<double>(valid);
        d = static_cast<float>((1.0 + static_cast<double>(d)) / (agr * agr));
      }
      row[j] = {d, out1 ? nb + 1 : nb};
    }
    std::stable_sort(row.begin(), row.end(), [](const auto& a, const auto& b) {
      if (a.first != b.first) return a.first < b.first;
      return a.second < b.second;
    });
    for (int j = 0; j < K; ++j) {
      dist[static_cast<size_t>(i) * K + j] = row[j].first;
      idx[static_cast<size_t>(i) * K + j] = row[j].second;
    }
  }
}

struct RunOut {
  std::vector<int> res;
  std::vector<double> vect_acc;
  double accbest = 0.0;
  uint64_t hashes[3] = {0, 0, 0};
  int counters[8] = {0};
  int pls[2] = {0, 0};          // pls_coarsening attempted / accepted
  std::vector<int> cycle_diag;  // cycles x 5
};

// Run diagnostics of run_iteration (kodama_matrix.cpp:3290-3316).
void fill_run(RunOut& ro, const CoreOut& core, int run, const std::vector<int>& land, const std::vector<int>& init,
              int L, int cycles) {
  ro.vect_acc = core.vect_acc;
  ro.accbest = core.accbest;
  ro.hashes[0] = fnv_hash(land);
  ro.hashes[1] = fnv_hash(init);
  ro.hashes[2] = fnv_hash(core.folds);
  ro.counters[0] = run;
  ro.counters[1] = core.counters[0];
  ro.counters[2] = core.counters[9];
  ro.counters[3] = core.counters[10];
  ro.counters[4] = core.counters[11];
  ro.counters[5] = core.counters[12];
  ro.counters[6] = core.counters[13];
  ro.counters[7] = L;
  ro.pls[0] = core.counters[16];
  ro.pls[1] = core.counters[17];
  ro.cycle_diag.resize(static_cast<size_t>(cycles) * 5);
  for (int c = 0; c < cycles; ++c) {
    int* cd = ro.cycle_diag.data() + 5 * c;
    cd[0] = core.proposal_size[c];
    cd[1] = core.active_classes[c];
    cd[2] = core.accepted[c];
    cd[3] = core.improving[c];
    cd[4] = core.temperature[c];
  }
}

// starting / constrain / fixed (n entries each, null = none) are the
// semi-supervised inputs of run_kodama_matrix (kodama_matrix.cpp:3405-3420,
// run_iteration :3060-3117, :3277-3283).
void kodama_matrix(const float* x, int n, int d, const int* gidx_in, const float* gdist_in, int gk_in,
                   int index_base, const MatrixOpts& o, uint64_t seed,
                   int* res_out, double* acc_out, double* v_out, uint64_t* hashes_out, int* counters_out,
                   int* cycle_out, int* knn_idx_out, float* knn_dist_out, int* knn_k_out, double* timings,
                   int* pls_out, const int* starting = nullptr, const int* constrain_in = nullptr,
                   const int* fixed_in = nullptr) {
  const auto t0 = std::chrono::steady_clock::now();
  auto since = [](std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
  };
  if (n < 3) throw std::invalid_argument("KODAMAMatrix requires at least 3 rows.");
  if (o.runs < 1 || o.cycles < 0 || o.folds < 2) throw std::invalid_argument("invalid KODAMA.matrix options");
  int landmarks = o.landmarks > 0 ? o.landmarks : 10000;
  if (landmarks >= n) landmarks = static_cast<int>(std::ceil(static_cast<double>(n) * 0.75));
  landmarks = std::max(2, std::min(landmarks, n - 1));
  const int requested = o.graph_neighbors > 0 ? o.graph_neighbors : 100;
  const int neighbors = std::max(1, static_cast<int>(std::floor(std::min({
    static_cast<double>(landmarks), static_cast<double>(n) * 0.75 - 1.0, static_cast<double>(requested)}))));
  // normalize_external_graph (kodama_matrix.cpp:1292-1330)
  int mn = std::numeric_limits<int>::max(), mx = std::numeric_limits<int>::min();
  for (size_t i = 0; i < static_cast<size_t>(n) * gk_in; ++i) {
    if (gidx_in[i] < 0) continue;
    mn = std::min(mn, gidx_in[i]);
    mx = std::max(mx, gidx_in[i]);
  }
  const bool one_based = index_base == 1 || (index_base < 0 && mn >= 1 && mx <= n);
  const int K = std::max(1, std::min(std::min(gk_in, neighbors), gk_in));
  std::vector<int> gidx(static_cast<size_t>(n) * K, -1);
  std::vector<float> gdist(static_cast<size_t>(n) * K, std::numeric_limits<float>::infinity());
  for (int i = 0; i < n; ++i) {
    int col = 0;
    for (int j = 0; j < gk_in && col < K; ++j) {
      const size_t src = static_cast<size_t>(i) * gk_in + j;
      int id = gidx_in[src];
      if (one_based && id > 0) --id;
      if (id < 0 || id >= n || id == i) continue;
      const float dd = gdist_in[src];
      if (!std::isfinite(dd)) continue;
      gidx[static_cast<size_t>(i) * K + col] = id;
      gdist[static_cast<size_t>(i) * K + col] = std::max(0.0f, dd);
      ++col;
    }
  }
  const int splitting = o.splitting > 0 ? o.splitting : (n < 40000 ? 100 : 300);
  std::vector<int> all_rows(static_cast<size_t>(n));
  std::iota(all_rows.begin(), all_rows.end(), 0);
  std::vector<int> groups = all_rows;  // normalize_constrain: 1..n without a constraint
  for (int& g : groups) ++g;
  if (constrain_in != nullptr) groups = first_appearance_ids(constrain_in, all_rows);
  bool identity = true;
  for (int i = 0; i < n; ++i) identity = identity && groups[i] == i + 1;
  // shared landmark atlas (kodama_matrix.cpp:3662-3734)
  const int coarse_k = std::max(2, std::min(splitting, n));
  std::mt19937_64 shared_rng(seed + 1u);
  const std::vector<int> shared = kmeans_labels(x, n, d, coarse_k, shared_rng, 10, o.threads);
  const Strata strata = index_strata(shared, coarse_k);
  const double t_atlas = since(t0);
  const auto t1 = std::chrono::steady_clock::now();

  std::vector<RunOut> outs(static_cast<size_t>(o.runs));
  std::atomic<int> next{1};
  auto worker = [&]() {
    for (;;) {
      const int slot = next.fetch_add(1);
      if (slot > o.runs) break;
      RunOut& ro = outs[static_cast<size_t>(slot - 1)];
      const int run = slot - 1 + (o.first_run > 0 ? o.first_run : 1);
      std::mt19937_64 rng(seed + static_cast<uint64_t>(run));
      (void)rng();
      const std::vector<int> land = quota_sample(strata, landmarks, rng);
      const int L = static_cast<int>(land.size());
      std::vector<float> xl(static_cast<size_t>(L) * d);
      for (int i = 0; i < L; ++i) std::copy_n(x + static_cast<size_t>(land[i]) * d, d, xl.data() + static_cast<size_t>(i) * d);
      std::vector<int> xcon(static_cast<size_t>(L)), xfix(static_cast<size_t>(L), 0), init;
      if (identity) std::iota(xcon.begin(), xcon.end(), 1);
      else xcon = first_appearance_ids(groups.data(), land);
      if (fixed_in != nullptr)
        for (int i = 0; i < L; ++i) xfix[i] = fixed_in[land[i]] != 0 ? 1 : 0;
      if (starting != nullptr) {
        init.resize(static_cast<size_t>(L));
        for (int i = 0; i < L; ++i) init[i] = starting[land[i]];
      } else {
        const int init_k = std::max(2, std::min(splitting, L));
        init = kmeans_labels(xl.data(), L, d, init_k, rng, 10);
      }
      if (!identity) init = constrained_majority(init, xcon);
      // subset_graph_to_rows (kodama_matrix.cpp:1332-1365): one-based local ids
      std::vector<int> g2l(static_cast<size_t>(n), -1);
      for (int i = 0; i < L; ++i) g2l[land[i]] = i;
      std::vector<int> lidx(static_cast<size_t>(L) * K, -1);
      std::vector<float> ldist(static_cast<size_t>(L) * K, std::numeric_limits<float>::infinity());
      for (int i = 0; i < L; ++i) {
        int col = 0;
        for (int j = 0; j < K; ++j) {
          const size_t src = static_cast<size_t>(land[i]) * K + j;
          const int gnb = gidx[src];
          if (gnb < 0 || gnb >= n) continue;
          const int loc = g2l[gnb];
          if (loc < 0 || loc == i) continue;
          lidx[static_cast<size_t>(i) * K + col] = loc + 1;
          ldist[static_cast<size_t>(i) * K + col] = gdist[src];
          ++col;
        }
      }
      const std::vector<int>& constrain = xcon;
      auto finish = [&](RunOut& out_run) {
        if (!identity) out_run.res = constrained_majority(out_run.res, groups);
      };
      if (o.classifier == 1) {
        // PLS-LDA classifier (run_iteration, kodama_matrix.cpp:3105-3158, 3262-3276)
        CoreOpts co;
        co.cycles = o.cycles;
        co.evolutionary = starting == nullptr;
        co.guarded = true;
        co.absorption = true;
        co.adaptive = true;
        co.coarsening = true;
        co.seed = seed + static_cast<uint64_t>(run);
        PLSOpts po;
        po.folds = o.folds;
        po.stratified = false;
        po.cv_seed = seed + static_cast<uint64_t>(run);
        po.max_components = o.components;
        po.fixed_components = o.components;
        const CoreOut core = core_plslda(xl.data(), L, d, init, constrain, xfix, co, po);
        ro.res.assign(static_cast<size_t>(n), 0);
        for (int i = 0; i < L; ++i) ro.res[land[i]] = core.clbest[i];
        std::vector<char> is_land(static_cast<size_t>(n), 0);
        for (int r : land) is_land[r] = 1;
        std::vector<int> tpoints;
        for (int t = 0; t < n; ++t) if (!is_land[t]) tpoints.push_back(t);
        if (!tpoints.empty()) {
          std::vector<float> xt(tpoints.size() * static_cast<size_t>(d));
          for (size_t i = 0; i < tpoints.size(); ++i)
            std::copy_n(x + static_cast<size_t>(tpoints[i]) * d, d, xt.data() + i * d);
          const std::vector<int> proj =
              plslda_predict(xl.data(), L, d, core.clbest, xt.data(), static_cast<int>(tpoints.size()), po);
          for (size_t i = 0; i < tpoints.size(); ++i) ro.res[tpoints[i]] = proj[i];
        }
        finish(ro);
        fill_run(ro, core, run, land, init, L, o.cycles);
        continue;
      }
      CoreOpts co;
      co.cycles = o.cycles;
      co.k = std::max(o.knn_k, 1);
      co.folds = o.folds;
      co.stratified = false;
      co.evolutionary = starting == nullptr;
      co.guarded = true;
      co.absorption = true;
      co.adaptive = true;
      co.seed = seed + static_cast<uint64_t>(run);
      co.cv_seed = seed + static_cast<uint64_t>(run);
      co.metric = o.metric;
      const CoreOut core = core_knn_graph(lidx.data(), ldist.data(), L, K, -1, init, constrain, xfix, co);
      // projection of non-landmarks (kodama_matrix.cpp:3221-3261, majority_label :169)
      ro.res.assign(static_cast<size_t>(n), 0);
      for (int i = 0; i < L; ++i) ro.res[land[i]] = core.clbest[i];
      const int pk = std::max(1, o.knn_k);
      std::vector<char> is_land(static_cast<size_t>(n), 0);
      for (int r : land) is_land[r] = 1;
      std::vector<int> votes;
      for (int t = 0; t < n; ++t) {
        if (is_land[t]) continue;
        votes.clear();
        for (int j = 0; j < K && static_cast<int>(votes.size()) < pk; ++j) {
          const int gnb = gidx[static_cast<size_t>(t) * K + j];
          if (gnb < 0 || gnb >= n) continue;
          const int loc = g2l[gnb];
          if (loc >= 0) votes.push_back(core.clbest[loc]);
        }
        ro.res[t] = votes.empty() ? core.clbest.front() : majority_of(votes);
      }
      finish(ro);
      fill_run(ro, core, run, land, init, L, o.cycles);
    }
  };
  const int workers = std::max(1, std::min(o.threads, o.runs));
  std::vector<std::thread> pool;
  for (int w = 0; w < workers; ++w) pool.emplace_back(worker);
  for (auto& th : pool) th.join();
  const double t_runs = since(t1);

  for (int r = 0; r < o.runs; ++r) {
    const RunOut& ro = outs[r];
    std::copy(ro.res.begin(), ro.res.end(), res_out + static_cast<size_t>(r) * n);
    acc_out[r] = ro.accbest;
    for (int c = 0; c < o.cycles; ++c) v_out[static_cast<size_t>(r) * o.cycles + c] = ro.vect_acc[c];
    for (int h = 0; h < 3; ++h) hashes_out[3 * r + h] = ro.hashes[h];
    for (int c = 0; c < 8; ++c) counters_out[8 * r + c] = ro.counters[c];
    if (pls_out) {
      pls_out[2 * r] = ro.pls[0];
      pls_out[2 * r + 1] = ro.pls[1];
    }
    std::copy(ro.cycle_diag.begin(), ro.cycle_diag.end(), cycle_out + static_cast<size_t>(r) * o.cycles * 5);
  }
  *knn_k_out = o.materialize ? K : 0;
  if (o.materialize) {
    if (o.apply_dissim) dissimilarity(gidx.data(), gdist.data(), n, K, res_out, o.runs, false, false);
    for (size_t i = 0; i < gidx.size(); ++i) {
      knn_idx_out[i] = gidx[i] >= 0 ? gidx[i] + 1 : gidx[i];
      knn_dist_out[i] = gdist[i];
    }
  }
  if (timings) {
    timings[0] = since(t0);
    timings[2] = t_runs;
    timings[4] = t_atlas;
    timings[5] = timings[0];
  }
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C ABI for oracle/oracle.py.  Same argument conventions as the reference
// driver (oracle/ref_driver.cpp) so the two can be compared call for call.
// ---------------------------------------------------------------------------
extern "C" {

int orc_last_error(char* buf, int len) {
  if (len <= 0) return 0;
  std::strncpy(buf, orc::g_error.c_str(), static_cast<size_t>(len - 1));
  buf[len - 1] = '\0';
  return static_cast<int>(orc::g_error.size());
}

int orc_exact_knn(const float* x, int n, int d, int K, int* idx, float* dist, int threads) {
  try {
    orc::exact_knn(x, n, d, K, idx, dist, std::max(1, threads));
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

// The randomized SIMPLS start vector (plscv.cpp:833-838): p draws of
// std::normal_distribution<float> on std::mt19937(1).
int orc_pls_start(int p, float* out) {
  std::mt19937 gen(1u);
  std::normal_distribution<float> nd(0.0f, 1.0f);
  for (int j = 0; j < p; ++j) out[j] = nd(gen);
  return 0;
}

int orc_exact_knn_metric(const float* x, int n, int d, int K, int metric, int* idx, float* dist, int threads) {
  try {
    orc::exact_knn_metric(x, n, d, K, metric, idx, dist, std::max(1, threads));
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

int orc_exact_knn_rows(const float* x, int n, int d, int K, const int* rows, int nrows, int* idx, float* dist,
                       int threads) {
  try {
    orc::exact_knn(x, n, d, K, idx, dist, std::max(1, threads), rows, nrows);
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

int orc_kmeans(const float* x, int n, int p, int k, unsigned long long rng_seed, int discard,
               int max_iter, int* labels) {
  try {
    std::mt19937_64 rng(rng_seed);
    rng.discard(static_cast<unsigned long long>(discard));
    const auto l = orc::kmeans_labels(x, n, p, k, rng, max_iter);
    std::memcpy(labels, l.data(), sizeof(int) * l.size());
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

// Self-check of the x87 extended-precision model against the native
// long double on an x86-64 host (returns the number of mismatches, -1 where
// long double is not the x87 format).
int orc_ext80_selftest(int n, unsigned long long seed) {
#if defined(__x86_64__) && (__LDBL_MANT_DIG__ == 64)
  std::mt19937_64 g(seed);
  int bad = 0;
  auto to_ld = [](Ext80 v) { return v.m == 0 ? 0.0L : std::ldexp(static_cast<long double>(v.m), v.e); };
  for (int i = 0; i < n; ++i) {
    const uint64_t t = 1 + g() % 20000, c = 1 + g() % 20000, smp = 1 + g() % 200000;
    const Ext80 e1 = ext80_div(ext80_from_u64(t * c), ext80_from_u64(smp));
    const long double l1 = static_cast<long double>(t) * static_cast<long double>(c) / static_cast<long double>(smp);
    bad += to_ld(e1) != l1;
    const int base = ext80_floor_int(e1);
    bad += base != static_cast<int>(std::floor(l1));
    const Ext80 f1 = ext80_sub(e1, ext80_from_u64(static_cast<uint64_t>(base)));
    const long double lf = l1 - static_cast<long double>(base);
    bad += to_ld(f1) != lf;
    const uint64_t u = g();
    const Ext80 off = ext80_canonical(u);
    const long double loff = static_cast<long double>(u) / 18446744073709551616.0L;
    bad += to_ld(off) != loff;
    const uint64_t sel = g() % 20000;
    const Ext80 nx = ext80_add(off, ext80_from_u64(sel));
    const long double lnx = loff + static_cast<long double>(sel);
    bad += to_ld(nx) != lnx;
    const Ext80 cum = ext80_add(f1, ext80_add(off, f1));
    const long double lcum = lf + (loff + lf);
    bad += to_ld(cum) != lcum;
    bad += ext80_lt(nx, cum) != (lnx < lcum);
    bad += ext80_lt(f1, off) != (lf < loff);
  }
  return bad;
#else
  (void)n;
  (void)seed;
  return -1;
#endif
}

int orc_dot_x86(const float* a, const float* b, int n, float* out) {
  *out = orc::dot_x86_order(a, b, n);
  return 0;
}

// ext80 self-check hook: returns the quota vector for given strata offsets.
int orc_quota_sample(const int* offsets, int strata, const int* rows, int nrows, int target,
                     unsigned long long seed, int discard, int* out) {
  try {
    orc::Strata st;
    st.offsets.assign(offsets, offsets + strata + 1);
    st.rows.assign(rows, rows + nrows);
    std::mt19937_64 rng(seed);
    rng.discard(static_cast<unsigned long long>(discard));
    const auto v = orc::quota_sample(st, target, rng);
    std::memcpy(out, v.data(), sizeof(int) * v.size());
    return static_cast<int>(v.size()) == target ? 0 : 1;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

int orc_core_knn_graph(
  const int* gidx, const float* gdist, int samples, int gk, int index_base,
  const int* labels, const int* constrain, int has_constrain, const int* fixed, int has_fixed,
  const int* copts, unsigned long long seed, unsigned long long cv_seed,
  int* clbest, int* cvpredbest, int* folds, double* vect_acc, double* vect_score,
  int* proposal_size, int* active_classes, unsigned char* flags3, double* scal_out, int* int_out
) {
  try {
    orc::CoreOpts o;
    o.cycles = copts[0];
    o.k = copts[1];
    o.folds = copts[2];
    o.stratified = copts[3] != 0;
    o.evolutionary = copts[4] != 0;
    o.guarded = copts[5] != 0;
    o.absorption = copts[6] != 0;
    o.adaptive = copts[7] != 0;
    o.metric = copts[8];
    o.seed = seed;
    o.cv_seed = cv_seed;
    std::vector<int> lab(labels, labels + samples);
    std::vector<int> con = has_constrain ? std::vector<int>(constrain, constrain + samples) : std::vector<int>();
    std::vector<int> fix = has_fixed ? std::vector<int>(fixed, fixed + samples) : std::vector<int>();
    const auto r = orc::core_knn_graph(gidx, gdist, samples, gk, index_base, lab, con, fix, o);
    std::memcpy(clbest, r.clbest.data(), sizeof(int) * samples);
    std::memcpy(cvpredbest, r.cvpredbest.data(), sizeof(int) * samples);
    std::memcpy(folds, r.folds.data(), sizeof(int) * samples);
    for (int c = 0; c < o.cycles; ++c) {
      vect_acc[c] = r.vect_acc[c];
      vect_score[c] = r.vect_score[c];
      proposal_size[c] = r.proposal_size[c];
      active_classes[c] = r.active_classes[c];
      flags3[3 * c + 0] = r.accepted[c];
      flags3[3 * c + 1] = r.improving[c];
      flags3[3 * c + 2] = r.temperature[c];
    }
    scal_out[0] = r.accbest;
    scal_out[1] = r.scorebest;
    std::memcpy(int_out, r.counters, sizeof(int) * 16);
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

// KNNCV (exact search); predicted and fold_out have n entries.
int orc_knncv(const float* x, int n, int d, const int* labels, const int* constrain, int has_constrain, int k,
              int folds, int stratified, int metric, unsigned long long cv_seed, int* predicted, int* fold_out) {
  try {
    std::vector<int> lab(labels, labels + n);
    std::vector<int> con = has_constrain ? std::vector<int>(constrain, constrain + n) : std::vector<int>();
    std::vector<int> fo;
    const std::vector<int> pred = orc::knncv(x, n, d, lab, con, k, folds, stratified != 0, metric, cv_seed, fo);
    std::memcpy(predicted, pred.data(), sizeof(int) * n);
    std::memcpy(fold_out, fo.data(), sizeof(int) * n);
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

// CoreKNN (exact search); outputs as orc_core_knn_graph.
int orc_core_knn(
  const float* x, int n, int d, int metric,
  const int* labels, const int* constrain, int has_constrain, const int* fixed, int has_fixed,
  const int* copts, unsigned long long seed, unsigned long long cv_seed,
  int* clbest, int* cvpredbest, int* folds, double* vect_acc, double* vect_score,
  int* proposal_size, int* active_classes, unsigned char* flags3, double* scal_out, int* int_out
) {
  try {
    orc::CoreOpts o;
    o.cycles = copts[0];
    o.k = copts[1];
    o.folds = copts[2];
    o.stratified = copts[3] != 0;
    o.evolutionary = copts[4] != 0;
    o.guarded = copts[5] != 0;
    o.absorption = copts[6] != 0;
    o.adaptive = copts[7] != 0;
    o.seed = seed;
    o.cv_seed = cv_seed;
    std::vector<int> lab(labels, labels + n);
    std::vector<int> con = has_constrain ? std::vector<int>(constrain, constrain + n) : std::vector<int>();
    std::vector<int> fix = has_fixed ? std::vector<int>(fixed, fixed + n) : std::vector<int>();
    const auto r = orc::core_knn(x, n, d, lab, con, fix, o, metric);
    std::memcpy(clbest, r.clbest.data(), sizeof(int) * n);
    std::memcpy(cvpredbest, r.cvpredbest.data(), sizeof(int) * n);
    std::memcpy(folds, r.folds.data(), sizeof(int) * n);
    for (int c = 0; c < o.cycles; ++c) {
      vect_acc[c] = r.vect_acc[c];
      vect_score[c] = r.vect_score[c];
      proposal_size[c] = r.proposal_size[c];
      active_classes[c] = r.active_classes[c];
      flags3[3 * c + 0] = r.accepted[c];
      flags3[3 * c + 1] = r.improving[c];
      flags3[3 * c + 2] = r.temperature[c];
    }
    scal_out[0] = r.accbest;
    scal_out[1] = r.scorebest;
    std::memcpy(int_out, r.counters, sizeof(int) * 16);
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

// starting / constrain / fixed: n entries each, or null.
int orc_kodama_matrix_graph_data_ex(
  const float* x, int n, int d, const int* gidx, const float* gdist, int gk, int index_base,
  const int* o, unsigned long long seed,
  int* res, double* acc, double* v, unsigned long long* hashes, int* run_counters,
  int* cycle_diag, int* out_idx, float* out_dist, int* out_k, double* timings, int* pls_counters,
  const int* starting, const int* constrain, const int* fixed
) {
  try {
    orc::MatrixOpts mo{o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7], o[8], o[9], o[10], o[11], o[12], o[13]};
    if (timings) for (int i = 0; i < 6; ++i) timings[i] = 0.0;
    orc::kodama_matrix(x, n, d, gidx, gdist, gk, index_base, mo, seed, res, acc, v,
                       reinterpret_cast<uint64_t*>(hashes), run_counters, cycle_diag, out_idx, out_dist, out_k,
                       timings, pls_counters, starting, constrain, fixed);
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

int orc_kodama_matrix_graph_data(
  const float* x, int n, int d, const int* gidx, const float* gdist, int gk, int index_base,
  const int* o, unsigned long long seed,
  int* res, double* acc, double* v, unsigned long long* hashes, int* run_counters,
  int* cycle_diag, int* out_idx, float* out_dist, int* out_k, double* timings, int* pls_counters
) {
  return orc_kodama_matrix_graph_data_ex(x, n, d, gidx, gdist, gk, index_base, o, seed, res, acc, v, hashes,
                                         run_counters, cycle_diag, out_idx, out_dist, out_k, timings,
                                         pls_counters, nullptr, nullptr, nullptr);
}

namespace {
orc::PLSOpts pls_opts(const int* popts, unsigned long long cv_seed) {
  orc::PLSOpts o;
  o.folds = popts[0];
  o.stratified = popts[1] != 0;
  o.max_components = popts[2];
  o.fixed_components = popts[3];
  o.center = popts[4] != 0;
  o.scale = popts[5] != 0;
  o.cv_seed = cv_seed;
  return o;
}
}  // namespace

// Same conventions as ref_plsldacv (oracle/ref_driver.cpp).
int orc_plsldacv(const float* x, int n, int d, const int* labels, const int* constrain, int has_constrain,
                 const int* popts, unsigned long long cv_seed, int* predicted, int* folds,
                 int* selected_components, double* accuracy_by_components, double* seconds) {
  try {
    orc::PLSOpts o = pls_opts(popts, cv_seed);
    o.da = popts[7] != 0;
    std::vector<int> lab(labels, labels + n);
    std::vector<int> con = has_constrain ? std::vector<int>(constrain, constrain + n) : std::vector<int>();
    const auto t0 = std::chrono::steady_clock::now();
    const auto r = orc::plsldacv(x, n, d, lab, con, o);
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::memcpy(predicted, r.predicted.data(), sizeof(int) * n);
    std::memcpy(folds, r.folds.data(), sizeof(int) * n);
    *selected_components = r.selected_components;
    for (int i = 0; i < o.max_components; ++i) accuracy_by_components[i] = r.accuracy_by_components[i];
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

int orc_plsldapredict(const float* train, int n, int d, const int* labels, const float* test, int nt,
                       const int* popts, int* predicted) {
  try {
    const orc::PLSOpts o = pls_opts(popts, 1);
    std::vector<int> lab(labels, labels + n);
    const auto r = orc::plslda_predict(train, n, d, lab, test, nt, o);
    std::memcpy(predicted, r.data(), sizeof(int) * r.size());
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

// CorePLSLDA_CPU.  copts as orc_core_knn_graph plus copts[8] =
// auto_class_coarsening; popts as orc_plsldacv; int_out has 18 counters.
int orc_core_plslda(
  const float* x, int samples, int d, const int* labels, const int* constrain, int has_constrain,
  const int* fixed, int has_fixed, const int* copts, const int* popts, unsigned long long seed,
  unsigned long long cv_seed, int* clbest, int* cvpredbest, int* folds, double* vect_acc, double* vect_score,
  int* proposal_size, int* active_classes, unsigned char* flags3, double* scal_out, int* int_out
) {
  try {
    orc::CoreOpts o;
    o.cycles = copts[0];
    o.evolutionary = copts[4] != 0;
    o.guarded = copts[5] != 0;
    o.absorption = copts[6] != 0;
    o.adaptive = copts[7] != 0;
    o.coarsening = copts[8] != 0;
    o.seed = seed;
    const orc::PLSOpts po = pls_opts(popts, cv_seed);
    std::vector<int> lab(labels, labels + samples);
    std::vector<int> con = has_constrain ? std::vector<int>(constrain, constrain + samples) : std::vector<int>();
    std::vector<int> fix = has_fixed ? std::vector<int>(fixed, fixed + samples) : std::vector<int>();
    const auto r = orc::core_plslda(x, samples, d, lab, con, fix, o, po);
    std::memcpy(clbest, r.clbest.data(), sizeof(int) * samples);
    std::memcpy(cvpredbest, r.cvpredbest.data(), sizeof(int) * samples);
    std::memcpy(folds, r.folds.data(), sizeof(int) * samples);
    for (int c = 0; c < o.cycles; ++c) {
      vect_acc[c] = r.vect_acc[c];
      vect_score[c] = r.vect_score[c];
      proposal_size[c] = r.proposal_size[c];
      active_classes[c] = r.active_classes[c];
      flags3[3 * c + 0] = r.accepted[c];
      flags3[3 * c + 1] = r.improving[c];
      flags3[3 * c + 2] = r.temperature[c];
    }
    scal_out[0] = r.accbest;
    scal_out[1] = r.scorebest;
    std::memcpy(int_out, r.counters, sizeof(r.counters));
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

int orc_dissimilarity(int* gidx, float* gdist, int samples, int gk, const int* res, int runs, int /*threads*/) {
  try {
    orc::dissimilarity(gidx, gdist, samples, gk, res, runs, true, true);
    return 0;
  } catch (const std::exception& e) {
    orc::g_error = e.what();
    return 1;
  }
}

}  // extern "C"
