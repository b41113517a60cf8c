// Host-side planning of per-run random choices (see host_plan.h).
#include "host_plan.h"

#include "ext80.h"

#include <algorithm>
#include <iterator>
#include <map>
#include <numeric>
#include <stdexcept>
#include <unordered_map>

namespace kgb {

Strata index_strata(const std::vector<int>& labels, int strata) {
  if (strata < 1) throw std::invalid_argument("Landmark strata count must be positive.");
  Strata s;
  s.offsets.assign(static_cast<std::size_t>(strata) + 1, 0);
  s.rows.resize(labels.size());
  for (int l : labels) {
    if (l < 1 || l > strata) throw std::invalid_argument("Landmark stratum label is out of range.");
    ++s.offsets[static_cast<std::size_t>(l)];
  }
  for (int t = 1; t <= strata; ++t) s.offsets[t] += s.offsets[t - 1];
  std::vector<int> cursor = s.offsets;
  for (std::size_t r = 0; r < labels.size(); ++r) {
    s.rows[static_cast<std::size_t>(cursor[labels[r] - 1]++)] = static_cast<int>(r);
  }
  return s;
}

// Quota allocation: floor of each stratum's proportional share, then the
// residual slots by systematic sampling over the shuffled strata with one
// uniform offset, the cumulative fractional parts compared in x87 extended
// precision (ext80.h); then std::sample inside each stratum.
std::vector<int> quota_sample(const Strata& st, int target, std::mt19937_64& rng) {
  if (st.offsets.size() < 2 || st.offsets.front() != 0 ||
      st.offsets.back() != static_cast<int>(st.rows.size())) {
    throw std::invalid_argument("Invalid landmark strata index.");
  }
  const int samples = static_cast<int>(st.rows.size());
  target = std::max(1, std::min(target, samples));
  const int strata = static_cast<int>(st.offsets.size()) - 1;
  std::vector<int> quota(static_cast<std::size_t>(strata), 0);
  std::vector<Ext80> frac(static_cast<std::size_t>(strata), Ext80{0, 0});
  std::vector<int> order;
  order.reserve(static_cast<std::size_t>(strata));
  int assigned = 0;
  const Ext80 total = ext80_from_u64(static_cast<uint64_t>(samples));
  for (int s = 0; s < strata; ++s) {
    const int count = st.offsets[s + 1] - st.offsets[s];
    if (count <= 0) continue;
    order.push_back(s);
    const Ext80 expected =
        ext80_div(ext80_from_u64(static_cast<uint64_t>(target) * static_cast<uint64_t>(count)), total);
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
    std::vector<char> rounded(static_cast<std::size_t>(strata), 0);
    for (int s : order) {
      cumulative = ext80_add(cumulative, frac[s]);
      const Ext80 next = ext80_add(offset, ext80_from_u64(static_cast<uint64_t>(selected)));
      if (selected < residual && ext80_lt(next, cumulative)) {
        ++quota[s];
        rounded[s] = 1;
        ++selected;
      }
    }
    while (selected < residual) {
      int best = -1;
      Ext80 bestv{0, 0};
      for (int s : order) {
        if (rounded[s]) continue;
        if (best < 0 || ext80_lt(bestv, frac[s])) {
          bestv = frac[s];
          best = s;
        }
      }
      if (best < 0) throw std::runtime_error("Unable to complete the landmark quota allocation.");
      ++quota[best];
      rounded[best] = 1;
      ++selected;
    }
  }
  std::vector<int> out;
  out.reserve(static_cast<std::size_t>(target));
  for (int s = 0; s < strata; ++s) {
    if (quota[s] <= 0) continue;
    std::sample(st.rows.begin() + st.offsets[s], st.rows.begin() + st.offsets[s + 1], std::back_inserter(out),
                quota[s], rng);
  }
  if (static_cast<int>(out.size()) != target) {
    throw std::runtime_error("Landmark quota allocation produced the wrong sample size.");
  }
  std::sort(out.begin(), out.end());
  return out;
}

std::vector<int> permutation_head(int rows, uint64_t seed, int needed) {
  std::vector<int> perm(static_cast<std::size_t>(rows));
  std::iota(perm.begin(), perm.end(), 0);
  std::mt19937 g(static_cast<uint32_t>(seed));
  const int steps = std::min(needed, rows - 1);
  for (int r = 0; r < steps; ++r) {
    const int other = r + static_cast<int>(g() % static_cast<uint32_t>(rows - r));
    std::swap(perm[r], perm[other]);
  }
  perm.resize(static_cast<std::size_t>(std::min(needed, rows)));
  return perm;
}

uint64_t kmeans_seed_from_draw(uint64_t draw) { return (draw & 0x7fffffffULL) + 1u; }

std::vector<float> split_uniforms(int k) {
  std::mt19937 g(1234u);
  std::vector<float> u(static_cast<std::size_t>(std::max(k, 1)));
  for (auto& v : u) v = static_cast<float>(g()) / static_cast<float>(std::mt19937::max());
  return u;
}

std::vector<int> make_folds(const std::vector<int>& labels, const std::vector<int>& constrain, int folds,
                            bool stratified, uint64_t seed) {
  if (folds < 2) throw std::invalid_argument("Number of folds must be at least 2.");
  const int n = static_cast<int>(labels.size());
  std::mt19937_64 rng(seed);
  std::vector<int> out(static_cast<std::size_t>(n), 0);
  if (constrain.empty()) {
    if (stratified) {
      std::map<int, std::vector<int>> by_label;
      for (int i = 0; i < n; ++i) by_label[labels[i]].push_back(i);
      std::vector<int> load(static_cast<std::size_t>(folds));
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
      std::vector<int> order(static_cast<std::size_t>(n));
      std::iota(order.begin(), order.end(), 0);
      std::shuffle(order.begin(), order.end(), rng);
      for (std::size_t i = 0; i < order.size(); ++i) out[order[i]] = static_cast<int>(i % static_cast<std::size_t>(folds));
    }
    return out;
  }
  std::map<int, std::vector<int>> members;
  for (int i = 0; i < n; ++i) members[constrain[i]].push_back(i);
  std::vector<int> glabel, gsize;
  for (const auto& kv : members) {
    std::map<int, int> counts;
    for (int idx : kv.second) counts[labels[idx]]++;
    int bl = counts.begin()->first, bc = counts.begin()->second;
    for (const auto& lc : counts) {
      if (lc.second > bc) {
        bl = lc.first;
        bc = lc.second;
      }
    }
    glabel.push_back(bl);
    gsize.push_back(static_cast<int>(kv.second.size()));
  }
  const std::size_t G = glabel.size();
  std::vector<int> gfold(G, 0);
  if (stratified) {
    std::map<int, std::vector<std::size_t>> by_label;
    for (std::size_t g = 0; g < G; ++g) by_label[glabel[g]].push_back(g);
    std::vector<int> load(static_cast<std::size_t>(folds));
    for (auto& kv : by_label) {
      std::shuffle(kv.second.begin(), kv.second.end(), rng);
      std::fill(load.begin(), load.end(), 0);
      for (std::size_t g : kv.second) {
        const int f = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
        gfold[g] = f;
        load[f] += gsize[g];
      }
    }
  } else {
    std::vector<std::size_t> order(G);
    std::iota(order.begin(), order.end(), 0);
    std::shuffle(order.begin(), order.end(), rng);
    for (std::size_t i = 0; i < G; ++i) gfold[order[i]] = static_cast<int>(i % static_cast<std::size_t>(folds));
  }
  std::size_t g = 0;
  for (const auto& kv : members) {
    for (int idx : kv.second) out[idx] = gfold[g];
    ++g;
  }
  return out;
}

RunPlan plan_run(const Strata& strata, int landmarks, int init_k, uint64_t seed, int run) {
  RunPlan p;
  std::mt19937_64 rng(seed + static_cast<uint64_t>(run));
  (void)rng();
  p.landmarks = quota_sample(strata, landmarks, rng);
  const int L = static_cast<int>(p.landmarks.size());
  const int k = std::max(1, std::min(init_k, L));
  p.init_rows = permutation_head(L, kmeans_seed_from_draw(rng()), k);
  p.landmark_hash = fnv_hash(p.landmarks.data(), p.landmarks.size());
  return p;
}

FoldPlan plan_folds(int L, int folds, uint64_t seed, int run) {
  FoldPlan p;
  std::vector<int> order(static_cast<std::size_t>(L));
  std::iota(order.begin(), order.end(), 0);
  std::mt19937_64 frng(seed + static_cast<uint64_t>(run));
  std::shuffle(order.begin(), order.end(), frng);
  p.folds.resize(static_cast<std::size_t>(L));
  std::vector<int> fo(static_cast<std::size_t>(L));
  for (std::size_t i = 0; i < order.size(); ++i) {
    fo[order[i]] = static_cast<int>(i % static_cast<std::size_t>(folds));
    p.folds[order[i]] = static_cast<uint8_t>(fo[order[i]]);
  }
  p.fold_hash = fnv_hash(fo.data(), fo.size());
  return p;
}

uint64_t unordered_bucket_count(std::size_t n) {
  std::unordered_map<int, int> m;
  m.reserve(n);
  return static_cast<uint64_t>(m.bucket_count());
}

uint64_t fnv_hash(const int* v, std::size_t n) {
  uint64_t h = 1469598103934665603ull;
  for (std::size_t i = 0; i < n; ++i) {
    const uint32_t b = static_cast<uint32_t>(v[i]);
    for (int s = 0; s < 32; s += 8) {
      h ^= static_cast<uint8_t>((b >> s) & 0xffu);
      h *= 1099511628211ull;
    }
  }
  return h;
}

}  // namespace kgb
