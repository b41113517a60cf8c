// Host-side planning of per-run random choices (see host_plan.h).
#include "host_plan.h"


#include <algorithm>
#include <map>
#include <numeric>
#include <stdexcept>
#include <unordered_map>

namespace kgb {

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
