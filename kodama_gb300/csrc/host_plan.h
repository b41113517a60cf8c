// Host-side planning of the data-independent random choices that precede the
// device work: fold assignment and the atlas k-means seeding.  These are
// serial draws from the reference's std::mt19937_64 streams and are made here
// with the same libstdc++ engines and algorithms the reference uses.  The
// per-run landmark quota sample depends on the atlas and is drawn on the
// device (plan.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <random>
#include <vector>

namespace kgb {

// Folds of one run over L landmarks with the identity constraint, not
// stratified (make_folds, common.cpp:180-189): independent of the data, so
// they can be planned while the device builds the graph and the atlas.
struct FoldPlan {
  std::vector<uint8_t> folds;
  uint64_t fold_hash = 0;
};
FoldPlan plan_folds(int L, int folds, uint64_t seed, int run);

// First `needed` entries of the FAISS-compatible permutation
// (kodama_matrix.cpp:535-564) seeded with `seed`.
std::vector<int> permutation_head(int rows, uint64_t seed, int needed);

// The initial centroid rows of kmeans_labels for an engine state: consumes one
// draw, kseed = draw & 0x7fffffff, permutation seeded kseed + 1.
uint64_t kmeans_seed_from_draw(uint64_t draw);

// First k uniforms of mt19937(1234) as split_empty_kmeans_clusters draws them.
std::vector<float> split_uniforms(int k);

// make_folds (common.cpp:108-214).
std::vector<int> make_folds(const std::vector<int>& labels, const std::vector<int>& constrain, int folds,
                            bool stratified, uint64_t seed);

// Bucket count of std::unordered_map<int,int> after reserve(n) on this host's
// standard library (fixes the iteration order of core_objective_score).
uint64_t unordered_bucket_count(std::size_t n);

// FNV-1a over the little-endian bytes of each int (hash_integer_vector,
// kodama_matrix.cpp:1689-1699).
uint64_t fnv_hash(const int* v, std::size_t n);

}  // namespace kgb
