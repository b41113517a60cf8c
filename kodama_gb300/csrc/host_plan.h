// Host-side planning of the per-run random choices that precede the device
// work: landmark atlas strata, landmark quota sampling, fold assignment and
// k-means seeding.  These are serial draws from the reference's per-run
// std::mt19937_64 streams and are made here with the same libstdc++ engines
// and algorithms the reference uses, so each run sees the reference's exact
// landmark rows, folds and initial centroids.
#pragma once

#include <cstddef>
#include <cstdint>
#include <random>
#include <vector>

namespace kgb {

struct Strata {
  std::vector<int> offsets, rows;
};

// index_strata (kodama_matrix.cpp:806-828); labels are 1..strata.
Strata index_strata(const std::vector<int>& labels, int strata);

// One KODAMA.matrix run's plan (run_iteration, kodama_matrix.cpp:2897-2939 and
// :3091-3103): rng(seed+run); discard one draw; quota-sample landmarks; then
// the init k-means seed.
struct RunPlan {
  std::vector<int> landmarks;       // sorted global rows, size L
  std::vector<int> init_rows;       // init_k initial centroid rows (indices into landmarks)
  uint64_t landmark_hash = 0;
};

// Landmarks and initial centroid rows of one run (needs the atlas strata).
RunPlan plan_run(const Strata& strata, int landmarks, int init_k, uint64_t seed, int run);

// Folds of one run over L landmarks with the identity constraint, not
// stratified (make_folds, common.cpp:180-189): independent of the data, so
// they can be planned while the device builds the graph and the atlas.
struct FoldPlan {
  std::vector<uint8_t> folds;
  uint64_t fold_hash = 0;
};
FoldPlan plan_folds(int L, int folds, uint64_t seed, int run);

// quota_sample_landmarks (kodama_matrix.cpp:856-944, preserve_strata_order=false).
std::vector<int> quota_sample(const Strata& st, int target, std::mt19937_64& rng);

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
