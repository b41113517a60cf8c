// Per-run landmark planning on the device (plan.cu).
//
// run_kodama_matrix draws, for every run r, from one std::mt19937_64 seeded
// seed + r (kodama_matrix.cpp:2897): one discarded output, the quota sample
// of the landmarks over the shared atlas strata (quota_sample_landmarks,
// kodama_matrix.cpp:856-944), then the seed of the landmark k-means
// (kodama_matrix.cpp:699, 723).  plan_landmarks reproduces those draws and
// their outputs on the device, so the landmark rows never leave HBM.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace kgb {

struct PlanArgs {
  int n = 0;          // rows of the data
  int strata = 0;     // atlas clusters; labels are 1..strata
  int target = 0;     // landmarks per run (<= n)
  int init_k = 0;     // initial k-means centroids per run (1..target)
  int runs = 0;
  int first_run = 1;  // run id of problem 0
  uint64_t seed = 0;
  const int* atlas = nullptr;  // n atlas labels
  // outputs
  int* land = nullptr;         // runs x target, ascending rows
  int* nonland = nullptr;      // runs x (n - target), ascending rows (may be null)
  int* init_rows = nullptr;    // runs x init_k, indices into the run's landmarks
  uint64_t* land_hash = nullptr;  // runs (FNV-1a of the landmark rows, plan_land_hash)
  int* status = nullptr;       // 0 = ok; set non-zero on an invalid atlas or quota
  // scratch (plan_scratch_bytes)
  void* scratch = nullptr;
};

size_t plan_scratch_bytes(int n, int strata, int target, int runs);
// Landmarks and initial centroid rows of every run.
int plan_landmarks(const PlanArgs& a, cudaStream_t st);
// FNV-1a of each run's landmark rows (hash_integer_vector); serial per run, so
// it is queued off the critical path after plan_landmarks.
int plan_land_hash(const PlanArgs& a, cudaStream_t st);

}  // namespace kgb
