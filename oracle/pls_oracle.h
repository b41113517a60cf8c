// PLS-LDA restatement shared by the oracle translation units.
//
// TEST INFRASTRUCTURE ONLY (see kodama_oracle.cpp).
#pragma once

#include <cstdint>
#include <vector>

namespace orc {

std::vector<int> make_folds(const std::vector<int>& labels, const std::vector<int>& constrain,
                            int folds, bool stratified, uint64_t seed);

struct PLSOpts {
  int folds = 10;
  bool stratified = true;
  uint64_t cv_seed = 1;
  int max_components = 10;
  int fixed_components = 0;
  bool center = true;
  bool scale = true;
  bool da = false;  // PLSDACV (PLSMode::PLS_DA): one-hot regression on the scores instead of LDA
};

struct PLSCVOut {
  std::vector<int> predicted;
  std::vector<int> folds;
  int selected_components = 1;
  std::vector<double> accuracy_by_components;
};

// Per-fold standardised data of one matrix, the reference's fold cache
// (plscv.cpp:530-667); label independent for non-stratified folds.
struct PLSFoldData {
  std::vector<int> train, validation;
  std::vector<float> mean, scale;
  std::vector<float> x_train, x_val;  // row-major standardised rows
  std::vector<float> gram;            // p x p, empty until built
};

struct PLSFoldCache {
  std::vector<int> folds;
  std::vector<int> fold_ids;
  std::vector<PLSFoldData> data;
  bool gram_built = false;
};

PLSFoldCache pls_fold_cache(const float* x, int n, int p, const std::vector<int>& folds, const PLSOpts& o);
void pls_build_grams(PLSFoldCache& cache, int p);

// One PLSLDACV evaluation over a prepared fold cache.  use_gram selects the
// loading computation through the cached fold Gram (plscv.cpp:901-907).
PLSCVOut plsldacv_on_cache(const PLSFoldCache& cache, int n, int p, const std::vector<int>& labels,
                           const PLSOpts& o, bool use_gram);

// PLSLDACV_CPU (plscv.cpp:2930, run_plscv_host :2293-2507) without a fold cache.
PLSCVOut plsldacv(const float* x, int n, int p, const std::vector<int>& labels,
                  const std::vector<int>& constrain, const PLSOpts& o);

// PLSLDAPredict_CPU (plscv.cpp:2976-3005).
std::vector<int> plslda_predict(const float* train, int n, int p, const std::vector<int>& labels,
                                const float* test, int nt, const PLSOpts& o);

}  // namespace orc
