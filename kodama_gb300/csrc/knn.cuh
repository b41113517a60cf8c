// Exact kNN graph kernels (knn.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace kgb {

constexpr int kMaxSegments = 16;

size_t knn_bruteforce_scratch(int n, int K, int segments);
int knn_bruteforce(const float* x, int n, int d, int K, int segments, void* scratch, int* idx, float* dist,
                   cudaStream_t st);

// knn_bruteforce restricted to the *nrows rows listed in rows (read on the
// device): their results are written, the other rows' left untouched.
int knn_bruteforce_rows(const float* x, int n, int d, int K, int segments, const int* rows, const int* nrows,
                        void* scratch, int* idx, float* dist, cudaStream_t st);

// The same exact graph as knn_bruteforce through a tensor-core candidate
// search with an exact re-rank and a per-row certificate (knn_tc.cu); rows
// whose certificate fails are recomputed by knn_bruteforce_rows.
bool knn_tc_supported(int n, int d, int K);
size_t knn_tc_scratch(int n, int d, int K, int segments);
int knn_tc_graph(const float* x, int n, int d, int K, int segments, void* scratch, int* idx, float* dist,
                 cudaStream_t st);
// Rows of the last knn_tc_graph on this scratch that went to the fallback
// (asynchronous copy into host memory).
int knn_tc_fallback_count(const void* scratch, int n, int d, int K, int segments, int* out, cudaStream_t st);

// Rows of x (n x d) split into bfloat16 hi + lo parts (x = hi + lo + r,
// |r| <= 2^-16 |x|), dp = d rounded up to 16, coordinates permuted inside
// each 16-block so one lane's m16n8k16 fragment values are contiguous.
int bf16_split_rows(const float* x, int n, int d, int dp, uint16_t* xh, uint16_t* xl, cudaStream_t st);

// Fold-wise search: for each row the K nearest rows of other folds (folds[n]),
// ranked by (internal distance, row); inner = minus the inner product instead
// of the squared L2 distance.  idx -1 / dist +inf where fewer rows qualify;
// dist is the internal distance.  Scratch as knn_bruteforce_scratch.
int knn_fold_search(const float* x, int n, int d, int K, bool inner, const int* folds, int segments, void* scratch,
                    int* idx, float* dist, cudaStream_t st);

// Global exact graph under the inner product (metric 1) or cosine (metric 0,
// on rows already scaled by normalize_rows mode 2): for each row the K other
// rows of smallest internal distance, minus the inner product (float chain in
// coordinate order), ties to the smaller row; reported distance 1 + v
// (inner product) or max(0, 1 + v) (cosine).  Scratch as knn_bruteforce.
int knn_bruteforce_inner(const float* x, int n, int d, int K, int metric, int segments, void* scratch, int* idx,
                         float* dist, cudaStream_t st);

// Cosine search matrix: mode 0 = knncv.cpp:85-108, mode 1 = core.cpp:166-195,
// mode 2 = kodama_matrix.cpp:155-167.
int normalize_rows(const float* x, int n, int d, int mode, float* out, cudaStream_t st);

// Majority vote of every row over its K fold-wise neighbours (knncv.cpp:111-131).
int knn_vote(const int* idx, const float* dist, int n, int K, const int* labels, int* pred, cudaStream_t st);

// Evolution vote tables (n x w, 16-bit ids, score = -distance) from the
// fold-wise neighbours (n x K, w <= K).
int knn_fold_tables(const int* idx, const float* dist, int n, int K, int w, uint16_t* nb, float* sc,
                    cudaStream_t st);

}  // namespace kgb
