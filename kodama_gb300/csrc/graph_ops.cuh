// Graph-side kernels (graph_ops.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace kgb {

constexpr int kMaxProjectK = 256;

struct VoteTableArgs {
  int problems, L, n, K, w;
  const int* gidx;        // n x K zero-based, -1 = none
  const float* gdist;     // n x K
  const int* land;        // problems x L global rows, or nullptr = identity (L == n)
  const int* g2l;         // problems x n local index or -1, or nullptr = identity
  const uint8_t* folds;   // problems x L
  uint16_t* nb;           // problems x L x w
  float* sc;              // problems x L x w
  int score_one_minus;    // 0: score -(d*d) (Euclidean), 1: score 1 - d (cosine, inner product)
};

struct ReverseArgs {
  int problems, L, w;
  const uint16_t* nb;     // problems x L x w
  int* rev_off;           // problems x (L+1)
  uint16_t* rev_idx;      // problems x L x w
};

struct ProjectArgs {
  int problems, L, n, K, pk, C0max;
  const int* gidx;        // n x K zero-based
  const int* g2l;         // problems x n
  const uint16_t* clbest; // problems x L codes
  const int* code2label;  // problems x C0max
  int* res;               // problems x n labels
};

struct CodingArgs {
  int problems, n, k, C0max;
  const int* labels;      // problems x n, values 1..k
  uint16_t* codes;        // problems x n
  int* code2label;        // problems x C0max
  int* ncodes;            // problems
};

struct DissimArgs {
  int n, K, runs;
  int in_one_based, out_one_based;
  const int* idx;         // n x K
  const float* dist;      // n x K
  const int* lbs;         // n x runs labels (transposed result matrix)
  int* out_idx;
  float* out_dist;
};

int graph_minmax(const int* idx, size_t total, int* mm, cudaStream_t st);
int normalize_external(const int* in_idx, const float* in_dist, int n, int gk, int K, int base, const int* mm,
                       int* out_idx, float* out_dist, cudaStream_t st);
int normalize_indices(const int* in_idx, const float* in_dist, size_t total, int samples, int base, const int* mm,
                      int* out_idx, float* out_dist, cudaStream_t st);
int build_g2l(const int* land, int problems, int L, int n, int* g2l, cudaStream_t st);
int build_vote_tables(const VoteTableArgs& a, cudaStream_t st);
int build_reverse_tables(const ReverseArgs& a, cudaStream_t st);
int project_labels(const ProjectArgs& a, cudaStream_t st);
int code_labels(const CodingArgs& a, cudaStream_t st);
int fnv_rows(const int* data, int rows, int n, uint64_t* out, cudaStream_t st);
int transpose_runs(const int* res, int runs, int n, int* out, cudaStream_t st);
int dissimilarity(const DissimArgs& a, cudaStream_t st);

}  // namespace kgb
