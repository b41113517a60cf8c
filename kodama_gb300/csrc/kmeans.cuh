// Batched bit-exact k-means (kmeans.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace kgb {

struct KMeansBatch {
  int problems;
  int n;                    // rows per problem
  int d;
  int k;
  int max_iter;
  const float* x;           // device matrix (rows x d)
  const int* rows;          // problems x n row ids into x, or nullptr = identity (problems == 1)
  const float* pnorm;       // per row of x: dot(x_r, x_r)
  const int* init_rows;     // problems x k: initial centroid rows (indices into the problem's rows)
  const float* split_uniform; // mt19937(1234) uniforms for empty-cluster splitting (k entries)
  float* cent;              // problems x k x d
  float* cnorm;             // problems x k
  int* assign;              // problems x n (must start at -1)
  int* active;              // problems
  int* changed;             // problems
  int* labels;              // problems x n output, 1-based
  int* members;             // problems x n scratch: rows grouped by cluster
  int* offsets;             // problems x (k+1) scratch: cluster offsets in members
  float* fscratch;          // problems x (3k+1) scratch for empty-cluster splitting
  // tensor-core assignment (kmeans_tc_supported): x split into bf16 hi / lo
  // (bf16_split_rows, dp columns), scratch for the centroids' split; xh null =
  // every distance computed exactly
  const uint16_t* xh;
  const uint16_t* xl;
  int dp;
  uint16_t* ch;             // problems x k x dp
  uint16_t* cl;
  int tc_blocks;            // set by kmeans_run: 64-row blocks per CTA
  float tc_crel;            // set by kmeans_run: the error bound's factor
  int tc_cent_smem;         // set by kmeans_run: fp32 centroids staged in shared memory (else read from L2)
};

// The tensor-core assignment applies (d <= 64, k <= 128).
bool kmeans_tc_supported(int d, int k);

size_t kmeans_sort_smem(int k);
int kmeans_row_norms(const float* x, int n, int d, float* out, cudaStream_t st);
int kmeans_run(const KMeansBatch& b, cudaStream_t st);

}  // namespace kgb
