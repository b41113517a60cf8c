// Exact kNN graph kernels (knn.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace kgb {

constexpr int kMaxSegments = 16;

size_t knn_bruteforce_scratch(int n, int K, int segments);
int knn_bruteforce(const float* x, int n, int d, int K, int segments, void* scratch, int* idx, float* dist,
                   cudaStream_t st);

}  // namespace kgb
