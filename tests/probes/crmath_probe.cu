// Test probe: evaluates kgb::cr_exp / kgb::cr_log (kodama_gb300/csrc/crmath.cuh)
// on a host array, for tests/test_gpu_crmath.py.  Test infrastructure only.
#include <cuda_runtime.h>

#include "crmath.cuh"

namespace {
__global__ void probe_kernel(const double* x, int n, int op, double* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = op == 0 ? kgb::cr_exp(x[i]) : op == 1 ? kgb::cr_log(x[i]) : op == 2 ? exp(x[i]) : log(x[i]);
}
}  // namespace

extern "C" int crmath_probe(const double* x, int n, int op, double* out) {
  double *dx = nullptr, *dout = nullptr;
  if (cudaMalloc(&dx, sizeof(double) * n) != cudaSuccess) return 1;
  if (cudaMalloc(&dout, sizeof(double) * n) != cudaSuccess) return 1;
  cudaMemcpy(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice);
  probe_kernel<<<256, 256>>>(dx, n, op, dout);
  cudaMemcpy(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost);
  const int rc = cudaGetLastError() == cudaSuccess ? 0 : 1;
  cudaFree(dx);
  cudaFree(dout);
  return rc;
}
