// kgb_dissimilarity_inplace_device: the co-label proximity of
// kgb_dissimilarity_inplace, computed in place on buffers the caller already
// holds on the device, without allocating device memory.
//
// Who needs this: callers whose device memory is not theirs to allocate from.
// A PyTorch process whose caching allocator has reserved most of the GPU, a
// serving loop that must not call cudaMalloc/cudaFree once it is warm
// (cudaFree waits for the whole device, and a failed cudaMalloc mid-request
// is an outage), or a host whose device memory budget is fixed up front.
// They hand in device pointers and a stream; everything else this call needs
// lives in one statically sized __device__ array that the CUDA module
// carries.
//
// Scratch layout (kScratchBytes = 16 MiB, 256-byte aligned):
//   [0, 256)           header; int at offset 0 = "bad graph index seen" flag,
//                      cleared at the start of every call
//   [256, 16 MiB)      labels transposed to samples x runs (int32), which
//                      bounds samples * runs to kMaxLabelCells.
//
// The scratch is shared by every call on a device.  Two calls that overlap
// in time on one device (two host threads, or work still queued on another
// stream) race on it and give wrong results; callers must serialise them.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "graph_ops.cuh"
#include "../../include/kodama_gb300.h"
#include "launch_count.cuh"

namespace kgb {
void set_last_error(const char* msg);
}  // namespace kgb

namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;
constexpr size_t kHeaderBytes = 256;
constexpr size_t kMaxLabelCells = (kScratchBytes - kHeaderBytes) / sizeof(int);
constexpr int kMaxNeighbors = 2048;  // 8 warps x K x 8 bytes of shared memory <= 128 KB
constexpr unsigned kFullMask = 0xffffffffu;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];


// Flags any stored index outside {negative (missing)} U [1, n].
__global__ void check_one_based_kernel(const int* __restrict__ idx, size_t total, int n, int* bad) {
  for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int v = idx[e];
    if (v >= 0 && (v < 1 || v > n)) atomicExch(bad, 1);
  }
}

// One warp per graph row.  The warp reads its whole row (neighbour id and
// distance) before any lane writes, and no other warp touches that row, so
// the sorted row can be written back over the input.  Nothing is written
// when the check kernel flagged a bad index, so a rejected call leaves the
// graph as it was.  Arithmetic and ordering are those of the out-of-place
// kernel: d' = (1 + d) / agr^2 in double with agr = same / valid over runs
// where both labels are non-zero, +inf when nothing agrees, then a stable
// sort by (d', id).
__global__ void dissimilarity_inplace_kernel(int* __restrict__ idx, float* __restrict__ dist, int n, int K, int runs,
                                             const int* __restrict__ lbs, const int* __restrict__ bad) {
  if (*bad != 0) return;
  extern __shared__ unsigned char dsm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  float* kd = reinterpret_cast<float*>(dsm) + static_cast<size_t>(warp) * K;
  int* ki = reinterpret_cast<int*>(reinterpret_cast<float*>(dsm) + static_cast<size_t>(wpb) * K) +
            static_cast<size_t>(warp) * K;
  const int i = blockIdx.x * wpb + warp;
  if (i >= n) return;
  const int* li = lbs + static_cast<size_t>(i) * runs;
  for (int j = 0; j < K; ++j) {
    const size_t off = static_cast<size_t>(i) * K + j;
    const int stored = idx[off];
    const int nb = stored >= 0 ? stored - 1 : stored;
    float d = dist[off];
    if (nb < 0 || nb >= n || !isfinite(d)) {
      if (lane == 0) {
        kd[j] = INFINITY;
        ki[j] = stored;
      }
      continue;
    }
    const int* lj = lbs + static_cast<size_t>(nb) * runs;
    int same = 0, valid = 0;
    for (int r = lane; r < runs; r += 32) {
      const int x = li[r], y = lj[r];
      const int pv = (x != 0) & (y != 0);
      valid += pv;
      same += pv & (x == y);
    }
    same = __reduce_add_sync(kFullMask, same);
    valid = __reduce_add_sync(kFullMask, valid);
    if (lane == 0) {
      if (same == 0 || valid == 0) {
        d = INFINITY;
      } else {
        const double agr = __ddiv_rn(static_cast<double>(same), static_cast<double>(valid));
        d = static_cast<float>(__ddiv_rn(__dadd_rn(1.0, static_cast<double>(d)), __dmul_rn(agr, agr)));
      }
      kd[j] = d;
      ki[j] = nb + 1;
    }
  }
  __syncwarp();
  for (int j = lane; j < K; j += 32) {
    const float dj = kd[j];
    const int ij = ki[j];
    int rank = 0;
    for (int q = 0; q < K; ++q) {
      const float dq = kd[q];
      const int iq = ki[q];
      const bool less = dq < dj || (!(dj < dq) && iq < ij);
      const bool equal_before = !(dq < dj) && !(dj < dq) && iq == ij && q < j;
      rank += less || equal_before;
    }
    idx[static_cast<size_t>(i) * K + rank] = ij;
    dist[static_cast<size_t>(i) * K + rank] = dj;
  }
}

struct Fail {
  int code;
  std::string msg;
};

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Fail{KGB_ECUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}

// Device address of g_scratch on the current device.  It is looked up on
// every call (cheap once the module is loaded), so a call after a
// cudaDeviceReset, which reloads the module and may move the array, uses
// the array's new address.  The first lookup on a device may load the
// module onto it, which is why the first call per device must not happen
// while a stream is being captured.
unsigned char* scratch_here() {
  void* p = nullptr;
  ck(cudaGetSymbolAddress(&p, g_scratch), "cudaGetSymbolAddress(scratch)");
  return static_cast<unsigned char*>(p);
}

// Restores the caller's current device when the call ends.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int device) {
    ck(cudaGetDevice(&prev), "cudaGetDevice");
    ck(cudaSetDevice(device), "cudaSetDevice");
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

void run(int32_t* gidx, float* gdist, int32_t samples, int32_t gk, const int32_t* res, int32_t runs,
         int32_t device, void* stream) {
  if (gidx == nullptr || gdist == nullptr || res == nullptr) throw Fail{KGB_EINVAL, "null pointer"};
  if (runs <= 0 || samples <= 0 || gk <= 0) {
    throw Fail{KGB_EINVAL, "KODAMADissimilarityInPlace requires a non-empty graph and label matrix."};
  }
  if (static_cast<size_t>(samples) * static_cast<size_t>(runs) > kMaxLabelCells) {
    throw Fail{KGB_EINVAL, "kgb_dissimilarity_inplace_device: samples * runs = " +
                               std::to_string(static_cast<long long>(samples) * runs) + " exceeds the static scratch (" +
                               std::to_string(kMaxLabelCells) + " labels, 16 MiB); use kgb_dissimilarity_inplace"};
  }
  if (gk > kMaxNeighbors) {
    throw Fail{KGB_EINVAL, "kgb_dissimilarity_inplace_device: neighbors = " + std::to_string(gk) +
                               " exceeds the supported maximum of " + std::to_string(kMaxNeighbors)};
  }
  int ndev = 0;
  ck(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
  if (device < 0 || device >= ndev) {
    throw Fail{KGB_EINVAL, "kgb_dissimilarity_inplace_device: no CUDA device " + std::to_string(device)};
  }
  DeviceGuard guard(device);
  unsigned char* scratch = scratch_here();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int* bad = reinterpret_cast<int*>(scratch);
  int* lbs = reinterpret_cast<int*>(scratch + kHeaderBytes);
  const size_t total = static_cast<size_t>(samples) * gk;

  ck(cudaMemsetAsync(scratch, 0, kHeaderBytes, st), "clear scratch header");
  const size_t want = (total + 255) / 256;
  // each launch through cudaLaunchKernelEx, so its own status is checked and
  // an error left on the thread by earlier, unrelated work is left alone
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(want < 1024 ? want : 1024));
  cfg.blockDim = dim3(256);
  cfg.stream = st;
  ck(cudaLaunchKernelEx(&cfg, check_one_based_kernel, static_cast<const int*>(gidx), total, static_cast<int>(samples),
                        bad),
     "check indices");
  kgb::count_launch();
  ck(static_cast<cudaError_t>(kgb::transpose_runs(res, runs, samples, lbs, st)), "transpose");
  const int wpb = 8;
  const size_t smem = static_cast<size_t>(wpb) * gk * (sizeof(float) + sizeof(int));
  if (smem > 48 * 1024) {
    ck(cudaFuncSetAttribute(dissimilarity_inplace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            static_cast<int>(smem)),
       "shared memory size");
  }
  cfg.gridDim = dim3(static_cast<unsigned>((samples + wpb - 1) / wpb));
  cfg.blockDim = dim3(wpb * 32);
  cfg.dynamicSmemBytes = smem;
  ck(cudaLaunchKernelEx(&cfg, dissimilarity_inplace_kernel, static_cast<int*>(gidx), static_cast<float*>(gdist),
                        static_cast<int>(samples), static_cast<int>(gk), static_cast<int>(runs),
                        static_cast<const int*>(lbs), static_cast<const int*>(bad)),
     "dissimilarity");
  kgb::count_launch();
  int h_bad = 0;
  ck(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st), "read index check");
  ck(cudaStreamSynchronize(st), "synchronize");
  if (h_bad != 0) throw Fail{KGB_EINVAL, "KODAMADissimilarityInPlace expects public one-based graph indices."};
}

}  // namespace

extern "C" int kgb_dissimilarity_inplace_device(int32_t* gidx, float* gdist, int32_t samples, int32_t gk,
                                                const int32_t* res, int32_t runs, int32_t device, void* stream) {
  try {
    run(gidx, gdist, samples, gk, res, runs, device, stream);
    return KGB_OK;
  } catch (const Fail& f) {
    kgb::set_last_error(f.msg.c_str());
    return f.code;
  } catch (const std::exception& e) {
    kgb::set_last_error(e.what());
    return KGB_EINTERNAL;
  }
}
