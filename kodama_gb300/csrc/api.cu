// C ABI of the GB300 label-evolution engine (include/kodama_gb300.h).
//
// Host orchestration in C++; every per-row / per-cycle computation runs in the
// CUDA kernels of evolve.cu, kmeans.cu, graph_ops.cu and knn.cu.  There is no
// CPU fallback: without a device every compute entry point fails with
// KGB_ECUDA.
#include "../../include/kodama_gb300.h"
#include "evolve.cuh"
#include "graph_ops.cuh"
#include "host_plan.h"
#include "kmeans.cuh"
#include "knn.cuh"
#include "launch_count.cuh"
#include "pls.cuh"
#include "mlp.cuh"
#include "plan.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <memory>
#include <mutex>
#include <exception>
#include <functional>
#include <future>
#include <limits>
#include <map>
#include <numeric>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace kgb {
namespace {
std::atomic<long long> g_launches{0};
}
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long g_launches_value() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace kgb

namespace {

thread_local std::string g_error;

struct KgbError : std::runtime_error {
  int code;
  KgbError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const std::string& msg) { throw KgbError(code, msg); }

void ck(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation) fail(KGB_ENOMEM, std::string(what) + ": " + cudaGetErrorString(e));
  fail(KGB_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void ck_launch(int e, const char* what) { ck(static_cast<cudaError_t>(e), what); }

template <class F>
int guarded(F&& f) {
  try {
    f();
    return KGB_OK;
  } catch (const KgbError& e) {
    g_error = e.what();
    return e.code;
  } catch (const std::invalid_argument& e) {
    g_error = e.what();
    return KGB_EINVAL;
  } catch (const std::bad_alloc& e) {
    g_error = "host allocation failed";
    return KGB_ENOMEM;
  } catch (const std::exception& e) {
    g_error = e.what();
    return KGB_EINTERNAL;
  }
}

// Pinned host memory of a captured batch.  A CUDA graph replays its copies at
// every launch, so the host side of each copy must outlive the capture: the
// sources of host-to-device copies are kept here, and device-to-host copies
// land here and are delivered to their host destinations after each launch.
class CaptureArena {
 public:
  CaptureArena() = default;
  CaptureArena(const CaptureArena&) = delete;
  CaptureArena& operator=(const CaptureArena&) = delete;
  ~CaptureArena() {
    for (void* p : blocks_) cudaFreeHost(p);
  }
  void* keep(const void* src, size_t bytes) {
    void* p = get(bytes);
    if (bytes) std::memcpy(p, src, bytes);
    return p;
  }
  void* slot(void* dst, size_t bytes) {
    void* p = get(bytes);
    posts_.push_back(Post{dst, p, bytes});
    return p;
  }
  void deliver() const {
    for (const Post& q : posts_) std::memcpy(q.dst, q.src, q.bytes);
  }

 private:
  void* get(size_t bytes) {
    bytes = (std::max<size_t>(bytes, 1) + 63) / 64 * 64;
    if (bytes > left_) {
      const size_t cap = std::max<size_t>(bytes, size_t(8) << 20);
      void* p = nullptr;
      ck(cudaMallocHost(&p, cap), "cudaMallocHost");
      blocks_.push_back(p);
      cur_ = static_cast<char*>(p);
      left_ = cap;
    }
    void* p = cur_;
    cur_ += bytes;
    left_ -= bytes;
    return p;
  }
  struct Post {
    void* dst;
    const void* src;
    size_t bytes;
  };
  std::vector<void*> blocks_;
  std::vector<Post> posts_;
  char* cur_ = nullptr;
  size_t left_ = 0;
};

// Per-call device context: device selection, one stream, stream-ordered
// allocations released when the call ends.  In capture mode the context
// enqueues into two streams of a batch being captured into a CUDA graph: no
// host synchronisation, host copies through the batch's pinned arena, and the
// allocations freed inside the graph (release()).
class Ctx {
 public:
  Ctx(int device, cudaStream_t main, cudaStream_t side, CaptureArena* arena)
      : stream_(main), side_(side), arena_(arena), owns_streams_(false) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    ck(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device), "device attribute");
  }
  explicit Ctx(int device) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) fail(KGB_ECUDA, "no CUDA device is available");
    if (device < 0 || device >= count) fail(KGB_EINVAL, "CUDA device ordinal out of range");
    ck(cudaSetDevice(device), "cudaSetDevice");
    // the call's chain of dependent stages runs at the highest priority; bulk
    // work that overlaps it (the exact graph) at the lowest, so the block
    // scheduler hands free SMs to the chain first
    int least = 0, greatest = 0;
    ck(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
    ck(cudaStreamCreateWithPriority(&stream_, cudaStreamNonBlocking, greatest), "cudaStreamCreate");
    ck(cudaStreamCreateWithPriority(&side_, cudaStreamNonBlocking, greatest), "cudaStreamCreate");
    ck(cudaStreamCreateWithPriority(&bg_, cudaStreamNonBlocking, least), "cudaStreamCreate");
    ck(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device), "device attribute");
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  ~Ctx() {
    if (owns_streams_) {
      cudaStreamSynchronize(side_);  // side-stream work reads buffers freed below
      cudaStreamSynchronize(bg_);
      for (void* p : bufs_) cudaFreeAsync(p, stream_);
      cudaStreamSynchronize(stream_);
    }
    for (int i = 0; i < nev_; ++i) cudaEventDestroy(ev_[i]);
    for (int i = 0; i < njoin_; ++i) cudaEventDestroy(join_[i]);
    if (owns_streams_) {
      cudaStreamDestroy(bg_);
      cudaStreamDestroy(side_);
      cudaStreamDestroy(stream_);
    }
  }
  // Queues f's work on the low-priority background stream, after everything
  // queued on the main stream so far (or after the main-stream mark `after`):
  // while f runs, stream() is that stream (launches and allocations of f go
  // there).  Returns false, running nothing, in capture mode, where there is
  // no background stream.  Timing events a and b (marks on the background
  // stream) bracket f's work.
  template <class F>
  bool on_background(F&& f, int* a, int* b, int after = -1) {
    if (bg_ == nullptr) return false;
    const int e = after >= 0 ? after : mark();
    ck(cudaStreamWaitEvent(bg_, ev_[e], 0), "cudaStreamWaitEvent");
    std::swap(stream_, bg_);
    *a = mark();
    f();
    *b = mark();
    std::swap(stream_, bg_);
    return true;
  }
  // The main stream waits for everything queued on the background stream.
  void join_background() {
    if (bg_ == nullptr) return;
    if (njoin_ >= kMaxEvents) fail(KGB_EINTERNAL, "too many stream joins");
    ck(cudaEventCreateWithFlags(&join_[njoin_], cudaEventDisableTiming), "cudaEventCreate");
    ck(cudaEventRecord(join_[njoin_], bg_), "cudaEventRecord");
    ck(cudaStreamWaitEvent(stream_, join_[njoin_], 0), "cudaStreamWaitEvent");
    ++njoin_;
  }
  bool capturing() const { return arena_ != nullptr; }
  // Capture mode: joins the side stream and frees every allocation inside the
  // graph, after all the work queued so far.
  void release() {
    join();
    for (void* p : bufs_) ck(cudaFreeAsync(p, stream_), "cudaFreeAsync");
    bufs_.clear();
  }
  // A host wait for timing or for host-side steps; skipped inside a capture.
  void checkpoint() {
    if (!capturing()) sync();
  }
  // side stream for work that overlaps the main stream: fork() makes it wait
  // for everything queued on the main stream so far.
  cudaStream_t side() const { return side_; }
  bool has_background() const { return bg_ != nullptr; }
  void fork() {
    const int e = mark();
    ck(cudaStreamWaitEvent(side_, ev_[e], 0), "cudaStreamWaitEvent");
  }
  // side stream waits for event e only; join() makes the main stream wait for
  // everything queued on the side stream so far.
  void fork_after(int e) { ck(cudaStreamWaitEvent(side_, ev_[e], 0), "cudaStreamWaitEvent"); }
  void join() {
    if (njoin_ >= kMaxEvents) fail(KGB_EINTERNAL, "too many stream joins");
    ck(cudaEventCreateWithFlags(&join_[njoin_], cudaEventDisableTiming), "cudaEventCreate");
    ck(cudaEventRecord(join_[njoin_], side_), "cudaEventRecord");
    ck(cudaStreamWaitEvent(stream_, join_[njoin_], 0), "cudaStreamWaitEvent");
    ++njoin_;
  }
  // Copies device memory to the host as soon as event e has completed, on the
  // side stream, and waits for that copy only (the main stream runs on).
  template <class T>
  void download_after(T* host, const T* dev, size_t count, int e) {
    ck(cudaStreamWaitEvent(side_, ev_[e], 0), "cudaStreamWaitEvent");
    if (count) ck(cudaMemcpyAsync(host, dev, count * sizeof(T), cudaMemcpyDeviceToHost, side_), "D2H");
    ck(cudaStreamSynchronize(side_), "stream synchronize");
  }
  // CUDA events on the call's stream, for per-stage device timings.
  int mark() {
    if (nev_ >= kMaxEvents) return nev_ - 1;
    ck(cudaEventCreate(&ev_[nev_]), "cudaEventCreate");
    ck(cudaEventRecord(ev_[nev_], stream_), "cudaEventRecord");
    return nev_++;
  }
  double ms(int a, int b) {
    float v = 0.0f;
    if (capturing() || a < 0 || b < 0 || cudaEventElapsedTime(&v, ev_[a], ev_[b]) != cudaSuccess) return 0.0;
    return static_cast<double>(v);
  }
  Ctx(const Ctx&) = delete;
  Ctx& operator=(const Ctx&) = delete;

  template <class T>
  T* alloc(size_t count) {
    void* p = nullptr;
    const size_t bytes = std::max<size_t>(1, count * sizeof(T));
    ck(cudaMallocAsync(&p, bytes, stream_), "cudaMallocAsync");
    bufs_.push_back(p);
    return static_cast<T*>(p);
  }
  template <class T>
  T* upload(const T* host, size_t count) {
    T* d = alloc<T>(count);
    h2d(d, host, count);
    return d;
  }
  // host -> existing device buffer, on the main stream
  template <class T>
  void h2d(T* dev, const T* host, size_t count) {
    if (!count) return;
    const void* src = capturing() ? arena_->keep(host, count * sizeof(T)) : static_cast<const void*>(host);
    ck(cudaMemcpyAsync(dev, src, count * sizeof(T), cudaMemcpyHostToDevice, stream_), "H2D");
  }
  template <class T>
  void download(T* host, const T* dev, size_t count) {
    download_on(stream_, host, dev, count);
  }
  template <class T>
  void download_side(T* host, const T* dev, size_t count) {
    download_on(side_, host, dev, count);
  }
  void sync() {
    if (capturing()) fail(KGB_EINTERNAL, "host synchronisation inside a captured batch");
    ck(cudaStreamSynchronize(stream_), "stream synchronize");
    ck(cudaStreamSynchronize(side_), "stream synchronize");
    if (bg_ != nullptr) ck(cudaStreamSynchronize(bg_), "stream synchronize");
  }
  cudaStream_t stream() const { return stream_; }
  int sms() const { return sms_; }

 private:
  template <class T>
  void download_on(cudaStream_t s, T* host, const T* dev, size_t count) {
    if (!count) return;
    void* dst = capturing() ? arena_->slot(host, count * sizeof(T)) : static_cast<void*>(host);
    ck(cudaMemcpyAsync(dst, dev, count * sizeof(T), cudaMemcpyDeviceToHost, s), "D2H");
  }
  static constexpr int kMaxEvents = 32;
  cudaStream_t stream_ = nullptr;
  cudaStream_t side_ = nullptr;
  cudaStream_t bg_ = nullptr;  // low-priority background stream (not in capture mode)
  CaptureArena* arena_ = nullptr;
  bool owns_streams_ = true;
  int sms_ = 1;
  std::vector<void*> bufs_;
  cudaEvent_t ev_[kMaxEvents];
  int nev_ = 0;
  cudaEvent_t join_[kMaxEvents];
  int njoin_ = 0;
};

// Pinned host staging for large device-to-host results (one buffer per host
// thread, grown on demand and kept): copying into pageable user memory
// directly is several times slower than a pinned copy plus a host memcpy.
class PinnedStage {
 public:
  ~PinnedStage() {
    if (p_) cudaFreeHost(p_);
  }
  void* get(size_t bytes) {
    if (bytes > cap_) {
      if (p_) cudaFreeHost(p_);
      p_ = nullptr;
      cap_ = 0;
      ck(cudaMallocHost(&p_, bytes), "cudaMallocHost");
      cap_ = bytes;
    }
    return p_;
  }

 private:
  void* p_ = nullptr;
  size_t cap_ = 0;
};

thread_local PinnedStage g_stage;

struct Clock {
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  double lap() {
    const auto now = std::chrono::steady_clock::now();
    const double s = std::chrono::duration<double>(now - t).count();
    t = now;
    return s;
  }
};

kgb_policy default_policy() {
  kgb_policy p;
  p.prediction_guidance = 1;
  p.adaptive_proposal_size = 1;
  p.transition_proposal = 1;
  p.stochastic_acceptance = 1;
  p.diversity_multiplier = 1;
  p.pls_transition_coarsening = 1;
  p.pls_fragmentation_penalty = 1;
  p.reject_single_class = 1;
  return p;
}

bool policy_is_zero(const kgb_policy& p) {
  return !p.prediction_guidance && !p.adaptive_proposal_size && !p.transition_proposal &&
         !p.stochastic_acceptance && !p.diversity_multiplier && !p.pls_transition_coarsening &&
         !p.pls_fragmentation_penalty && !p.reject_single_class;
}

// Label coding of one problem: codes = ranks among the sorted distinct labels.
struct Coding {
  std::vector<int> code2label;
  std::vector<uint16_t> codes;
  bool nocollide = true;
};

Coding code_labels(const int* labels, int n, uint64_t bucket_count) {
  Coding c;
  c.code2label.assign(labels, labels + n);
  std::sort(c.code2label.begin(), c.code2label.end());
  c.code2label.erase(std::unique(c.code2label.begin(), c.code2label.end()), c.code2label.end());
  if (c.code2label.size() > 65535) fail(KGB_EINVAL, "more than 65535 distinct labels");
  c.codes.resize(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) {
    c.codes[i] = static_cast<uint16_t>(std::lower_bound(c.code2label.begin(), c.code2label.end(), labels[i]) -
                                       c.code2label.begin());
  }
  for (int l : c.code2label) {
    if (l < 0 || static_cast<uint64_t>(l) >= bucket_count) c.nocollide = false;
  }
  return c;
}

// normalize_constrain / factor_subset (kodama_matrix.cpp:183-201, 988-1001):
// group ids 1.. by first appearance of values[rows[i]].
std::vector<int> first_appearance_ids(const int* values, const std::vector<int>& rows) {
  std::map<int, int> ids;
  std::vector<int> out(rows.size(), 0);
  for (size_t i = 0; i < rows.size(); ++i) {
    auto it = ids.find(values[rows[i]]);
    if (it == ids.end()) it = ids.emplace(values[rows[i]], static_cast<int>(ids.size()) + 1).first;
    out[i] = it->second;
  }
  return out;
}

// majority_label (kodama_matrix.cpp:169-181): the most frequent value, ties to
// the smaller value.
int majority_value(const std::vector<int>& values) {
  std::map<int, int> counts;
  for (int v : values) counts[v] += 1;
  int bl = counts.begin()->first, bc = counts.begin()->second;
  for (const auto& kv : counts)
    if (kv.second > bc || (kv.second == bc && kv.first < bl)) {
      bl = kv.first;
      bc = kv.second;
    }
  return bl;
}

// constrained_majority (kodama_matrix.cpp:1003-1011), in place on n labels.
void constrained_majority(int* labels, const int* groups, size_t n) {
  std::map<int, std::vector<int>> by;
  for (size_t i = 0; i < n; ++i) by[groups[i]].push_back(labels[i]);
  std::map<int, int> lab;
  for (const auto& kv : by) lab[kv.first] = majority_value(kv.second);
  for (size_t i = 0; i < n; ++i) labels[i] = lab[groups[i]];
}

// Status word of the device landmark planning (plan.cu): non-zero when the
// atlas labels or the quota allocation were inconsistent.
void check_plan_status(const int* d_status) {
  int v = 0;
  ck(cudaMemcpy(&v, d_status, sizeof(int), cudaMemcpyDeviceToHost), "D2H");
  if (v != 0) fail(KGB_EINTERNAL, "Landmark quota allocation produced the wrong sample size.");
}

int host_threads(int requested) {
  if (requested > 0) return requested;
  const unsigned hc = std::thread::hardware_concurrency();
  return hc ? static_cast<int>(std::min(hc, 32u)) : 4;
}

template <class F>
void parallel_for(int n, int threads, F&& f) {
  threads = std::max(1, std::min(threads, n));
  if (threads == 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> pool;
  std::vector<std::exception_ptr> errs(static_cast<size_t>(threads));
  for (int t = 0; t < threads; ++t) {
    pool.emplace_back([&, t]() {
      try {
        for (int i = t; i < n; i += threads) f(i);
      } catch (...) {
        errs[t] = std::current_exception();
      }
    });
  }
  for (auto& th : pool) th.join();
  for (auto& e : errs) if (e) std::rethrow_exception(e);
}

struct EvolveBuffers {
  uint16_t* clbest;
  uint16_t* cvpredbest;
  double* vect_acc;
  double* vect_score;
  int* psize;
  int* active;
  uint8_t* flags;
  int* counters;
  double* best;
  int* status;
};

// Common launcher of the persistent kernel for `problems` problems of L rows.
EvolveBuffers run_evolution(Ctx& ctx, kgb::EvolveParams P, int C0max) {
  const int problems = P.problems, L = P.L, T = P.T;
  EvolveBuffers b;
  b.clbest = ctx.alloc<uint16_t>(static_cast<size_t>(problems) * L);
  b.cvpredbest = ctx.alloc<uint16_t>(static_cast<size_t>(problems) * L);
  b.vect_acc = ctx.alloc<double>(static_cast<size_t>(problems) * std::max(T, 1));
  b.vect_score = ctx.alloc<double>(static_cast<size_t>(problems) * std::max(T, 1));
  b.psize = ctx.alloc<int>(static_cast<size_t>(problems) * std::max(T, 1));
  b.active = ctx.alloc<int>(static_cast<size_t>(problems) * std::max(T, 1));
  b.flags = ctx.alloc<uint8_t>(static_cast<size_t>(problems) * std::max(T, 1) * 3);
  b.counters = ctx.alloc<int>(static_cast<size_t>(problems) * 16);
  b.best = ctx.alloc<double>(static_cast<size_t>(problems) * 2);
  b.status = ctx.alloc<int>(static_cast<size_t>(problems));
  P.clbest = b.clbest;
  P.cvpredbest = b.cvpredbest;
  P.vect_acc = b.vect_acc;
  P.vect_score = b.vect_score;
  P.proposal_size = b.psize;
  P.active = b.active;
  P.flags = b.flags;
  P.counters = b.counters;
  P.best = b.best;
  P.status = b.status;
  P.C0max = C0max;
  P.trans = ctx.alloc<int>(static_cast<size_t>(problems) * C0max * C0max);
  P.foldcnt = ctx.alloc<int>(static_cast<size_t>(problems) * P.F * C0max);
  const int grid = std::min(problems, ctx.sms());
  constexpr size_t kSmemBudget = 224 * 1024;
  const size_t Lp = (static_cast<size_t>(L) + 7) / 8 * 8;
  // prefer (in order): rows, transitions in shared memory
  bool placed = false;
  size_t smem = 0;
  for (int option = 0; option < 4 && !placed; ++option) {
    const bool rows = option < 2;
    const bool trans = (option % 2) == 0;
    smem = kgb::evolve_smem_bytes(L, C0max, rows, trans);
    if (smem <= kSmemBudget) {
      placed = true;
      P.smem_rows = rows;
      P.smem_trans = trans;
    }
  }
  if (!placed) fail(KGB_EINVAL, "too many distinct labels for the evolution kernel");
  P.rows_scratch = P.smem_rows ? nullptr
                               : ctx.alloc<uint16_t>(static_cast<size_t>(grid) * kgb::kEvolveRowArrays * Lp);
  P.raw_scratch = ctx.alloc<uint64_t>(static_cast<size_t>(grid) * (L / 2 + 64));
  if (P.smem_trans) P.trans = nullptr;
  {
    int* roff = ctx.alloc<int>(static_cast<size_t>(problems) * (L + 1));
    uint16_t* ridx = ctx.alloc<uint16_t>(static_cast<size_t>(problems) * L * P.w);
    kgb::ReverseArgs ra{};
    ra.problems = problems;
    ra.L = L;
    ra.w = P.w;
    ra.nb = P.nb;
    ra.rev_off = roff;
    ra.rev_idx = ridx;
    ck_launch(kgb::build_reverse_tables(ra, ctx.stream()), "reverse tables");
    P.rev_off = roff;
    P.rev_idx = ridx;
  }
  {
    std::vector<double> psq(static_cast<size_t>(L) + 1);
    const double nd = static_cast<double>(L);
    for (int c = 0; c <= L; ++c) {
      const double q = static_cast<double>(c) / nd;
      psq[c] = q * q;
    }
    P.psq = ctx.upload(psq.data(), psq.size());
  }
  ck_launch(kgb::evolve_launch(P, grid, smem, ctx.stream()), "evolution kernel launch");
  return b;
}

// ---------------------------------------------------------------------------
// PLS-LDA (pls.cu): fold slices, device buffers, the evolution cycle loop
// ---------------------------------------------------------------------------

// The SIMPLS start vector (plscv.cpp:833-838): the reference's own engine and
// distribution from the same libstdc++, hence the same floats.
std::vector<float> pls_start_vector(int p) {
  std::mt19937 gen(1u);
  std::normal_distribution<float> nd(0.0f, 1.0f);
  std::vector<float> w(static_cast<size_t>(p));
  for (float& v : w) v = nd(gen);
  return w;
}

// Slices of R problems of L rows: fold ids renumbered densely per problem (the
// reference visits only the fold ids that occur), training and validation
// rows of each slice ascending.  Predict mode: one slice per problem, every
// row trains.
struct PlsSlices {
  int F = 1;
  std::vector<int> train_off, train_idx, val_off, val_idx, ntrain, present;
  std::vector<uint8_t> folds8;
};

// Slices (r, f) of R problems of L rows: training rows = the rows outside
// fold f (every row in predict mode), validation rows = fold f, both
// ascending; fold ids are made dense per problem.  Sized by counting first
// and filled in parallel over the problems (this runs while the device
// works, and a serial push_back build of 500 slices took longer than that).
PlsSlices pls_slices(const std::vector<std::vector<int>>& folds, int R, int L, bool predict) {
  PlsSlices sl;
  const int threads = host_threads(0);
  std::vector<int> dense(predict ? 0 : static_cast<size_t>(R) * L);
  std::vector<int> nf(static_cast<size_t>(R), 1);
  if (!predict) {
    parallel_for(R, threads, [&](int r) {
      std::vector<int> ids = folds[r];
      std::sort(ids.begin(), ids.end());
      ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
      nf[r] = static_cast<int>(ids.size());
      int* dr = dense.data() + static_cast<size_t>(r) * L;
      for (int i = 0; i < L; ++i)
        dr[i] = static_cast<int>(std::lower_bound(ids.begin(), ids.end(), folds[r][i]) - ids.begin());
    });
    sl.F = 0;
    for (int r = 0; r < R; ++r) sl.F = std::max(sl.F, nf[r]);
    if (sl.F > 255) fail(KGB_EINVAL, "at most 255 folds are supported");
    sl.folds8.resize(static_cast<size_t>(R) * L);
  }
  const int F = sl.F;
  // validation counts per slice, then the offsets
  std::vector<int> nval(static_cast<size_t>(R) * F, 0);
  if (!predict)
    parallel_for(R, threads, [&](int r) {
      const int* dr = dense.data() + static_cast<size_t>(r) * L;
      int* c = nval.data() + static_cast<size_t>(r) * F;
      for (int i = 0; i < L; ++i) ++c[dr[i]];
    });
  const size_t S = static_cast<size_t>(R) * F;
  sl.train_off.resize(S + 1);
  sl.val_off.resize(S + 1);
  sl.ntrain.resize(S);
  sl.present.resize(S);
  sl.train_off[0] = 0;
  sl.val_off[0] = 0;
  for (size_t q = 0; q < S; ++q) {
    sl.ntrain[q] = L - nval[q];
    sl.train_off[q + 1] = sl.train_off[q] + sl.ntrain[q];
    sl.val_off[q + 1] = sl.val_off[q] + nval[q];
    sl.present[q] = static_cast<int>(q % F) < nf[q / F] ? 1 : 0;
  }
  sl.train_idx.resize(static_cast<size_t>(sl.train_off[S]));
  sl.val_idx.resize(static_cast<size_t>(sl.val_off[S]));
  parallel_for(R, threads, [&](int r) {
    const int* dr = predict ? nullptr : dense.data() + static_cast<size_t>(r) * L;
    for (int f = 0; f < F; ++f) {
      const size_t q = static_cast<size_t>(r) * F + f;
      int* tr = sl.train_idx.data() + sl.train_off[q];
      int* va = sl.val_idx.data() + sl.val_off[q];
      for (int i = 0; i < L; ++i) {
        if (dr != nullptr && dr[i] == f) *va++ = i;
        else *tr++ = i;
      }
    }
    if (!predict)
      for (int i = 0; i < L; ++i) sl.folds8[static_cast<size_t>(r) * L + i] = static_cast<uint8_t>(dr[i]);
  });
  return sl;
}

// One problem's slices padded with absent (empty) slices up to F.
PlsSlices pad_slices(PlsSlices sl, int F) {
  for (int f = sl.F; f < F; ++f) {
    sl.train_off.push_back(sl.train_off.back());
    sl.val_off.push_back(sl.val_off.back());
    sl.ntrain.push_back(0);
    sl.present.push_back(0);
  }
  sl.F = std::max(sl.F, F);
  return sl;
}

// Host preparation that depends only on (seed, run, L): the fold plans and,
// for the PLS classifier, the cross-validation slices over them.  Started on
// host threads at the beginning of a call, so it overlaps the graph and the
// k-means on the device.
struct FoldWork {
  std::vector<kgb::FoldPlan> plans;
  PlsSlices slices;
  bool has_slices = false;
};

FoldWork plan_fold_work(int M, int L, int F, uint64_t seed, int first_run, int nthreads, bool pls) {
  FoldWork w;
  w.plans.resize(static_cast<size_t>(M));
  parallel_for(M, nthreads, [&](int r) { w.plans[r] = kgb::plan_folds(L, F, seed, first_run + r); });
  if (pls) {
    std::vector<std::vector<int>> fl(static_cast<size_t>(M));
    for (int r = 0; r < M; ++r) fl[r].assign(w.plans[r].folds.begin(), w.plans[r].folds.end());
    w.slices = pls_slices(fl, M, L, false);
    w.has_slices = true;
  }
  return w;
}

struct PlsBuffers {
  kgb::PlsPrepArgs prep{};
  kgb::PlsEvalArgs ev{};
  int S = 0;
  std::vector<int> ntrain, present;
};

// Device room for slices that change at every evaluation (stratified folds of
// the labels being evaluated): one problem of n rows and up to F slices.
struct PlsSliceRoom {
  int* train_off = nullptr;
  int* train_idx = nullptr;
  int* val_off = nullptr;
  int* val_idx = nullptr;
  uint8_t* folds = nullptr;
  float* logprior = nullptr;
  int* lp_off = nullptr;
};

// logf(max(k / nt, FLT_MIN)) for every count k of a class of each slice, one
// table per distinct training size.
void pls_logprior_tables(const std::vector<int>& ntrain, std::vector<float>& tables, std::vector<int>& lp_off) {
  std::map<int, int> table_of;
  tables.clear();
  lp_off.assign(ntrain.size(), 0);
  for (size_t s2 = 0; s2 < ntrain.size(); ++s2) {
    const int nt = ntrain[s2];
    auto it = table_of.find(nt);
    if (it == table_of.end()) {
      it = table_of.emplace(nt, static_cast<int>(tables.size())).first;
      const float den = static_cast<float>(std::max(1, nt));
      for (int k = 0; k <= nt; ++k)
        tables.push_back(std::log(std::max(static_cast<float>(k) / den, std::numeric_limits<float>::min())));
    }
    lp_off[s2] = it->second;
  }
}

// Statistics, standardised rows and evaluation scratch of a set of slices.
// d_X: R x L x p rows; d_Xv: R x NV x p rows to predict (predict mode) or null.
// Whether the label cross-product of an evaluation lives in shared memory.
bool pls_s_in_smem(int p, int C0max, int requested, int max_components, bool tiles_after_s, bool few_slices) {
  const size_t two_ctas = 110 * 1024;
  const size_t bytes = kgb::pls_eval_smem(p, C0max, requested, max_components, true, tiles_after_s);
  return bytes <= two_ctas || (few_slices && bytes <= 200 * 1024);
}

PlsBuffers pls_buffers(Ctx& ctx, const float* d_X, int R, int L, int p, const PlsSlices& sl, int C0max,
                       int max_components, int requested, bool center, bool scale, const float* d_Xv, int NV) {
  PlsBuffers b;
  const int F = sl.F, S = R * F;
  b.S = S;
  b.ntrain = sl.ntrain;
  b.present = sl.present;
  if (requested > kgb::kPlsMaxComponents || max_components > kgb::kPlsMaxComponents)
    fail(KGB_EINVAL, "at most 64 PLS components are supported by the CUDA PLS-LDA kernel");
  // the cross-product in shared memory when two CTAs still fit on an SM
  // (evaluations that compute scores in the fit hold the score tiles beside
  // it); with no more slices than SMs one CTA per SM costs nothing
  const bool s_in_smem = pls_s_in_smem(p, C0max, requested, max_components, true, S <= ctx.sms());
  if (kgb::pls_eval_smem(p, C0max, requested, max_components, s_in_smem, true) > 200 * 1024)
    fail(KGB_EINVAL, "too many features, classes or components for the PLS-LDA kernel");
  cudaStream_t st = ctx.stream();
  kgb::PlsPrepArgs& a = b.prep;
  a.problems = R;
  a.F = F;
  a.L = L;
  a.p = p;
  a.center = center;
  a.scale = scale;
  a.X = d_X;
  int* d_toff = ctx.upload(sl.train_off.data(), sl.train_off.size());
  int* d_tidx = sl.train_idx.empty() ? ctx.alloc<int>(1) : ctx.upload(sl.train_idx.data(), sl.train_idx.size());
  a.train_off = d_toff;
  a.train_idx = d_tidx;
  a.mean = ctx.alloc<float>(static_cast<size_t>(S) * p);
  a.sdev = ctx.alloc<float>(static_cast<size_t>(S) * p);
  a.Z = ctx.alloc<float>(static_cast<size_t>(S) * L * p);
  a.xsum = ctx.alloc<float>(static_cast<size_t>(S) * p);
  a.zexp = ctx.alloc<int>(static_cast<size_t>(S) * p);
  a.Xv = d_Xv;
  a.NV = NV;
  a.Zv = d_Xv != nullptr ? ctx.alloc<float>(static_cast<size_t>(R) * NV * p) : nullptr;
  a.gram = nullptr;
  ck_launch(kgb::pls_prepare(a, st), "PLS fold preparation");

  kgb::PlsEvalArgs& e = b.ev;
  e.problems = R;
  e.F = F;
  e.L = L;
  e.p = p;
  e.C0max = C0max;
  e.max_components = max_components;
  e.requested = requested;
  e.predict_mode = d_Xv != nullptr;
  e.s_in_smem = s_in_smem ? 1 : 0;
  e.tiles_after_s = 1;  // no fold Gram yet: every slice computes scores in the fit
  e.Z = a.Z;
  e.xsum = a.xsum;
  e.zexp = a.zexp;
  e.gram = nullptr;
  e.use_gram = ctx.alloc<uint8_t>(S);
  ck(cudaMemsetAsync(const_cast<uint8_t*>(e.use_gram), 0, S, st), "memset");
  e.folds = e.predict_mode ? nullptr : ctx.upload(sl.folds8.data(), sl.folds8.size());
  e.train_off = d_toff;
  e.train_idx = d_tidx;
  e.val_off = ctx.upload(sl.val_off.data(), sl.val_off.size());
  e.val_idx = sl.val_idx.empty() ? ctx.alloc<int>(1) : ctx.upload(sl.val_idx.data(), sl.val_idx.size());
  e.Zv = a.Zv;
  e.NV = NV;
  const std::vector<float> w0 = pls_start_vector(p);
  e.w0 = ctx.upload(w0.data(), w0.size());
  std::vector<float> tables;
  std::vector<int> lp_off;
  pls_logprior_tables(sl.ntrain, tables, lp_off);
  e.logprior = ctx.upload(tables.data(), tables.size());
  e.lp_off = ctx.upload(lp_off.data(), lp_off.size());
  e.pred = ctx.alloc<uint16_t>(static_cast<size_t>(R) * (e.predict_mode ? NV : L));
  e.eval_comp = ctx.alloc<int>(S);
  e.status = ctx.alloc<int>(S);
  e.s_scr = ctx.alloc<float>(static_cast<size_t>(S) * p * C0max);
  e.W = ctx.alloc<float>(static_cast<size_t>(S) * p * max_components);
  e.V = ctx.alloc<float>(static_cast<size_t>(S) * p * max_components);
  e.T = ctx.alloc<float>(static_cast<size_t>(S) * L * requested);
  e.Tt = ctx.alloc<float>(static_cast<size_t>(S) * L * requested);
  e.pos = ctx.alloc<uint16_t>(static_cast<size_t>(S) * L);
  e.posok = ctx.alloc<uint8_t>(static_cast<size_t>(S) * L);
  e.sc = ctx.alloc<float>(static_cast<size_t>(S) * L);
  return b;
}

// Moves one problem's slice set (pad_slices to the buffers' S) into the
// room and recomputes the fold statistics and standardised rows.
void pls_refresh_slices(Ctx& ctx, PlsBuffers& b, const PlsSliceRoom& room, const PlsSlices& sl, int n) {
  if (sl.F != b.S) fail(KGB_EINTERNAL, "slice count changed");
  ctx.h2d(room.train_off, sl.train_off.data(), sl.train_off.size());
  ctx.h2d(room.train_idx, sl.train_idx.data(), sl.train_idx.size());
  ctx.h2d(room.val_off, sl.val_off.data(), sl.val_off.size());
  ctx.h2d(room.val_idx, sl.val_idx.data(), sl.val_idx.size());
  ctx.h2d(room.folds, sl.folds8.data(), static_cast<size_t>(n));
  std::vector<float> tables;
  std::vector<int> lp_off;
  pls_logprior_tables(sl.ntrain, tables, lp_off);
  ctx.h2d(room.logprior, tables.data(), tables.size());
  ctx.h2d(room.lp_off, lp_off.data(), lp_off.size());
  b.ntrain = sl.ntrain;
  b.present = sl.present;
  b.prep.train_off = room.train_off;
  b.prep.train_idx = room.train_idx;
  b.ev.train_off = room.train_off;
  b.ev.train_idx = room.train_idx;
  b.ev.val_off = room.val_off;
  b.ev.val_idx = room.val_idx;
  b.ev.folds = room.folds;
  b.ev.logprior = room.logprior;
  b.ev.lp_off = room.lp_off;
  ck_launch(kgb::pls_prepare(b.prep, ctx.stream()), "PLS fold preparation");
}

// Builds the fold Gram matrices (slices with at least p training rows) and
// switches the evaluation to the Gram loadings, as the reference's fold cache
// does from the second evaluation of a data epoch on.
void pls_enable_gram(Ctx& ctx, PlsBuffers& b) {
  const int S = b.S, p = b.prep.p;
  std::vector<uint8_t> want(static_cast<size_t>(S));
  for (int s2 = 0; s2 < S; ++s2) want[s2] = p <= b.ntrain[s2] ? 1 : 0;
  uint8_t* d_want = const_cast<uint8_t*>(b.ev.use_gram);
  ctx.h2d(d_want, want.data(), want.size());
  b.prep.gram = ctx.alloc<float>(static_cast<size_t>(S) * p * p);
  ck_launch(kgb::pls_build_gram(b.prep, d_want, ctx.stream()), "fold Gram");
  b.ev.gram = b.prep.gram;
  b.ev.tiles_after_s = std::all_of(want.begin(), want.end(), [](uint8_t v) { return v != 0; }) ? 0 : 1;
  b.ev.s_in_smem = pls_s_in_smem(p, b.ev.C0max, b.ev.requested, b.ev.max_components, b.ev.tiles_after_s != 0,
                                 S <= ctx.sms())
                       ? 1
                       : 0;
}

// Host class lists of coded labels: rows grouped by code, ascending within.
void class_lists_host(const std::vector<uint16_t>& codes, int C0max, std::vector<int>& off,
                      std::vector<uint16_t>& rows) {
  off.assign(static_cast<size_t>(C0max) + 1, 0);
  for (uint16_t c : codes) off[c + 1]++;
  for (int c = 0; c < C0max; ++c) off[c + 1] += off[c];
  std::vector<int> pos(off.begin(), off.end() - 1);
  rows.resize(codes.size());
  for (size_t i = 0; i < codes.size(); ++i) rows[pos[codes[i]]++] = static_cast<uint16_t>(i);
}

// Status words of PLS-LDA fits read back after the call's work: with a sink
// the check is deferred to pls_status_check (the captured batch path).
struct PlsStatusSink {
  std::vector<std::vector<int>> status;
  std::vector<std::vector<uint8_t>> present;
};

void pls_status_check(const std::vector<int>& status, const std::vector<uint8_t>& present) {
  for (size_t s2 = 0; s2 < status.size(); ++s2) {
    if (!present[s2]) continue;
    if (status[s2] == 1) fail(KGB_EINTERNAL, "CPU float32 SIMPLS found no supervised latent direction.");
    if (status[s2] == 2) fail(KGB_EINTERNAL, "Float32 PLS-LDA Cholesky factorization failed.");
  }
}

void pls_check_status(Ctx& ctx, const PlsBuffers& b, PlsStatusSink* sink = nullptr) {
  if (sink != nullptr) {
    sink->status.emplace_back(static_cast<size_t>(b.S));
    sink->present.emplace_back(b.present.begin(), b.present.end());
    ctx.download(sink->status.back().data(), b.ev.status, static_cast<size_t>(b.S));
    return;
  }
  std::vector<int> status(static_cast<size_t>(b.S));
  ctx.download(status.data(), b.ev.status, status.size());
  ctx.sync();
  pls_status_check(status, std::vector<uint8_t>(b.present.begin(), b.present.end()));
}

// maximize_core with the PLS-LDA predictor for P.problems problems whose
// slices are in `b`: the cycle loop of alternating evolution steps and CV
// evaluations.  P carries everything but the outputs and scratch.
// before_eval (may be empty) runs before every evaluation (the labels to
// evaluate are in b.ev.labels); with it the fold Gram is never used.
EvolveBuffers run_pls_evolution(Ctx& ctx, kgb::EvolveParams P, PlsBuffers& b, int C0max, bool coarsening,
                                const kgb_policy& pol, PlsStatusSink* sink = nullptr,
                                const std::function<void()>& before_eval = {}) {
  const int problems = P.problems, L = P.L, T = P.T;
  cudaStream_t st = ctx.stream();
  EvolveBuffers eb;
  eb.clbest = ctx.alloc<uint16_t>(static_cast<size_t>(problems) * L);
  eb.cvpredbest = ctx.alloc<uint16_t>(static_cast<size_t>(problems) * L);
  eb.vect_acc = ctx.alloc<double>(static_cast<size_t>(problems) * std::max(T, 1));
  eb.vect_score = ctx.alloc<double>(static_cast<size_t>(problems) * std::max(T, 1));
  eb.psize = ctx.alloc<int>(static_cast<size_t>(problems) * std::max(T, 1));
  eb.active = ctx.alloc<int>(static_cast<size_t>(problems) * std::max(T, 1));
  eb.flags = ctx.alloc<uint8_t>(static_cast<size_t>(problems) * std::max(T, 1) * 3);
  eb.counters = ctx.alloc<int>(static_cast<size_t>(problems) * 18);
  eb.best = ctx.alloc<double>(static_cast<size_t>(problems) * 2);
  eb.status = ctx.alloc<int>(static_cast<size_t>(problems));
  P.clbest = eb.clbest;
  P.cvpredbest = eb.cvpredbest;
  P.vect_acc = eb.vect_acc;
  P.vect_score = eb.vect_score;
  P.proposal_size = eb.psize;
  P.active = eb.active;
  P.flags = eb.flags;
  P.counters = eb.counters;
  P.best = eb.best;
  P.status = eb.status;
  P.C0max = C0max;
  P.w = 1;
  P.trans = ctx.alloc<int>(static_cast<size_t>(problems) * C0max * C0max);
  const int grid = problems;
  constexpr size_t kSmemBudget = 200 * 1024;
  const size_t Lp = (static_cast<size_t>(L) + 7) / 8 * 8;
  bool placed = false;
  size_t smem = 0;
  for (int option = 0; option < 4 && !placed; ++option) {
    const bool rows = option < 2;
    const bool trans = (option % 2) == 0;
    smem = kgb::evolve_smem_bytes(L, C0max, rows, trans);
    if (smem <= kSmemBudget) {
      placed = true;
      P.smem_rows = rows;
      P.smem_trans = trans;
    }
  }
  if (!placed) fail(KGB_EINVAL, "too many distinct labels for the evolution kernel");
  P.rows_scratch = P.smem_rows ? nullptr
                               : ctx.alloc<uint16_t>(static_cast<size_t>(grid) * kgb::kEvolveRowArrays * Lp);
  P.raw_scratch = ctx.alloc<uint64_t>(static_cast<size_t>(grid) * (L / 2 + 64));
  if (P.smem_trans) P.trans = nullptr;
  {
    std::vector<double> psq(static_cast<size_t>(L) + 1);
    const double nd = static_cast<double>(L);
    for (int c = 0; c <= L; ++c) {
      const double q = static_cast<double>(c) / nd;
      psq[c] = q * q;
    }
    P.psq = ctx.upload(psq.data(), psq.size());
  }
  kgb::EvolvePlsParams Q{};
  Q.base = P;
  Q.state = ctx.alloc<kgb::PlsRunState>(problems);
  Q.rng = ctx.alloc<kgb::Mt64State>(problems);
  Q.cur = ctx.alloc<uint16_t>(static_cast<size_t>(problems) * L);
  Q.curpred = ctx.alloc<uint16_t>(static_cast<size_t>(problems) * L);
  Q.cl = ctx.alloc<uint16_t>(static_cast<size_t>(problems) * L);
  Q.pred = b.ev.pred;
  Q.class_off = ctx.alloc<int>(static_cast<size_t>(problems) * (C0max + 1));
  Q.class_rows = ctx.alloc<uint16_t>(static_cast<size_t>(problems) * L);
  {
    // entropy terms p*log(p), p = k/L, rounded as core_objective_score does
    std::vector<double> plogp(static_cast<size_t>(L) + 1, 0.0);
    const double nd = static_cast<double>(L);
    for (int k = 1; k <= L; ++k) {
      const double q = static_cast<double>(k) / nd;
      plogp[k] = q * std::log(q);
    }
    Q.plogp = ctx.upload(plogp.data(), plogp.size());
    Q.logn = std::log(nd);
    std::vector<double> klogk(static_cast<size_t>(L) + 1, 0.0), logk(static_cast<size_t>(L) + 1, 0.0);
    for (int k = 1; k <= L; ++k) {
      logk[k] = std::log(static_cast<double>(k));
      klogk[k] = static_cast<double>(k) * logk[k];
    }
    Q.klogk = ctx.upload(klogk.data(), klogk.size());
    Q.logk = ctx.upload(logk.data(), logk.size());
  }
  Q.coarsening = coarsening;
  Q.pol_coarsen = pol.pls_transition_coarsening != 0;
  Q.pol_frag = pol.pls_fragmentation_penalty != 0;
  b.ev.labels = Q.cl;
  b.ev.class_off = Q.class_off;
  b.ev.class_rows = Q.class_rows;
  Q.phase = 0;
  Q.cycle = 0;
  ck_launch(kgb::evolve_pls_launch(Q, grid, smem, st), "PLS evolution step");
  for (int cycle = 0; cycle <= T; ++cycle) {
    if (before_eval) {
      before_eval();
    } else if (cycle == 1) {
      pls_enable_gram(ctx, b);
    }
    ck_launch(kgb::pls_evaluate(b.ev, st), "PLS-LDA evaluation");
    Q.phase = 1;
    Q.cycle = cycle;
    ck_launch(kgb::evolve_pls_launch(Q, grid, smem, st), "PLS evolution step");
  }
  pls_check_status(ctx, b, sink);
  // leave the best labels' class lists in b.ev for a projection
  b.ev.labels = eb.clbest;
  return eb;
}


void check_metric(int metric) {
  if (metric != KGB_METRIC_COSINE && metric != KGB_METRIC_INNER_PRODUCT && metric != KGB_METRIC_EUCLIDEAN)
    fail(KGB_EINVAL, "unknown distance metric");
}

void validate_matrix_options(const kgb_matrix_options* o) {
  if (o == nullptr) fail(KGB_EINVAL, "options pointer is null");
  if (o->runs < 1) fail(KGB_EINVAL, "KODAMAMatrixOptions::runs must be positive.");
  if (o->cycles < 0) fail(KGB_EINVAL, "KODAMAMatrixOptions::cycles must be non-negative.");
  if (o->folds < 2) fail(KGB_EINVAL, "KODAMAMatrixOptions::folds must be at least two.");
  if (o->folds > 255) fail(KGB_EINVAL, "at most 255 folds are supported");
  check_metric(o->metric);
}

// The KODAMA.matrix path after the global graph (n x K zero-based, compacted,
// distances finite >= 0) is resident on the device.
// The bf16 hi / lo split of the data matrix, made once per call and shared
// by the k-means runs that use the tensor-core assignment.
struct TcSplit {
  uint16_t* xh = nullptr;
  uint16_t* xl = nullptr;
  int dp = 0;
};

void tc_kmeans_inputs(Ctx& ctx, kgb::KMeansBatch& B, const float* d_x, int n, int d, TcSplit& split) {
  if (!kgb::kmeans_tc_supported(d, B.k)) return;
  if (split.xh == nullptr) {
    split.dp = (d + 15) / 16 * 16;
    split.xh = ctx.alloc<uint16_t>(static_cast<size_t>(n) * split.dp);
    split.xl = ctx.alloc<uint16_t>(static_cast<size_t>(n) * split.dp);
    ck_launch(kgb::bf16_split_rows(d_x, n, d, split.dp, split.xh, split.xl, ctx.stream()), "bf16 split");
  }
  B.xh = split.xh;
  B.xl = split.xl;
  B.dp = split.dp;
  B.ch = ctx.alloc<uint16_t>(static_cast<size_t>(B.problems) * B.k * split.dp);
  B.cl = ctx.alloc<uint16_t>(static_cast<size_t>(B.problems) * B.k * split.dp);
}

// Host side of one KODAMA.matrix call between its enqueue and its finalize:
// where the results land when the device work completes, and what the
// finalize needs to fill kgb_matrix_result.
struct MatrixTail {
  int n = 0, K = 0, M = 0, T = 0, L = 0, r0 = 1, cstride = 16;
  bool pls = false, want_graph = false, apply_dissimilarity = false, graph_here = false;
  void* res_stage = nullptr;  // pinned copy of res (host results only)
  size_t res_bytes = 0;
  std::vector<double> best, v;
  std::vector<int> psize, active, counters;
  std::vector<uint8_t> flags;
  std::vector<uint64_t> land_hash, init_hash, fold_hash;
  int plan_status = 0;
  PlsStatusSink pls_status;
  std::vector<int> gi;
  std::vector<float> gd;
  int ev_start = -1, ev_atlas = -1, ev_graph = -1, ev_init = -1, ev_tables = -1, ev_evo0 = -1, ev_evo1 = -1,
      ev_proj = -1, ev_dis = -1, ev_bg0 = -1, ev_bg1 = -1;
  bool graph_bg = false;  // the graph was built on the background stream (ev_bg0 .. ev_bg1)
};

// build_graph (may be empty): queues the kNN graph into d_gidx / d_gdist.  It
// needs only x, so outside a captured batch it runs on the low-priority
// background stream beside the landmark planning and the landmark k-means
// (from the start of the call, beside the atlas k-means too, when it is the
// longer branch), and is joined before anything reads the graph; in a
// captured batch it runs right after the atlas.  Queues
// the whole call; the results are read by matrix_finalize once the device
// work is done (no host wait on the plain path, so a batch can capture it).
void matrix_from_device_graph(Ctx& ctx, const float* d_x, int n, int d, int* d_gidx, float* d_gdist, int K,
                              const kgb_matrix_options* o, kgb_matrix_result* out, Clock& clk, int ev_start,
                              int ev_graph, std::future<FoldWork>& folds_future,
                              MatrixTail& tail, const std::function<void()>& build_graph = {}) {
  const kgb_policy pol = policy_is_zero(o->policy) ? default_policy() : o->policy;
  int landmarks = o->landmarks > 0 ? o->landmarks : 10000;
  if (landmarks >= n) landmarks = static_cast<int>(std::ceil(static_cast<double>(n) * 0.75));
  landmarks = std::max(2, std::min(landmarks, n - 1));
  const int splitting = o->splitting > 0 ? o->splitting : (n < 40000 ? 100 : 300);
  const int coarse_k = std::max(2, std::min(splitting, n));
  const int M = o->runs, T = o->cycles, F = o->folds;
  const uint64_t seed = o->seed;
  const int knn_k = std::max(o->knn_k, 1);
  const int w = std::max(1, std::min(knn_k, K));
  const bool pls = o->classifier == 1;
  TcSplit tc_split;
  if (o->classifier != 0 && o->classifier != 1) fail(KGB_EINVAL, "Unsupported KODAMA.matrix classifier.");
  if (!pls && w > 32) fail(KGB_EINVAL, "knn.k above 32 is not supported by the vote kernel");
  if (!pls && knn_k > kgb::kMaxProjectK) fail(KGB_EINVAL, "knn.k too large for the projection kernel");
  if (pls && o->components < 1) fail(KGB_EINVAL, "PLSOptions::max_components must be positive.");
  cudaStream_t st = ctx.stream();

  // Where the background graph starts.  Its CTAs, once resident, hold the SMs
  // that the atlas k-means' many short launches wait for, so it starts after
  // the atlas -- unless it is the longer branch: the candidate search grows as
  // n^2 d and the atlas plus the landmark stage about as n, and from about
  // n = 40000 at d = 64 (N=20000, d=50: graph 2 ms, atlas + landmarks 6.5 ms;
  // N=100000: 55 ms against 25 ms) the graph starts with the call.
  const bool graph_first = static_cast<double>(n) * n * d >= 1.0e11;
  int ev_bg0 = -1, ev_bg1 = -1, ev_planned = -1;
  bool graph_bg = static_cast<bool>(build_graph) && graph_first &&
                  ctx.on_background([&]() { build_graph(); }, &ev_bg0, &ev_bg1);

  // shared landmark atlas (kodama_matrix.cpp:3662-3734)
  float* d_pnorm = ctx.alloc<float>(n);
  ck_launch(kgb::kmeans_row_norms(d_x, n, d, d_pnorm, st), "row norms");
  std::mt19937_64 shared_rng(seed + 1u);
  const int ck_atlas = std::max(1, std::min(coarse_k, n));
  const std::vector<int> atlas_init = kgb::permutation_head(n, kgb::kmeans_seed_from_draw(shared_rng()), ck_atlas);
  const int kmax = std::max(ck_atlas, splitting);
  const std::vector<float> split_u = kgb::split_uniforms(kmax);
  float* d_split = ctx.upload(split_u.data(), split_u.size());
  int* d_atlas_labels = ctx.alloc<int>(n);
  {
    kgb::KMeansBatch B{};
    B.problems = 1;
    B.n = n;
    B.d = d;
    B.k = ck_atlas;
    B.max_iter = 10;
    B.x = d_x;
    B.rows = nullptr;
    B.pnorm = d_pnorm;
    B.init_rows = ctx.upload(atlas_init.data(), atlas_init.size());
    B.split_uniform = d_split;
    B.cent = ctx.alloc<float>(static_cast<size_t>(ck_atlas) * d);
    B.cnorm = ctx.alloc<float>(ck_atlas);
    B.assign = ctx.alloc<int>(n);
    ck(cudaMemsetAsync(B.assign, 0xff, sizeof(int) * n, st), "memset");
    B.active = ctx.alloc<int>(1);
    B.changed = ctx.alloc<int>(1);
    B.labels = d_atlas_labels;
    B.members = ctx.alloc<int>(n);
    B.offsets = ctx.alloc<int>(ck_atlas + 1);
    B.fscratch = ctx.alloc<float>(3 * ck_atlas + 1);
    tc_kmeans_inputs(ctx, B, d_x, n, d, tc_split);
    ck_launch(kgb::kmeans_run(B, st), "atlas k-means");
  }
  const int ev_atlas = ctx.mark();
  const bool graph_here = static_cast<bool>(build_graph) && !ctx.has_background();
  if (graph_here) {
    build_graph();
    ev_graph = ctx.mark();
  }
  out->timings[2] = clk.lap();

  // per-run landmarks and k-means seeds, drawn on the device from the atlas
  // (side stream); quota_sample returns exactly
  // min(target, n) rows
  const int init_k = std::max(2, std::min(splitting, landmarks));
  const int kk = std::max(1, std::min(init_k, landmarks));
  const int r0 = o->first_run > 0 ? o->first_run : 1;
  const int L = landmarks;
  int* d_land = ctx.alloc<int>(static_cast<size_t>(M) * L);
  int* d_nonland = pls && n > L ? ctx.alloc<int>(static_cast<size_t>(M) * (n - L)) : nullptr;
  int* d_plan_init = ctx.alloc<int>(static_cast<size_t>(M) * kk);
  uint64_t* d_land_hash = ctx.alloc<uint64_t>(M);
  int* d_plan_status = ctx.alloc<int>(1);
  int* d_km_assign = nullptr;
  {
    ck(cudaMemsetAsync(d_plan_status, 0, sizeof(int), st), "memset");
    kgb::PlanArgs pa;
    pa.n = n;
    pa.strata = coarse_k;
    pa.target = L;
    pa.init_k = kk;
    pa.runs = M;
    pa.first_run = r0;
    pa.seed = seed;
    pa.atlas = d_atlas_labels;
    pa.land = d_land;
    pa.nonland = d_nonland;
    pa.init_rows = d_plan_init;
    pa.land_hash = d_land_hash;
    pa.status = d_plan_status;
    pa.scratch = ctx.alloc<char>(kgb::plan_scratch_bytes(n, coarse_k, L, M));
    ctx.fork();  // after the atlas and the status reset
    ck_launch(kgb::plan_landmarks(pa, ctx.side()), "landmark planning");
    // the landmark k-means' assignment scratch is cleared beside the
    // planning, so that the k-means launch is the first thing the main
    // stream runs once the planning ends
    if (o->starting_labels == nullptr) {
      d_km_assign = ctx.alloc<int>(static_cast<size_t>(M) * L);
      ck(cudaMemsetAsync(d_km_assign, 0xff, sizeof(int) * static_cast<size_t>(M) * L, st), "memset");
    }
    ctx.join();
    ev_planned = ctx.mark();
    // the serial landmark hashes stay on the side stream, beside the k-means
    ck_launch(kgb::plan_land_hash(pa, ctx.side()), "landmark hashes");
  }
  out->timings[5] = 0.0;
  std::vector<int> land;  // host copy, semi-supervised inputs only
  if (o->starting_labels != nullptr || o->constrain != nullptr || o->fixed != nullptr) {
    land.resize(static_cast<size_t>(M) * L);
    ctx.download(land.data(), d_land, land.size());
    ctx.sync();
    check_plan_status(d_plan_status);
  }
  int* d_init_labels = ctx.alloc<int>(static_cast<size_t>(M) * L);
  // semi-supervised inputs (run_kodama_matrix, kodama_matrix.cpp:3405-3420;
  // run_iteration :3060-3117): starting labels replace the k-means start,
  // a constraint groups the rows (normalize_constrain), fixed rows keep
  // their labels
  const bool has_start = o->starting_labels != nullptr;
  std::vector<int> groups_all;
  bool identity_groups = true;
  if (o->constrain != nullptr) {
    std::vector<int> all(static_cast<size_t>(n));
    std::iota(all.begin(), all.end(), 0);
    groups_all = first_appearance_ids(o->constrain, all);
    for (int i = 0; i < n && identity_groups; ++i) identity_groups = groups_all[i] == i + 1;
  }
  const bool semi = has_start || !identity_groups;
  std::vector<int> xcon;  // M x L landmark group ids (non-identity constraint)
  if (!identity_groups) {
    xcon.resize(static_cast<size_t>(M) * L);
    parallel_for(M, host_threads(o->host_threads), [&](int r) {
      const std::vector<int> lr(land.begin() + static_cast<size_t>(r) * L, land.begin() + static_cast<size_t>(r + 1) * L);
      const std::vector<int> ids = first_appearance_ids(groups_all.data(), lr);
      std::copy(ids.begin(), ids.end(), xcon.begin() + static_cast<size_t>(r) * L);
    });
  }
  if (!has_start) {
    kgb::KMeansBatch B{};
    B.problems = M;
    B.n = L;
    B.d = d;
    B.k = kk;
    B.max_iter = 10;
    B.x = d_x;
    B.rows = d_land;
    B.pnorm = d_pnorm;
    B.init_rows = d_plan_init;
    B.split_uniform = d_split;
    B.cent = ctx.alloc<float>(static_cast<size_t>(M) * kk * d);
    B.cnorm = ctx.alloc<float>(static_cast<size_t>(M) * kk);
    B.assign = d_km_assign;
    B.active = ctx.alloc<int>(M);
    B.changed = ctx.alloc<int>(M);
    B.labels = d_init_labels;
    B.members = ctx.alloc<int>(static_cast<size_t>(M) * L);
    B.offsets = ctx.alloc<int>(static_cast<size_t>(M) * (kk + 1));
    B.fscratch = ctx.alloc<float>(static_cast<size_t>(M) * (3 * kk + 1));
    tc_kmeans_inputs(ctx, B, d_x, n, d, tc_split);
    ck_launch(kgb::kmeans_run(B, st), "landmark k-means");
  }
  // the background graph becomes ready with the landmark k-means and is
  // queued after it, so the k-means' CTAs (a whole SM each) are placed first
  // and the graph fills the SMs they leave
  if (static_cast<bool>(build_graph) && !graph_first && !graph_here)
    graph_bg = ctx.on_background([&]() { build_graph(); }, &ev_bg0, &ev_bg1, ev_planned);
  // folds (and the PLS slices) were planned on the host while the device worked
  FoldWork fold_work = folds_future.get();
  std::vector<kgb::FoldPlan>& fold_plans = fold_work.plans;
  // label coding and the initial-label hashes on the device; with
  // semi-supervised inputs the start labels are built and coded on the host
  const uint64_t bc = kgb::unordered_bucket_count(static_cast<size_t>(L));
  std::vector<Coding> semi_codes;
  int C0max = std::max(F, kk);
  if (semi) {
    std::vector<int> init_host(static_cast<size_t>(M) * L);
    if (has_start) {
      for (size_t i = 0; i < init_host.size(); ++i) init_host[i] = o->starting_labels[land[i]];
    } else {
      ctx.download(init_host.data(), d_init_labels, init_host.size());
      ctx.sync();
    }
    semi_codes.resize(static_cast<size_t>(M));
    parallel_for(M, host_threads(o->host_threads), [&](int r) {
      int* lr = init_host.data() + static_cast<size_t>(r) * L;
      if (!identity_groups) {
        const int* gr = xcon.data() + static_cast<size_t>(r) * L;
        constrained_majority(lr, gr, static_cast<size_t>(L));
        // a constraint keeps every group inside one fold (make_folds,
        // common.cpp:190-214), so the folds follow the start labels
        const std::vector<int> fo = kgb::make_folds(std::vector<int>(lr, lr + L), std::vector<int>(gr, gr + L), F,
                                                    false, seed + static_cast<uint64_t>(r0 + r));
        fold_plans[r].folds.assign(fo.begin(), fo.end());
        fold_plans[r].fold_hash = kgb::fnv_hash(fo.data(), fo.size());
      }
      semi_codes[r] = code_labels(lr, L, bc);
    });
    if (!identity_groups) fold_work.has_slices = false;  // the folds follow the start labels
    for (const auto& c : semi_codes) C0max = std::max<int>(C0max, static_cast<int>(c.code2label.size()));
    ck(cudaMemcpyAsync(d_init_labels, init_host.data(), sizeof(int) * init_host.size(), cudaMemcpyHostToDevice, st),
       "H2D");
    ctx.sync();
  }
  std::vector<uint8_t> folds(static_cast<size_t>(M) * L);
  for (int r = 0; r < M; ++r) {
    std::copy(fold_plans[r].folds.begin(), fold_plans[r].folds.end(), folds.begin() + static_cast<size_t>(r) * L);
  }
  uint8_t* d_folds = ctx.upload(folds.data(), folds.size());
  uint16_t* d_codes = ctx.alloc<uint16_t>(static_cast<size_t>(M) * L);
  int* d_c2l = ctx.alloc<int>(static_cast<size_t>(M) * C0max);
  int* d_ncodes = ctx.alloc<int>(M);
  uint64_t* d_init_hash = ctx.alloc<uint64_t>(M);
  std::vector<uint8_t> nocol(static_cast<size_t>(M), 1);
  if (semi) {
    std::vector<uint16_t> codes(static_cast<size_t>(M) * L);
    std::vector<int> c2l(static_cast<size_t>(M) * C0max, 0), ncodes(static_cast<size_t>(M));
    for (int r = 0; r < M; ++r) {
      std::copy(semi_codes[r].codes.begin(), semi_codes[r].codes.end(), codes.begin() + static_cast<size_t>(r) * L);
      std::copy(semi_codes[r].code2label.begin(), semi_codes[r].code2label.end(),
                c2l.begin() + static_cast<size_t>(r) * C0max);
      ncodes[r] = static_cast<int>(semi_codes[r].code2label.size());
      nocol[r] = semi_codes[r].nocollide ? 1 : 0;
    }
    ck(cudaMemcpyAsync(d_codes, codes.data(), sizeof(uint16_t) * codes.size(), cudaMemcpyHostToDevice, st), "H2D");
    ck(cudaMemcpyAsync(d_c2l, c2l.data(), sizeof(int) * c2l.size(), cudaMemcpyHostToDevice, st), "H2D");
    ck(cudaMemcpyAsync(d_ncodes, ncodes.data(), sizeof(int) * ncodes.size(), cudaMemcpyHostToDevice, st), "H2D");
    ctx.sync();
    ctx.fork();
    ck_launch(kgb::fnv_rows(d_init_labels, M, L, d_init_hash, ctx.side()), "label hashes");
  } else {
    kgb::CodingArgs ca{};
    ca.problems = M;
    ca.n = L;
    ca.k = kk;
    ca.C0max = C0max;
    ca.labels = d_init_labels;
    ca.codes = d_codes;
    ca.code2label = d_c2l;
    ca.ncodes = d_ncodes;
    ck_launch(kgb::code_labels(ca, st), "label coding");
    // the serial FNV hashes overlap the evolution on the side stream
    ctx.fork();
    ck_launch(kgb::fnv_rows(d_init_labels, M, L, d_init_hash, ctx.side()), "label hashes");
  }
  tail.init_hash.assign(static_cast<size_t>(M), 0);
  ctx.download_side(tail.init_hash.data(), d_init_hash, static_cast<size_t>(M));
  out->timings[7] = 0.0;
  out->timings[3] = clk.lap();

  const int ev_init = ctx.mark();
  std::vector<uint64_t> seeds(static_cast<size_t>(M));
  for (int r = 0; r < M; ++r) seeds[r] = seed + static_cast<uint64_t>(r0 + r);
  std::vector<int> identity(static_cast<size_t>(L));
  for (int i = 0; i < L; ++i) identity[i] = i;
  std::vector<int> goff(static_cast<size_t>(L) + 1);
  for (int i = 0; i <= L; ++i) goff[i] = i;
  kgb::EvolveParams P{};
  P.problems = M;
  P.L = L;
  P.w = w;
  P.T = T;
  P.F = F;
  P.G = L;
  P.singleton = identity_groups ? 1 : 0;
  P.evolutionary = has_start ? 0 : 1;
  P.guarded = 1;
  P.absorption = 1;
  P.adaptive = 1;
  P.pol_guidance = pol.prediction_guidance != 0;
  P.pol_adaptive = pol.adaptive_proposal_size != 0;
  P.pol_transition = pol.transition_proposal != 0;
  P.pol_stochastic = pol.stochastic_acceptance != 0;
  P.pol_diversity = pol.diversity_multiplier != 0;
  P.pol_reject1 = pol.reject_single_class != 0;
  P.bucket_count = bc;
  P.init = d_codes;
  P.code2label = d_c2l;
  P.ncodes = d_ncodes;
  P.nocollide = ctx.upload(nocol.data(), nocol.size());
  P.folds = d_folds;
  P.fixed = nullptr;
  P.goff = ctx.upload(goff.data(), goff.size());
  P.gmem = ctx.upload(identity.data(), identity.size());
  if (!identity_groups || o->fixed != nullptr) {
    // one block of groups and fixed flags per run: groups in ascending id
    // (maximize_core's std::map), members in landmark order
    std::vector<int> pg_off(static_cast<size_t>(M) * (L + 1)), pg_mem(static_cast<size_t>(M) * L),
        pg_cnt(static_cast<size_t>(M));
    std::vector<int> pfix(o->fixed != nullptr ? static_cast<size_t>(M) * L : 0);
    parallel_for(M, host_threads(o->host_threads), [&](int r) {
      int* off = pg_off.data() + static_cast<size_t>(r) * (L + 1);
      int* mem = pg_mem.data() + static_cast<size_t>(r) * L;
      if (identity_groups) {
        for (int i = 0; i <= L; ++i) off[i] = i;
        for (int i = 0; i < L; ++i) mem[i] = i;
        pg_cnt[r] = L;
      } else {
        std::map<int, std::vector<int>> members;
        for (int i = 0; i < L; ++i) members[xcon[static_cast<size_t>(r) * L + i]].push_back(i);
        int g = 0, pos = 0;
        off[0] = 0;
        for (const auto& kv : members) {
          for (int m : kv.second) mem[pos++] = m;
          off[++g] = pos;
        }
        pg_cnt[r] = g;
      }
      if (o->fixed != nullptr)
        for (int i = 0; i < L; ++i)
          pfix[static_cast<size_t>(r) * L + i] = o->fixed[land[static_cast<size_t>(r) * L + i]] != 0 ? 1 : 0;
    });
    P.per_problem_groups = 1;
    P.goff = ctx.upload(pg_off.data(), pg_off.size());
    P.gmem = ctx.upload(pg_mem.data(), pg_mem.size());
    P.gcount = ctx.upload(pg_cnt.data(), pg_cnt.size());
    if (o->fixed != nullptr) P.fixed = ctx.upload(pfix.data(), pfix.size());
  }
  P.seeds = ctx.upload(seeds.data(), seeds.size());
  EvolveBuffers eb{};
  int* d_res = nullptr;
  int ev_tables = 0, ev_evo0 = 0, ev_evo1 = 0, ev_proj = 0;
  int cstride = 16;
  if (graph_bg) ctx.join_background();  // everything below may read the graph
  if (pls) {
    // PLS-LDA classifier (run_iteration, kodama_matrix.cpp:3105-3158, 3262-3276):
    // CorePLSLDA on the landmark rows of every run, PLSLDAPredict for the rest
    cstride = 18;
    const int p = d;
    float* d_xl = ctx.alloc<float>(static_cast<size_t>(M) * L * p);
    ck_launch(kgb::pls_gather_rows(d_x, p, d_land, static_cast<size_t>(M) * L, d_xl, st), "landmark rows");
    const bool planned = fold_work.has_slices && fold_work.slices.folds8.size() == static_cast<size_t>(M) * L;
    PlsSlices sl;
    if (planned) {
      sl = std::move(fold_work.slices);
    } else {
      std::vector<std::vector<int>> fl(static_cast<size_t>(M));
      for (int r = 0; r < M; ++r) fl[r].assign(fold_plans[r].folds.begin(), fold_plans[r].folds.end());
      sl = pls_slices(fl, M, L, false);
    }
    const int comps = o->components;
    PlsBuffers b = pls_buffers(ctx, d_xl, M, L, p, sl, C0max, comps, comps, true, true, nullptr, 0);
    ev_tables = ctx.mark();
    ev_evo0 = ev_tables;
    eb = run_pls_evolution(ctx, P, b, C0max, true, pol, &tail.pls_status);
    ev_evo1 = ctx.mark();
    const int NV = n - L;
    int* d_test = d_nonland != nullptr ? d_nonland : ctx.alloc<int>(1);
    d_res = ctx.alloc<int>(static_cast<size_t>(M) * n);
    uint16_t* d_proj = ctx.alloc<uint16_t>(static_cast<size_t>(M) * std::max(NV, 1));
    if (NV > 0) {
      float* d_xt = ctx.alloc<float>(static_cast<size_t>(M) * NV * p);
      ck_launch(kgb::pls_gather_rows(d_x, p, d_test, static_cast<size_t>(M) * NV, d_xt, st), "test rows");
      const int ncomp = std::max(1, std::min({comps, p, std::max(1, L - 1)}));
      const PlsSlices sp = pls_slices({}, M, L, true);
      PlsBuffers pb = pls_buffers(ctx, d_xl, M, L, p, sp, C0max, ncomp, ncomp, true, true, d_xt, NV);
      pb.ev.labels = eb.clbest;
      pb.ev.class_off = b.ev.class_off;
      pb.ev.class_rows = b.ev.class_rows;
      ck_launch(kgb::pls_evaluate(pb.ev, st), "PLS-LDA projection");
      pls_check_status(ctx, pb, &tail.pls_status);
      d_proj = pb.ev.pred;
    }
    ck_launch(kgb::pls_assemble_result(M, n, L, std::max(NV, 0), d_land, d_test, eb.clbest, d_proj, d_c2l, C0max,
                                       d_res, st),
              "result rows");
    ev_proj = ctx.mark();
    ctx.checkpoint();
    out->timings[4] = clk.lap();
  } else {
  // per-run fold-filtered vote tables over the landmark subgraph
  int* d_g2l = ctx.alloc<int>(static_cast<size_t>(M) * n);
  ck_launch(kgb::build_g2l(d_land, M, L, n, d_g2l, st), "landmark index");
  uint16_t* d_nb = ctx.alloc<uint16_t>(static_cast<size_t>(M) * L * w);
  float* d_sc = ctx.alloc<float>(static_cast<size_t>(M) * L * w);
  {
    kgb::VoteTableArgs a{};
    a.problems = M;
    a.L = L;
    a.n = n;
    a.K = K;
    a.w = w;
    a.gidx = d_gidx;
    a.gdist = d_gdist;
    a.land = d_land;
    a.g2l = d_g2l;
    a.folds = d_folds;
    a.nb = d_nb;
    a.sc = d_sc;
    a.score_one_minus = o->metric != KGB_METRIC_EUCLIDEAN;
    ck_launch(kgb::build_vote_tables(a, st), "vote tables");
  }
  ev_tables = ctx.mark();
  P.nb = d_nb;
  P.sc = d_sc;
  if (o->proposal_weights != nullptr) {
    float* master = ctx.upload(o->proposal_weights, kgb::kMlpParams);
    float* rounded = ctx.alloc<float>(kgb::kMlpParams);
    uint32_t* frag = ctx.alloc<uint32_t>(kgb::kMlpFragWords);
    ck_launch(kgb::mlp_round_params(master, rounded, st), "proposal weights");
    ck_launch(kgb::mlp_pack_params(rounded, frag, st), "proposal weights");
    P.mlp = frag;
    P.mlp_greedy = o->proposal_greedy != 0;
  }
  const bool snap = out->snapshot_features != nullptr && out->snapshot_flags != nullptr;
  if (snap) {
    P.snap_cycle = o->snapshot_cycle;
    P.snap_feat = ctx.alloc<float>(static_cast<size_t>(M) * L * kgb::kMlpIn);
    P.snap_cur = ctx.alloc<uint16_t>(static_cast<size_t>(M) * L);
    P.snap_pred = ctx.alloc<uint16_t>(static_cast<size_t>(M) * L);
    ck(cudaMemsetAsync(P.snap_feat, 0, sizeof(float) * M * L * kgb::kMlpIn, st), "memset");
    ck(cudaMemsetAsync(P.snap_cur, 0, sizeof(uint16_t) * M * L, st), "memset");
    ck(cudaMemsetAsync(P.snap_pred, 0, sizeof(uint16_t) * M * L, st), "memset");
  }
  ev_evo0 = ctx.mark();
  eb = run_evolution(ctx, P, C0max);
  ev_evo1 = ctx.mark();
  if (snap) {
    const size_t ML = static_cast<size_t>(M) * L;
    std::vector<uint16_t> scur(ML), spred(ML), best(ML);
    ctx.download(out->snapshot_features, P.snap_feat, ML * kgb::kMlpIn);
    ctx.download(scur.data(), P.snap_cur, ML);
    ctx.download(spred.data(), P.snap_pred, ML);
    ctx.download(best.data(), eb.clbest, ML);
    ctx.sync();
    for (size_t i = 0; i < ML; ++i)
      out->snapshot_flags[i] = static_cast<uint8_t>((scur[i] != spred[i] ? 1 : 0) | (best[i] == spred[i] ? 2 : 0));
  }

  // projection of non-landmarks and result matrix
  d_res = ctx.alloc<int>(static_cast<size_t>(M) * n);
  {
    kgb::ProjectArgs a{};
    a.problems = M;
    a.L = L;
    a.n = n;
    a.K = K;
    a.pk = knn_k;
    a.C0max = C0max;
    a.gidx = d_gidx;
    a.g2l = d_g2l;
    a.clbest = eb.clbest;
    a.code2label = P.code2label;
    a.res = d_res;
    ck_launch(kgb::project_labels(a, st), "projection");
  }
  ev_proj = ctx.mark();
  ctx.checkpoint();
  out->timings[4] = clk.lap();
  }

  if (!identity_groups) {
    // the result rows take their groups' majority labels (run_iteration,
    // kodama_matrix.cpp:3277-3283)
    std::vector<int> res_host(static_cast<size_t>(M) * n);
    ctx.download(res_host.data(), d_res, res_host.size());
    ctx.sync();
    parallel_for(M, host_threads(o->host_threads), [&](int r) {
      constrained_majority(res_host.data() + static_cast<size_t>(r) * n, groups_all.data(), static_cast<size_t>(n));
    });
    ck(cudaMemcpyAsync(d_res, res_host.data(), sizeof(int) * res_host.size(), cudaMemcpyHostToDevice, st), "H2D");
    ctx.sync();
  }

  // outputs: queued here, read by matrix_finalize
  tail.n = n;
  tail.K = K;
  tail.M = M;
  tail.T = T;
  tail.L = L;
  tail.r0 = r0;
  tail.cstride = cstride;
  tail.pls = pls;
  tail.res_bytes = sizeof(int) * static_cast<size_t>(M) * n;
  if (out->res_on_device) {
    ck(cudaMemcpyAsync(out->res, d_res, tail.res_bytes, cudaMemcpyDeviceToDevice, st), "D2D");
  } else {
    if (ctx.capturing()) fail(KGB_EINTERNAL, "a captured batch keeps its label matrices on the device");
    tail.res_stage = g_stage.get(tail.res_bytes);
    ck(cudaMemcpyAsync(tail.res_stage, d_res, tail.res_bytes, cudaMemcpyDeviceToHost, st), "D2H");
  }
  tail.best.assign(static_cast<size_t>(M) * 2, 0.0);
  tail.v.assign(static_cast<size_t>(M) * T, 0.0);
  tail.psize.assign(static_cast<size_t>(M) * T, 0);
  tail.active.assign(static_cast<size_t>(M) * T, 0);
  tail.counters.assign(static_cast<size_t>(M) * cstride, 0);
  tail.flags.assign(static_cast<size_t>(M) * T * 3, 0);
  ctx.download(tail.best.data(), eb.best, tail.best.size());
  ctx.download(tail.v.data(), eb.vect_acc, tail.v.size());
  ctx.download(tail.psize.data(), eb.psize, tail.psize.size());
  ctx.download(tail.active.data(), eb.active, tail.active.size());
  ctx.download(tail.flags.data(), eb.flags, tail.flags.size());
  ctx.download(tail.counters.data(), eb.counters, tail.counters.size());
  tail.want_graph = o->materialize_graph && out->knn_idx != nullptr && out->knn_dist != nullptr;
  tail.apply_dissimilarity = o->apply_dissimilarity != 0;
  if (tail.want_graph) {
    if (out->knn_cap < K) fail(KGB_EINVAL, "knn_cap is smaller than the graph width");
    tail.gi.assign(static_cast<size_t>(n) * K, 0);
    tail.gd.assign(static_cast<size_t>(n) * K, 0.0f);
    if (o->apply_dissimilarity) {
      int* d_lbs = ctx.alloc<int>(static_cast<size_t>(M) * n);
      ck_launch(kgb::transpose_runs(d_res, M, n, d_lbs, st), "transpose");
      int* d_oidx = ctx.alloc<int>(static_cast<size_t>(n) * K);
      float* d_odist = ctx.alloc<float>(static_cast<size_t>(n) * K);
      kgb::DissimArgs a{};
      a.n = n;
      a.K = K;
      a.runs = M;
      a.in_one_based = 0;
      a.out_one_based = 1;
      a.idx = d_gidx;
      a.dist = d_gdist;
      a.lbs = d_lbs;
      a.out_idx = d_oidx;
      a.out_dist = d_odist;
      ck_launch(kgb::dissimilarity(a, st), "dissimilarity");
      ctx.download(tail.gi.data(), d_oidx, tail.gi.size());
      ctx.download(tail.gd.data(), d_odist, tail.gd.size());
    } else {
      ctx.download(tail.gi.data(), d_gidx, tail.gi.size());
      ctx.download(tail.gd.data(), d_gdist, tail.gd.size());
    }
  }
  tail.ev_dis = ctx.mark();
  tail.land_hash.assign(static_cast<size_t>(M), 0);
  ctx.download_side(tail.land_hash.data(), d_land_hash, tail.land_hash.size());
  ctx.download(&tail.plan_status, d_plan_status, 1);
  tail.fold_hash.resize(static_cast<size_t>(M));
  for (int r = 0; r < M; ++r) tail.fold_hash[r] = fold_plans[r].fold_hash;
  tail.graph_here = graph_here;
  tail.graph_bg = graph_bg;
  tail.ev_bg0 = ev_bg0;
  tail.ev_bg1 = ev_bg1;
  tail.ev_start = ev_start;
  tail.ev_atlas = ev_atlas;
  tail.ev_graph = ev_graph;
  tail.ev_init = ev_init;
  tail.ev_tables = ev_tables;
  tail.ev_evo0 = ev_evo0;
  tail.ev_evo1 = ev_evo1;
  tail.ev_proj = ev_proj;
}

// Fills kgb_matrix_result from a completed call's tail (ctx null: no stage
// timings, as for a captured batch).
void matrix_finalize(Ctx* ctx, MatrixTail& t, kgb_matrix_result* out, Clock& clk) {
  if (t.plan_status != 0) fail(KGB_EINTERNAL, "Landmark quota allocation produced the wrong sample size.");
  for (size_t i = 0; i < t.pls_status.status.size(); ++i) pls_status_check(t.pls_status.status[i], t.pls_status.present[i]);
  const int M = t.M, T = t.T, n = t.n, K = t.K, L = t.L;
  if (t.res_stage != nullptr) std::memcpy(out->res, t.res_stage, t.res_bytes);
  if (!t.v.empty()) std::memcpy(out->v, t.v.data(), sizeof(double) * t.v.size());
  const double t_dl = clk.lap();
  auto ms = [&](int a, int b) { return ctx == nullptr ? 0.0 : ctx->ms(a, b); };
  if (t.graph_bg) {
    // the graph beside the atlas and the landmark initialisation
    out->kernel_ms[0] = ms(t.ev_bg0, t.ev_bg1);
    out->kernel_ms[1] = ms(t.ev_start, t.ev_atlas);
    out->kernel_ms[2] = ms(t.ev_atlas, t.ev_init);
  } else if (t.graph_here) {
    // order on the device: atlas, graph, landmark initialisation
    out->kernel_ms[0] = ms(t.ev_atlas, t.ev_graph);
    out->kernel_ms[1] = ms(t.ev_start, t.ev_atlas);
    out->kernel_ms[2] = ms(t.ev_graph, t.ev_init);
  } else {
    out->kernel_ms[0] = ms(t.ev_start, t.ev_graph);
    out->kernel_ms[1] = ms(t.ev_graph, t.ev_atlas);
    out->kernel_ms[2] = ms(t.ev_atlas, t.ev_init);
  }
  out->kernel_ms[3] = ms(t.ev_init, t.ev_tables);
  out->kernel_ms[4] = ms(t.ev_evo0, t.ev_evo1);
  out->kernel_ms[5] = ms(t.ev_evo1, t.ev_proj);
  out->kernel_ms[6] = ms(t.ev_proj, t.ev_dis);
  out->kernel_ms[7] = ms(t.ev_start, t.ev_dis);
  if (t.want_graph) {
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < K; ++j) {
        int v = t.gi[static_cast<size_t>(i) * K + j];
        if (!t.apply_dissimilarity && v >= 0) v += 1;
        out->knn_idx[static_cast<size_t>(i) * out->knn_cap + j] = v;
        out->knn_dist[static_cast<size_t>(i) * out->knn_cap + j] = t.gd[static_cast<size_t>(i) * K + j];
      }
    }
    out->knn_k = K;
  } else {
    out->knn_k = 0;
  }
  out->timings[6] = clk.lap() + t_dl;
  for (int r = 0; r < M; ++r) {
    out->acc[r] = t.best[2 * r];
    if (out->run_hashes) {
      out->run_hashes[3 * r + 0] = t.land_hash[r];
      out->run_hashes[3 * r + 1] = t.init_hash[r];
      out->run_hashes[3 * r + 2] = t.fold_hash[r];
    }
    const int* c = t.counters.data() + static_cast<size_t>(r) * t.cstride;
    if (out->pls_counters) {
      out->pls_counters[2 * r] = t.pls ? c[16] : 0;
      out->pls_counters[2 * r + 1] = t.pls ? c[17] : 0;
    }
    if (out->run_counters) {
      int* rc = out->run_counters + 8 * r;
      rc[0] = t.r0 + r;
      rc[1] = c[0];
      rc[2] = c[9];
      rc[3] = c[10];
      rc[4] = c[11];
      rc[5] = c[12];
      rc[6] = c[13];
      rc[7] = L;
    }
    if (out->cycle_diag) {
      for (int cy = 0; cy < T; ++cy) {
        int* cd = out->cycle_diag + (static_cast<size_t>(r) * T + cy) * 5;
        const size_t o1 = static_cast<size_t>(r) * T + cy;
        cd[0] = t.psize[o1];
        cd[1] = t.active[o1];
        cd[2] = t.flags[3 * o1 + 0];
        cd[3] = t.flags[3 * o1 + 1];
        cd[4] = t.flags[3 * o1 + 2];
      }
    }
  }
  out->effective_landmarks = L;
}

// The exact kNN graph of d_x (n x d, device) into d_idx / d_dist (n x K),
// self excluded, reported distances as the reference reports them
// (native_knn.cpp:1157-1164).  Euclidean: the tensor-core candidate search
// with its certificate where it applies (knn_tc.cu), else the brute force.
// Cosine (rows scaled as normalize_rows_for_cosine, kodama_matrix.cpp:155)
// and inner product: the brute-force search on minus the inner product.
// fallback_rows (host, may be null) receives how many rows the brute force
// computed.
void exact_graph(Ctx& ctx, const float* d_x, int n, int d, int K, int method, int metric, int* d_idx, float* d_dist,
                 int* fallback_rows) {
  const int segments = 4;
  if (metric != KGB_METRIC_EUCLIDEAN) {
    if (method == KGB_KNN_TENSOR) fail(KGB_EINVAL, "the tensor-core kNN search is for the Euclidean metric");
    const float* xs = d_x;
    if (metric == KGB_METRIC_COSINE) {
      float* xn = ctx.alloc<float>(static_cast<size_t>(n) * d);
      ck_launch(kgb::normalize_rows(d_x, n, d, 2, xn, ctx.stream()), "cosine rows");
      xs = xn;
    }
    void* scratch = ctx.alloc<unsigned char>(kgb::knn_bruteforce_scratch(n, K, segments));
    ck_launch(kgb::knn_bruteforce_inner(xs, n, d, K, metric, segments, scratch, d_idx, d_dist, ctx.stream()),
              "kNN graph");
    if (fallback_rows != nullptr) *fallback_rows = n;
    return;
  }
  const bool tc = method == KGB_KNN_TENSOR || (method == KGB_KNN_AUTO && kgb::knn_tc_supported(n, d, K));
  if (method == KGB_KNN_TENSOR && !kgb::knn_tc_supported(n, d, K))
    fail(KGB_EINVAL, "the tensor-core kNN search needs d <= 256, K <= 96 and n > 2 * (K + 16) + 64");
  if (tc) {
    void* scratch = ctx.alloc<unsigned char>(kgb::knn_tc_scratch(n, d, K, segments));
    ck_launch(kgb::knn_tc_graph(d_x, n, d, K, segments, scratch, d_idx, d_dist, ctx.stream()), "kNN graph");
    if (fallback_rows != nullptr) {
      int count = 0;
      ck_launch(kgb::knn_tc_fallback_count(scratch, n, d, K, segments, &count, ctx.stream()), "kNN graph");
      ctx.sync();
      *fallback_rows = count;
    }
  } else {
    void* scratch = ctx.alloc<unsigned char>(kgb::knn_bruteforce_scratch(n, K, segments));
    ck_launch(kgb::knn_bruteforce(d_x, n, d, K, segments, scratch, d_idx, d_dist, ctx.stream()), "kNN graph");
    if (fallback_rows != nullptr) *fallback_rows = n;
  }
}

// The exact graph a KODAMA.matrix call works on: under the cosine and
// inner-product metrics it then passes through normalize_external_graph
// (kodama_matrix.cpp:1292-1330), as the reference's graph-input path does
// with a caller graph, which clamps the reported distances at zero (1 - <x,y>
// can be negative).
void matrix_graph(Ctx& ctx, const float* d_x, int n, int d, int K, int metric, int* d_gidx, float* d_gdist) {
  if (metric == KGB_METRIC_EUCLIDEAN) {
    exact_graph(ctx, d_x, n, d, K, KGB_KNN_AUTO, metric, d_gidx, d_gdist, nullptr);
    return;
  }
  int* t_idx = ctx.alloc<int>(static_cast<size_t>(n) * K);
  float* t_dist = ctx.alloc<float>(static_cast<size_t>(n) * K);
  exact_graph(ctx, d_x, n, d, K, KGB_KNN_AUTO, metric, t_idx, t_dist, nullptr);
  int* d_mm = ctx.alloc<int>(2);
  ck_launch(kgb::graph_minmax(t_idx, static_cast<size_t>(n) * K, d_mm, ctx.stream()), "graph min/max");
  ck_launch(kgb::normalize_external(t_idx, t_dist, n, K, K, 0, d_mm, d_gidx, d_gdist, ctx.stream()),
            "graph normalisation");
}

// Landmarks and graph width of a call (run_kodama_matrix,
// kodama_matrix.cpp:3340-3350, and the graph width rule).
struct MatrixSizes {
  int landmarks, neighbors;
};
MatrixSizes matrix_sizes(int n, const kgb_matrix_options* opt) {
  int landmarks = opt->landmarks > 0 ? opt->landmarks : 10000;
  if (landmarks >= n) landmarks = static_cast<int>(std::ceil(static_cast<double>(n) * 0.75));
  landmarks = std::max(2, std::min(landmarks, n - 1));
  const int requested = opt->graph_neighbors > 0 ? opt->graph_neighbors : 100;
  const int neighbors = std::max(1, static_cast<int>(std::floor(std::min(
      {static_cast<double>(landmarks), static_cast<double>(n) * 0.75 - 1.0, static_cast<double>(requested)}))));
  return MatrixSizes{landmarks, neighbors};
}

// ---------------------------------------------------------------------------
// Batches of independent KODAMA.matrix problems in one captured CUDA graph.
//
// Every problem's plain raw-data path (matrix_from_device_graph) is queued,
// with no host synchronisation, into one of `lanes` stream pairs of a capture;
// the graph therefore holds `lanes` independent chains that the device runs
// side by side, and each problem's allocations are graph memory nodes freed
// at the end of its chain, so memory is reused along a chain.  The problems'
// data sit in one persistent device buffer and their label matrices in
// persistent device buffers; everything else goes through the capture arena.
// The schedule (lanes, and the order problems are dealt to the lanes) is
// picked by timing candidate graphs on the first call for a batch shape and
// kept for later calls; the last graph is replayed while the shape stays.
// ---------------------------------------------------------------------------
struct BatchProblem {
  MatrixTail tail;
  kgb_matrix_result shadow{};  // the capture's view of the result (label matrix on the device)
  int* d_res = nullptr;
  size_t x_off = 0;
  double cost = 0.0;
};

struct BatchGraph {
  std::string key;
  int device = 0, lanes = 0, order = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t root = nullptr;
  std::vector<cudaStream_t> streams;
  CaptureArena arena;
  std::vector<std::unique_ptr<BatchProblem>> problems;
  float* d_x = nullptr;
  size_t nodes = 0, kernel_nodes = 0;
  BatchGraph() = default;
  BatchGraph(const BatchGraph&) = delete;
  BatchGraph& operator=(const BatchGraph&) = delete;
  ~BatchGraph() {
    if (root) cudaStreamSynchronize(root);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& p : problems)
      if (p->d_res) cudaFree(p->d_res);
    if (d_x) cudaFree(d_x);
    for (cudaStream_t st : streams) cudaStreamDestroy(st);
    if (root) cudaStreamDestroy(root);
  }
};

std::mutex g_batch_mu;
std::unique_ptr<BatchGraph> g_batch;                  // the last captured batch
std::map<std::string, std::pair<int, int>> g_tuned;   // batch shape -> (lanes, order)

void check_batch_problem(const kgb_matrix_problem& q) {
  if (q.x == nullptr || q.result == nullptr) fail(KGB_EINVAL, "null pointer");
  if (q.n < 3) fail(KGB_EINVAL, "KODAMAMatrix requires at least 3 rows.");
  if (q.d < 1) fail(KGB_EINVAL, "Input matrix must have at least one column.");
  validate_matrix_options(&q.options);
  const kgb_matrix_result* r = q.result;
  if (r->res == nullptr || r->acc == nullptr || r->v == nullptr) fail(KGB_EINVAL, "null result buffer");
  if (r->res_on_device) fail(KGB_EINVAL, "a batch returns the label matrices in host memory");
  if (q.options.starting_labels != nullptr || q.options.constrain != nullptr || q.options.fixed != nullptr)
    fail(KGB_EINVAL, "semi-supervised inputs are not supported in a batch");
  if (q.options.proposal_weights != nullptr) fail(KGB_EINVAL, "the learned proposal is not supported in a batch");
  if (r->snapshot_features != nullptr || r->snapshot_flags != nullptr)
    fail(KGB_EINVAL, "proposal snapshots are not supported in a batch");
}

// Everything the captured work depends on, so a replay is only taken for the
// same shapes and options.
std::string batch_key(const kgb_matrix_problem* probs, int count, int device) {
  std::string k = std::to_string(device) + ":" + std::to_string(count);
  for (int i = 0; i < count; ++i) {
    const kgb_matrix_problem& q = probs[i];
    const kgb_matrix_options& o = q.options;
    char buf[512];
    std::snprintf(buf, sizeof(buf), "|%d,%d,%d,%d,%d,%d,%d,%d,%d,%d,%d,%d,%d,%d,%d,%llu,%d%d%d%d%d%d%d%d,%d,%d,%d",
                  q.n, q.d, o.runs, o.cycles, o.landmarks, o.splitting, o.graph_neighbors, o.folds, o.knn_k,
                  o.classifier, o.components, o.materialize_graph, o.apply_dissimilarity, o.metric, o.first_run,
                  static_cast<unsigned long long>(o.seed), o.policy.prediction_guidance,
                  o.policy.adaptive_proposal_size, o.policy.transition_proposal, o.policy.stochastic_acceptance,
                  o.policy.diversity_multiplier, o.policy.pls_transition_coarsening,
                  o.policy.pls_fragmentation_penalty, o.policy.reject_single_class,
                  q.result->knn_idx != nullptr && q.result->knn_dist != nullptr ? q.result->knn_cap : -1,
                  q.result->run_hashes != nullptr, q.result->cycle_diag != nullptr);
    k += buf;
  }
  return k;
}

// Relative device cost of a problem, for dealing the longest first: the
// graph (n^2 d), the k-means and the evolution (M T L per cycle, with PLS
// heavier by its per-cycle fits over d features).
double batch_cost(const kgb_matrix_problem& q) {
  const double n = q.n, d = q.d, M = q.options.runs, T = q.options.cycles + 1;
  const double L = matrix_sizes(q.n, &q.options).landmarks;
  const double graph = n * n * d * 1e-9;
  const double evolve = q.options.classifier == 1 ? M * T * L * (d + 20.0) * 2e-9 : M * T * L * 4e-9;
  return graph + evolve + M * L * d * 1e-8;
}

std::unique_ptr<BatchGraph> build_batch(const kgb_matrix_problem* probs, int count, int device, int lanes,
                                        int order, const std::string& key) {
  auto g = std::make_unique<BatchGraph>();
  g->key = key;
  g->device = device;
  g->lanes = lanes;
  g->order = order;
  ck(cudaSetDevice(device), "cudaSetDevice");
  ck(cudaStreamCreateWithFlags(&g->root, cudaStreamNonBlocking), "cudaStreamCreate");
  for (int l = 0; l < 2 * lanes; ++l) {
    cudaStream_t st;
    ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    g->streams.push_back(st);
  }
  size_t xf = 0;
  for (int i = 0; i < count; ++i) {
    auto bp = std::make_unique<BatchProblem>();
    bp->x_off = xf;
    xf += static_cast<size_t>(probs[i].n) * probs[i].d;
    bp->cost = batch_cost(probs[i]);
    ck(cudaMalloc(&bp->d_res, sizeof(int) * static_cast<size_t>(probs[i].options.runs) * probs[i].n), "cudaMalloc");
    bp->shadow = *probs[i].result;
    bp->shadow.res = bp->d_res;
    bp->shadow.res_on_device = 1;
    g->problems.push_back(std::move(bp));
  }
  ck(cudaMalloc(&g->d_x, sizeof(float) * std::max<size_t>(xf, 1)), "cudaMalloc");
  // deal the problems to the lanes: longest first to the least loaded lane,
  // or in the given order round robin
  std::vector<int> idx(static_cast<size_t>(count));
  std::iota(idx.begin(), idx.end(), 0);
  std::vector<std::vector<int>> lane_of(static_cast<size_t>(lanes));
  if (order == 1) {
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return g->problems[a]->cost > g->problems[b]->cost; });
    std::vector<double> load(static_cast<size_t>(lanes), 0.0);
    for (int i : idx) {
      const int l = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
      lane_of[l].push_back(i);
      load[l] += g->problems[i]->cost;
    }
  } else {
    for (int i : idx) lane_of[i % lanes].push_back(i);
  }
  std::vector<std::unique_ptr<Ctx>> ctxs;
  std::vector<cudaEvent_t> evs;
  auto event = [&]() {
    cudaEvent_t e;
    ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    evs.push_back(e);
    return e;
  };
  ck(cudaStreamBeginCapture(g->root, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture");
  try {
    const cudaEvent_t e0 = event();
    ck(cudaEventRecord(e0, g->root), "cudaEventRecord");
    for (int l = 0; l < lanes; ++l) {
      cudaStream_t mainst = g->streams[2 * l], sidest = g->streams[2 * l + 1];
      ck(cudaStreamWaitEvent(mainst, e0, 0), "cudaStreamWaitEvent");
      ck(cudaStreamWaitEvent(sidest, e0, 0), "cudaStreamWaitEvent");
      for (int i : lane_of[l]) {
        const kgb_matrix_problem& q = probs[i];
        BatchProblem& bp = *g->problems[i];
        ctxs.push_back(std::make_unique<Ctx>(device, mainst, sidest, &g->arena));
        Ctx& ctx = *ctxs.back();
        const MatrixSizes sz = matrix_sizes(q.n, &q.options);
        const int K = sz.neighbors, landmarks = sz.landmarks;
        const int M = q.options.runs, F = q.options.folds;
        const int first_run = q.options.first_run > 0 ? q.options.first_run : 1;
        const uint64_t seed = q.options.seed;
        const bool pls_classifier = q.options.classifier == 1;
        std::future<FoldWork> folds = std::async(std::launch::deferred, [=]() {
          return plan_fold_work(M, landmarks, F, seed, first_run, 1, pls_classifier);
        });
        const float* d_x = g->d_x + bp.x_off;
        const int ev_start = ctx.mark();
        int* d_gidx = ctx.alloc<int>(static_cast<size_t>(q.n) * K);
        float* d_gdist = ctx.alloc<float>(static_cast<size_t>(q.n) * K);
        kgb_matrix_options o = q.options;
        o.device = device;
        Clock clk;
        matrix_from_device_graph(ctx, d_x, q.n, q.d, d_gidx, d_gdist, K, &o, &bp.shadow, clk, ev_start, -1, folds,
                                 bp.tail, [&]() {
                                   matrix_graph(ctx, d_x, q.n, q.d, K, o.metric, d_gidx, d_gdist);
                                 });
        ctx.release();
      }
      const cudaEvent_t done = event();
      ck(cudaEventRecord(done, mainst), "cudaEventRecord");
      ck(cudaStreamWaitEvent(g->root, done, 0), "cudaStreamWaitEvent");
    }
    ck(cudaStreamEndCapture(g->root, &g->graph), "cudaStreamEndCapture");
  } catch (...) {
    cudaGraph_t broken = nullptr;
    cudaStreamEndCapture(g->root, &broken);
    if (broken) cudaGraphDestroy(broken);
    cudaGetLastError();
    ctxs.clear();
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
    throw;
  }
  ctxs.clear();
  for (cudaEvent_t e : evs) cudaEventDestroy(e);
  ck(cudaGraphInstantiate(&g->exec, g->graph, 0), "cudaGraphInstantiate");
  size_t nn = 0;
  ck(cudaGraphGetNodes(g->graph, nullptr, &nn), "cudaGraphGetNodes");
  std::vector<cudaGraphNode_t> nodes(nn);
  if (nn) ck(cudaGraphGetNodes(g->graph, nodes.data(), &nn), "cudaGraphGetNodes");
  g->nodes = nn;
  for (cudaGraphNode_t nd : nodes) {
    cudaGraphNodeType ty;
    if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) ++g->kernel_nodes;
  }
  return g;
}

// One replay: data in, graph, label matrices out; returns the graph's device
// time in ms.
double run_batch(BatchGraph& g, const kgb_matrix_problem* probs, int count) {
  ck(cudaSetDevice(g.device), "cudaSetDevice");
  cudaEvent_t e0, e1;
  ck(cudaEventCreate(&e0), "cudaEventCreate");
  ck(cudaEventCreate(&e1), "cudaEventCreate");
  for (int i = 0; i < count; ++i)
    ck(cudaMemcpyAsync(g.d_x + g.problems[i]->x_off, probs[i].x, sizeof(float) * static_cast<size_t>(probs[i].n) * probs[i].d,
                       cudaMemcpyHostToDevice, g.root),
       "H2D");
  ck(cudaEventRecord(e0, g.root), "cudaEventRecord");
  ck(cudaGraphLaunch(g.exec, g.root), "cudaGraphLaunch");
  ck(cudaEventRecord(e1, g.root), "cudaEventRecord");
  for (int i = 0; i < count; ++i)
    ck(cudaMemcpyAsync(probs[i].result->res, g.problems[i]->d_res,
                       sizeof(int) * static_cast<size_t>(probs[i].options.runs) * probs[i].n, cudaMemcpyDeviceToHost,
                       g.root),
       "D2H");
  const cudaError_t e = cudaStreamSynchronize(g.root);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ck(e, "batch graph");
  g.arena.deliver();
  return static_cast<double>(ms);
}

void batch_entry(const kgb_matrix_problem* probs, int count, const kgb_batch_options* bo, kgb_batch_report* rep) {
  if (probs == nullptr || count < 1) fail(KGB_EINVAL, "a batch needs at least one problem");
  for (int i = 0; i < count; ++i) check_batch_problem(probs[i]);
  const int device = bo != nullptr ? bo->device : 0;
  int devcount = 0;
  if (cudaGetDeviceCount(&devcount) != cudaSuccess || devcount <= 0) fail(KGB_ECUDA, "no CUDA device is available");
  if (device < 0 || device >= devcount) fail(KGB_EINVAL, "CUDA device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_batch_mu);
  const std::string key = batch_key(probs, count, device);
  Clock clk;
  double tune_ms = 0.0;
  bool rebuilt = false;
  int lanes = bo != nullptr ? bo->lanes : 0, order = bo != nullptr ? bo->order : 0;
  if (lanes < 0 || lanes > 64) fail(KGB_EINVAL, "lanes must lie in [0, 64]");
  if (order < 0 || order > 2) fail(KGB_EINVAL, "order must be 0, 1 or 2");
  if (lanes == 0 || order == 0) {
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      if (lanes == 0) lanes = it->second.first;
      if (order == 0) order = it->second.second;
    } else {
      // autotune on a sample of at most 64 problems spread over the cost
      // range: the lane count first (longest-first dealing), then the order
      // at that lane count; each candidate graph is captured and timed once
      std::vector<int> byc(static_cast<size_t>(count));
      std::iota(byc.begin(), byc.end(), 0);
      std::stable_sort(byc.begin(), byc.end(),
                       [&](int a, int b) { return batch_cost(probs[a]) > batch_cost(probs[b]); });
      const int ns = std::min(count, 64);
      std::vector<kgb_matrix_problem> sample;
      for (int i = 0; i < ns; ++i) sample.push_back(probs[byc[static_cast<size_t>(i) * count / ns]]);
      const std::string skey = "tune:" + batch_key(sample.data(), ns, device);
      auto time_schedule = [&](int cl, int co) {
        g_batch.reset();
        g_batch = build_batch(sample.data(), ns, device, cl, co, skey);
        return run_batch(*g_batch, sample.data(), ns);
      };
      double best = 0.0;
      int bl = 0, bo2 = order != 0 ? order : 1;
      for (int cl : {4, 8, 16, 32}) {
        if (lanes != 0 && cl != lanes) continue;
        if (lanes == 0 && cl > ns && cl != 4) continue;
        const double ms = time_schedule(cl, bo2);
        if (bl == 0 || ms < best) {
          best = ms;
          bl = cl;
        }
      }
      if (order == 0) {
        const double ms = time_schedule(bl, 2);
        if (ms < best) bo2 = 2;
      }
      g_batch.reset();
      g_tuned[key] = {bl, bo2};
      lanes = bl;
      order = bo2;
      tune_ms = clk.lap() * 1000.0;
      rebuilt = true;
    }
  }
  if (!g_batch || g_batch->key != key || g_batch->lanes != lanes || g_batch->order != order) {
    g_batch.reset();
    g_batch = build_batch(probs, count, device, lanes, order, key);
    rebuilt = true;
  }
  const double dev_ms = run_batch(*g_batch, probs, count);
  for (int i = 0; i < count; ++i) {
    kgb_matrix_result* out = probs[i].result;
    for (double& t : out->timings) t = 0.0;
    for (double& t : out->kernel_ms) t = 0.0;
    Clock fclk;
    matrix_finalize(nullptr, g_batch->problems[i]->tail, out, fclk);
  }
  if (rep != nullptr) {
    rep->lanes = lanes;
    rep->order = order;
    rep->graph_nodes = static_cast<int32_t>(g_batch->nodes);
    rep->kernel_nodes = static_cast<int32_t>(g_batch->kernel_nodes);
    rep->rebuilt = rebuilt ? 1 : 0;
    rep->device_ms = dev_ms;
    rep->tune_ms = tune_ms;
  }
}

void matrix_entry(const float* x, bool x_on_device, int n, int d, const int32_t* gidx, const float* gdist, int gk,
                  int index_base, const kgb_matrix_options* opt, kgb_matrix_result* out) {
  if (x == nullptr || out == nullptr) fail(KGB_EINVAL, "null pointer");
  if (n < 3) fail(KGB_EINVAL, "KODAMAMatrix requires at least 3 rows.");
  if (d < 1) fail(KGB_EINVAL, "Input matrix must have at least one column.");
  validate_matrix_options(opt);
  if (out->res == nullptr || out->acc == nullptr || out->v == nullptr) fail(KGB_EINVAL, "null result buffer");
  Clock total, clk;
  for (double& t : out->timings) t = 0.0;
  for (double& t : out->kernel_ms) t = 0.0;
  Ctx ctx(opt->device);
  int landmarks = opt->landmarks > 0 ? opt->landmarks : 10000;
  if (landmarks >= n) landmarks = static_cast<int>(std::ceil(static_cast<double>(n) * 0.75));
  landmarks = std::max(2, std::min(landmarks, n - 1));
  const int requested = opt->graph_neighbors > 0 ? opt->graph_neighbors : 100;
  const int neighbors = std::max(1, static_cast<int>(std::floor(std::min(
      {static_cast<double>(landmarks), static_cast<double>(n) * 0.75 - 1.0, static_cast<double>(requested)}))));
  // fold planning depends only on (seed, run, L): start it on host threads now
  const int M = opt->runs, F = opt->folds, nthreads = host_threads(opt->host_threads);
  const int first_run = opt->first_run > 0 ? opt->first_run : 1;
  const uint64_t seed = opt->seed;
  const bool pls_classifier = opt->classifier == 1;
  std::future<FoldWork> folds_future = std::async(std::launch::async, [=]() {
    return plan_fold_work(M, landmarks, F, seed, first_run, nthreads, pls_classifier);
  });
  const int ev_start = ctx.mark();
  const float* d_x = x_on_device ? x : ctx.upload(x, static_cast<size_t>(n) * d);
  int K;
  int* d_gidx;
  float* d_gdist;
  if (gidx != nullptr) {
    K = std::max(1, std::min(gk, neighbors));
    const int* d_in_idx = ctx.upload(gidx, static_cast<size_t>(n) * gk);
    const float* d_in_dist = ctx.upload(gdist, static_cast<size_t>(n) * gk);
    int* d_mm = ctx.alloc<int>(2);
    ck_launch(kgb::graph_minmax(d_in_idx, static_cast<size_t>(n) * gk, d_mm, ctx.stream()), "graph min/max");
    d_gidx = ctx.alloc<int>(static_cast<size_t>(n) * K);
    d_gdist = ctx.alloc<float>(static_cast<size_t>(n) * K);
    ck_launch(kgb::normalize_external(d_in_idx, d_in_dist, n, gk, K, index_base, d_mm, d_gidx, d_gdist,
                                      ctx.stream()), "graph normalisation");
  } else {
    // raw data: the graph is queued after the atlas k-means (see
    // matrix_from_device_graph), beside the landmark planning
    K = neighbors;
    d_gidx = ctx.alloc<int>(static_cast<size_t>(n) * K);
    d_gdist = ctx.alloc<float>(static_cast<size_t>(n) * K);
    out->timings[1] = clk.lap();
    MatrixTail tail;
    matrix_from_device_graph(ctx, d_x, n, d, d_gidx, d_gdist, K, opt, out, clk, ev_start, -1, folds_future, tail,
                             [&]() { matrix_graph(ctx, d_x, n, d, K, opt->metric, d_gidx, d_gdist); });
    ctx.sync();
    matrix_finalize(&ctx, tail, out, clk);
    out->timings[0] = total.lap();
    return;
  }
  const int ev_graph = ctx.mark();
  ctx.sync();
  out->timings[1] = clk.lap();
  MatrixTail tail;
  matrix_from_device_graph(ctx, d_x, n, d, d_gidx, d_gdist, K, opt, out, clk, ev_start, ev_graph, folds_future,
                           tail);
  ctx.sync();
  matrix_finalize(&ctx, tail, out, clk);
  out->timings[0] = total.lap();
}

// Label evolution of `problems` problems over the same `samples` rows
// (maximize_core, core.cpp:1269-1549, with predict_precomputed_knn): folds
// from each problem's labels (make_folds, common.cpp:108-214), groups from
// `constrain` (ascending values, members in row order; nullptr = singletons)
// and `fixed` flags shared by all problems, vote tables of width w filled by
// tables(folds, d_folds, d_nb, d_sc), all problems in one persistent launch.
template <class Tables>
void core_knn_run(Ctx& ctx, int samples, int problems, const int32_t* labels, const uint64_t* seeds,
                  const uint64_t* cv_seeds, const int32_t* constrain, const int32_t* fixed,
                  const kgb_core_options* opt, int w, kgb_core_result* out, Tables&& tables) {
  if (samples > 65535) fail(KGB_EINVAL, "at most 65535 samples per problem are supported");
  if (problems < 1) fail(KGB_EINVAL, "problems must be positive");
  if (opt->cycles < 0) fail(KGB_EINVAL, "Core cycles must be non-negative.");
  check_metric(opt->metric);
  if (opt->k < 1) fail(KGB_EINVAL, "KNNOptions::k must be positive.");
  if (opt->folds < 2) fail(KGB_EINVAL, "Number of folds must be at least 2.");
  if (opt->folds > 255) fail(KGB_EINVAL, "at most 255 folds are supported");
  if (w > 32) fail(KGB_EINVAL, "knn.k above 32 is not supported by the vote kernel");
  const kgb_policy pol = policy_is_zero(opt->policy) ? default_policy() : opt->policy;
  cudaStream_t st = ctx.stream();
  std::vector<int> goff, gmem;
  if (constrain == nullptr) {
    goff.reserve(static_cast<size_t>(samples) + 1);
    for (int i = 0; i <= samples; ++i) goff.push_back(i);
    for (int i = 0; i < samples; ++i) gmem.push_back(i);
  } else {
    std::map<int, std::vector<int>> members;
    for (int i = 0; i < samples; ++i) members[constrain[i]].push_back(i);
    goff.push_back(0);
    for (const auto& kv : members) {
      gmem.insert(gmem.end(), kv.second.begin(), kv.second.end());
      goff.push_back(static_cast<int>(gmem.size()));
    }
  }
  const std::vector<int> con = constrain ? std::vector<int>(constrain, constrain + samples) : std::vector<int>();
  const uint64_t bc = kgb::unordered_bucket_count(static_cast<size_t>(samples));
  std::vector<Coding> codings(static_cast<size_t>(problems));
  std::vector<std::vector<int>> folds(static_cast<size_t>(problems));
  parallel_for(problems, host_threads(0), [&](int p) {
    const int* lab = labels + static_cast<size_t>(p) * samples;
    codings[p] = code_labels(lab, samples, bc);
    folds[p] = kgb::make_folds(std::vector<int>(lab, lab + samples), con, opt->folds, opt->stratified != 0,
                               cv_seeds[p]);
  });
  int C0max = opt->folds;
  for (const auto& c : codings) C0max = std::max<int>(C0max, static_cast<int>(c.code2label.size()));
  std::vector<uint16_t> codes(static_cast<size_t>(problems) * samples);
  std::vector<int> c2l(static_cast<size_t>(problems) * C0max, 0), ncodes(static_cast<size_t>(problems));
  std::vector<uint8_t> nocol(static_cast<size_t>(problems)), fo8(static_cast<size_t>(problems) * samples);
  for (int p = 0; p < problems; ++p) {
    std::copy(codings[p].codes.begin(), codings[p].codes.end(), codes.begin() + static_cast<size_t>(p) * samples);
    std::copy(codings[p].code2label.begin(), codings[p].code2label.end(), c2l.begin() + static_cast<size_t>(p) * C0max);
    ncodes[p] = static_cast<int>(codings[p].code2label.size());
    nocol[p] = codings[p].nocollide ? 1 : 0;
    for (int i = 0; i < samples; ++i) fo8[static_cast<size_t>(p) * samples + i] = static_cast<uint8_t>(folds[p][i]);
  }
  uint8_t* d_folds = ctx.upload(fo8.data(), fo8.size());
  uint16_t* d_nb = ctx.alloc<uint16_t>(static_cast<size_t>(problems) * samples * w);
  float* d_sc = ctx.alloc<float>(static_cast<size_t>(problems) * samples * w);
  tables(folds, d_folds, d_nb, d_sc);
  kgb::EvolveParams P{};
  P.problems = problems;
  P.L = samples;
  P.w = w;
  P.T = opt->cycles;
  P.F = opt->folds;
  P.G = static_cast<int>(goff.size()) - 1;
  P.singleton = constrain == nullptr;
  P.evolutionary = opt->evolutionary_search != 0;
  P.guarded = opt->guarded_diversity != 0;
  P.absorption = opt->many_to_one_absorption != 0;
  P.adaptive = opt->adaptive_proposal_size != 0;
  P.pol_guidance = pol.prediction_guidance != 0;
  P.pol_adaptive = pol.adaptive_proposal_size != 0;
  P.pol_transition = pol.transition_proposal != 0;
  P.pol_stochastic = pol.stochastic_acceptance != 0;
  P.pol_diversity = pol.diversity_multiplier != 0;
  P.pol_reject1 = pol.reject_single_class != 0;
  P.bucket_count = bc;
  P.nb = d_nb;
  P.sc = d_sc;
  P.init = ctx.upload(codes.data(), codes.size());
  P.code2label = ctx.upload(c2l.data(), c2l.size());
  P.ncodes = ctx.upload(ncodes.data(), ncodes.size());
  P.nocollide = ctx.upload(nocol.data(), nocol.size());
  P.folds = d_folds;
  P.fixed = fixed != nullptr ? ctx.upload(fixed, static_cast<size_t>(samples)) : nullptr;
  P.goff = ctx.upload(goff.data(), goff.size());
  P.gmem = ctx.upload(gmem.data(), gmem.size());
  P.seeds = ctx.upload(seeds, static_cast<size_t>(problems));
  const EvolveBuffers eb = run_evolution(ctx, P, C0max);
  const int T = opt->cycles;
  std::vector<uint16_t> hb(static_cast<size_t>(problems) * samples), hp(hb.size());
  std::vector<double> best(static_cast<size_t>(problems) * 2);
  std::vector<int> counters(static_cast<size_t>(problems) * 16);
  ctx.download(hb.data(), eb.clbest, hb.size());
  ctx.download(hp.data(), eb.cvpredbest, hp.size());
  ctx.download(best.data(), eb.best, best.size());
  ctx.download(counters.data(), eb.counters, counters.size());
  std::vector<double> va(static_cast<size_t>(problems) * T), vs(va.size());
  std::vector<int> ps(va.size()), ac(va.size());
  std::vector<uint8_t> fl(va.size() * 3);
  ctx.download(va.data(), eb.vect_acc, va.size());
  ctx.download(vs.data(), eb.vect_score, vs.size());
  ctx.download(ps.data(), eb.psize, ps.size());
  ctx.download(ac.data(), eb.active, ac.size());
  ctx.download(fl.data(), eb.flags, fl.size());
  ctx.sync();
  for (int p = 0; p < problems; ++p) {
    kgb_core_result& r = out[p];
    const int* map = c2l.data() + static_cast<size_t>(p) * C0max;
    for (int i = 0; i < samples; ++i) {
      const size_t o1 = static_cast<size_t>(p) * samples + i;
      if (r.clbest) r.clbest[i] = map[hb[o1]];
      if (r.cvpredbest) r.cvpredbest[i] = map[hp[o1]];
      if (r.fold_assignments) r.fold_assignments[i] = folds[p][i];
    }
    for (int c = 0; c < T; ++c) {
      const size_t o1 = static_cast<size_t>(p) * T + c;
      if (r.vect_acc) r.vect_acc[c] = va[o1];
      if (r.vect_score) r.vect_score[c] = vs[o1];
      if (r.proposal_size) r.proposal_size[c] = ps[o1];
      if (r.active_classes) r.active_classes[c] = ac[o1];
      if (r.flags) {
        r.flags[3 * c] = fl[3 * o1];
        r.flags[3 * c + 1] = fl[3 * o1 + 1];
        r.flags[3 * c + 2] = fl[3 * o1 + 2];
      }
    }
    r.accbest = best[2 * p];
    r.scorebest = best[2 * p + 1];
    std::memset(r.counters, 0, sizeof(r.counters));
    std::memcpy(r.counters, counters.data() + static_cast<size_t>(p) * 16, sizeof(int) * 16);
  }
}

// CoreKNNGraph over one graph for `problems` label vectors: the graph's
// fold-filtered neighbours as vote tables (precompute_knn_cv_graph,
// core.cpp:624-688).
void core_graph_problems(const int32_t* gidx, const float* gdist, int samples, int gk, int index_base, int problems,
                         const int32_t* labels, const uint64_t* seeds, const uint64_t* cv_seeds,
                         const int32_t* constrain, const int32_t* fixed, const kgb_core_options* opt,
                         kgb_core_result* out) {
  Ctx ctx(opt->device);
  cudaStream_t st = ctx.stream();
  const size_t total = static_cast<size_t>(samples) * gk;
  const int* d_in_idx = ctx.upload(gidx, total);
  const float* d_in_dist = ctx.upload(gdist, total);
  int* d_mm = ctx.alloc<int>(2);
  ck_launch(kgb::graph_minmax(d_in_idx, total, d_mm, st), "graph min/max");
  int* d_gidx = ctx.alloc<int>(total);
  float* d_gdist = ctx.alloc<float>(total);
  ck_launch(kgb::normalize_indices(d_in_idx, d_in_dist, total, samples, index_base, d_mm, d_gidx, d_gdist, st),
            "graph normalisation");
  const int w = std::max(1, std::min(opt->k, gk));
  core_knn_run(ctx, samples, problems, labels, seeds, cv_seeds, constrain, fixed, opt, w, out,
               [&](const std::vector<std::vector<int>>&, uint8_t* d_folds, uint16_t* d_nb, float* d_sc) {
                 kgb::VoteTableArgs a{};
                 a.problems = problems;
                 a.L = samples;
                 a.n = samples;
                 a.K = gk;
                 a.w = w;
                 a.gidx = d_gidx;
                 a.gdist = d_gdist;
                 a.land = nullptr;
                 a.g2l = nullptr;
                 a.folds = d_folds;
                 a.nb = d_nb;
                 a.sc = d_sc;
                 a.score_one_minus = opt->metric != KGB_METRIC_EUCLIDEAN;
                 ck_launch(kgb::build_vote_tables(a, st), "vote tables");
               });
}

// Every fold keeps training rows (knncv.cpp:142, core.cpp:705; a
// std::runtime_error there).
void check_training_rows(const std::vector<int>& folds) {
  std::map<int, int> size;
  for (int f : folds) size[f]++;
  for (const auto& kv : size)
    if (kv.second == static_cast<int>(folds.size())) fail(KGB_EINTERNAL, "KNN fold has no training samples.");
}

// The search matrix of a metric on the device: cosine rows normalised
// (mode 0 = knncv.cpp:85-108, 1 = core.cpp:166-195), else x itself.
const float* search_matrix(Ctx& ctx, const float* d_x, int n, int d, int metric, int mode) {
  if (metric != KGB_METRIC_COSINE) return d_x;
  float* xs = ctx.alloc<float>(static_cast<size_t>(n) * d);
  ck_launch(kgb::normalize_rows(d_x, n, d, mode, xs, ctx.stream()), "search matrix");
  return xs;
}


}  // namespace

namespace kgb {
// Lets entry points defined in other translation units report a message
// through kgb_last_error().
void set_last_error(const char* msg) { g_error = msg; }
}  // namespace kgb

// Resident data and exact kNN graph of KODAMAGraph (see kgb_graph_create).
struct kgb_graph_handle {
  std::mutex mu;
  int device = 0, n = 0, d = 0, K = 0, metric = KGB_METRIC_EUCLIDEAN;
  float* d_x = nullptr;
  int* d_idx = nullptr;
  float* d_dist = nullptr;
  ~kgb_graph_handle() {
    if (d_x) cudaFree(d_x);
    if (d_idx) cudaFree(d_idx);
    if (d_dist) cudaFree(d_dist);
  }
};

extern "C" {

int kgb_last_error(char* buf, size_t len) {
  if (buf != nullptr && len > 0) {
    std::strncpy(buf, g_error.c_str(), len - 1);
    buf[len - 1] = '\0';
  }
  return static_cast<int>(g_error.size());
}

const char* kgb_version(void) { return "kodama_gb300 0.1 (sm_103a)"; }

int kgb_kodama_matrix_from_graph_data(const float* x, int32_t n, int32_t d, const int32_t* gidx,
                                      const float* gdist, int32_t gk, int32_t index_base,
                                      const kgb_matrix_options* opt, kgb_matrix_result* out) {
  return guarded([&]() {
    if (gidx == nullptr || gdist == nullptr) fail(KGB_EINVAL, "null graph pointer");
    if (gk <= 0) fail(KGB_EINVAL, "NeighborGraph.neighbors must be positive.");
    matrix_entry(x, false, n, d, gidx, gdist, gk, index_base, opt, out);
  });
}

int kgb_kodama_matrix(const float* x, int32_t n, int32_t d, const kgb_matrix_options* opt, kgb_matrix_result* out) {
  return guarded([&]() { matrix_entry(x, false, n, d, nullptr, nullptr, 0, -1, opt, out); });
}

int kgb_kodama_matrix_resident(const float* x_device, int32_t n, int32_t d, const kgb_matrix_options* opt,
                               kgb_matrix_result* out) {
  return guarded([&]() { matrix_entry(x_device, true, n, d, nullptr, nullptr, 0, -1, opt, out); });
}

int kgb_kodama_matrix_batch(const kgb_matrix_problem* problems, int32_t count, const kgb_batch_options* options,
                            kgb_batch_report* report) {
  return guarded([&]() { batch_entry(problems, count, options, report); });
}

int kgb_graph_create(const float* x, int32_t n, int32_t d, int32_t neighbors, int32_t metric, int32_t device,
                     kgb_graph_handle** out) {
  return guarded([&]() {
    if (x == nullptr || out == nullptr) fail(KGB_EINVAL, "null pointer");
    *out = nullptr;
    check_metric(metric);
    if (n < 3) fail(KGB_EINVAL, "KODAMAGraph requires at least 3 rows.");
    if (d < 1) fail(KGB_EINVAL, "Input matrix must have at least one column.");
    if (neighbors < 1) fail(KGB_EINVAL, "KODAMAGraphOptions::neighbors must be positive.");
    auto g = std::make_unique<kgb_graph_handle>();
    g->device = device;
    g->n = n;
    g->d = d;
    g->K = std::min(neighbors, n - 1);
    g->metric = metric;
    Ctx ctx(device);
    ck(cudaMalloc(&g->d_x, sizeof(float) * static_cast<size_t>(n) * d), "cudaMalloc");
    ck(cudaMalloc(&g->d_idx, sizeof(int) * static_cast<size_t>(n) * g->K), "cudaMalloc");
    ck(cudaMalloc(&g->d_dist, sizeof(float) * static_cast<size_t>(n) * g->K), "cudaMalloc");
    ctx.h2d(g->d_x, x, static_cast<size_t>(n) * d);
    exact_graph(ctx, g->d_x, n, d, g->K, KGB_KNN_AUTO, metric, g->d_idx, g->d_dist, nullptr);
    ctx.sync();
    *out = g.release();
  });
}

int kgb_graph_info(const kgb_graph_handle* g, int32_t* n, int32_t* d, int32_t* neighbors) {
  return guarded([&]() {
    if (g == nullptr) fail(KGB_EINVAL, "null handle");
    if (n) *n = g->n;
    if (d) *d = g->d;
    if (neighbors) *neighbors = g->K;
  });
}

int kgb_graph_materialize(kgb_graph_handle* g, int32_t* idx, float* dist) {
  return guarded([&]() {
    if (g == nullptr || idx == nullptr || dist == nullptr) fail(KGB_EINVAL, "null pointer");
    std::lock_guard<std::mutex> lock(g->mu);
    Ctx ctx(g->device);
    const size_t total = static_cast<size_t>(g->n) * g->K;
    ctx.download(idx, g->d_idx, total);
    ctx.download(dist, g->d_dist, total);
    ctx.sync();
    for (size_t i = 0; i < total; ++i)
      if (idx[i] >= 0) idx[i] += 1;  // one-based, as NeighborGraph leaves KODAMAGraph
  });
}

int kgb_kodama_matrix_graph(kgb_graph_handle* g, const kgb_matrix_options* opt, kgb_matrix_result* out) {
  return guarded([&]() {
    if (g == nullptr || out == nullptr) fail(KGB_EINVAL, "null pointer");
    validate_matrix_options(opt);
    if (out->res == nullptr || out->acc == nullptr || out->v == nullptr) fail(KGB_EINVAL, "null result buffer");
    std::lock_guard<std::mutex> lock(g->mu);
    Clock total, clk;
    for (double& t : out->timings) t = 0.0;
    for (double& t : out->kernel_ms) t = 0.0;
    const int n = g->n, d = g->d;
    kgb_matrix_options o = *opt;
    o.device = g->device;
    Ctx ctx(g->device);
    const MatrixSizes sz = matrix_sizes(n, &o);
    const int K = std::max(1, std::min(g->K, sz.neighbors));
    const int M = o.runs, F = o.folds, nthreads = host_threads(o.host_threads);
    const int first_run = o.first_run > 0 ? o.first_run : 1;
    const uint64_t seed = o.seed;
    const int landmarks = sz.landmarks;
    const bool pls_classifier = o.classifier == 1;
    std::future<FoldWork> folds_future = std::async(std::launch::async, [=]() {
      return plan_fold_work(M, landmarks, F, seed, first_run, nthreads, pls_classifier);
    });
    const int ev_start = ctx.mark();
    int* d_gidx = g->d_idx;
    float* d_gdist = g->d_dist;
    if (K < g->K || g->metric != KGB_METRIC_EUCLIDEAN) {
      // the first K columns, as normalize_external_graph trims a wider graph
      // (and clamps at zero the distances 1 - <x,y> of a non-Euclidean graph)
      int* d_mm = ctx.alloc<int>(2);
      ck_launch(kgb::graph_minmax(g->d_idx, static_cast<size_t>(n) * g->K, d_mm, ctx.stream()), "graph min/max");
      d_gidx = ctx.alloc<int>(static_cast<size_t>(n) * K);
      d_gdist = ctx.alloc<float>(static_cast<size_t>(n) * K);
      ck_launch(kgb::normalize_external(g->d_idx, g->d_dist, n, g->K, K, 0, d_mm, d_gidx, d_gdist, ctx.stream()),
                "graph normalisation");
    }
    const int ev_graph = ctx.mark();
    out->timings[1] = clk.lap();
    MatrixTail tail;
    matrix_from_device_graph(ctx, g->d_x, n, d, d_gidx, d_gdist, K, &o, out, clk, ev_start, ev_graph, folds_future,
                             tail);
    ctx.sync();
    matrix_finalize(&ctx, tail, out, clk);
    out->timings[0] = total.lap();
  });
}

void kgb_graph_destroy(kgb_graph_handle* g) {
  if (g == nullptr) return;
  {
    std::lock_guard<std::mutex> lock(g->mu);
    cudaSetDevice(g->device);
  }
  delete g;
}

int64_t kgb_launch_count(void) { return kgb::g_launches_value(); }

int kgb_core_knn_graph_batch(const int32_t* gidx, const float* gdist, int32_t samples, int32_t gk,
                             int32_t index_base, int32_t problems, const int32_t* labels,
                             const uint64_t* seeds, const uint64_t* cv_seeds, const kgb_core_options* opt,
                             kgb_core_result* out) {
  return guarded([&]() {
    if (gidx == nullptr || gdist == nullptr || labels == nullptr || seeds == nullptr || cv_seeds == nullptr ||
        opt == nullptr || out == nullptr) {
      fail(KGB_EINVAL, "null pointer");
    }
    if (samples < 2) fail(KGB_EINVAL, "CoreKNNGraph requires at least two samples.");
    if (gk <= 0) fail(KGB_EINVAL, "NeighborGraph.neighbors must be positive.");
    core_graph_problems(gidx, gdist, samples, gk, index_base, problems, labels, seeds, cv_seeds, nullptr, nullptr,
                        opt, out);
  });
}

int kgb_knn_graph(const float* x, int32_t n, int32_t d, int32_t K, int32_t device, int32_t* idx, float* dist) {
  return kgb_knn_graph_ex(x, n, d, K, device, KGB_KNN_AUTO, idx, dist, nullptr);
}

int kgb_knn_graph_ex(const float* x, int32_t n, int32_t d, int32_t K, int32_t device, int32_t method,
                     int32_t* idx, float* dist, int32_t* fallback_rows) {
  return guarded([&]() {
    if (x == nullptr || idx == nullptr || dist == nullptr) fail(KGB_EINVAL, "null pointer");
    if (n < 1 || d < 1 || K < 1) fail(KGB_EINVAL, "invalid kNN graph dimensions");
    if (method != KGB_KNN_AUTO && method != KGB_KNN_BRUTE_FORCE && method != KGB_KNN_TENSOR)
      fail(KGB_EINVAL, "unknown kNN search method");
    Ctx ctx(device);
    const float* d_x = ctx.upload(x, static_cast<size_t>(n) * d);
    int* d_idx = ctx.alloc<int>(static_cast<size_t>(n) * K);
    float* d_dist = ctx.alloc<float>(static_cast<size_t>(n) * K);
    int fb = 0;
    exact_graph(ctx, d_x, n, d, K, method, KGB_METRIC_EUCLIDEAN, d_idx, d_dist, &fb);
    ctx.download(idx, d_idx, static_cast<size_t>(n) * K);
    ctx.download(dist, d_dist, static_cast<size_t>(n) * K);
    ctx.sync();
    if (fallback_rows != nullptr) *fallback_rows = fb;
  });
}

int kgb_knn_graph_metric(const float* x, int32_t n, int32_t d, int32_t K, int32_t metric, int32_t device,
                         int32_t* idx, float* dist) {
  return guarded([&]() {
    if (x == nullptr || idx == nullptr || dist == nullptr) fail(KGB_EINVAL, "null pointer");
    if (n < 1 || d < 1 || K < 1) fail(KGB_EINVAL, "invalid kNN graph dimensions");
    check_metric(metric);
    Ctx ctx(device);
    const float* d_x = ctx.upload(x, static_cast<size_t>(n) * d);
    int* d_idx = ctx.alloc<int>(static_cast<size_t>(n) * K);
    float* d_dist = ctx.alloc<float>(static_cast<size_t>(n) * K);
    exact_graph(ctx, d_x, n, d, K, KGB_KNN_AUTO, metric, d_idx, d_dist, nullptr);
    ctx.download(idx, d_idx, static_cast<size_t>(n) * K);
    ctx.download(dist, d_dist, static_cast<size_t>(n) * K);
    ctx.sync();
  });
}

int kgb_dissimilarity_inplace(int32_t* gidx, float* gdist, int32_t samples, int32_t gk, const int32_t* res,
                              int32_t runs, int32_t device) {
  return guarded([&]() {
    if (gidx == nullptr || gdist == nullptr || res == nullptr) fail(KGB_EINVAL, "null pointer");
    if (runs <= 0 || samples <= 0 || gk <= 0) {
      fail(KGB_EINVAL, "KODAMADissimilarityInPlace requires a non-empty graph and label matrix.");
    }
    const size_t total = static_cast<size_t>(samples) * gk;
    for (size_t i = 0; i < total; ++i) {
      const int v = gidx[i];
      if (v < 0) continue;
      if (v < 1 || v > samples) fail(KGB_EINVAL, "KODAMADissimilarityInPlace expects public one-based graph indices.");
    }
    Ctx ctx(device);
    cudaStream_t st = ctx.stream();
    int* d_idx = ctx.upload(gidx, total);
    float* d_dist = ctx.upload(gdist, total);
    const int* d_res = ctx.upload(res, static_cast<size_t>(runs) * samples);
    int* d_lbs = ctx.alloc<int>(static_cast<size_t>(runs) * samples);
    ck_launch(kgb::transpose_runs(d_res, runs, samples, d_lbs, st), "transpose");
    int* d_oidx = ctx.alloc<int>(total);
    float* d_odist = ctx.alloc<float>(total);
    kgb::DissimArgs a{};
    a.n = samples;
    a.K = gk;
    a.runs = runs;
    a.in_one_based = 1;
    a.out_one_based = 1;
    a.idx = d_idx;
    a.dist = d_dist;
    a.lbs = d_lbs;
    a.out_idx = d_oidx;
    a.out_dist = d_odist;
    ck_launch(kgb::dissimilarity(a, st), "dissimilarity");
    ctx.download(gidx, d_oidx, total);
    ctx.download(gdist, d_odist, total);
    ctx.sync();
  });
}

namespace {
void check_pls_options(const kgb_pls_options* o) {
  if (o->max_components < 1) fail(KGB_EINVAL, "PLSOptions::max_components must be positive.");
  if (o->fixed_components < 0) fail(KGB_EINVAL, "PLSOptions::fixed_components must be non-negative.");
  if (o->fixed_components > o->max_components)
    fail(KGB_EINVAL, "PLSOptions::fixed_components cannot exceed max_components.");
}

int plscv_entry(const float* x, int32_t n, int32_t p, const int32_t* labels, const int32_t* constrain,
                const kgb_pls_options* opt, int32_t* predicted, int32_t* fold_assignments,
                int32_t* selected_components, double* accuracy_by_components, bool da);
}  // namespace

int kgb_plsldacv(const float* x, int32_t n, int32_t p, const int32_t* labels, const int32_t* constrain,
                 const kgb_pls_options* opt, int32_t* predicted, int32_t* fold_assignments,
                 int32_t* selected_components, double* accuracy_by_components) {
  return plscv_entry(x, n, p, labels, constrain, opt, predicted, fold_assignments, selected_components,
                     accuracy_by_components, false);
}

int kgb_plsdacv(const float* x, int32_t n, int32_t p, const int32_t* labels, const int32_t* constrain,
                const kgb_pls_options* opt, int32_t* predicted, int32_t* fold_assignments,
                int32_t* selected_components, double* accuracy_by_components) {
  return plscv_entry(x, n, p, labels, constrain, opt, predicted, fold_assignments, selected_components,
                     accuracy_by_components, true);
}

}  // extern "C"

namespace {
// run_plscv_host (plscv.cpp:2293-2507) for PLSLDACV (da = false) and PLSDACV.
int plscv_entry(const float* x, int32_t n, int32_t p, const int32_t* labels, const int32_t* constrain,
                const kgb_pls_options* opt, int32_t* predicted, int32_t* fold_assignments,
                int32_t* selected_components, double* accuracy_by_components, bool da) {
  return guarded([&]() {
    if (x == nullptr || labels == nullptr || opt == nullptr || predicted == nullptr) fail(KGB_EINVAL, "null pointer");
    if (n < 1 || p < 1) fail(KGB_EINVAL, da ? "PLSDACV requires a non-empty matrix." : "PLSLDACV requires a non-empty matrix.");
    if (n > 65535) fail(KGB_EINVAL, "at most 65535 rows are supported");
    check_pls_options(opt);
    const std::vector<int> lab(labels, labels + n);
    const std::vector<int> con = constrain ? std::vector<int>(constrain, constrain + n) : std::vector<int>();
    const std::vector<int> folds = kgb::make_folds(lab, con, opt->folds, opt->stratified != 0, opt->cv_seed);
    const Coding cd = code_labels(labels, n, 1);
    const int C0max = std::max(2, static_cast<int>(cd.code2label.size()));
    const int requested = opt->fixed_components > 0 ? opt->fixed_components : opt->max_components;
    Ctx ctx(opt->device);
    const float* d_x = ctx.upload(x, static_cast<size_t>(n) * p);
    const PlsSlices sl = pls_slices({folds}, 1, n, false);
    PlsBuffers b = pls_buffers(ctx, d_x, 1, n, p, sl, C0max, opt->max_components, requested, opt->center != 0,
                               opt->scale != 0, nullptr, 0);
    std::vector<int> off;
    std::vector<uint16_t> rows;
    class_lists_host(cd.codes, C0max, off, rows);
    b.ev.labels = ctx.upload(cd.codes.data(), cd.codes.size());
    b.ev.class_off = ctx.upload(off.data(), off.size());
    b.ev.class_rows = ctx.upload(rows.data(), rows.size());
    b.ev.da_mode = da ? 1 : 0;
    ck_launch(kgb::pls_evaluate(b.ev, ctx.stream()), da ? "PLS-DA evaluation" : "PLS-LDA evaluation");
    std::vector<uint16_t> pc(static_cast<size_t>(n));
    std::vector<int> comp(static_cast<size_t>(b.S));
    ctx.download(pc.data(), b.ev.pred, pc.size());
    ctx.download(comp.data(), b.ev.eval_comp, comp.size());
    pls_check_status(ctx, b);
    int evaluated = requested;
    for (int s2 = 0; s2 < b.S; ++s2)
      if (b.present[s2]) evaluated = std::min(evaluated, comp[s2]);
    const int best = std::min(evaluated, opt->max_components);
    int ok = 0;
    for (int i = 0; i < n; ++i) {
      predicted[i] = cd.code2label[pc[i]];
      ok += predicted[i] == labels[i];
    }
    if (fold_assignments) std::copy(folds.begin(), folds.end(), fold_assignments);
    if (selected_components) *selected_components = best;
    if (accuracy_by_components) {
      for (int c = 0; c < opt->max_components; ++c) accuracy_by_components[c] = 0.0;
      accuracy_by_components[best - 1] = static_cast<double>(ok) / static_cast<double>(n);
    }
  });
}

}  // namespace

extern "C" {

int kgb_plslda_predict(const float* train, int32_t n, int32_t p, const int32_t* labels, const float* test,
                       int32_t nt, const kgb_pls_options* opt, int32_t* predicted) {
  return guarded([&]() {
    if (train == nullptr || labels == nullptr || opt == nullptr || (nt > 0 && (test == nullptr || predicted == nullptr)))
      fail(KGB_EINVAL, "PLSLDAPredict input matrix pointer is null.");
    if (n <= 0 || nt <= 0 || p <= 0) return;
    if (n > 65535) fail(KGB_EINVAL, "at most 65535 training rows are supported");
    const Coding cd = code_labels(labels, n, 1);
    if (cd.code2label.size() == 1) {
      for (int i = 0; i < nt; ++i) predicted[i] = cd.code2label[0];
      return;
    }
    const int C0max = static_cast<int>(cd.code2label.size());
    const int requested = opt->fixed_components > 0 ? opt->fixed_components : opt->max_components;
    const int ncomp = std::max(1, std::min({requested, static_cast<int>(p), std::max(1, static_cast<int>(n) - 1)}));
    Ctx ctx(opt->device);
    const float* d_x = ctx.upload(train, static_cast<size_t>(n) * p);
    const float* d_t = ctx.upload(test, static_cast<size_t>(nt) * p);
    const PlsSlices sl = pls_slices({}, 1, n, true);
    PlsBuffers b = pls_buffers(ctx, d_x, 1, n, p, sl, C0max, ncomp, ncomp, opt->center != 0, opt->scale != 0, d_t, nt);
    std::vector<int> off;
    std::vector<uint16_t> rows;
    class_lists_host(cd.codes, C0max, off, rows);
    b.ev.labels = ctx.upload(cd.codes.data(), cd.codes.size());
    b.ev.class_off = ctx.upload(off.data(), off.size());
    b.ev.class_rows = ctx.upload(rows.data(), rows.size());
    ck_launch(kgb::pls_evaluate(b.ev, ctx.stream()), "PLS-LDA evaluation");
    std::vector<uint16_t> pc(static_cast<size_t>(nt));
    ctx.download(pc.data(), b.ev.pred, pc.size());
    pls_check_status(ctx, b);
    for (int i = 0; i < nt; ++i) predicted[i] = cd.code2label[pc[i]];
  });
}

int kgb_core_plslda(const float* x, int32_t n, int32_t p, const int32_t* labels, const int32_t* constrain,
                    const int32_t* fixed, const kgb_core_options* opt, const kgb_pls_options* pls,
                    kgb_core_result* out) {
  return guarded([&]() {
    if (x == nullptr || labels == nullptr || opt == nullptr || pls == nullptr || out == nullptr)
      fail(KGB_EINVAL, "null pointer");
    if (n < 2 || p < 1) fail(KGB_EINVAL, "CorePLSLDA requires at least two rows.");
    if (n > 65535) fail(KGB_EINVAL, "at most 65535 rows are supported");
    if (opt->cycles < 0) fail(KGB_EINVAL, "Core cycles must be non-negative.");
    check_pls_options(pls);
    const bool strat = pls->stratified != 0;
    const kgb_policy pol = policy_is_zero(opt->policy) ? default_policy() : opt->policy;
    const std::vector<int> lab(labels, labels + n);
    const std::vector<int> con = constrain ? std::vector<int>(constrain, constrain + n) : std::vector<int>();
    const std::vector<int> folds = kgb::make_folds(lab, con, pls->folds, strat, pls->cv_seed);
    const uint64_t bc = kgb::unordered_bucket_count(static_cast<size_t>(n));
    const Coding cd = code_labels(labels, n, bc);
    const int C0 = static_cast<int>(cd.code2label.size());
    const int C0max = std::max(2, C0);
    // groups: singletons without a constraint, else ascending constrain values
    std::vector<int> goff, gmem;
    int G = n;
    if (con.empty()) {
      for (int i = 0; i <= n; ++i) goff.push_back(i);
      for (int i = 0; i < n; ++i) gmem.push_back(i);
    } else {
      std::map<int, std::vector<int>> members;
      for (int i = 0; i < n; ++i) members[con[i]].push_back(i);
      goff.push_back(0);
      for (const auto& kv : members) {
        gmem.insert(gmem.end(), kv.second.begin(), kv.second.end());
        goff.push_back(static_cast<int>(gmem.size()));
      }
      G = static_cast<int>(members.size());
    }
    const int requested = pls->fixed_components > 0 ? pls->fixed_components : pls->max_components;
    Ctx ctx(pls->device);
    const float* d_x = ctx.upload(x, static_cast<size_t>(n) * p);
    // stratified folds follow the labels under evaluation (core_pls_lda: each
    // evaluation is a fresh PLSLDACV, core.cpp:1626-1646), so the slices are
    // rebuilt before every evaluation and no fold Gram is kept
    const PlsSlices sl = strat ? pad_slices(pls_slices({folds}, 1, n, false), pls->folds)
                               : pls_slices({folds}, 1, n, false);
    PlsBuffers b = pls_buffers(ctx, d_x, 1, n, p, sl, C0max, pls->max_components, requested, pls->center != 0,
                               pls->scale != 0, nullptr, 0);
    PlsSliceRoom room;
    std::function<void()> refresh;
    if (strat) {
      const int F = sl.F;
      room.train_off = ctx.alloc<int>(static_cast<size_t>(F) + 1);
      room.train_idx = ctx.alloc<int>(static_cast<size_t>(F) * n);
      room.val_off = ctx.alloc<int>(static_cast<size_t>(F) + 1);
      room.val_idx = ctx.alloc<int>(static_cast<size_t>(n));
      room.folds = ctx.alloc<uint8_t>(static_cast<size_t>(n));
      room.logprior = ctx.alloc<float>(static_cast<size_t>(F) * (n + 1));
      room.lp_off = ctx.alloc<int>(static_cast<size_t>(F));
      refresh = [&, F]() {
        std::vector<uint16_t> codes(static_cast<size_t>(n));
        ctx.download(codes.data(), b.ev.labels, codes.size());
        ctx.sync();
        std::vector<int> cur(static_cast<size_t>(n));
        for (int i = 0; i < n; ++i) cur[i] = cd.code2label[codes[i]];
        const std::vector<int> fo = kgb::make_folds(cur, con, pls->folds, true, pls->cv_seed);
        const PlsSlices s2 = pad_slices(pls_slices({fo}, 1, n, false), F);
        if (s2.F != F) fail(KGB_EINTERNAL, "more folds than the stratified slice room holds");
        pls_refresh_slices(ctx, b, room, s2, n);
      };
    }
    std::vector<int> c2l(static_cast<size_t>(C0max), 0);
    std::copy(cd.code2label.begin(), cd.code2label.end(), c2l.begin());
    const int nco = C0;
    const uint8_t nocol = cd.nocollide ? 1 : 0;
    const uint64_t seed = opt->seed;
    kgb::EvolveParams P{};
    P.problems = 1;
    P.L = n;
    P.T = opt->cycles;
    P.F = sl.F;
    P.G = G;
    P.singleton = con.empty() ? 1 : 0;
    P.evolutionary = opt->evolutionary_search != 0;
    P.guarded = opt->guarded_diversity != 0;
    P.absorption = opt->many_to_one_absorption != 0;
    P.adaptive = opt->adaptive_proposal_size != 0;
    P.pol_guidance = pol.prediction_guidance != 0;
    P.pol_adaptive = pol.adaptive_proposal_size != 0;
    P.pol_transition = pol.transition_proposal != 0;
    P.pol_stochastic = pol.stochastic_acceptance != 0;
    P.pol_diversity = pol.diversity_multiplier != 0;
    P.pol_reject1 = pol.reject_single_class != 0;
    P.bucket_count = bc;
    P.init = ctx.upload(cd.codes.data(), cd.codes.size());
    P.code2label = ctx.upload(c2l.data(), c2l.size());
    P.ncodes = ctx.upload(&nco, 1);
    P.nocollide = ctx.upload(&nocol, 1);
    P.folds = b.ev.folds;
    P.fixed = fixed ? ctx.upload(fixed, static_cast<size_t>(n)) : nullptr;
    P.goff = ctx.upload(goff.data(), goff.size());
    P.gmem = ctx.upload(gmem.data(), gmem.size());
    P.seeds = ctx.upload(&seed, 1);
    const EvolveBuffers eb =
        run_pls_evolution(ctx, P, b, C0max, opt->auto_class_coarsening != 0, pol, nullptr, refresh);
    const int T = opt->cycles;
    std::vector<uint16_t> cb(static_cast<size_t>(n)), cp(static_cast<size_t>(n));
    std::vector<double> va(static_cast<size_t>(std::max(T, 1))), vs(va.size()), best(2);
    std::vector<int> ps(va.size()), ac(va.size()), counters(18);
    std::vector<uint8_t> fl(va.size() * 3);
    ctx.download(cb.data(), eb.clbest, cb.size());
    ctx.download(cp.data(), eb.cvpredbest, cp.size());
    ctx.download(va.data(), eb.vect_acc, va.size());
    ctx.download(vs.data(), eb.vect_score, vs.size());
    ctx.download(ps.data(), eb.psize, ps.size());
    ctx.download(ac.data(), eb.active, ac.size());
    ctx.download(fl.data(), eb.flags, fl.size());
    ctx.download(counters.data(), eb.counters, counters.size());
    ctx.download(best.data(), eb.best, best.size());
    ctx.sync();
    for (int i = 0; i < n; ++i) {
      if (out->clbest) out->clbest[i] = cd.code2label[cb[i]];
      if (out->cvpredbest) out->cvpredbest[i] = cd.code2label[cp[i]];
      if (out->fold_assignments) out->fold_assignments[i] = folds[i];
    }
    for (int c = 0; c < T; ++c) {
      if (out->vect_acc) out->vect_acc[c] = va[c];
      if (out->vect_score) out->vect_score[c] = vs[c];
      if (out->proposal_size) out->proposal_size[c] = ps[c];
      if (out->active_classes) out->active_classes[c] = ac[c];
      if (out->flags)
        for (int q = 0; q < 3; ++q) out->flags[3 * c + q] = fl[3 * c + q];
    }
    out->accbest = best[0];
    out->scorebest = best[1];
    for (int q = 0; q < 18; ++q) out->counters[q] = counters[q];
  });
}

int kgb_proposal_train(const float* features, const uint8_t* targets, int32_t n, int32_t epochs, int32_t batch,
                       float learning_rate, uint64_t seed, const float* weights_init, int32_t device,
                       float* weights_out, float* loss_per_epoch) {
  return guarded([&]() {
    if (features == nullptr || targets == nullptr || weights_out == nullptr) fail(KGB_EINVAL, "null pointer");
    if (n < 1 || epochs < 0 || batch < 1) fail(KGB_EINVAL, "invalid training sizes");
    std::vector<float> w(kgb::kMlpParams, 0.0f);
    if (weights_init != nullptr) {
      std::copy(weights_init, weights_init + kgb::kMlpParams, w.begin());
    } else {
      // He-uniform weights, zero biases, from a seeded engine
      std::mt19937_64 rng(seed);
      auto fill = [&](int off, int count, int fan_in) {
        const float a = std::sqrt(6.0f / static_cast<float>(fan_in));
        std::uniform_real_distribution<float> u(-a, a);
        for (int i = 0; i < count; ++i) w[off + i] = u(rng);
      };
      fill(kgb::kMlpW1, kgb::kMlpIn * kgb::kMlpHidden, kgb::kMlpIn);
      fill(kgb::kMlpW2, kgb::kMlpHidden * kgb::kMlpHidden, kgb::kMlpHidden);
      fill(kgb::kMlpW3, kgb::kMlpHidden, kgb::kMlpHidden);
    }
    Ctx ctx(device);
    cudaStream_t st = ctx.stream();
    const float* d_feat = ctx.upload(features, static_cast<size_t>(n) * kgb::kMlpIn);
    const uint8_t* d_tgt = ctx.upload(targets, static_cast<size_t>(n));
    float* master = ctx.upload(w.data(), w.size());
    float* rounded = ctx.alloc<float>(kgb::kMlpParams);
    float* m = ctx.alloc<float>(kgb::kMlpParams);
    float* v = ctx.alloc<float>(kgb::kMlpParams);
    float* grad = ctx.alloc<float>(kgb::kMlpParams);
    ck(cudaMemsetAsync(m, 0, sizeof(float) * kgb::kMlpParams, st), "memset");
    ck(cudaMemsetAsync(v, 0, sizeof(float) * kgb::kMlpParams, st), "memset");
    const int bsz = std::min(batch, n);
    const int nb = (n + bsz - 1) / bsz;
    float* partial = ctx.alloc<float>(static_cast<size_t>((bsz + kgb::kMlpGradBlock - 1) / kgb::kMlpGradBlock) *
                                      (kgb::kMlpParams + 1));
    float* d_loss = ctx.alloc<float>(nb);
    int* d_idx = ctx.alloc<int>(n);
    std::vector<int> order(static_cast<size_t>(n));
    std::vector<float> losses(static_cast<size_t>(nb));
    int step = 0;
    for (int ep = 0; ep < epochs; ++ep) {
      std::iota(order.begin(), order.end(), 0);
      std::mt19937_64 rng(seed + 1000003ull * static_cast<uint64_t>(ep + 1));
      std::shuffle(order.begin(), order.end(), rng);
      ck(cudaMemcpyAsync(d_idx, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st), "H2D");
      for (int b = 0; b < nb; ++b) {
        const int rows = std::min(bsz, n - b * bsz);
        ck_launch(kgb::mlp_round_params(master, rounded, st), "round");
        ck_launch(kgb::mlp_gradient(rounded, d_feat, d_tgt, d_idx + static_cast<size_t>(b) * bsz, rows, partial, grad,
                                    d_loss + b, st),
                  "gradient");
        ck_launch(kgb::mlp_adam(master, m, v, grad, learning_rate, ++step, st), "adam");
      }
      ctx.download(losses.data(), d_loss, losses.size());
      ctx.sync();  // `order` is rewritten next epoch
      if (loss_per_epoch) {
        double acc = 0.0;
        for (float l : losses) acc += l;
        loss_per_epoch[ep] = static_cast<float>(acc / nb);
      }
    }
    ctx.download(weights_out, master, kgb::kMlpParams);
    ctx.sync();
  });
}

int kgb_proposal_gradient(const float* weights, const float* features, const uint8_t* targets, int32_t n,
                          int32_t device, float* grad, float* loss) {
  return guarded([&]() {
    if (weights == nullptr || features == nullptr || targets == nullptr || grad == nullptr || loss == nullptr)
      fail(KGB_EINVAL, "null pointer");
    if (n < 1) fail(KGB_EINVAL, "no rows");
    Ctx ctx(device);
    cudaStream_t st = ctx.stream();
    float* master = ctx.upload(weights, kgb::kMlpParams);
    float* rounded = ctx.alloc<float>(kgb::kMlpParams);
    ck_launch(kgb::mlp_round_params(master, rounded, st), "round");
    std::vector<int> idx(static_cast<size_t>(n));
    std::iota(idx.begin(), idx.end(), 0);
    float* partial = ctx.alloc<float>(static_cast<size_t>((n + kgb::kMlpGradBlock - 1) / kgb::kMlpGradBlock) *
                                      (kgb::kMlpParams + 1));
    float* d_grad = ctx.alloc<float>(kgb::kMlpParams);
    float* d_loss = ctx.alloc<float>(1);
    ck_launch(kgb::mlp_gradient(rounded, ctx.upload(features, static_cast<size_t>(n) * kgb::kMlpIn),
                                ctx.upload(targets, static_cast<size_t>(n)), ctx.upload(idx.data(), idx.size()), n,
                                partial, d_grad, d_loss, st),
              "gradient");
    ctx.download(grad, d_grad, kgb::kMlpParams);
    ctx.download(loss, d_loss, 1);
    ctx.sync();
  });
}

int kgb_proposal_predict(const float* weights, const float* features, int32_t n, int32_t device, float* logits) {
  return guarded([&]() {
    if (weights == nullptr || features == nullptr || logits == nullptr) fail(KGB_EINVAL, "null pointer");
    if (n < 1) return;
    Ctx ctx(device);
    cudaStream_t st = ctx.stream();
    float* master = ctx.upload(weights, kgb::kMlpParams);
    float* rounded = ctx.alloc<float>(kgb::kMlpParams);
    uint32_t* frag = ctx.alloc<uint32_t>(kgb::kMlpFragWords);
    ck_launch(kgb::mlp_round_params(master, rounded, st), "round");
    ck_launch(kgb::mlp_pack_params(rounded, frag, st), "pack");
    float* d_out = ctx.alloc<float>(n);
    ck_launch(kgb::mlp_predict(frag, ctx.upload(features, static_cast<size_t>(n) * kgb::kMlpIn), n, d_out, st),
              "predict");
    ctx.download(logits, d_out, n);
    ctx.sync();
  });
}

int kgb_core_knn_graph(const int32_t* gidx, const float* gdist, int32_t samples, int32_t gk, int32_t index_base,
                       const int32_t* labels, const int32_t* constrain, const int32_t* fixed,
                       const kgb_core_options* opt, kgb_core_result* out) {
  return guarded([&]() {
    if (gidx == nullptr || gdist == nullptr || labels == nullptr || opt == nullptr || out == nullptr)
      fail(KGB_EINVAL, "null pointer");
    if (samples < 2) fail(KGB_EINVAL, "NeighborGraph samples must be at least 2.");
    if (gk <= 0) fail(KGB_EINVAL, "NeighborGraph.neighbors must be positive.");
    const uint64_t s = opt->seed, cs = opt->cv_seed;
    core_graph_problems(gidx, gdist, samples, gk, index_base, 1, labels, &s, &cs, constrain, fixed, opt, out);
  });
}

int kgb_knncv(const float* x, int32_t n, int32_t d, const int32_t* labels, const int32_t* constrain,
              const kgb_knn_options* opt, int32_t* predicted, int32_t* fold_assignments) {
  return guarded([&]() {
    if (x == nullptr) fail(KGB_EINVAL, "MatrixView data pointer is null.");
    if (labels == nullptr || opt == nullptr || predicted == nullptr) fail(KGB_EINVAL, "null pointer");
    if (n < 1 || d < 1) fail(KGB_EINVAL, "Input matrix must have at least one row and one column.");
    if (opt->k < 1) fail(KGB_EINVAL, "KNNOptions::k must be positive.");
    if (opt->folds < 2) fail(KGB_EINVAL, "Number of folds must be at least 2.");
    if (n > 65535) fail(KGB_EINVAL, "at most 65535 rows are supported");
    check_metric(opt->metric);
    const std::vector<int> lab(labels, labels + n);
    const std::vector<int> con = constrain ? std::vector<int>(constrain, constrain + n) : std::vector<int>();
    const std::vector<int> folds = kgb::make_folds(lab, con, opt->folds, opt->stratified != 0, opt->cv_seed);
    check_training_rows(folds);
    const int K = std::min(opt->k, n - 1);
    Ctx ctx(opt->device);
    cudaStream_t st = ctx.stream();
    const float* d_x = ctx.upload(x, static_cast<size_t>(n) * d);
    const float* xs = search_matrix(ctx, d_x, n, d, opt->metric, 0);
    const int* d_folds = ctx.upload(folds.data(), folds.size());
    int* d_idx = ctx.alloc<int>(static_cast<size_t>(n) * K);
    float* d_dist = ctx.alloc<float>(static_cast<size_t>(n) * K);
    const int segments = 4;
    void* scratch = ctx.alloc<unsigned char>(kgb::knn_bruteforce_scratch(n, K, segments));
    ck_launch(kgb::knn_fold_search(xs, n, d, K, opt->metric != KGB_METRIC_EUCLIDEAN, d_folds, segments, scratch,
                                   d_idx, d_dist, st),
              "fold-wise kNN");
    int* d_pred = ctx.alloc<int>(static_cast<size_t>(n));
    ck_launch(kgb::knn_vote(d_idx, d_dist, n, K, ctx.upload(labels, static_cast<size_t>(n)), d_pred, st), "vote");
    ctx.download(predicted, d_pred, static_cast<size_t>(n));
    ctx.sync();
    if (fold_assignments) std::copy(folds.begin(), folds.end(), fold_assignments);
  });
}

int kgb_core_knn(const float* x, int32_t n, int32_t d, int32_t metric, const int32_t* labels,
                 const int32_t* constrain, const int32_t* fixed, const kgb_core_options* opt,
                 kgb_core_result* out) {
  return guarded([&]() {
    if (x == nullptr) fail(KGB_EINVAL, "MatrixView data pointer is null.");
    if (labels == nullptr || opt == nullptr || out == nullptr) fail(KGB_EINVAL, "null pointer");
    if (n < 1 || d < 1) fail(KGB_EINVAL, "Input matrix must have at least one row and one column.");
    if (n < 2) fail(KGB_EINVAL, "CoreKNN requires at least two samples.");
    check_metric(metric);
    if (opt->k < 1) fail(KGB_EINVAL, "KNNOptions::k must be positive.");
    if (opt->folds < 2) fail(KGB_EINVAL, "Number of folds must be at least 2.");
    {
      const std::vector<int> con = constrain ? std::vector<int>(constrain, constrain + n) : std::vector<int>();
      check_training_rows(kgb::make_folds(std::vector<int>(labels, labels + n), con, opt->folds,
                                          opt->stratified != 0, opt->cv_seed));
    }
    const int w = std::min(opt->k, n - 1);
    const uint64_t s = opt->seed, cs = opt->cv_seed;
    Ctx ctx(opt->device);
    cudaStream_t st = ctx.stream();
    const float* d_x = ctx.upload(x, static_cast<size_t>(n) * d);
    const float* xs = search_matrix(ctx, d_x, n, d, metric, 1);
    core_knn_run(ctx, n, 1, labels, &s, &cs, constrain, fixed, opt, w, out,
                 [&](const std::vector<std::vector<int>>& folds, uint8_t*, uint16_t* d_nb, float* d_sc) {
                   const int* d_folds = ctx.upload(folds[0].data(), folds[0].size());
                   int* d_idx = ctx.alloc<int>(static_cast<size_t>(n) * w);
                   float* d_dist = ctx.alloc<float>(static_cast<size_t>(n) * w);
                   const int segments = 4;
                   void* scratch = ctx.alloc<unsigned char>(kgb::knn_bruteforce_scratch(n, w, segments));
                   ck_launch(kgb::knn_fold_search(xs, n, d, w, metric != KGB_METRIC_EUCLIDEAN, d_folds, segments,
                                                  scratch, d_idx, d_dist, st),
                             "fold-wise kNN");
                   ck_launch(kgb::knn_fold_tables(d_idx, d_dist, n, w, w, d_nb, d_sc, st), "vote tables");
                 });
  });
}

}  // extern "C"
