// Shared definitions for the HSS GB300 library: status codes, error plumbing,
// the kernel-parameter block and small device helpers.
#pragma once

#include <cuda_runtime.h>
#include <map>
#include <memory>
#include <atomic>
#include <mutex>
#include <exception>
#include <thread>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/hssgpu.h"

namespace hss {

// Exception carrying an hss status code; every extern "C" entry point catches
// it and returns the code, so no C++ exception crosses the C boundary.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define HSS_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e__ = (call);                                                 \
    if (e__ != cudaSuccess)                                                   \
      throw ::hss::Error(HSS_ERR_CUDA, std::string(#call) + ": " +            \
                                           cudaGetErrorString(e__));          \
  } while (0)

#define HSS_REQUIRE(cond, code, msg)                                          \
  do {                                                                        \
    if (!(cond)) throw ::hss::Error((code), (msg));                           \
  } while (0)

inline void check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    throw Error(HSS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Helmholtz constants: s = h^2 kh^2 / 4 (the imaginary factor of the off-diagonal
// entries), w = 1 + kh^2 (i/4) dr (the diagonal) and the weights 2 exp(-(j 0.3)^2),
// j = 0..21, of the Hankel-integral trapezoid rule (j = 0 unused).  The weights travel in
// the kernel parameters, so no per-device state has to be uploaded before a launch.
constexpr int kHankelNodes = 21;
constexpr double kHankelStep = 0.3;
struct HelmDev {
  double kh, s, w_re, w_im;
  double hw[kHankelNodes + 1];
};
HelmDev make_helm_dev(const hss_kernel_params& kp);

// Device copy of hss_kernel_params with derived constants.  HSS_SL_H_2D blocks of the HSS
// solvers are generated in the real 2 x 2 embedding (point-table entries 2i and 2i + 1 are
// the real and imaginary components of point i): entry (t, s) is Re K for (even, even) and
// (odd, odd), Im K for (odd, even) and -Im K for (even, odd).
struct KernelDev {
  int flag;
  double h2half;  // h*h*0.5
  double b_alpha, b_x0, b_y0, b_isig;
  double c_alpha, c_x0, c_y0, c_isig;
  HelmDev helm;
};

inline KernelDev make_kernel_dev(const hss_kernel_params& p) {
  KernelDev k;
  k.flag = p.flag;
  k.h2half = p.h * p.h * 0.5;
  k.b_alpha = p.b_alpha; k.b_x0 = p.b_x0; k.b_y0 = p.b_y0; k.b_isig = p.b_isig;
  k.c_alpha = p.c_alpha; k.c_x0 = p.c_x0; k.c_y0 = p.c_y0; k.c_isig = p.c_isig;
  k.helm = make_helm_dev(p);
  return k;
}

// Structure-of-arrays point table on the device (real points, then proxies).
struct PointsDev {
  const double* x;
  const double* y;
  const double* nx;
  const double* ny;
  const double* w;
  const double* kap;
};

// RAII device buffer.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t cnt) { alloc(cnt); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t cnt) {
    release();
    n = cnt;
    if (cnt) {
      cudaError_t e = cudaMalloc(&p, cnt * sizeof(T));
      if (e != cudaSuccess) {
        p = nullptr; n = 0;
        throw Error(HSS_ERR_NOMEM, "cudaMalloc of " + std::to_string(cnt * sizeof(T)) + " bytes failed");
      }
    }
  }
  // grow-only: keeps the current allocation (and every pointer into it) when large enough
  void ensure(size_t cnt) {
    if (n < cnt) alloc(cnt);
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void upload(const std::vector<T>& h, cudaStream_t s) {
    if (h.size() > n) alloc(h.size());
    if (!h.empty())
      HSS_CUDA(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void zero(cudaStream_t s) {
    if (n) HSS_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
};

// Grow-only pinned host block (small device->host reads without pageable staging).
struct PinnedBuf {
  double* p = nullptr;
  size_t n = 0;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  void ensure(size_t cnt) {
    if (n >= cnt) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    HSS_CUDA(cudaMallocHost(&p, cnt * sizeof(double)));
    n = cnt;
  }
};

template <typename T>
inline void download(std::vector<T>& h, const T* d, size_t cnt, cudaStream_t s) {
  h.resize(cnt);
  if (cnt) HSS_CUDA(cudaMemcpyAsync(h.data(), d, cnt * sizeof(T), cudaMemcpyDeviceToHost, s));
}

// Instantiated CUDA graphs of fixed launch sequences, keyed by the number of
// right-hand sides.
// The two streams of a plan whose steps run concurrently: the critical chain on a
// high-priority stream, the steps off it on a low-priority one; one event per step.
struct PlanStreams {
  cudaStream_t crit = nullptr, side = nullptr;
  cudaEvent_t fork = nullptr, jc = nullptr, js = nullptr;
  std::vector<cudaEvent_t> ev;
  explicit PlanStreams(size_t nsteps) {
    int least = 0, greatest = 0;
    HSS_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    HSS_CUDA(cudaStreamCreateWithPriority(&crit, cudaStreamNonBlocking, greatest));
    HSS_CUDA(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, least));
    for (cudaEvent_t* e : {&fork, &jc, &js}) HSS_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    ev.assign(nsteps, nullptr);
    for (auto& e : ev) HSS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  ~PlanStreams() {
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {fork, jc, js})
      if (e) cudaEventDestroy(e);
    if (crit) cudaStreamDestroy(crit);
    if (side) cudaStreamDestroy(side);
  }
  PlanStreams(const PlanStreams&) = delete;
  PlanStreams& operator=(const PlanStreams&) = delete;
  // fork both streams from s / join both back into s
  void fork_from(cudaStream_t s) {
    HSS_CUDA(cudaEventRecord(fork, s));
    HSS_CUDA(cudaStreamWaitEvent(crit, fork, 0));
    HSS_CUDA(cudaStreamWaitEvent(side, fork, 0));
  }
  void join_into(cudaStream_t s) {
    HSS_CUDA(cudaEventRecord(jc, crit));
    HSS_CUDA(cudaEventRecord(js, side));
    HSS_CUDA(cudaStreamWaitEvent(s, jc, 0));
    HSS_CUDA(cudaStreamWaitEvent(s, js, 0));
  }
};

struct GraphCache {
  std::map<int, cudaGraphExec_t> g;
  GraphCache() = default;
  GraphCache(const GraphCache&) = delete;
  GraphCache& operator=(const GraphCache&) = delete;
  ~GraphCache() { clear(); }
  void clear() {
    for (auto& kv : g) cudaGraphExecDestroy(kv.second);
    g.clear();
  }
};

// Capture body() on the stream into a graph once per key, then replay it.
template <typename F>
inline void run_graph(GraphCache& gc, int key, cudaStream_t s, bool enabled, F&& body) {
  if (!enabled) {
    body();
    return;
  }
  auto it = gc.g.find(key);
  if (it == gc.g.end()) {
    cudaGraph_t graph = nullptr;
    HSS_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      body();
    } catch (...) {
      cudaStreamEndCapture(s, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    HSS_CUDA(cudaStreamEndCapture(s, &graph));
    cudaGraphExec_t ex = nullptr;
    // per-node priorities: kernels captured from a high-priority stream keep their priority
    cudaError_t e = cudaGraphInstantiateWithFlags(&ex, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    HSS_REQUIRE(e == cudaSuccess, HSS_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    it = gc.g.emplace(key, ex).first;
  }
  HSS_CUDA(cudaGraphLaunch(it->second, s));
}

// One-time setup per CUDA device (function attributes, which cudaFuncSetAttribute sets for
// the current device only).  run() calls f() the first time it is reached with a given
// device current; the flags are per device and guarded by a mutex, so several host threads
// and several devices in one process each get the setup exactly once.
struct PerDeviceOnce {
  static constexpr int kMaxDevices = 256;
  std::mutex mu;
  bool done[kMaxDevices] = {};
  template <typename F>
  void run(F&& f) {
    int dev = 0;
    HSS_CUDA(cudaGetDevice(&dev));
    HSS_REQUIRE(dev >= 0 && dev < kMaxDevices, HSS_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev]) return;
    f();
    done[dev] = true;
  }
};

// Host-side parallel loop over [0, n): chunks handed out dynamically to up to
// hardware_concurrency() threads; the first exception of any chunk is rethrown.
template <typename F>
inline void parallel_for(int n, F&& f, int min_per_thread = 64) {
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nt = std::max(1, std::min(hw, n / std::max(1, min_per_thread)));
  if (nt <= 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<int> next(0);
  std::exception_ptr err = nullptr;
  std::atomic<bool> failed(false);
  const int chunk = std::max(1, n / (nt * 8));
  auto work = [&] {
    try {
      for (;;) {
        const int i0 = next.fetch_add(chunk);
        if (i0 >= n || failed.load()) break;
        const int i1 = std::min(n, i0 + chunk);
        for (int i = i0; i < i1; ++i) f(i);
      }
    } catch (...) {
      if (!failed.exchange(true)) err = std::current_exception();
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(work);
  work();
  for (auto& t : th) t.join();
  if (err) std::rethrow_exception(err);
}

}  // namespace hss
