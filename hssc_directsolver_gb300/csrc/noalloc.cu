// Batched block inversion that allocates no device memory.
//
// Some callers cannot call cudaMalloc/cudaFree once they are running: hosts
// whose device memory is owned by their own pool allocator (which a second
// allocator would fragment or exceed), and latency-bound loops in which
// cudaMalloc and cudaFree would synchronise the device.  This entry point
// serves them: the caller passes the matrices and the info array, and all the
// scratch the blocked Gauss-Jordan inversion needs (descriptors, pivots,
// bookkeeping, panel rows and the column-permutation buffer) comes from one
// fixed array in device global memory, declared below.
//
// Limits and sharing:
//  * the array holds NOALLOC_SCRATCH_BYTES (16 MiB); every GPU that loads this
//    library holds it until the process exits;
//  * a call needs batch * (n*n + 2*32*n) doubles + batch * (n + GJ_AUX) ints +
//    the descriptors, and at most NOALLOC_MAX_BATCH matrices; larger calls are
//    rejected with HSS_ERR_ARG before any work;
//  * every call uses the same array and leaves its contents behind, so calls
//    that overlap on the GPU (different streams or threads, without ordering)
//    race on it and must not be issued.  The info entries, which must start at
//    zero, are cleared by each call.
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; later calls reuse it.
//    That first call may also load this library's device code on the device
//    (CUDA loads modules lazily), so make it before any stream capture.  A
//    cudaDeviceReset destroys the array with the context: the cached address is
//    then stale, so do not use this entry point after resetting a device.
#include <mutex>

#include "dense.cuh"

namespace hss {

constexpr size_t NOALLOC_SCRATCH_BYTES = 16u << 20;
constexpr int NOALLOC_MAX_BATCH = 256;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// device address of g_noalloc_scratch, per device (the host symbol is only a stand-in)
static unsigned char* scratch_ptr_for_current_device() {
  static std::mutex mu;
  static unsigned char* ptrs[NOALLOC_MAX_DEVICES] = {};
  int dev = 0;
  HSS_CUDA(cudaGetDevice(&dev));
  HSS_REQUIRE(dev >= 0 && dev < NOALLOC_MAX_DEVICES, HSS_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!ptrs[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    HSS_REQUIRE(e == cudaSuccess && p != nullptr, HSS_ERR_CUDA,
                std::string("cudaGetSymbolAddress of the inversion scratch: ") + cudaGetErrorString(e));
    ptrs[dev] = static_cast<unsigned char*>(p);
  }
  return ptrs[dev];
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

void batched_inverse_noalloc(double* d_A, int n, int batch, int* d_info, cudaStream_t s) {
  HSS_REQUIRE(d_A && d_info && n > 0 && batch > 0, HSS_ERR_ARG, "bad arguments");
  HSS_REQUIRE(batch <= NOALLOC_MAX_BATCH, HSS_ERR_ARG,
              "no-allocation inverse: batch exceeds " + std::to_string(NOALLOC_MAX_BATCH));
  const size_t nn = (size_t)n;
  const size_t b_desc = align256((size_t)batch * sizeof(InvP<double>));
  const size_t b_ipiv = align256((size_t)batch * nn * sizeof(int));
  const size_t b_aux = align256((size_t)batch * GJ_AUX * sizeof(int));
  const size_t b_w = align256((size_t)batch * 2 * GJ_NB * nn * sizeof(double));
  const size_t b_wf = align256((size_t)batch * nn * nn * sizeof(double));
  const size_t need = b_desc + b_ipiv + b_aux + b_w + b_wf;
  HSS_REQUIRE(need <= NOALLOC_SCRATCH_BYTES, HSS_ERR_ARG,
              "no-allocation inverse: needs " + std::to_string(need) + " bytes of scratch, the fixed array holds " +
                  std::to_string(NOALLOC_SCRATCH_BYTES));
  unsigned char* base = scratch_ptr_for_current_device();
  auto* dP = reinterpret_cast<InvP<double>*>(base);
  int* ipiv = reinterpret_cast<int*>(base + b_desc);
  int* aux = reinterpret_cast<int*>(base + b_desc + b_ipiv);
  double* W = reinterpret_cast<double*>(base + b_desc + b_ipiv + b_aux);
  double* Wf = reinterpret_cast<double*>(base + b_desc + b_ipiv + b_aux + b_w);
  InvP<double> P[NOALLOC_MAX_BATCH];  // host descriptors on the stack
  for (int b = 0; b < batch; ++b)
    P[b] = InvP<double>{d_A + (size_t)b * nn * nn, n, n, ipiv + (size_t)b * nn, W + (size_t)b * 2 * GJ_NB * nn,
                        Wf + (size_t)b * nn * nn, d_info + b, aux + (size_t)b * GJ_AUX};
  HSS_CUDA(cudaMemsetAsync(d_info, 0, batch * sizeof(int), s));
  // pageable source: the copy is staged before cudaMemcpyAsync returns
  HSS_CUDA(cudaMemcpyAsync(dP, P, batch * sizeof(InvP<double>), cudaMemcpyHostToDevice, s));
  invert_batched<double>(dP, batch, n, s);
  HSS_CUDA(cudaStreamSynchronize(s));
}

}  // namespace hss
