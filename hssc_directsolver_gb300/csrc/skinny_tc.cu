// Skinny products on the tensor cores (tcgen05): digit packing, the persistent product
// kernel and its split-K reduction.  Format and accuracy are described in skinny_tc.cuh.
//
// Kernel structure (one CTA per SM, 192 threads):
//   warp 4, lane 0  producer: streams each work item's packed A blocks into a ring of
//                   TC_STAGES shared-memory stages with bulk copies (cp.async.bulk, the TMA
//                   engine) completing on per-stage mbarriers;
//   warp 5, lane 0  MMA issuer: one tcgen05.mma (M = 128, N = 32, K = 16, bf16 -> fp32) per
//                   digit slice and stage into the item's TMEM accumulators; tcgen05.commit
//                   frees the stage and, after the item's last stage, signals the epilogue;
//   warps 0-3       cut the right-hand sides of the next items into bf16 digits (the B
//                   operand, two buffers), then read the accumulators of the finished item
//                   (one TMEM lane per row), add the digit pairs in integers and write FP64.
// Accumulators are double-buffered in TMEM (2 x 256 columns), so the epilogue of one item
// overlaps the loads and MMAs of the next.  Every wait is bounded by the global timer; a
// wait that gives up sets the error word, and the CTA drains its copies in flight and
// frees its TMEM before it exits.
#include <algorithm>
#include <climits>
#include <queue>

#include "skinny_tc.cuh"

namespace hss {

namespace {

constexpr int TC_THREADS = 320;  // 4 epilogue warps, 4 digit warps, producer, MMA issuer
constexpr uint32_t TC_BBYTES = (TC_KITEM / 8) * 512;  // 30 K cores x 4 row groups x 128 B
constexpr int TC_BDEPTH = 2;  // right-hand-side digit buffers: items prepared ahead of the MMAs
constexpr int TC_MAXIT = 512; // work items per CTA: their geometry is staged in shared memory
constexpr int TC_MAXPART = 16; // parts of one row tile (CTAs sharing its K range)
template <int S>
constexpr uint32_t tc_abytes() { return (uint32_t)S * (TC_ROWS / 8) * 256; }
template <int S>
constexpr size_t tc_smem() { return TC_BDEPTH * TC_BBYTES + TC_STAGES * tc_abytes<S>() + 512 + TC_MAXIT * 16; }
constexpr unsigned long long TC_WAIT_NS = 2000000000ULL;  // 2 s per wait

// instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both K-major,
// N = 32 (bits 17-22 hold N/8), M = 128 (bits 24-28 hold M/16)
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(32 >> 3) << 17) |
                              ((uint32_t)(TC_ROWS >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase of `bar` with the given parity.  Gives up (false) when another role
// aborted the CTA or after TC_WAIT_NS, which sets the abort flag and the error word.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_f, int* err) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  for (unsigned it = 1;; ++it) {
    if (mbar_try(bar, parity)) return true;
    if ((it & 63) == 0) {
      if (*abort_f) return false;
      if (gtimer() - t0 > TC_WAIT_NS) {
        *abort_f = 1;
        atomicExch(err, 1);
        return false;
      }
    }
  }
}
// bounded wait that ignores the abort flag (draining copies before exit)
__device__ __forceinline__ void mbar_wait_drain(uint32_t bar, uint32_t parity) {
  const unsigned long long t0 = gtimer();
  while (!mbar_try(bar, parity))
    if (gtimer() - t0 > TC_WAIT_NS) return;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor, no swizzle: start, leading-dimension byte offset (the
// K-direction step between core matrices), stride byte offset (the M/N-direction step
// between 8-row groups), descriptor version 1 (bits 46-48)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(TC_IDESC), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 24 consecutive accumulator columns of this thread's TMEM lane (completed by tmem_ld_wait)
__device__ __forceinline__ void tmem_ld24_issue(uint32_t taddr, uint32_t (&v)[24]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
               : "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
                 "=r"(v[23])
               : "r"(taddr + 16));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// named barrier `id` over one 128-thread role group (four warps)
__device__ __forceinline__ void named_sync128(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
// true on every thread of the group iff `ok` holds on all of them (named barrier `id`)
__device__ __forceinline__ bool all128(int id, bool ok) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %2, 0;\n bar.red.and.pred q, %1, 128, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"(id), "r"((uint32_t)ok)
      : "memory");
  return r != 0;
}
// an FP32 holding an integer of magnitude < 2^22, as an int (exact; adds 1.5 * 2^23)
__device__ __forceinline__ int exact_f32_int(uint32_t bits) {
  return __float_as_int(__uint_as_float(bits) + 12582912.0f) - 0x4B400000;
}

// Row / column exponent: |x| < 2^(e - 1) for every x whose biased exponent field is <= ef.
__device__ __forceinline__ int exp_field(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}
__device__ __forceinline__ int scale_exp(int ef) { return ef == 0 ? -1021 : ef - 1021; }

// round(x * 2^(8S - e)) for |x| < 2^(e - 1), from the bits of x (no FP64 arithmetic)
template <int S>
__device__ __forceinline__ long long tc_fixed(double x, int e) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ef = (int)((b >> 52) & 0x7FF);
  if (ef == 0) return 0;  // zero or subnormal: below every scale in use
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = e - 8 * S + 1075 - ef;  // x 2^(8S - e) = m 2^-sh
  long long v;
  if (sh >= 60) v = 0;
  else if (sh > 0) v = (long long)((m + (1ull << (sh - 1))) >> sh);
  else v = (long long)(m << (-sh));
  return (b >> 63) ? -v : v;
}

// v = sum_j d[j] 256^(S-1-j): the low S-1 digits balanced in [-128, 127], the top digit
// takes the rest (|d[0]| <= 128 for |v| <= 2^(8S-1))
template <int S>
__device__ __forceinline__ void tc_digits(long long v, int (&d)[S]) {
#pragma unroll
  for (int j = S - 1; j >= 1; --j) {
    const int q = (int)(((v + 128) & 255) - 128);
    d[j] = q;
    v = (v - q) >> 8;
  }
  d[0] = (int)v;
}

// bf16 bits of a small integer (exact: at most 8 significant bits)
__device__ __forceinline__ uint32_t bf16_digit(int q) {
  const float f = __int_as_float(0x4B400000 + q) - 12582912.0f;
  return __float_as_uint(f) >> 16;
}

// v * 2^e as a double, rounded to nearest (ties to even), from integer operations only:
// GB300 runs int -> double conversions and FP64 arithmetic at a small fraction of its
// integer rate.  Results outside the normal range take the FP64 path.
__device__ __forceinline__ double int_scaled(long long v, int e) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = (unsigned long long)v & 0x8000000000000000ull;
  unsigned long long u = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
  const int nb = 64 - __clzll(u);  // significant bits
  unsigned long long m;
  int top = nb - 1;                // exponent of the leading bit
  if (nb <= 53) {
    m = u << (53 - nb);
  } else {
    const int sh = nb - 53;
    m = u >> sh;
    const unsigned long long rem = u & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (m & 1ull))) ++m;
    if (m == (1ull << 53)) {
      m >>= 1;
      ++top;
    }
  }
  const int be = top + e + 1023;
  if (be <= 0 || be >= 2047) return ldexp((double)v, e);
  return __longlong_as_double((long long)(sgn | ((unsigned long long)be << 52) | (m & 0xFFFFFFFFFFFFFull)));
}

// x >> sh rounded to nearest (ties up), sh >= 1; 0 when the shift removes every bit
__device__ __forceinline__ long long shr_round(long long x, int sh) {
  if (sh >= 62) return 0;
  return (x + (1LL << (sh - 1))) >> sh;
}

// Running sum (at, ae) += t 2^e of integer products with exponents: the sum is held 2^hb
// below its largest term's scale, so <= 2^hb terms of magnitude < 2^61 add without overflow
// (hb = 0 keeps a single term exact).
__device__ __forceinline__ void acc_add(long long& at, int& ae, long long t, int e, bool first, int hb) {
  const int e7 = e + hb;
  if (first) {
    at = hb ? shr_round(t, hb) : t;
    ae = e7;
    return;
  }
  if (e7 > ae) {
    at = shr_round(at, e7 - ae);
    ae = e7;
  }
  at += shr_round(t, ae - e);
}

__device__ __forceinline__ double seg_val(const TcPackP& p, int r, int k) {
  if (k < p.K[0]) return p.sign[0] * p.A[0][r + (size_t)k * p.lda[0]];
  k -= p.K[0];
  if (k < p.K[1]) return p.sign[1] * p.A[1][r + (size_t)k * p.lda[1]];
  k -= p.K[1];
  return p.sign[2] * p.A[2][r + (size_t)k * p.lda[2]];
}

// right-hand-side entries come from L2 (__ldcg): in a chained launch they were written by
// other CTAs during an earlier phase
__device__ __forceinline__ double b_val(const TcProd& p, int k, int c) {
  if (k < p.K[0]) return __ldcg(p.B[0] + k + (size_t)c * p.ldb[0]);
  k -= p.K[0];
  if (k < p.K[1]) return __ldcg(p.B[1] + k + (size_t)c * p.ldb[1]);
  k -= p.K[1];
  return __ldcg(p.B[2] + k + (size_t)c * p.ldb[2]);
}

// Wait (one thread) until every CTA has finished phase `cnt` (the counter reaches n), bounded
// by the global timer like the mbarrier waits.
__device__ __forceinline__ bool phase_wait(const int* cnt, int n, volatile int* abort_f, int* err) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(cnt) : "memory");
  if (v >= n) return true;
  const unsigned long long t0 = gtimer();
  for (unsigned it = 1;; ++it) {
    __nanosleep(64);
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(cnt) : "memory");
    if (v >= n) return true;
    if ((it & 63) == 0) {
      if (*abort_f) return false;
      if (gtimer() - t0 > TC_WAIT_NS) {
        *abort_f = 1;
        atomicExch(err, 1);
        return false;
      }
    }
  }
}

__global__ void k_tc_rexp(const TcPackP* __restrict__ P) {
  const TcPackP p = P[blockIdx.y];
  const int Kt = p.K[0] + p.K[1] + p.K[2];
  for (int r = blockIdx.x * 256 + threadIdx.x; r < p.M; r += gridDim.x * 256) {
    int ef = 0;
    for (int k = 0; k < Kt; ++k) ef = max(ef, exp_field(seg_val(p, r, k)));
    p.rexp[r] = scale_exp(ef);
  }
}

template <int S>
__global__ void k_tc_pack(const TcPackP* __restrict__ P) {
  const TcPackP p = P[blockIdx.y];
  const int Kt = p.K[0] + p.K[1] + p.K[2];
  const int Kp = (Kt + 15) & ~15, Mp = (p.M + 7) & ~7;
  const long long work = (long long)(Kp / 8) * Mp;
  for (long long w = blockIdx.x * 256LL + threadIdx.x; w < work; w += (long long)gridDim.x * 256) {
    const int r = (int)(w % Mp), cc = (int)(w / Mp);
    const int e = (r < p.M) ? p.rexp[r] : 0;
    uint32_t pk[S][4];
#pragma unroll
    for (int j = 0; j < S; ++j) pk[j][0] = pk[j][1] = pk[j][2] = pk[j][3] = 0u;
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
      const int k = cc * 8 + kk;
      const double a = (r < p.M && k < Kt) ? seg_val(p, r, k) : 0.0;
      int d[S];
      tc_digits<S>(tc_fixed<S>(a, e), d);
#pragma unroll
      for (int j = 0; j < S; ++j) pk[j][kk >> 1] |= bf16_digit(d[j]) << (16 * (kk & 1));
    }
    const int t = r / TC_ROWS, rt = min(TC_ROWS, Mp - TC_ROWS * t);
    const int q = cc >> 1, c = cc & 1, g = (r % TC_ROWS) >> 3, rr = r & 7;
    const size_t base = (size_t)t * (Kp / TC_KS) * S * (TC_ROWS / 8) * 256 + (size_t)q * S * (rt / 8) * 256;
#pragma unroll
    for (int j = 0; j < S; ++j) {
      uint4 v = make_uint4(pk[j][0], pk[j][1], pk[j][2], pk[j][3]);
      *reinterpret_cast<uint4*>(p.out + base + (size_t)j * (rt / 8) * 256 + g * 256 + c * 128 + rr * 16) = v;
    }
  }
}

template <int S>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_skinny_tc(const TcProd* __restrict__ P, const int4* __restrict__ items, const int* __restrict__ cta_off,
                double alpha, double beta, long long* __restrict__ part, int* __restrict__ err, int nphase,
                int* __restrict__ pdone) {
  constexpr uint32_t AB = tc_abytes<S>();
  constexpr int TMAX = S + 1;          // digit pairs kept: weight 256^-t, t <= S + 1
  constexpr int TMID = (TMAX + 1) / 2; // pairs t <= TMID in the high integer, the rest in the low one
  constexpr int UP = 20, DOWN = 8 * (TMAX - TMID) - UP;
  static_assert(DOWN >= 0, "digit pair split");
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* Bbuf = sm;
  unsigned char* Abuf = sm + TC_BDEPTH * TC_BBYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(Abuf + TC_STAGES * AB);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * TC_STAGES + 4 + 2 * TC_BDEPTH);
  volatile int* abort_f = reinterpret_cast<volatile int*>(tslot + 1);
  volatile int* last_f = reinterpret_cast<volatile int*>(tslot + 2);
  int* xexp = reinterpret_cast<int*>(tslot + 4);  // [8 item slots][4 columns]
  int* red = xexp + 32;                           // [2][4 prep warps][4 columns]
  // per item: product, tile | rows << 16, first | end K << 16, K steps | flags << 16
  int4* gtab = reinterpret_cast<int4*>(reinterpret_cast<unsigned char*>(bars) + 512);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i0 = cta_off[blockIdx.x], nit = cta_off[blockIdx.x + 1] - i0;
  const uint32_t bar0 = smem_u32(bars);
  auto FULL = [&](int s) { return bar0 + 8u * s; };
  auto EMPTY = [&](int s) { return bar0 + 8u * (TC_STAGES + s); };
  // per accumulator set a (item j % 2): DONE (MMAs finished), TFREE (accumulators read);
  // per B buffer b (item j % TC_BDEPTH): BREADY (digits written), BFREE (MMAs reading it done)
  auto DONE = [&](int a) { return bar0 + 8u * (2 * TC_STAGES + a); };
  auto TFREE = [&](int a) { return bar0 + 8u * (2 * TC_STAGES + 2 + a); };
  auto BREADY = [&](int b) { return bar0 + 8u * (2 * TC_STAGES + 4 + b); };
  auto BFREE = [&](int b) { return bar0 + 8u * (2 * TC_STAGES + 4 + TC_BDEPTH + b); };

  if (tid == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(FULL(s), 1);
      mbar_init(EMPTY(s), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(DONE(a), 1);
      mbar_init(TFREE(a), 128);
    }
    for (int b = 0; b < TC_BDEPTH; ++b) {
      mbar_init(BREADY(b), 128);
      mbar_init(BFREE(b), 1);
    }
    *abort_f = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // rows 24..31 of every B buffer (no right-hand side) stay zero
  constexpr int KC = TC_KITEM / 8;  // K cores of a B buffer
  for (int e = tid; e < TC_BDEPTH * KC * 8; e += TC_THREADS) {
    const int buf = e / (KC * 8), kc = (e / 8) % KC, part16 = e & 7;
    *reinterpret_cast<uint4*>(Bbuf + buf * TC_BBYTES + kc * 512 + 3 * 128 + part16 * 16) = make_uint4(0, 0, 0, 0);
  }
  for (int e = tid; e < nit; e += TC_THREADS) {  // item geometry, once (global loads off the pipeline)
    const int4 w = items[i0 + e];
    const TcProd& p = P[w.x];
    const int Kp = (p.K[0] + p.K[1] + p.K[2] + 15) & ~15, Mp = (p.M + 7) & ~7;
    const int rt = min(TC_ROWS, Mp - TC_ROWS * (w.y & 1023));
    gtab[e] = make_int4(w.x, w.y | (rt << 16), w.z, (Kp / TC_KS) | (w.w << 16));
  }
  if (warp == 9) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tslot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  // item geometry
  struct Geo {
    int prod, t, ph, rt, kb, ke, nks;
  };
  auto geo = [&](int j) {
    const int4 w = gtab[j];
    Geo g;
    g.prod = w.x;
    g.t = w.y & 1023;
    g.ph = (w.y >> 10) & 63;
    g.rt = w.y >> 16;
    g.kb = w.z & 0xFFFF;
    g.ke = w.z >> 16;
    g.nks = w.w & 0xFFFF;
    return g;
  };

  if (warp == 8) {
    if (lane == 0) {
      // producer
      int gs = 0;
      bool ok = true;
      for (int j = 0; j < nit && ok; ++j) {
        const Geo g = geo(j);
        // a stage holds spp consecutive K steps (one contiguous copy): 128 rows' worth
        const uint32_t step_bytes = (uint32_t)S * (g.rt / 8) * 256;
        const int spp = TC_ROWS / g.rt, q0 = g.kb / TC_KS, q1 = g.ke / TC_KS;
        const unsigned char* tile = P[g.prod].A + (size_t)g.t * g.nks * AB;
        for (int q = q0; q < q1; q += spp, ++gs) {
          const int s = gs % TC_STAGES;
          if (gs >= TC_STAGES && !mbar_wait(EMPTY(s), ((gs / TC_STAGES) - 1) & 1, abort_f, err)) {
            ok = false;
            break;
          }
          const uint32_t bytes = step_bytes * (uint32_t)min(spp, q1 - q);
          mbar_expect_tx(FULL(s), bytes);
          bulk_g2s(smem_u32(Abuf + s * AB), tile + (size_t)q * step_bytes, bytes, FULL(s));
        }
      }
      if (!ok)  // let the copies in flight land before the CTA exits
        for (int h = max(0, gs - TC_STAGES); h < gs; ++h) mbar_wait_drain(FULL(h % TC_STAGES), (h / TC_STAGES) & 1);
    }
  } else if (warp == 9) {
    if (lane == 0) {
      // MMA issuer
      int gs = 0;
      bool ok = true;
      for (int j = 0; j < nit && ok; ++j) {
        const int a = j & 1, bi = j % TC_BDEPTH;
        if (!mbar_wait(BREADY(bi), (j / TC_BDEPTH) & 1, abort_f, err)) break;
        if (j >= 2 && !mbar_wait(TFREE(a), ((j - 2) >> 1) & 1, abort_f, err)) break;
        tc_fence_after();
        const Geo g = geo(j);
        const uint32_t bb = smem_u32(Bbuf + bi * TC_BBYTES);
        const uint32_t dcol = tmem + (uint32_t)a * 256;
        const uint32_t step_bytes = (uint32_t)S * (g.rt / 8) * 256;
        const int spp = TC_ROWS / g.rt, nq = (g.ke - g.kb) / TC_KS;
        for (int q = 0; q < nq; q += spp, ++gs) {
          const int s = gs % TC_STAGES;
          if (!mbar_wait(FULL(s), (gs / TC_STAGES) & 1, abort_f, err)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const int nst = min(spp, nq - q);
          for (int u = 0; u < nst; ++u) {
            const uint32_t ab = smem_u32(Abuf + s * AB) + (uint32_t)u * step_bytes;
            const uint64_t bd = sdesc(bb + (uint32_t)(q + u) * 1024, 512, 128);
#pragma unroll
            for (int i = 0; i < S; ++i)
              tc_mma(dcol + (uint32_t)i * 32, sdesc(ab + (uint32_t)(i * (g.rt / 8) * 256), 128, 256), bd,
                     (q + u) > 0 ? 1u : 0u);
          }
          tc_commit(EMPTY(s));
        }
        if (ok) {
          tc_commit(DONE(a));
          tc_commit(BFREE(bi));
        }
      }
      // MMAs in flight finish before the accumulators are freed
      if (!ok && gs > 0) mbar_wait_drain(EMPTY((gs - 1) % TC_STAGES), ((gs - 1) / TC_STAGES) & 1);
    }
  } else if (warp >= 4) {
    // right-hand-side digits of item j into B buffer j % TC_BDEPTH once the MMAs of item
    // j - TC_BDEPTH (the buffer's previous reader) are done
    const int ptid = tid - 128, pw = warp - 4;
    for (int j = 0; j < nit; ++j) {
      const int a = j % TC_BDEPTH;
      if (j >= TC_BDEPTH && !all128(1, mbar_wait(BFREE(a), ((j - TC_BDEPTH) / TC_BDEPTH) & 1, abort_f, err)))
        break;
      const Geo g = geo(j);
      if (g.ph > 0 && (j == 0 || geo(j - 1).ph != g.ph)) {
        // the right-hand sides of phase ph are the outputs of phase ph - 1 on every CTA
        bool ok = true;
        if (ptid == 0) ok = phase_wait(pdone + g.ph - 1, (int)gridDim.x, abort_f, err);
        if (!all128(1, ok)) break;
      }
      named_sync128(1);
      const TcProd& p = P[g.prod];
      const int c = ptid & 3, oct = ptid >> 2;
      const int Kt = p.K[0] + p.K[1] + p.K[2];
      const int k0 = g.kb + oct * 8;
      const bool live = (c < p.r) && (k0 < g.ke);
      double xv[8];
      int mef = 0;
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        const int k = k0 + kk;
        xv[kk] = (live && k < Kt) ? b_val(p, k, c) : 0.0;
        mef = max(mef, exp_field(xv[kk]));
      }
      mef = max(mef, __shfl_xor_sync(0xffffffffu, mef, 4));
      mef = max(mef, __shfl_xor_sync(0xffffffffu, mef, 8));
      mef = max(mef, __shfl_xor_sync(0xffffffffu, mef, 16));
      if (lane < 4) red[((j & 1) * 4 + pw) * 4 + lane] = mef;
      named_sync128(1);
      int m = 0;
#pragma unroll
      for (int w = 0; w < 4; ++w) m = max(m, red[((j & 1) * 4 + w) * 4 + c]);
      const int e = scale_exp(m);
      if (ptid < 4) xexp[(j & 7) * 4 + ptid] = e;
      if (k0 < g.ke) {
        uint32_t pk[S][4];
#pragma unroll
        for (int jj = 0; jj < S; ++jj) pk[jj][0] = pk[jj][1] = pk[jj][2] = pk[jj][3] = 0u;
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
          int d[S];
          tc_digits<S>(tc_fixed<S>(xv[kk], e), d);
#pragma unroll
          for (int jj = 0; jj < S; ++jj) pk[jj][kk >> 1] |= bf16_digit(d[jj]) << (16 * (kk & 1));
        }
        unsigned char* bb = Bbuf + a * TC_BBYTES + (k0 - g.kb) / 8 * 512;
#pragma unroll
        for (int jj = 0; jj < S; ++jj) {
          const int n = jj * 4 + c;
          *reinterpret_cast<uint4*>(bb + (n >> 3) * 128 + (n & 7) * 16) = make_uint4(pk[jj][0], pk[jj][1], pk[jj][2], pk[jj][3]);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(BREADY(a));
    }
  } else {
    // epilogue (128 threads; thread = TMEM lane = tile row)
    long long acc_t[4] = {0, 0, 0, 0};  // running sum of the current part
    int acc_e[4] = {0, 0, 0, 0};
    // phases [arrived, upto) are finished on this CTA: publish its outputs and count it in
    int arrived = 0;
    auto arrive = [&](int upto) {
      if (upto <= arrived) return;
      __threadfence();
      named_sync128(2);
      if (tid == 0)
        for (int ph = arrived; ph < upto; ++ph) atomicAdd(pdone + ph, 1);
      arrived = upto;
    };
    arrive(nit > 0 ? geo(0).ph : nphase);  // phases without items on this CTA
    for (int j = 0; j < nit; ++j) {
      const int a = j & 1;
      // the 128 threads leave together: a thread left behind would wait in a barrier
      if (!all128(2, mbar_wait(DONE(a), (j >> 1) & 1, abort_f, err))) break;
      tc_fence_after();
      const Geo g = geo(j);
      const TcProd& p = P[g.prod];
      int xe[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) xe[c] = xexp[(j & 7) * 4 + c];
      int sacc[TMAX - 1][4];
#pragma unroll
      for (int t = 0; t < TMAX - 1; ++t) sacc[t][0] = sacc[t][1] = sacc[t][2] = sacc[t][3] = 0;
      const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)a * 256;
#pragma unroll
      for (int i0s = 0; i0s < S; i0s += 3) {
        uint32_t v[3][24];
#pragma unroll
        for (int u = 0; u < 3; ++u)
          if (i0s + u < S) tmem_ld24_issue(lane_base + (uint32_t)(i0s + u) * 32, v[u]);
        tmem_ld_wait();
#pragma unroll
        for (int u = 0; u < 3; ++u) {
          const int i = i0s + u;
          if (i >= S) continue;
#pragma unroll
          for (int jx = 0; jx < S; ++jx) {
            const int t = i + jx + 2;
            if (t <= TMAX) {
#pragma unroll
              for (int c = 0; c < 4; ++c) sacc[t - 2][c] += exact_f32_int(v[u][jx * 4 + c]);
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(TFREE(a));
      const int row = TC_ROWS * g.t + tid;
      const bool mine = tid < g.rt && row < p.M;
      long long tot[4];
      int E[4];
      const int er = mine ? p.rexp[row] : 0;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        long long hi = 0, lo = 0;
#pragma unroll
        for (int t = 2; t <= TMID; ++t) hi += (long long)sacc[t - 2][c] << (8 * (TMID - t));
#pragma unroll
        for (int t = TMID + 1; t <= TMAX; ++t) lo += (long long)sacc[t - 2][c] << (8 * (TMAX - t));
        // one integer: |hi| < 2^42 moves up by UP bits, lo (weight 2^(8 (TMID - TMAX)) of hi's)
        // down by DOWN bits, dropping < 2^-52 of the product's scale
        tot[c] = (hi << UP) + (lo >> DOWN);
        E[c] = er + xe[c] - 8 * TMID - UP;
      }
      const int flags = gtab[j].w >> 16;
      const bool first = flags & 1, last = (flags >> 1) & 1;
      const int hb = (flags >> 2) & 7, part_q = (flags >> 5) & 15, np = (flags >> 9) & 31;
#pragma unroll
      for (int c = 0; c < 4; ++c) acc_add(acc_t[c], acc_e[c], tot[c], E[c], first, hb);
      if (!last) continue;  // the next chunk of this part follows on this CTA (same phase)
      if (np == 1) {
        if (mine) {
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            if (c >= p.r) continue;
            const double y = int_scaled(acc_t[c], acc_e[c]);
            double* cp = p.C + row + (size_t)c * p.ldc;
            if (alpha == 1.0 && beta == 0.0) *cp = y;  // no FP64 arithmetic on the common path
            else *cp = (beta == 0.0) ? alpha * y : alpha * y + beta * *cp;
          }
        }
      } else {
        // several parts: publish (integer, exponent); the CTA finishing the tile's last part adds all
        if (mine) {
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            if (c >= p.r) continue;
            long long* pp = part + p.part_off + (((long long)part_q * p.M + row) * 4 + c) * 2;
            pp[0] = acc_t[c];
            pp[1] = acc_e[c];
          }
        }
        __threadfence();
        named_sync128(2);
        if (tid == 0) *last_f = (atomicAdd(p.cnt + g.t, 1) == np - 1) ? 1 : 0;
        named_sync128(2);
        if (*last_f) {
          __threadfence();
          if (mine) {
            const long long step = (long long)p.M * 8;
            const int pb = 32 - __clz(np - 1);  // headroom bits for np terms
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              if (c >= p.r) continue;
              const long long* pp = part + p.part_off + ((long long)row * 4 + c) * 2;
              long long vt[TC_MAXPART];
              int ve[TC_MAXPART];
#pragma unroll
              for (int q = 0; q < TC_MAXPART; ++q) {  // every load issued before any is used
                vt[q] = q < np ? __ldcg(pp + q * step) : 0;
                ve[q] = q < np ? (int)__ldcg(pp + q * step + 1) : -100000;
              }
              int emax = ve[0];
#pragma unroll
              for (int q = 1; q < TC_MAXPART; ++q) emax = max(emax, ve[q]);
              long long sum = 0;
#pragma unroll
              for (int q = 0; q < TC_MAXPART; ++q)
                if (q < np) sum += shr_round(vt[q], emax - ve[q] + pb);
              const double y = int_scaled(sum, emax + pb);
              double* cp = p.C + row + (size_t)c * p.ldc;
              if (alpha == 1.0 && beta == 0.0) *cp = y;
              else *cp = (beta == 0.0) ? alpha * y : alpha * y + beta * *cp;
            }
          }
          named_sync128(2);
          if (tid == 0) p.cnt[g.t] = 0;  // every part has been counted: ready for the next launch
        }
      }
      arrive(j + 1 < nit ? geo(j + 1).ph : nphase);
    }
    arrive(nphase);
    // the last CTA to finish every phase resets the phase counters for the next launch (every
    // CTA's digit warps have passed all their phase waits by now)
    if (tid == 0 && atomicAdd(pdone + nphase, 1) == (int)gridDim.x - 1) {
      for (int ph = 0; ph <= nphase; ++ph) atomicExch(pdone + ph, 0);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 9) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

int sm_count() {
  int dev = 0, n = 0;
  HSS_CUDA(cudaGetDevice(&dev));
  HSS_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  return std::max(1, n);
}

}  // namespace

size_t tc_packed_bytes(int M, int K) {
  const size_t Mp = ((size_t)M + 7) & ~(size_t)7, Kp = ((size_t)K + 15) & ~(size_t)15;
  return Mp * Kp * TC_S * 2;
}

void tc_pack(const TcPackP* dP, int batch, int maxM, int maxK, cudaStream_t s) {
  if (batch <= 0 || maxM <= 0 || maxK <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "tc_pack: batch too large");
  k_tc_rexp<<<dim3(std::max(1, std::min(ceil_div(maxM, 256), 64)), batch), 256, 0, s>>>(dP);
  check_launch("k_tc_rexp");
  const long long work = (long long)((maxK + 15) / 8) * ((maxM + 7) & ~7);
  k_tc_pack<TC_S><<<dim3(std::max(1, std::min(ceil_div(work, 256), 2048)), batch), 256, 0, s>>>(dP);
  check_launch("k_tc_pack");
}

void TcStep::build(const std::vector<TcProd>& P0, double al, double be, int* d_err, cudaStream_t s) {
  build(std::vector<std::vector<TcProd>>{P0}, al, be, d_err, s);
}

void TcStep::build(const std::vector<std::vector<TcProd>>& phases, double al, double be, int* d_err,
                   cudaStream_t s) {
  HSS_REQUIRE(d_err != nullptr, HSS_ERR_ARG, "tensor-core product: no error word");
  HSS_REQUIRE(!phases.empty() && phases.size() <= 63, HSS_ERR_ARG, "tensor-core product: 1..63 phases");
  err = d_err;
  alpha = al;
  beta = be;
  nphase = (int)phases.size();
  std::vector<TcProd> P;
  std::vector<int> phase_of;
  for (int ph = 0; ph < nphase; ++ph)
    for (auto& q : phases[ph]) {
      P.push_back(q);
      phase_of.push_back(ph);
    }
  nprod = (int)P.size();
  const int nsm = sm_count();
  // row tiles of every product, in product order; cost = rows x K steps (+ a fixed cost per chunk)
  struct Tile { int prod, t, rt, nks, ph; };
  std::vector<Tile> tiles;
  std::vector<long long> ptotal(nphase, 0);
  maxM = 0;
  for (int i = 0; i < nprod; ++i) {
    TcProd& p = P[i];
    HSS_REQUIRE(p.r >= 1 && p.r <= TC_NR && p.M > 0, HSS_ERR_ARG, "tensor-core product: 1..4 columns");
    const int Kt = p.K[0] + p.K[1] + p.K[2];
    HSS_REQUIRE(Kt > 0 && Kt < 65536 - 16, HSS_ERR_ARG, "tensor-core product: K outside 1..65519");
    HSS_REQUIRE((reinterpret_cast<uintptr_t>(p.A) & 15) == 0, HSS_ERR_ARG, "tensor-core product: A not 16-byte aligned");
    const int Kp = (Kt + 15) & ~15, Mp = (p.M + 7) & ~7;
    const int nt = (Mp + TC_ROWS - 1) / TC_ROWS;
    HSS_REQUIRE(nt <= 1024, HSS_ERR_ARG, "tensor-core product: more than 1024 row tiles");
    p.ksplit = (Kp + TC_KITEM - 1) / TC_KITEM;
    maxM = std::max(maxM, p.M);
    for (int t = 0; t < nt; ++t) {
      const int rt = std::min(TC_ROWS, Mp - TC_ROWS * t);
      tiles.push_back(Tile{i, t, rt, Kp / TC_KS, phase_of[i]});
      ptotal[phase_of[i]] += (long long)rt * (Kp / TC_KS);
    }
  }
  // Linear partition: every CTA takes an equal share of rows x K steps.  Whole tiles go to
  // the current CTA while they fit; a tile larger than a quarter of the share is cut at a K
  // step so that the CTA is filled (at most TC_MAXPART parts per tile); the CTAs of one tile
  // meet in the in-kernel reduction.
  const int ntile = (int)tiles.size();
  // Per phase, cut the tiles' K steps, in order and weighted by their rows, into runs of
  // equal weight, one per CTA; a run boundary may fall inside a tile (its parts then meet in
  // the kernel's final add).  A tile of weight w spans at most w / share + 2 runs, so a
  // phase uses fewer CTAs when needed to keep every tile within TC_MAXPART parts.  A chain
  // of phases runs on every SM (one CTA each, all resident: a cooperative launch).
  grid = nphase > 1 ? nsm : std::max(1, std::min(nsm, ntile * TC_MAXPART));
  struct Seg { int tile, s0, s1; };
  std::vector<std::vector<Seg>> per(grid);
  {
    int tb = 0;
    for (int ph = 0; ph < nphase; ++ph) {
      int te = tb;
      long long maxw = 1;
      while (te < ntile && tiles[te].ph == ph) {
        maxw = std::max(maxw, (long long)tiles[te].rt * tiles[te].nks);
        ++te;
      }
      if (te == tb) continue;
      const long long total = ptotal[ph];
      const int g = std::max(1, std::min(grid, (int)std::min<long long>((long long)(te - tb) * TC_MAXPART,
                                                                        (TC_MAXPART - 2) * total / maxw)));
      const long long share = (total + g - 1) / g;
      long long w0 = 0;  // weight before the current tile
      for (int ti = tb; ti < te; ++ti) {
        const Tile& T = tiles[ti];
        int s0 = 0;
        while (s0 < T.nks) {
          const long long pos = w0 + (long long)s0 * T.rt;  // weight at step s0
          const int c = (int)std::min<long long>(g - 1, pos / share);
          const long long end = (c == g - 1) ? LLONG_MAX : (long long)(c + 1) * share;
          const long long room = end - pos;  // steps of this tile before the run's end (at least one)
          const int take = (int)std::max<long long>(1, std::min<long long>(T.nks - s0, (room + T.rt - 1) / T.rt));
          per[c].push_back(Seg{ti, s0, s0 + take});
          s0 += take;
        }
        w0 += (long long)T.rt * T.nks;
      }
      tb = te;
    }
  }
  if (nphase == 1)
    while (grid > 1 && per[grid - 1].empty()) --grid;
  // parts per tile, counters and part-sum slots
  std::vector<int> tparts(ntile, 0);
  for (auto& v : per)
    for (auto& sg : v) ++tparts[sg.tile];
  std::vector<int> pslots(nprod, 1), tfirst(nprod, -1);
  for (int ti = 0; ti < ntile; ++ti) {
    HSS_REQUIRE(tparts[ti] >= 1 && tparts[ti] <= TC_MAXPART, HSS_ERR_ARG, "tensor-core product: tile split too far");
    pslots[tiles[ti].prod] = std::max(pslots[tiles[ti].prod], tparts[ti]);
    if (tfirst[tiles[ti].prod] < 0) tfirst[tiles[ti].prod] = ti;
  }
  long long poff = 0;
  for (int i = 0; i < nprod; ++i) {
    P[i].nparts = pslots[i];
    P[i].part_off = poff;
    if (pslots[i] > 1) poff += (long long)pslots[i] * P[i].M * 4 * 2;
  }
  cnt.alloc(std::max(ntile, 1));
  cnt.zero(s);
  for (int i = 0; i < nprod; ++i) P[i].cnt = cnt.p + tfirst[i];  // tiles of a product are consecutive
  // items: chunks of <= TC_KITEM columns of each segment, in segment order per CTA
  std::vector<int> qnext(ntile, 0);
  std::vector<int4> flat;
  std::vector<int> off(grid + 1, 0);
  constexpr int CH = TC_KITEM / TC_KS;  // K steps per chunk
  for (int c = 0; c < grid; ++c) {
    for (auto& sg : per[c]) {
      const Tile& T = tiles[sg.tile];
      const int q = qnext[sg.tile]++;
      const int nch = (sg.s1 - sg.s0 + CH - 1) / CH;
      int hb = 0;  // headroom bits of the part's running sum: 2^hb >= its chunk count
      while ((1 << hb) < nch) ++hb;
      HSS_REQUIRE(hb <= 7, HSS_ERR_ARG, "tensor-core product: part of more than 128 chunks");
      for (int ch = 0; ch < nch; ++ch) {
        const int a0 = sg.s0 + ch * CH, a1 = std::min(sg.s1, a0 + CH);
        const int flags = ((ch == 0) ? 1 : 0) | ((ch == nch - 1) ? 2 : 0) | (hb << 2) | (q << 5) | (tparts[sg.tile] << 9);
        flat.push_back(make_int4(T.prod, T.t | (T.ph << 10), (a0 * TC_KS) | ((a1 * TC_KS) << 16), flags));
      }
    }
    HSS_REQUIRE((int)flat.size() - off[c] <= TC_MAXIT, HSS_ERR_ARG, "tensor-core product: too many work items for one launch");
    off[c + 1] = (int)flat.size();
  }
  pdone.alloc(nphase + 1);
  pdone.zero(s);
  prods.alloc(P.size());
  items.alloc(std::max<size_t>(flat.size(), 1));
  cta_off.alloc(off.size());
  part.alloc(std::max<long long>(poff, 1));
  HSS_CUDA(cudaMemcpyAsync(prods.p, P.data(), P.size() * sizeof(TcProd), cudaMemcpyHostToDevice, s));
  HSS_CUDA(cudaMemcpyAsync(items.p, flat.data(), flat.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  HSS_CUDA(cudaMemcpyAsync(cta_off.p, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  HSS_CUDA(cudaStreamSynchronize(s));  // host vectors go out of scope
}

void TcStep::run(cudaStream_t s) const {
  if (grid <= 0) return;
  static PerDeviceOnce attr_once;
  attr_once.run([] {
    HSS_CUDA(cudaFuncSetAttribute(k_skinny_tc<TC_S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)tc_smem<TC_S>()));
  });
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(TC_THREADS, 1, 1);
  cfg.dynamicSmemBytes = tc_smem<TC_S>();
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;  // the phases of a chain wait on every CTA
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = nphase > 1 ? 1 : 0;
  HSS_CUDA(cudaLaunchKernelEx(&cfg, k_skinny_tc<TC_S>, prods.p, items.p, cta_off.p, alpha, beta, part.p, err,
                              nphase, pdone.p));
  check_launch("k_skinny_tc");
}

}  // namespace hss
