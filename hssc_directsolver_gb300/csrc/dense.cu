// Batched dense linear algebra kernels (FP64 and FP32) for the HSS levels.
#include "dense.cuh"

#include <cfloat>
#include <cmath>
#include <type_traits>
#include <cooperative_groups.h>

namespace hss {

// ---------------------------------------------------------------------------
// Block reductions
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over a 256-thread block; every thread gets the result.
template <typename R>
__device__ R block_sum256(R v, R* sh /* >= 8 */) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  R t = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) t += sh[i];
  __syncthreads();
  return t;
}

// Arg-max of val over a 256-thread block, lowest index among equal maxima.
// Threads with no candidate pass val = -1, idx = INT_MAX.
template <typename R>
__device__ void block_argmax256(R& val, int& idx, R* shv, int* shi) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    R ov = __shfl_xor_sync(0xffffffffu, val, o);
    int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > val || (ov == val && oi < idx)) { val = ov; idx = oi; }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) { shv[w] = val; shi[w] = idx; }
  __syncthreads();
  val = shv[0];
  idx = shi[0];
#pragma unroll
  for (int i = 1; i < 8; ++i) {
    if (shv[i] > val || (shv[i] == val && shi[i] < idx)) { val = shv[i]; idx = shi[i]; }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Tiled GEMM: 64x64 output tile, K step 16, 256 threads, 4x4 per thread.
// ---------------------------------------------------------------------------
template <typename R, bool TA, bool TB>
__global__ void __launch_bounds__(256) k_gemm(const GemmP<R>* __restrict__ P, R alpha, R beta) {
  const GemmP<R> p = P[blockIdx.z];
  const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  if (m0 >= p.M || n0 >= p.N) return;
  __shared__ R As[16][64 + 1];
  __shared__ R Bs[16][64 + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  R acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = R(0);
  for (int k0 = 0; k0 < p.K; k0 += 16) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + 256 * r;
      int i, kk;
      if (!TA) { i = e & 63; kk = e >> 6; } else { kk = e & 15; i = e >> 4; }
      const int gi = m0 + i, gk = k0 + kk;
      R v = R(0);
      if (gi < p.M && gk < p.K)
        v = TA ? p.A[gk + (size_t)gi * p.lda] : p.A[gi + (size_t)gk * p.lda];
      As[kk][i] = v;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + 256 * r;
      int j, kk;
      if (!TB) { kk = e & 15; j = e >> 4; } else { j = e & 63; kk = e >> 6; }
      const int gj = n0 + j, gk = k0 + kk;
      R v = R(0);
      if (gj < p.N && gk < p.K)
        v = TB ? p.B[gj + (size_t)gk * p.ldb] : p.B[gk + (size_t)gj * p.ldb];
      Bs[kk][j] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      R a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gi = m0 + tx + 16 * i;
    if (gi >= p.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gj = n0 + ty + 16 * j;
      if (gj >= p.N) continue;
      R* c = p.C + gi + (size_t)gj * p.ldc;
      *c = (beta == R(0)) ? alpha * acc[i][j] : alpha * acc[i][j] + beta * (*c);
    }
  }
}

template <typename R>
void gemm_batched(const GemmP<R>* dP, int batch, int maxM, int maxN, bool tA, bool tB, R alpha,
                  R beta, cudaStream_t s) {
  if (batch <= 0 || maxM <= 0 || maxN <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "gemm batch too large");
  dim3 grid(ceil_div(maxM, 64), ceil_div(maxN, 64), batch);
  HSS_REQUIRE(grid.y <= 65535, HSS_ERR_ARG, "gemm N too large");
  if (!tA && !tB) k_gemm<R, false, false><<<grid, 256, 0, s>>>(dP, alpha, beta);
  else if (!tA && tB) k_gemm<R, false, true><<<grid, 256, 0, s>>>(dP, alpha, beta);
  else if (tA && !tB) k_gemm<R, true, false><<<grid, 256, 0, s>>>(dP, alpha, beta);
  else k_gemm<R, true, true><<<grid, 256, 0, s>>>(dP, alpha, beta);
  check_launch("k_gemm");
}

// ---------------------------------------------------------------------------
// Skinny GEMM: C (M x N, N <= 8) = alpha*A(M x K)*B(K x N) + beta*C.
//
// The right-hand-side products of a solve.  A CTA owns 32*V rows (V = 16-byte
// vector width: 4 floats or 2 doubles per lane); its 8 warps take interleaved
// k of the CTA's K range; B is staged in shared memory in chunks of SK_KC rows
// so every k costs one 16-byte load of A and a broadcast shared-memory read of
// B.  Under-filled launches split K over ksplit CTAs whose partial sums go to a
// workspace and are added in a fixed order by k_skinny_reduce, so results are
// bitwise reproducible.
// ---------------------------------------------------------------------------
template <typename R> struct Vec16;
template <> struct Vec16<float> { using T = float4; static constexpr int V = 4; };
template <> struct Vec16<double> { using T = double2; static constexpr int V = 2; };

constexpr int SK_KC = 128;

template <typename R>
__device__ __forceinline__ void unpack16(const typename Vec16<R>::T& t, R* a);
template <>
__device__ __forceinline__ void unpack16<float>(const float4& t, float* a) { a[0] = t.x; a[1] = t.y; a[2] = t.z; a[3] = t.w; }
template <>
__device__ __forceinline__ void unpack16<double>(const double2& t, double* a) { a[0] = t.x; a[1] = t.y; }

template <typename R, int NR>
__global__ void __launch_bounds__(256) k_skinny(const GemmP<R>* __restrict__ P, R alpha, R beta, int ksplit,
                                                R* __restrict__ part, int mmax) {
  using VT = typename Vec16<R>::T;
  constexpr int V = Vec16<R>::V;
  constexpr int ROWS = 32 * V;
  const GemmP<R> p = P[blockIdx.z];
  const int row0 = blockIdx.x * ROWS;
  if (row0 >= p.M) return;
  const int N = p.N;
  const int kper = (((p.K + ksplit - 1) / ksplit) + 7) & ~7;
  const int kb = blockIdx.y * kper, ke = min(p.K, kb + kper);
  __shared__ __align__(16) R Bs[SK_KC][NR];
  __shared__ R red[8][NR][ROWS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int r = row0 + lane * V;
  const bool vec_ok = ((p.lda % V) == 0) && ((reinterpret_cast<uintptr_t>(p.A) & 15) == 0);
  R acc[V][NR];
#pragma unroll
  for (int v = 0; v < V; ++v)
#pragma unroll
    for (int c = 0; c < NR; ++c) acc[v][c] = R(0);
  for (int kc = kb; kc < ke; kc += SK_KC) {
    const int kn = min(SK_KC, ke - kc);
    __syncthreads();
    for (int e = threadIdx.x; e < SK_KC * NR; e += 256) {
      const int kk = e % SK_KC, c = e / SK_KC;
      Bs[kk][c] = (kk < kn && c < N) ? p.B[(size_t)(kc + kk) + (size_t)c * p.ldb] : R(0);
    }
    __syncthreads();
    for (int kk = w; kk < kn; kk += 8) {
      const R* col = p.A + (size_t)(kc + kk) * p.lda;
      R a[V];
      if (vec_ok && r + V <= p.M) {
        unpack16<R>(__ldg(reinterpret_cast<const VT*>(col + r)), a);
      } else {
#pragma unroll
        for (int v = 0; v < V; ++v) a[v] = (r + v < p.M) ? __ldg(col + r + v) : R(0);
      }
      R b[NR];
#pragma unroll
      for (int c = 0; c < NR; ++c) b[c] = Bs[kk][c];
#pragma unroll
      for (int v = 0; v < V; ++v)
#pragma unroll
        for (int c = 0; c < NR; ++c) acc[v][c] += a[v] * b[c];
    }
  }
#pragma unroll
  for (int v = 0; v < V; ++v)
#pragma unroll
    for (int c = 0; c < NR; ++c) red[w][c][lane * V + v] = acc[v][c];
  __syncthreads();
  for (int e = threadIdx.x; e < ROWS * N; e += 256) {
    const int rr = e % ROWS, c = e / ROWS;
    const int row = row0 + rr;
    if (row >= p.M) continue;
    R t = red[0][c][rr];
#pragma unroll
    for (int q = 1; q < 8; ++q) t += red[q][c][rr];
    if (ksplit == 1) {
      R* cp = p.C + row + (size_t)c * p.ldc;
      *cp = (beta == R(0)) ? alpha * t : alpha * t + beta * (*cp);
    } else {
      part[(((size_t)blockIdx.z * ksplit + blockIdx.y) * 8 + c) * mmax + row] = t;
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_skinny_reduce(const GemmP<R>* __restrict__ P, R alpha, R beta, int ksplit,
                                                       const R* __restrict__ part, int mmax) {
  const GemmP<R> p = P[blockIdx.y];
  for (int e = blockIdx.x * 256 + threadIdx.x; e < p.M * p.N; e += gridDim.x * 256) {
    const int row = e % p.M, c = e / p.M;
    R t = R(0);
    for (int y = 0; y < ksplit; ++y) t += part[(((size_t)blockIdx.y * ksplit + y) * 8 + c) * mmax + row];
    R* cp = p.C + row + (size_t)c * p.ldc;
    *cp = (beta == R(0)) ? alpha * t : alpha * t + beta * (*cp);
  }
}

// ---- double-float skinny product ----------------------------------------
// (sh, sl) += (ah + al) * (bh + bl) to ~2^-48 relative: p + e = ah*bh exactly
// (FMA error term), t = ah*bl + al*bh + e, TwoSum (Knuth) of sh and p, then a
// Fast2Sum renormalisation keeps |sl| <= ulp(sh)/2.  al*bl (2^-48) is dropped.
// Intrinsics keep the compiler from contracting or reassociating any step.
__device__ __forceinline__ void df_madd(float& sh, float& sl, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  const float e = __fmaf_rn(ah, bh, -p);
  const float t = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, e));
  const float s = __fadd_rn(sh, p);
  const float bb = __fsub_rn(s, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  const float lo = __fadd_rn(sl, __fadd_rn(err, t));
  const float hi = __fadd_rn(s, lo);
  sl = __fsub_rn(lo, __fsub_rn(hi, s));
  sh = hi;
}

// x = hi + lo to 2^-47 relative using integer operations only (GB300 runs
// double<->float conversions on its narrow FP64 pipe): hi keeps the sign, the
// exponent and the top 23 stored mantissa bits, lo the remaining 29 bits,
// renormalised and truncated to 24.  Entries below 2^-102 lose lo (float
// underflow); outside the float exponent range the FP64 conversion is used.
__device__ __forceinline__ void split_d2f(double x, float& hi, float& lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned int sign = (unsigned int)(u >> 32) & 0x80000000u;
  const int e = (int)((u >> 52) & 0x7FF);
  const int ef = e - 896;
  if ((u << 1) == 0ULL) {  // +-0 (padding and structural zeros stay off the FP64 pipe)
    hi = __uint_as_float(sign);
    lo = 0.f;
    return;
  }
  if (ef <= 0 || ef >= 255) {
    hi = __double2float_rn(x);
    lo = 0.f;
    return;
  }
  hi = __uint_as_float(sign | ((unsigned int)ef << 23) | (unsigned int)((u >> 29) & 0x7FFFFFu));
  const unsigned int ml = (unsigned int)(u & 0x1FFFFFFFu);
  const int lz = __clz(ml);
  const int efl = e - 917 - lz;
  if (ml == 0u || efl <= 0) {
    lo = 0.f;
    return;
  }
  const int sh = lz - 8;
  const unsigned int mm = (sh >= 0) ? (ml << sh) : (ml >> (-sh));
  lo = __uint_as_float(sign | ((unsigned int)efl << 23) | (mm & 0x7FFFFFu));
}

// (ah, al) += (bh, bl): TwoSum of the high parts, the low parts and the error
// added, Fast2Sum renormalisation.  FP32 pipes only.
__device__ __forceinline__ void df_add(float& ah, float& al, float bh, float bl) {
  const float s = __fadd_rn(ah, bh);
  const float bb = __fsub_rn(s, ah);
  const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
  const float lo = __fadd_rn(__fadd_rn(al, bl), err);
  const float hi = __fadd_rn(s, lo);
  al = __fsub_rn(lo, __fsub_rn(hi, s));
  ah = hi;
}

// (ah, al) *= (bh, bl) to ~2^-47 (exact high product plus cross terms).
__device__ __forceinline__ void df_mul(float& ah, float& al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  const float e = __fmaf_rn(ah, bh, -p);
  const float t = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, e));
  const float hi = __fadd_rn(p, t);
  al = __fsub_rn(t, __fsub_rn(hi, p));
  ah = hi;
}

// double nearest-below-rounding of hi + lo (|lo| <= ulp(hi)/2), integer operations
// only: hi's 24-bit significand widened to 53 bits, lo's aligned and added or
// subtracted, one renormalisation step.  Zero, tiny, huge and non-finite hi take
// the FP64 conversion path.
__device__ __forceinline__ double df_to_double(float hi, float lo) {
  const unsigned int hb = __float_as_uint(hi), lb = __float_as_uint(lo);
  const int eh = (int)((hb >> 23) & 0xFF), el = (int)((lb >> 23) & 0xFF);
  if ((hb << 1) == 0u && (lb << 1) == 0u) return __longlong_as_double((long long)((unsigned long long)hb << 32));
  if (eh == 0 || eh == 255 || el == 255) return (double)hi + (double)lo;
  long long M = (long long)((1ULL << 52) | ((unsigned long long)(hb & 0x7FFFFFu) << 29));
  int e = eh + 896;  // double biased exponent of hi
  if (el != 0) {
    const long long L = (long long)((1u << 23) | (lb & 0x7FFFFFu));
    const int g = eh - el;  // >= 24 after renormalisation
    long long Ls = 0;
    if (g <= 29) Ls = L << (29 - g);
    else if (g < 29 + 24) Ls = L >> (g - 29);
    M = ((hb ^ lb) & 0x80000000u) ? M - Ls : M + Ls;
    if (M >= (1LL << 53)) { M >>= 1; ++e; }
    else if (M < (1LL << 52)) { M <<= 1; --e; }
  }
  const unsigned long long bits = ((unsigned long long)(hb & 0x80000000u) << 32) | ((unsigned long long)e << 52) |
                                  ((unsigned long long)M & ((1ULL << 52) - 1));
  return __longlong_as_double((long long)bits);
}

// out = alpha * t + beta * C for a double-float t, stored as FP64.
__device__ __forceinline__ double df_epilogue(float th, float tl, float ah, float al, double beta, double c) {
  df_mul(th, tl, ah, al);
  if (beta != 0.0) {
    float ch, cl, bh, bl;
    split_d2f(c, ch, cl);
    split_d2f(beta, bh, bl);
    df_mul(ch, cl, bh, bl);
    df_add(th, tl, ch, cl);
  }
  return df_to_double(th, tl);
}

// Sum of a double-float value over a warp (xor butterfly); every lane gets the same (h, l).
__device__ __forceinline__ void warp_sum_df(float& h, float& l) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, h, o), ol = __shfl_xor_sync(0xffffffffu, l, o);
    df_add(h, l, oh, ol);
  }
}

// Paired-FP32 SIMD (sm_100+ f32x2): two lanes of FP32 per instruction, used for
// the two rows a thread owns.  Values are 64-bit registers {row0, row1}.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 x2_add(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_sub(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_mul(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_fma(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f32x2 x2_pack(float a, float b) {
  f32x2 d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(a), "f"(b));
  return d;
}
__device__ __forceinline__ void x2_unpack(f32x2 d, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(d));
}

// df_madd on two rows at once.  bh2 = (bh, bh), bhn2 = -bh2, bln2 = -(bl, bl).
// en = ah*(-bh) + p = -(exact error of p); tn = -(ah*bl + al*bh + e).  The high
// sum takes the TwoSum of p; every low-order term (its rounding error and tn)
// goes into sl, renormalised only at the end: the loop-carried chain is one add
// for sh and one for sl, so the eight accumulators of a thread overlap.  sl then
// carries ~2^-24 |sl| per step, ~K 2^-48 of the sum over K steps.
__device__ __forceinline__ void df_madd_x2(f32x2& sh, f32x2& sl, f32x2 ah, f32x2 al, f32x2 bh2, f32x2 bhn2,
                                           f32x2 bln2) {
  const f32x2 p = x2_mul(ah, bh2);
  const f32x2 en = x2_fma(ah, bhn2, p);
  const f32x2 tn = x2_fma(ah, bln2, x2_fma(al, bhn2, en));
  const f32x2 s = x2_add(sh, p);
  const f32x2 bb = x2_sub(s, sh);
  const f32x2 err = x2_add(x2_sub(sh, x2_sub(s, bb)), x2_sub(p, bb));
  sl = x2_add(sl, x2_sub(err, tn));
  sh = s;
}

// Operand access of the double-float skinny kernel for a plain or a segmented product.
__device__ __forceinline__ int dfd_K(const GemmP<double>& p) { return p.K; }
__device__ __forceinline__ const float2* dfd_col(const GemmP<double>& p, int k) {
  return reinterpret_cast<const float2*>(p.A) + (size_t)k * p.lda;
}
__device__ __forceinline__ double dfd_b(const GemmP<double>& p, int k, int c) { return p.B[k + (size_t)c * p.ldb]; }
__device__ __forceinline__ bool dfd_vec_ok(const GemmP<double>& p) {
  return (p.lda % 2) == 0 && (reinterpret_cast<uintptr_t>(p.A) & 15) == 0;
}
__device__ __forceinline__ int dfd_K(const SegGemmP& p) { return p.K[0] + p.K[1] + p.K[2]; }
__device__ __forceinline__ int dfd_seg(const SegGemmP& p, int& k) {
  if (k < p.K[0]) return 0;
  k -= p.K[0];
  if (k < p.K[1]) return 1;
  k -= p.K[1];
  return 2;
}
// (selects rather than an indexed member array: a dynamic index would put the
// descriptor in local memory)
__device__ __forceinline__ const float2* dfd_col(const SegGemmP& p, int k) {
  const int sg = dfd_seg(p, k);
  const double* a = sg == 0 ? p.A[0] : (sg == 1 ? p.A[1] : p.A[2]);
  const int ld = sg == 0 ? p.lda[0] : (sg == 1 ? p.lda[1] : p.lda[2]);
  return reinterpret_cast<const float2*>(a) + (size_t)k * ld;
}
__device__ __forceinline__ double dfd_b(const SegGemmP& p, int k, int c) {
  const int sg = dfd_seg(p, k);
  const double* b = sg == 0 ? p.B[0] : (sg == 1 ? p.B[1] : p.B[2]);
  const int ld = sg == 0 ? p.ldb[0] : (sg == 1 ? p.ldb[1] : p.ldb[2]);
  const double sn = sg == 0 ? p.sign[0] : (sg == 1 ? p.sign[1] : p.sign[2]);
  return sn * b[k + (size_t)c * ld];
}
__device__ __forceinline__ bool dfd_vec_ok(const SegGemmP& p) {
  bool ok = true;
#pragma unroll
  for (int sg = 0; sg < 3; ++sg)
    if (p.K[sg] > 0) ok = ok && (p.lda[sg] % 2) == 0 && (reinterpret_cast<uintptr_t>(p.A[sg]) & 15) == 0;
  return ok;
}

constexpr int SKD_STAGES = 4;  // cp.async columns in flight per thread (<= 4 right-hand sides)

// One element of a double-float copy in the pair-interleaved layout of split_df: the
// 16-byte block holding elements (2i, 2i+1) of the array is (h_2i, h_2i+1, l_2i, l_2i+1).
// Arrays start on 16-byte boundaries, so an element's slot follows from its address.
__device__ __forceinline__ void dfd_elem(const float2* e, float& h, float& l) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(e);
  const float* blk = reinterpret_cast<const float*>(a & ~(uintptr_t)15);
  const int par = (int)((a >> 3) & 1);
  h = __ldg(blk + par);
  l = __ldg(blk + 2 + par);
}

// Column step of the cp.async ring: GemmP columns advance by a fixed stride, segmented
// columns are looked up (they may cross into the next segment).
template <typename D>
struct DfCols {
  const char* base;
  size_t step;
  __device__ __forceinline__ DfCols(const D& p, int k0, int r) {
    if constexpr (std::is_same<D, GemmP<double>>::value) {
      base = reinterpret_cast<const char*>(dfd_col(p, k0) + r);
      step = (size_t)8 * p.lda * sizeof(float2);
    } else {
      base = nullptr;
      step = 0;
    }
  }
  // address of row r of column k0 + 8 it
  __device__ __forceinline__ const void* at(const D& p, int k0, int it, int r) const {
    if constexpr (std::is_same<D, GemmP<double>>::value) return base + (size_t)it * step;
    else return dfd_col(p, k0 + 8 * it) + r;
  }
};

template <int NR, typename D>
__global__ void __launch_bounds__(256, (NR > 4) ? 3 : 4) k_skinny_df(const D* __restrict__ P, double alpha, double beta,
                                                   int ksplit, double* __restrict__ part, int mmax) {
  constexpr int V = 2;  // one 16-byte load = the (hi, hi, lo, lo) block of two rows
  constexpr int KC = (NR > 4) ? SK_KC / 2 : SK_KC;  // static shared memory under 48 KB
  constexpr int ROWS = 32 * V;
  const D p = P[blockIdx.z];
  const int row0 = blockIdx.x * ROWS;
  if (row0 >= p.M) return;
  const int N = p.N;
  const int Kt = dfd_K(p);
  const int kper = (((Kt + ksplit - 1) / ksplit) + 7) & ~7;
  const int kb = blockIdx.y * kper, ke = min(Kt, kb + kper);
  // per column: (bh, bh) x NR, (-bh, -bh) x NR, (-bl, -bl) x NR, read two right-hand sides
  // per 16-byte load
  __shared__ __align__(16) f32x2 Bs[KC][3][NR];
  __shared__ float2 red[8][NR][ROWS];
  __shared__ __align__(16) ulonglong2 ring[(NR <= 4) ? SKD_STAGES : 1][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int r = row0 + lane * V;
  const bool vec_ok = dfd_vec_ok(p);
  f32x2 sh[NR], sl[NR];  // {row r, row r+1} accumulators
#pragma unroll
  for (int c = 0; c < NR; ++c) { sh[c] = 0ULL; sl[c] = 0ULL; }
  auto madd = [&](f32x2 ah, f32x2 al, const f32x2* b) {
#pragma unroll
    for (int c = 0; c < NR; c += 2) {
      const ulonglong2 bh = *reinterpret_cast<const ulonglong2*>(b + c);
      const ulonglong2 bn = *reinterpret_cast<const ulonglong2*>(b + NR + c);
      const ulonglong2 bl = *reinterpret_cast<const ulonglong2*>(b + 2 * NR + c);
      df_madd_x2(sh[c], sl[c], ah, al, bh.x, bn.x, bl.x);
      df_madd_x2(sh[c + 1], sl[c + 1], ah, al, bh.y, bn.y, bl.y);
    }
  };
  for (int kc = kb; kc < ke; kc += KC) {
    const int kn = min(KC, ke - kc);
    __syncthreads();
    for (int e = threadIdx.x; e < KC * NR; e += 256) {
      const int kk = e % KC, c = e / KC;
      const double x = (kk < kn && c < N) ? dfd_b(p, kc + kk, c) : 0.0;
      float xh, xl;
      split_d2f(x, xh, xl);
      Bs[kk][0][c] = x2_pack(xh, xh);
      Bs[kk][1][c] = x2_pack(-xh, -xh);
      Bs[kk][2][c] = x2_pack(-xl, -xl);
    }
    __syncthreads();
    if constexpr (NR <= 4) {
      if (vec_ok) {
        // cp.async ring: each thread keeps its next SKD_STAGES columns' 16 bytes in
        // flight into its own shared-memory slots (it reads only what it copied, so
        // the per-thread group wait is the only synchronisation needed).  With even
        // leading dimensions a row pair inside the matrix is a whole 16-byte block
        // (for odd M the partner of the last row is padding of the same column).
        const int niter = (w < kn) ? (kn - w + 7) / 8 : 0;
        const int nv = (r < p.M) ? 16 : 0;
        const DfCols<D> cols(p, kc + w, nv ? r : 0);
        const void* dummy = dfd_col(p, kc);
        const unsigned ring0 = (unsigned)__cvta_generic_to_shared(&ring[0][threadIdx.x]);
        auto issue = [&](int it) {
          const bool live = it < niter;
          const void* src = live ? cols.at(p, kc + w, it, nv ? r : 0) : dummy;
          const unsigned dst = ring0 + (unsigned)((it % SKD_STAGES) * 256 * sizeof(ulonglong2));
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(live ? nv : 0));
          asm volatile("cp.async.commit_group;\n" ::);
        };
#pragma unroll
        for (int it = 0; it < SKD_STAGES; ++it) issue(it);
        for (int it = 0; it < niter; ++it) {
          asm volatile("cp.async.wait_group %0;\n" ::"n"(SKD_STAGES - 1));
          const ulonglong2 a = ring[it % SKD_STAGES][threadIdx.x];
          madd(a.x, a.y, &Bs[w + 8 * it][0][0]);
          issue(it + SKD_STAGES);
        }
        asm volatile("cp.async.wait_all;\n" ::);
        continue;
      }
    }
    // software-pipelined: the next column's 16 bytes are in flight during this column's math
    auto load = [&](int kk) -> ulonglong2 {
      const float2* col = dfd_col(p, kc + kk);
      if (vec_ok && r < p.M) return __ldg(reinterpret_cast<const ulonglong2*>(col + r));
      float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
      if (r < p.M) dfd_elem(col + r, h0, l0);
      if (r + 1 < p.M) dfd_elem(col + r + 1, h1, l1);
      return make_ulonglong2(x2_pack(h0, h1), x2_pack(l0, l1));
    };
    ulonglong2 cur = (w < kn) ? load(w) : make_ulonglong2(0ULL, 0ULL);
    for (int kk = w; kk < kn; kk += 8) {
      const ulonglong2 nxt = (kk + 8 < kn) ? load(kk + 8) : make_ulonglong2(0ULL, 0ULL);
      madd(cur.x, cur.y, &Bs[kk][0][0]);
      cur = nxt;
    }
  }
#pragma unroll
  for (int c = 0; c < NR; ++c) {
    const f32x2 hi = x2_add(sh[c], sl[c]);  // Fast2Sum renormalisation
    const f32x2 lo = x2_sub(sl[c], x2_sub(hi, sh[c]));
    float h0, h1, l0, l1;
    x2_unpack(hi, h0, h1);
    x2_unpack(lo, l0, l1);
    red[w][c][lane * V] = make_float2(h0, l0);
    red[w][c][lane * V + 1] = make_float2(h1, l1);
  }
  __syncthreads();
  float alh, all;
  split_d2f(alpha, alh, all);
  for (int e = threadIdx.x; e < ROWS * N; e += 256) {
    const int rr = e % ROWS, c = e / ROWS;
    const int row = row0 + rr;
    if (row >= p.M) continue;
    float th = red[0][c][rr].x, tl = red[0][c][rr].y;
#pragma unroll
    for (int q = 1; q < 8; ++q) df_add(th, tl, red[q][c][rr].x, red[q][c][rr].y);
    if (ksplit == 1) {
      double* cp = p.C + row + (size_t)c * p.ldc;
      *cp = df_epilogue(th, tl, alh, all, beta, (beta == 0.0) ? 0.0 : *cp);
    } else {
      reinterpret_cast<float2*>(part)[(((size_t)blockIdx.z * ksplit + blockIdx.y) * 8 + c) * mmax + row] =
          make_float2(th, tl);
    }
  }
}

// split-K partials of k_skinny_df (float pairs) summed in double-float arithmetic.
// Block (64 rows of one right-hand side of one product) x 4 slice groups: group g sums
// the slices y = g mod 4 in order, and the four group sums are combined as
// (0 + 1) + (2 + 3).
template <typename D>
__global__ void __launch_bounds__(256) k_skinny_reduce_df(const D* __restrict__ P, double alpha,
                                                          double beta, int ksplit, const double* __restrict__ part,
                                                          int mmax) {
  const D p = P[blockIdx.z];
  const int c = blockIdx.y;
  if (c >= p.N || (int)blockIdx.x * 64 >= p.M) return;
  const float2* pp = reinterpret_cast<const float2*>(part);
  const int g = threadIdx.x >> 6, rr = threadIdx.x & 63;
  const int row = blockIdx.x * 64 + rr;
  __shared__ float2 gs[4][64];
  float th = 0.f, tl = 0.f;
  if (row < p.M) {
#pragma unroll 4
    for (int y = g; y < ksplit; y += 4) {
      const float2 q = pp[(((size_t)blockIdx.z * ksplit + y) * 8 + c) * mmax + row];
      df_add(th, tl, q.x, q.y);
    }
  }
  gs[g][rr] = make_float2(th, tl);
  __syncthreads();
  if (g != 0 || row >= p.M) return;
  float h0 = gs[0][rr].x, l0 = gs[0][rr].y, h2 = gs[2][rr].x, l2 = gs[2][rr].y;
  df_add(h0, l0, gs[1][rr].x, gs[1][rr].y);
  df_add(h2, l2, gs[3][rr].x, gs[3][rr].y);
  df_add(h0, l0, h2, l2);
  float alh, all;
  split_d2f(alpha, alh, all);
  double* cp = p.C + row + (size_t)c * p.ldc;
  *cp = df_epilogue(h0, l0, alh, all, beta, (beta == 0.0) ? 0.0 : *cp);
}

// Pair-interleaved float-pair copy: elements (2i, 2i+1) become the 16-byte block
// (h_2i, h_2i+1, l_2i, l_2i+1), so a row pair of a column is one load whose halves are
// the paired-FP32 operands directly.  An odd count leaves a zero partner in the last
// block (dst holds n rounded up to even elements).
__global__ void k_split_df(const double* __restrict__ src, float4* __restrict__ dst, long long n) {
  const long long npair = (n + 1) / 2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npair; i += (long long)gridDim.x * blockDim.x) {
    const double x0 = src[2 * i];
    const double x1 = (2 * i + 1 < n) ? src[2 * i + 1] : 0.0;
    const float h0 = __double2float_rn(x0), h1 = __double2float_rn(x1);
    dst[i] = make_float4(h0, h1, __double2float_rn(__dsub_rn(x0, (double)h0)), __double2float_rn(__dsub_rn(x1, (double)h1)));
  }
}

void split_df(const double* src, double* dst, long long n, cudaStream_t s) {
  if (n <= 0) return;
  HSS_REQUIRE((reinterpret_cast<uintptr_t>(dst) & 15) == 0, HSS_ERR_ARG, "split_df: destination not 16-byte aligned");
  const long long npair = (n + 1) / 2;
  k_split_df<<<std::min(ceil_div(npair, 256), 4096), 256, 0, s>>>(src, reinterpret_cast<float4*>(dst), n);
  check_launch("k_split_df");
}

// ---- double-float tiled GEMM ----------------------------------------------
// C = alpha op(A) op(B) + beta C for FP64 operands in memory, computed in
// double-float arithmetic (~2^-47 per product).  64x64 tile, K step 16, 256
// threads, 4x4 outputs per thread as two f32x2 row pairs.  Tiles are split
// into (hi, lo) floats with integer operations while staging; the B tile is
// also kept negated for the exact-product error terms.  The accumulators are
// renormalised after every K step and combined to FP64 with integer operations.
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) k_gemm_df(const GemmP<double>* __restrict__ P, double alpha, double beta) {
  const GemmP<double> p = P[blockIdx.z];
  const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  if (m0 >= p.M || n0 >= p.N) return;
  __shared__ float Ah[16][64 + 1], Al[16][64 + 1];
  __shared__ float Bh[16][64 + 1], Bhn[16][64 + 1], Bln[16][64 + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  f32x2 sh[2][4], sl[2][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) { sh[i][j] = 0ULL; sl[i][j] = 0ULL; }
  for (int k0 = 0; k0 < p.K; k0 += 16) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + 256 * r;
      int i, kk;
      if (!TA) { i = e & 63; kk = e >> 6; } else { kk = e & 15; i = e >> 4; }
      const int gi = m0 + i, gk = k0 + kk;
      double v = 0.0;
      if (gi < p.M && gk < p.K) v = TA ? p.A[gk + (size_t)gi * p.lda] : p.A[gi + (size_t)gk * p.lda];
      float h, l;
      split_d2f(v, h, l);
      Ah[kk][i] = h;
      Al[kk][i] = l;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + 256 * r;
      int j, kk;
      if (!TB) { kk = e & 15; j = e >> 4; } else { j = e & 63; kk = e >> 6; }
      const int gj = n0 + j, gk = k0 + kk;
      double v = 0.0;
      if (gj < p.N && gk < p.K) v = TB ? p.B[gj + (size_t)gk * p.ldb] : p.B[gk + (size_t)gj * p.ldb];
      float h, l;
      split_d2f(v, h, l);
      Bh[kk][j] = h;
      Bhn[kk][j] = -h;
      Bln[kk][j] = -l;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < 16; ++kk) {
      const f32x2 ah0 = x2_pack(Ah[kk][tx], Ah[kk][tx + 16]), al0 = x2_pack(Al[kk][tx], Al[kk][tx + 16]);
      const f32x2 ah1 = x2_pack(Ah[kk][tx + 32], Ah[kk][tx + 48]), al1 = x2_pack(Al[kk][tx + 32], Al[kk][tx + 48]);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = ty + 16 * j;
        const float bh = Bh[kk][c], bhn = Bhn[kk][c], bln = Bln[kk][c];
        const f32x2 bh2 = x2_pack(bh, bh), bhn2 = x2_pack(bhn, bhn), bln2 = x2_pack(bln, bln);
        df_madd_x2(sh[0][j], sl[0][j], ah0, al0, bh2, bhn2, bln2);
        df_madd_x2(sh[1][j], sl[1][j], ah1, al1, bh2, bhn2, bln2);
      }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const f32x2 hi = x2_add(sh[i][j], sl[i][j]);
        sl[i][j] = x2_sub(sl[i][j], x2_sub(hi, sh[i][j]));
        sh[i][j] = hi;
      }
    __syncthreads();
  }
  float alh, all;
  split_d2f(alpha, alh, all);
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    float h[2], l[2];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      x2_unpack(sh[i][j], h[0], h[1]);
      x2_unpack(sl[i][j], l[0], l[1]);
      const int gj = n0 + ty + 16 * j;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int gi = m0 + tx + 16 * (2 * i + u);
        if (gi >= p.M || gj >= p.N) continue;
        double* c = p.C + gi + (size_t)gj * p.ldc;
        *c = df_epilogue(h[u], l[u], alh, all, beta, (beta == 0.0) ? 0.0 : *c);
      }
    }
  }
}

void gemm_batched_df(const GemmP<double>* dP, int batch, int maxM, int maxN, bool tA, bool tB, double alpha,
                     double beta, cudaStream_t s) {
  if (batch <= 0 || maxM <= 0 || maxN <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "gemm batch too large");
  dim3 grid(ceil_div(maxM, 64), ceil_div(maxN, 64), batch);
  HSS_REQUIRE(grid.y <= 65535, HSS_ERR_ARG, "gemm N too large");
  if (!tA && !tB) k_gemm_df<false, false><<<grid, 256, 0, s>>>(dP, alpha, beta);
  else if (!tA && tB) k_gemm_df<false, true><<<grid, 256, 0, s>>>(dP, alpha, beta);
  else if (tA && !tB) k_gemm_df<true, false><<<grid, 256, 0, s>>>(dP, alpha, beta);
  else k_gemm_df<true, true><<<grid, 256, 0, s>>>(dP, alpha, beta);
  check_launch("k_gemm_df");
}

template <typename R>
int skinny_ksplit(int batch, int maxM, int maxK) {
  constexpr int ROWS = 32 * Vec16<R>::V;
  const long long ctas = (long long)ceil_div(maxM, ROWS) * batch;
  if (ctas >= 304 || maxK < 256) return 1;
  int ks = (int)std::min<long long>(16, (304 + ctas - 1) / ctas);
  ks = std::max(1, std::min(ks, maxK / 128));
  return ks;
}

template <typename R>
void gemm_skinny_split(const GemmP<R>* dP, int batch, int maxM, int maxN, R alpha, R beta, int ksplit, R* part,
                       cudaStream_t s) {
  if (batch <= 0 || maxM <= 0) return;
  HSS_REQUIRE(batch <= 65535 && maxN <= 8, HSS_ERR_ARG, "skinny gemm: batch <= 65535 and N <= 8");
  HSS_REQUIRE(ksplit == 1 || part != nullptr, HSS_ERR_ARG, "skinny gemm: split-K needs a workspace");
  constexpr int ROWS = 32 * Vec16<R>::V;
  dim3 grid(ceil_div(maxM, ROWS), ksplit, batch);
  if (maxN <= 4) k_skinny<R, 4><<<grid, 256, 0, s>>>(dP, alpha, beta, ksplit, part, maxM);
  else k_skinny<R, 8><<<grid, 256, 0, s>>>(dP, alpha, beta, ksplit, part, maxM);
  check_launch("k_skinny");
  if (ksplit > 1) {
    const int gx = std::max(1, std::min(ceil_div((long long)maxM * maxN, 256), 64));
    k_skinny_reduce<R><<<dim3(gx, batch), 256, 0, s>>>(dP, alpha, beta, ksplit, part, maxM);
    check_launch("k_skinny_reduce");
  }
}

int skinny_ksplit_df(int batch, int maxM, int maxK) {
  const long long ctas = (long long)ceil_div(maxM, 64) * batch;
  if (ctas >= 1216 || maxK < 128) return 1;
  int ks = (int)std::min<long long>(32, (1216 + ctas - 1) / ctas);
  ks = std::max(1, std::min(ks, maxK / 64));
  return ks;
}

template <typename D>
static void skinny_df_launch(const D* dP, int batch, int maxM, int maxN, double alpha, double beta, int ksplit,
                             double* part, cudaStream_t s) {
  if (batch <= 0 || maxM <= 0) return;
  HSS_REQUIRE(batch <= 65535 && maxN <= 8, HSS_ERR_ARG, "skinny gemm: batch <= 65535 and N <= 8");
  HSS_REQUIRE(ksplit == 1 || part != nullptr, HSS_ERR_ARG, "skinny gemm: split-K needs a workspace");
  dim3 grid(ceil_div(maxM, 64), ksplit, batch);
  if (maxN <= 4) k_skinny_df<4, D><<<grid, 256, 0, s>>>(dP, alpha, beta, ksplit, part, maxM);
  else k_skinny_df<8, D><<<grid, 256, 0, s>>>(dP, alpha, beta, ksplit, part, maxM);
  check_launch("k_skinny_df");
  if (ksplit > 1) {
    k_skinny_reduce_df<D><<<dim3(ceil_div(maxM, 64), maxN, batch), 256, 0, s>>>(dP, alpha, beta, ksplit, part, maxM);
    check_launch("k_skinny_reduce_df");
  }
}

void gemm_skinny_split_df(const GemmP<double>* dP, int batch, int maxM, int maxN, double alpha, double beta,
                          int ksplit, double* part, cudaStream_t s) {
  skinny_df_launch(dP, batch, maxM, maxN, alpha, beta, ksplit, part, s);
}

void gemm_skinny_split_df(const SegGemmP* dP, int batch, int maxM, int maxN, double alpha, double beta,
                          int ksplit, double* part, cudaStream_t s) {
  skinny_df_launch(dP, batch, maxM, maxN, alpha, beta, ksplit, part, s);
}

template <typename R>
void gemm_skinny(const GemmP<R>* dP, int batch, int maxM, R alpha, R beta, cudaStream_t s) {
  gemm_skinny_split<R>(dP, batch, maxM, 8, alpha, beta, 1, nullptr, s);
}

// ---------------------------------------------------------------------------
// Blocked Gauss-Jordan inversion with partial pivoting.
//
// Per block of GJ_NB columns:
//  1. k_gj_panel_cl: one thread-block cluster per matrix factors the panel
//     (all n rows x GJ_NB columns) held in the distributed shared memory of the
//     cluster (rows split across the CTAs).  Pivot search, pivot-row exchange
//     and elimination run on the panel columns only; the interchanges are
//     recorded in ipiv.
//  2. k_gj_gather: the row interchanges of the block are composed into a row
//     map; the rows it touches (panel rows and the rows they displaced) are
//     copied, for every non-panel column, into W.
//  3. k_gj_update: every non-panel column is permuted and updated with the
//     panel: A(:,c) = base(:,c) + P * W(pivot rows, c), base being 0 on the
//     panel rows, the displaced row content on the displaced rows and A(:,c)
//     elsewhere.
// The cluster barriers are reached the same number of times by every CTA of
// a cluster (all of them take the same pivot decisions), so they cannot hang.
// ---------------------------------------------------------------------------
namespace cg = cooperative_groups;

template <typename R>
__device__ void block_argmax_any(R& val, int& idx, R* shv, int* shi) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    R ov = __shfl_xor_sync(0xffffffffu, val, o);
    int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > val || (ov == val && oi < idx)) { val = ov; idx = oi; }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) { shv[w] = val; shi[w] = idx; }
  __syncthreads();
  val = shv[0];
  idx = shi[0];
  for (int i = 1; i < nw; ++i)
    if (shv[i] > val || (shv[i] == val && shi[i] < idx)) { val = shv[i]; idx = shi[i]; }
  __syncthreads();
}

// 256 threads: a clustered panel holds at most 256 rows per CTA (one row per thread), and the
// per-column chain of block barriers is shorter with 8 warps than with 16 (FP64 inversion
// 0.56 -> 0.50 s at N = 65536)
constexpr int GJ_THREADS = 256;

template <typename R>
__global__ void __launch_bounds__(GJ_THREADS) k_gj_panel_cl(const InvP<R>* __restrict__ P, int j0, int rows_per) {
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks();
  const int crank = (int)cl.block_rank();
  const InvP<R> p = P[blockIdx.x / C];
  const int n = p.n;
  if (j0 >= n) return;        // same for the whole cluster
  if (*p.info != 0) return;   // read before any CTA of this launch can write it
  extern __shared__ __align__(16) unsigned char s_raw[];
  R* pan = reinterpret_cast<R*>(s_raw);  // rows_per x GJ_NB, ld rows_per
  __shared__ R s_slot_v;
  __shared__ int s_slot_i;
  __shared__ R rowJ[GJ_NB], rowP[GJ_NB], s_row[GJ_NB];
  __shared__ R shv[32];
  __shared__ int shi[32];
  __shared__ R s_gv;
  __shared__ int s_gi;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int r0 = crank * rows_per, r1 = min(n, r0 + rows_per);
  const int jend = min(j0 + GJ_NB, n), nbk = jend - j0;
  R* A = p.A;
  const size_t lda = p.lda;
  for (int e = tid; e < rows_per * nbk; e += nt) {
    const int i = e % rows_per, c = e / rows_per;
    pan[i + c * rows_per] = (r0 + i < r1) ? A[(r0 + i) + (size_t)(j0 + c) * lda] : R(0);
  }
  __syncthreads();
  bool failed = false;
  for (int j = j0; j < jend; ++j) {
    const int jj = j - j0;
    R best = R(-1);
    int bi = INT_MAX;
    for (int i = max(j, r0) + tid; i < r1; i += nt) {
      const R v = fabs(pan[(i - r0) + jj * rows_per]);
      if (v > best) { best = v; bi = i; }
    }
    block_argmax_any(best, bi, shv, shi);
    if (tid == 0) { s_slot_v = best; s_slot_i = bi; }
    cl.sync();
    if (tid == 0) {
      R gv = R(-1);
      int gi = INT_MAX;
      for (int q = 0; q < C; ++q) {
        const R v = *cl.map_shared_rank(&s_slot_v, q);
        const int i = *cl.map_shared_rank(&s_slot_i, q);
        if (v > gv || (v == gv && i < gi)) { gv = v; gi = i; }
      }
      s_gv = gv;
      s_gi = gi;
    }
    __syncthreads();
    best = s_gv;
    bi = s_gi;
    if (bi == INT_MAX || !(best > R(0)) || !isfinite(best)) {
      if (crank == 0 && tid == 0) *p.info = (best == R(0)) ? (j + 1) : -1;
      failed = true;
      break;
    }
    const int oj = j / rows_per, ob = bi / rows_per;
    if (tid < nbk) {
      rowJ[tid] = *cl.map_shared_rank(&pan[(j - oj * rows_per) + tid * rows_per], oj);
      rowP[tid] = *cl.map_shared_rank(&pan[(bi - ob * rows_per) + tid * rows_per], ob);
    }
    cl.sync();  // every CTA holds rows j and bi before any CTA rewrites them
    // the pivot reciprocal is formed by the nbk threads that scale the pivot row only
    // (an FP64 division in every thread would cost more than the column's update)
    if (tid < nbk) {
      const R rpt = R(1) / rowP[jj];
      s_row[tid] = (tid == jj) ? rpt : rowP[tid] * rpt;
    }
    if (crank == 0 && tid == 0) p.ipiv[j] = bi;
    __syncthreads();
    const R rp = s_row[jj];
    for (int i = r0 + tid; i < r1; i += nt) {
      R* row = pan + (i - r0);
      if (i == j) {
        for (int c = 0; c < nbk; ++c) row[c * rows_per] = s_row[c];
        continue;
      }
      const bool moved = (i == bi);
      const R aij = moved ? rowJ[jj] : row[jj * rows_per];
      for (int c = 0; c < nbk; ++c) {
        if (c == jj) continue;
        const R cur = moved ? rowJ[c] : row[c * rows_per];
        row[c * rows_per] = cur - aij * s_row[c];
      }
      row[jj * rows_per] = -aij * rp;
    }
    __syncthreads();
  }
  if (!failed) {
    for (int e = tid; e < rows_per * nbk; e += nt) {
      const int i = e % rows_per, c = e / rows_per;
      if (r0 + i < r1) A[(r0 + i) + (size_t)(j0 + c) * lda] = pan[i + c * rows_per];
    }
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
}

// Compose the block's interchanges into a row map and copy the touched rows
// of every non-panel column into W: rows 0..nbk-1 = new panel rows, rows
// GJ_NB.. = new content of the displaced rows.  aux = [np, prow[GJ_NB], ...].
template <typename R>
__global__ void __launch_bounds__(256) k_gj_gather(const InvP<R>* __restrict__ P, int j0) {
  const InvP<R> p = P[blockIdx.y];
  const int n = p.n;
  if (j0 >= n) return;
  if (*p.info != 0) return;
  const int jend = min(j0 + GJ_NB, n), nbk = jend - j0;
  __shared__ int pos[2 * GJ_NB], src[2 * GJ_NB];
  __shared__ int s_np;
  __shared__ int rsrc[GJ_NB], psrc[GJ_NB];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (w == 0) {
    // warp 0 composes the block's interchanges: pos lists the rows touched (first-touch
    // order, at most 2 GJ_NB), src[q] the row whose content ends up in row pos[q]; a
    // lookup is one ballot over the list
    int cnt = 0;
    auto find = [&](int r) {
      const unsigned m0 = __ballot_sync(0xffffffffu, lane < cnt && pos[lane] == r);
      const unsigned m1 = __ballot_sync(0xffffffffu, lane + 32 < cnt && pos[lane + 32] == r);
      if (m0) return __ffs(m0) - 1;
      if (m1) return 31 + __ffs(m1);
      if (lane == 0) {
        pos[cnt] = r;
        src[cnt] = r;
      }
      __syncwarp();
      return cnt++;
    };
    for (int j = j0; j < jend; ++j) {
      const int a = find(j), b = find(p.ipiv[j]);
      if (lane == 0) {
        const int t = src[a];
        src[a] = src[b];
        src[b] = t;
      }
      __syncwarp();
    }
    for (int r = 0; r < nbk; ++r) {
      const int q = find(j0 + r);  // every row of the block was touched above
      if (lane == 0) rsrc[r] = src[q];
    }
    // the displaced rows outside the block, in list order
    int np = 0;
    for (int base = 0; base < cnt; base += 32) {
      const int q = base + lane;
      const bool take = q < cnt && (pos[q] < j0 || pos[q] >= jend) && src[q] != pos[q];
      const unsigned mk = __ballot_sync(0xffffffffu, take);
      if (take) {
        const int slot = np + __popc(mk & ((1u << lane) - 1u));
        psrc[slot] = src[q];
        if (blockIdx.x == 0) p.aux[1 + slot] = pos[q];
      }
      np += __popc(mk);
    }
    if (lane == 0) {
      s_np = np;
      if (blockIdx.x == 0) p.aux[0] = np;
    }
  }
  __syncthreads();
  // one warp per non-panel column: lane r copies the block's row r (and displaced row r)
  const int np = s_np;
  const R* __restrict__ A = p.A;
  R* __restrict__ W = p.W;
  const size_t lda = p.lda;
  const int ra = (lane < nbk) ? rsrc[lane] : 0, rb = (lane < np) ? psrc[lane] : 0;
  const int nwarp = gridDim.x * (blockDim.x >> 5);
  for (int c = blockIdx.x * (blockDim.x >> 5) + w; c < n; c += nwarp) {
    if (c >= j0 && c < jend) continue;
    const R* col = A + (size_t)c * lda;
    const R v0 = (lane < nbk) ? col[ra] : R(0);
    const R v1 = (lane < np) ? col[rb] : R(0);
    R* wc = W + (size_t)c * 2 * GJ_NB;
    if (lane < nbk) wc[lane] = v0;
    if (lane < np) wc[GJ_NB + lane] = v1;
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_gj_update(const InvP<R>* __restrict__ P, int j0) {
  const InvP<R> p = P[blockIdx.z];
  const int n = p.n;
  if (j0 >= n) return;
  if (*p.info != 0) return;
  const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  if (m0 >= n || n0 >= n) return;
  const int jend = min(j0 + GJ_NB, n), nbk = jend - j0;
  __shared__ R Ps[GJ_NB][64 + 1];
  __shared__ R Ws[GJ_NB][64 + 1];
  __shared__ int rowq[64];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  R* A = p.A;
  const size_t lda = p.lda;
  const int np = p.aux[0];
  if (tid < 64) {
    const int gi = m0 + tid;
    int q = -1;
    for (int t = 0; t < np; ++t)
      if (p.aux[1 + t] == gi) q = t;
    rowq[tid] = q;
  }
  for (int e = tid; e < 64 * GJ_NB; e += 256) {
    const int i = e & 63, r = e >> 6;
    const int gi = m0 + i;
    Ps[r][i] = (gi < n && r < nbk) ? A[gi + (size_t)(j0 + r) * lda] : R(0);
  }
  for (int e = tid; e < 64 * GJ_NB; e += 256) {
    const int r = e % GJ_NB, j = e / GJ_NB;
    const int gj = n0 + j;
    Ws[r][j] = (gj < n && r < nbk) ? p.W[r + (size_t)gj * 2 * GJ_NB] : R(0);
  }
  __syncthreads();
  R acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = R(0);
  for (int r = 0; r < nbk; ++r) {
    R a[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = Ps[r][tx + 16 * i];
#pragma unroll
    for (int j = 0; j < 4; ++j) b[j] = Ws[r][ty + 16 * j];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gj = n0 + ty + 16 * j;
    if (gj >= n || (gj >= j0 && gj < jend)) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int li = tx + 16 * i, gi = m0 + li;
      if (gi >= n) continue;
      R* c = A + gi + (size_t)gj * lda;
      R base;
      if (gi >= j0 && gi < jend) base = R(0);
      else if (rowq[li] >= 0) base = p.W[GJ_NB + rowq[li] + (size_t)gj * 2 * GJ_NB];
      else base = *c;
      *c = base + acc[i][j];
    }
  }
}

// k_gj_update in double-float arithmetic for FP64 matrices: the rank-32 panel
// product on the FP32 pipes (f32x2 row pairs), then added to the gathered base.
__global__ void __launch_bounds__(256) k_gj_update_df(const InvP<double>* __restrict__ P, int j0) {
  const InvP<double> p = P[blockIdx.z];
  const int n = p.n;
  if (j0 >= n) return;
  if (*p.info != 0) return;
  const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  if (m0 >= n || n0 >= n) return;
  const int jend = min(j0 + GJ_NB, n), nbk = jend - j0;
  __shared__ float Ph[GJ_NB][64 + 1], Pl[GJ_NB][64 + 1];
  __shared__ float Wh[GJ_NB][64 + 1], Whn[GJ_NB][64 + 1], Wln[GJ_NB][64 + 1];
  __shared__ int rowq[64];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double* A = p.A;
  const size_t lda = p.lda;
  const int np = p.aux[0];
  if (tid < 64) {
    const int gi = m0 + tid;
    int q = -1;
    for (int t = 0; t < np; ++t)
      if (p.aux[1 + t] == gi) q = t;
    rowq[tid] = q;
  }
  for (int e = tid; e < 64 * GJ_NB; e += 256) {
    const int i = e & 63, r = e >> 6;
    const int gi = m0 + i;
    float h, l;
    split_d2f((gi < n && r < nbk) ? A[gi + (size_t)(j0 + r) * lda] : 0.0, h, l);
    Ph[r][i] = h;
    Pl[r][i] = l;
  }
  for (int e = tid; e < 64 * GJ_NB; e += 256) {
    const int r = e % GJ_NB, j = e / GJ_NB;
    const int gj = n0 + j;
    float h, l;
    split_d2f((gj < n && r < nbk) ? p.W[r + (size_t)gj * 2 * GJ_NB] : 0.0, h, l);
    Wh[r][j] = h;
    Whn[r][j] = -h;
    Wln[r][j] = -l;
  }
  __syncthreads();
  f32x2 sh[2][4], sl[2][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) { sh[i][j] = 0ULL; sl[i][j] = 0ULL; }
  for (int r = 0; r < nbk; ++r) {
    const f32x2 ah0 = x2_pack(Ph[r][tx], Ph[r][tx + 16]), al0 = x2_pack(Pl[r][tx], Pl[r][tx + 16]);
    const f32x2 ah1 = x2_pack(Ph[r][tx + 32], Ph[r][tx + 48]), al1 = x2_pack(Pl[r][tx + 32], Pl[r][tx + 48]);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = ty + 16 * j;
      const f32x2 bh2 = x2_pack(Wh[r][c], Wh[r][c]), bhn2 = x2_pack(Whn[r][c], Whn[r][c]),
                  bln2 = x2_pack(Wln[r][c], Wln[r][c]);
      df_madd_x2(sh[0][j], sl[0][j], ah0, al0, bh2, bhn2, bln2);
      df_madd_x2(sh[1][j], sl[1][j], ah1, al1, bh2, bhn2, bln2);
    }
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float h[2], l[2];
      const f32x2 hi = x2_add(sh[i][j], sl[i][j]);
      const f32x2 lo = x2_sub(sl[i][j], x2_sub(hi, sh[i][j]));
      x2_unpack(hi, h[0], h[1]);
      x2_unpack(lo, l[0], l[1]);
      const int gj = n0 + ty + 16 * j;
      if (gj >= n || (gj >= j0 && gj < jend)) continue;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int li = tx + 16 * (2 * i + u), gi = m0 + li;
        if (gi >= n) continue;
        double* c = A + gi + (size_t)gj * lda;
        double base;
        if (gi >= j0 && gi < jend) base = 0.0;
        else if (rowq[li] >= 0) base = p.W[GJ_NB + rowq[li] + (size_t)gj * 2 * GJ_NB];
        else base = *c;
        float bh, bl;
        split_d2f(base, bh, bl);
        float th = h[u], tl = l[u];
        df_add(th, tl, bh, bl);
        *c = df_to_double(th, tl);
      }
    }
}

// Column permutation undoing the row interchanges (applied in reverse).
template <typename R>
__global__ void k_gj_perm(const InvP<R>* __restrict__ P) {
  const InvP<R> p = P[blockIdx.x];
  if (threadIdx.x != 0) return;
  if (*p.info != 0) return;
  // reuse ipiv storage after reading: build arr in W's first column block
  int* arr = reinterpret_cast<int*>(p.W);  // W holds >= GJ_NB*n reals >= n ints
  for (int j = 0; j < p.n; ++j) arr[j] = j;
  for (int j = p.n - 1; j >= 0; --j) {
    const int q = p.ipiv[j];
    if (q != j) { const int t = arr[j]; arr[j] = arr[q]; arr[q] = t; }
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_gj_colgather(const InvP<R>* __restrict__ P) {
  const InvP<R> p = P[blockIdx.y];
  if (*p.info != 0) return;
  const int n = p.n;
  const int* arr = reinterpret_cast<const int*>(p.W);
  const long long tot = (long long)n * n;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int i = (int)(e % n), j = (int)(e / n);
    p.Wfull[e] = p.A[i + (size_t)arr[j] * p.lda];
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_gj_copyback(const InvP<R>* __restrict__ P) {
  const InvP<R> p = P[blockIdx.y];
  if (*p.info != 0) return;
  const int n = p.n;
  const long long tot = (long long)n * n;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int i = (int)(e % n), j = (int)(e / n);
    p.A[i + (size_t)j * p.lda] = p.Wfull[e];
  }
}

template <typename R>
static int gj_cluster(int n, int batch, int& rows_per) {
  int C = 1;
  if (batch < 152 && n > 256) {
    while (C < 8 && (n + C - 1) / C > 256) C *= 2;
  }
  rows_per = (n + C - 1) / C;
  // blocks above 6400 rows take the non-portable 16-CTA cluster (n up to 12800)
  while ((size_t)rows_per * GJ_NB * sizeof(R) > 200 * 1024 && C < 16) {
    C *= 2;
    rows_per = (n + C - 1) / C;
  }
  return C;
}

// A cluster launch of C CTAs must fit on the GPU at once: 16-CTA clusters need the
// non-portable opt-in and one GPC with 16 SMs of free shared memory.  Returns an error
// status instead of launching what cannot be co-scheduled.
template <typename K>
static void require_cluster_fits(K kernel, cudaLaunchConfig_t& cfg, int C) {
  if (C <= 8) return;
  int nclusters = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, kernel, &cfg);
  HSS_REQUIRE(e == cudaSuccess && nclusters > 0, HSS_ERR_ARG,
              "block too large: a 16-CTA cluster panel does not fit on this GPU");
}

template <typename R>
void invert_batched(const InvP<R>* dP, int batch, int maxn, cudaStream_t s, bool df) {
  if (batch <= 0 || maxn <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "invert batch too large");
  int rows_per = 0;
  const int C = gj_cluster<R>(maxn, batch, rows_per);
  const size_t smem = (size_t)rows_per * GJ_NB * sizeof(R);
  HSS_REQUIRE(smem <= 200 * 1024, HSS_ERR_ARG, "block too large for the cluster panel (n > 12800)");
  static PerDeviceOnce attr_once;  // per R instantiation; attributes are per device
  attr_once.run([] {
    HSS_CUDA(cudaFuncSetAttribute(k_gj_panel_cl<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    HSS_CUDA(cudaFuncSetAttribute(k_gj_panel_cl<R>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  });
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(batch * C, 1, 1);
  cfg.blockDim = dim3(GJ_THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  require_cluster_fits(k_gj_panel_cl<R>, cfg, C);
  const int gcols = std::max(1, std::min(ceil_div(maxn, 64), 128));  // <= 8 columns per warp up to n = 8192
  for (int j0 = 0; j0 < maxn; j0 += GJ_NB) {
    HSS_CUDA(cudaLaunchKernelEx(&cfg, k_gj_panel_cl<R>, dP, j0, rows_per));
    k_gj_gather<R><<<dim3(gcols, batch), 256, 0, s>>>(dP, j0);
    check_launch("k_gj_gather");
    dim3 g(ceil_div(maxn, 64), ceil_div(maxn, 64), batch);
    if constexpr (std::is_same<R, double>::value) {
      if (df) {
        k_gj_update_df<<<g, 256, 0, s>>>(dP, j0);
        check_launch("k_gj_update_df");
        continue;
      }
    }
    k_gj_update<R><<<g, 256, 0, s>>>(dP, j0);
    check_launch("k_gj_update");
  }
  k_gj_perm<R><<<batch, 32, 0, s>>>(dP);
  check_launch("k_gj_perm");
  const int gx = std::max(1, std::min(ceil_div((long long)maxn * maxn, 256), 1024));
  k_gj_colgather<R><<<dim3(gx, batch), 256, 0, s>>>(dP);
  check_launch("k_gj_colgather");
  k_gj_copyback<R><<<dim3(gx, batch), 256, 0, s>>>(dP);
  check_launch("k_gj_copyback");
}


// ---------------------------------------------------------------------------
// Blocked Householder least squares.
// ---------------------------------------------------------------------------
// Householder factorization of the panel A[j0:m, j0:jend], one thread-block
// cluster per problem with the panel rows split over the CTAs' shared memory
// (two cluster barriers per column: the norm and the reflector dot products
// are summed over the cluster in a fixed order).  Writes R into A, the explicit
// reflectors into V (rows j0..m-1, ld m) and the compact-WY factor Tf.
constexpr int QR_THREADS = 512;

template <typename R>
__global__ void __launch_bounds__(QR_THREADS) k_qr_panel_cl(const QrP<R>* __restrict__ P, int j0, int cap_rows) {
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks();
  const int crank = (int)cl.block_rank();
  const QrP<R> p = P[blockIdx.x / C];
  if (j0 >= p.kf) return;  // same for the whole cluster
  extern __shared__ __align__(16) unsigned char s_raw[];
  R* pan = reinterpret_cast<R*>(s_raw);  // rows_per x QR_NB, ld rows_per
  __shared__ R slot1[2];
  __shared__ R slot2[QR_NB];
  __shared__ R s_dot[QR_NB];
  __shared__ R s_hh[2];
  __shared__ R s_tau[QR_NB];
  __shared__ R sh[32];
  __shared__ R s_gram[QR_NB][QR_NB + 1];
  __shared__ R s_tf[QR_NB][QR_NB + 1];
  const int m = p.m, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nt >> 5;
  const int jend = min(j0 + QR_NB, p.kf), nbk = jend - j0;
  const int mm = m - j0;
  const int rows_per = (mm + C - 1) / C;
  const int r0 = j0 + crank * rows_per, r1 = min(m, r0 + rows_per);
  R* A = p.A;
  const size_t lda = p.lda;
  (void)cap_rows;
  for (int e = tid; e < rows_per * QR_NB; e += nt) {
    const int i = e % rows_per, c = e / rows_per;
    pan[i + c * rows_per] = (c < nbk && r0 + i < r1) ? A[(r0 + i) + (size_t)(j0 + c) * lda] : R(0);
  }
  __syncthreads();
  for (int j = j0; j < jend; ++j) {
    const int jj = j - j0;
    // squared norm of the column below the diagonal, summed over the cluster
    R part = R(0);
    for (int i = max(j + 1, r0) + tid; i < r1; i += nt) {
      const R v = pan[(i - r0) + jj * rows_per];
      part += v * v;
    }
    part = warp_sum(part);
    __syncthreads();
    if (lane == 0) sh[w] = part;
    __syncthreads();
    if (tid == 0) {
      R t = R(0);
      for (int q = 0; q < nw; ++q) t += sh[q];
      slot1[0] = t;
      // the owner of row j publishes alpha before anyone may rewrite it
      if (j >= r0 && j < r1) slot1[1] = pan[(j - r0) + jj * rows_per];
    }
    cl.sync();
    // the column's Householder scalars: thread 0 gathers the cluster's partial norms and
    // forms them once (not one FP64 square root and two divisions per thread)
    const int oj = (j - j0) / rows_per;
    if (tid == 0) {
      R xn2 = R(0);
      for (int q = 0; q < C; ++q) xn2 += *cl.map_shared_rank(&slot1[0], q);
      const R alpha = *cl.map_shared_rank(&slot1[1], oj);
      R tau0, beta0, scal0;
      if (xn2 == R(0)) { tau0 = R(0); beta0 = alpha; scal0 = R(0); }
      else {
        beta0 = -copysign(sqrt(alpha * alpha + xn2), alpha);
        tau0 = (beta0 - alpha) / beta0;
        scal0 = R(1) / (alpha - beta0);
      }
      s_tau[jj] = tau0;
      s_hh[0] = beta0;
      s_hh[1] = scal0;
    }
    __syncthreads();
    const R tau = s_tau[jj], beta = s_hh[0], scal = s_hh[1];
    // reflector into the panel column (v_j = 1 on the diagonal row)
    for (int i = r0 + tid; i < r1; i += nt) {
      R* x = pan + (i - r0) + jj * rows_per;
      if (i > j) *x = *x * scal;
      else if (i == j) *x = R(1);
    }
    __syncthreads();
    // partial dot products v . a_c for the remaining panel columns
    for (int c = jj + 1 + w; c < nbk; c += nw) {
      R d = R(0);
      for (int i = max(j, r0) + lane; i < r1; i += 32) d += pan[(i - r0) + jj * rows_per] * pan[(i - r0) + c * rows_per];
      d = warp_sum(d);
      if (lane == 0) slot2[c] = d;
    }
    cl.sync();
    if (tid < nbk && tid > jj) {
      R t = R(0);
      for (int q = 0; q < C; ++q) t += *cl.map_shared_rank(&slot2[tid], q);
      s_dot[tid] = t * tau;
    }
    __syncthreads();
    for (int e = tid; e < rows_per * nbk; e += nt) {
      const int i = e % rows_per, c = e / rows_per;
      const int gi = r0 + i;
      if (c <= jj || gi >= r1 || gi < j) continue;
      pan[i + c * rows_per] -= s_dot[c] * pan[i + jj * rows_per];
    }
    if (crank == oj && tid == 0) p.diag[j] = fabs(beta);
    // beta goes to the R diagonal when the panel is written back
    if (tid == 0) s_dot[jj] = beta;
    __syncthreads();
  }
  // partial Gram matrix V^T V of the own rows
  for (int e = tid; e < nbk * nbk; e += nt) {
    const int a = e % nbk, b = e / nbk;
    R d = R(0);
    if (a < b)
      for (int i = r0; i < r1; ++i) {
        const int gi = i;
        const R va = (gi >= j0 + a) ? pan[(i - r0) + a * rows_per] : R(0);
        const R vb = (gi >= j0 + b) ? pan[(i - r0) + b * rows_per] : R(0);
        d += va * vb;
      }
    s_gram[a][b] = d;
  }
  // V (explicit, zero above the diagonal) and the panel back to A (R on and above the diagonal)
  for (int e = tid; e < rows_per * QR_NB; e += nt) {
    const int i = e % rows_per, c = e / rows_per;
    const int gi = r0 + i;
    if (gi >= r1) continue;
    R v = R(0);
    if (c < nbk) {
      const int gj = j0 + c;
      if (gi > gj) v = pan[i + c * rows_per];
      else if (gi == gj) v = R(1);
    }
    p.V[(gi - j0) + (size_t)c * m] = v;
  }
  cl.sync();
  if (crank == 0) {
    // rows j0..jend-1 of the panel (R block) are owned by the first CTAs: gather R's
    // upper triangle and the strict-lower reflector part is not needed in A
    for (int e = tid; e < nbk * nbk; e += nt) {
      const int a = e % nbk, b = e / nbk;  // row j0+a, column j0+b
      if (a > b) continue;
      const int gi = j0 + a;
      const int o = (gi - j0) / rows_per;
      R v;
      if (a == b) v = s_dot[b];  // beta of column b (same in every CTA)
      else v = *cl.map_shared_rank(&pan[(gi - j0 - o * rows_per) + b * rows_per], o);
      A[gi + (size_t)(j0 + b) * lda] = v;
    }
    // cluster totals of the Gram entries, stored in place: each entry is read (all
    // ranks, its own included) and then overwritten by the one thread that owns it
    for (int e = tid; e < nbk * nbk; e += nt) {
      const int a = e % nbk, b = e / nbk;
      if (a >= b) continue;
      R t = R(0);
      for (int q = 0; q < C; ++q) t += cl.map_shared_rank(&s_gram[0][0], q)[a * (QR_NB + 1) + b];
      s_gram[a][b] = t;
    }
    for (int e = tid; e < QR_NB * QR_NB; e += nt) s_tf[e % QR_NB][e / QR_NB] = R(0);
    __syncthreads();
    // compact-WY factor, one column at a time (the column's entries in parallel)
    for (int b = 0; b < nbk; ++b) {
      if (tid == 0) s_tf[b][b] = s_tau[b];
      if (tid < b) {
        const int a = tid;
        R t = R(0);
        for (int c = a; c < b; ++c) t += s_tf[a][c] * s_gram[c][b];
        s_tf[a][b] = -s_tau[b] * t;
      }
      __syncthreads();
    }
    for (int e = tid; e < QR_NB * QR_NB; e += nt) p.Tf[e] = s_tf[e % QR_NB][e / QR_NB];
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
}

// k_qr_panel_cl in double-float arithmetic, for the FP64 problems of the double-float
// modes: the panel is held as float pairs in the cluster's shared memory (the same 8 bytes
// per entry), and the column norms, reflector dot products, rank-1 panel updates and the
// Gram matrix run on the FP32 pipes (~2^-48 relative).  The Householder scalars, the
// cluster totals of the squared norms, the Gram totals and the compact-WY factor stay in
// FP64.  Same cluster layout, barriers, fixed summation order and outputs (R in A, V, Tf,
// diag) as k_qr_panel_cl.
__global__ void __launch_bounds__(QR_THREADS) k_qr_panel_cl_df(const QrP<double>* __restrict__ P, int j0) {
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks();
  const int crank = (int)cl.block_rank();
  const QrP<double> p = P[blockIdx.x / C];
  if (j0 >= p.kf) return;  // same for the whole cluster
  extern __shared__ __align__(16) unsigned char s_raw[];
  float2* pan = reinterpret_cast<float2*>(s_raw);  // rows_per x QR_NB, ld rows_per
  __shared__ float2 slot1[2];      // partial squared norm; alpha (owner of row j)
  __shared__ float2 slot2[QR_NB];  // partial reflector dot products
  __shared__ float2 s_dot[QR_NB];  // tau (v . a_c), cluster totals
  __shared__ float s_hf[4];        // scal and tau as float pairs
  __shared__ double s_tau[QR_NB], s_beta[QR_NB];
  __shared__ float shh[QR_THREADS / 32], shl[QR_THREADS / 32];
  __shared__ double s_gram[QR_NB][QR_NB + 1];
  __shared__ double s_tf[QR_NB][QR_NB + 1];
  const int m = p.m, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nt >> 5;
  const int jend = min(j0 + QR_NB, p.kf), nbk = jend - j0;
  const int mm = m - j0;
  const int rows_per = (mm + C - 1) / C;
  const int r0 = j0 + crank * rows_per, r1 = min(m, r0 + rows_per);
  double* A = p.A;
  const size_t lda = p.lda;
  for (int e = tid; e < rows_per * QR_NB; e += nt) {
    const int i = e % rows_per, c = e / rows_per;
    float h = 0.f, l = 0.f;
    if (c < nbk && r0 + i < r1) split_d2f(A[(r0 + i) + (size_t)(j0 + c) * lda], h, l);
    pan[i + c * rows_per] = make_float2(h, l);
  }
  __syncthreads();
  for (int j = j0; j < jend; ++j) {
    const int jj = j - j0;
    // squared norm of the column below the diagonal: CTA total in double-float
    float nh = 0.f, nl = 0.f;
    for (int i = max(j + 1, r0) + tid; i < r1; i += nt) {
      const float2 v = pan[(i - r0) + jj * rows_per];
      df_madd(nh, nl, v.x, v.y, v.x, v.y);
    }
    warp_sum_df(nh, nl);
    __syncthreads();
    if (lane == 0) { shh[w] = nh; shl[w] = nl; }
    __syncthreads();
    if (tid == 0) {
      float th = shh[0], tl = shl[0];
      for (int q = 1; q < nw; ++q) df_add(th, tl, shh[q], shl[q]);
      slot1[0] = make_float2(th, tl);
      // the owner of row j publishes alpha before anyone may rewrite it
      if (j >= r0 && j < r1) slot1[1] = pan[(j - r0) + jj * rows_per];
    }
    cl.sync();
    // the column's Householder scalars in FP64, by thread 0 of every CTA
    const int oj = (j - j0) / rows_per;
    if (tid == 0) {
      double xn2 = 0.0;
      for (int q = 0; q < C; ++q) {
        const float2 t = *cl.map_shared_rank(&slot1[0], q);
        xn2 += (double)t.x + (double)t.y;
      }
      const float2 a = *cl.map_shared_rank(&slot1[1], oj);
      const double alpha = (double)a.x + (double)a.y;
      double tau = 0.0, beta = alpha, scal = 0.0;
      if (xn2 != 0.0) {
        beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
        tau = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      s_tau[jj] = tau;
      s_beta[jj] = beta;
      split_d2f(scal, s_hf[0], s_hf[1]);
      split_d2f(tau, s_hf[2], s_hf[3]);
    }
    __syncthreads();
    // reflector into the panel column (v_j = 1 on the diagonal row)
    const float sch = s_hf[0], scl = s_hf[1];
    for (int i = r0 + tid; i < r1; i += nt) {
      float2* x = pan + (i - r0) + jj * rows_per;
      if (i > j) {
        float2 v = *x;
        df_mul(v.x, v.y, sch, scl);
        *x = v;
      } else if (i == j) {
        *x = make_float2(1.f, 0.f);
      }
    }
    __syncthreads();
    // partial dot products v . a_c for the remaining panel columns
    for (int c = jj + 1 + w; c < nbk; c += nw) {
      float dh = 0.f, dl = 0.f;
      for (int i = max(j, r0) + lane; i < r1; i += 32) {
        const float2 v = pan[(i - r0) + jj * rows_per], a = pan[(i - r0) + c * rows_per];
        df_madd(dh, dl, v.x, v.y, a.x, a.y);
      }
      warp_sum_df(dh, dl);
      if (lane == 0) slot2[c] = make_float2(dh, dl);
    }
    cl.sync();
    if (tid < nbk && tid > jj) {
      float th = 0.f, tl = 0.f;
      for (int q = 0; q < C; ++q) {
        const float2 t = *cl.map_shared_rank(&slot2[tid], q);
        df_add(th, tl, t.x, t.y);
      }
      df_mul(th, tl, s_hf[2], s_hf[3]);
      s_dot[tid] = make_float2(th, tl);
    }
    __syncthreads();
    for (int e = tid; e < rows_per * nbk; e += nt) {
      const int i = e % rows_per, c = e / rows_per;
      const int gi = r0 + i;
      if (c <= jj || gi >= r1 || gi < j) continue;
      const float2 v = pan[i + jj * rows_per], d = s_dot[c];
      float2 a = pan[i + c * rows_per];
      df_madd(a.x, a.y, -d.x, -d.y, v.x, v.y);
      pan[i + c * rows_per] = a;
    }
    if (crank == oj && tid == 0) p.diag[j] = fabs(s_beta[jj]);
    __syncthreads();
  }
  // partial Gram matrix V^T V of the own rows (v_b is zero above row j0 + b)
  for (int e = tid; e < nbk * nbk; e += nt) {
    const int a = e % nbk, b = e / nbk;
    float dh = 0.f, dl = 0.f;
    if (a < b)
      for (int i = max(r0, j0 + b); i < r1; ++i) {
        const float2 va = pan[(i - r0) + a * rows_per], vb = pan[(i - r0) + b * rows_per];
        df_madd(dh, dl, va.x, va.y, vb.x, vb.y);
      }
    s_gram[a][b] = (double)dh + (double)dl;
  }
  // V (explicit, zero above the diagonal) back to FP64
  for (int e = tid; e < rows_per * QR_NB; e += nt) {
    const int i = e % rows_per, c = e / rows_per;
    const int gi = r0 + i;
    if (gi >= r1) continue;
    double v = 0.0;
    if (c < nbk) {
      const int gj = j0 + c;
      if (gi > gj) {
        const float2 t = pan[i + c * rows_per];
        v = df_to_double(t.x, t.y);
      } else if (gi == gj) {
        v = 1.0;
      }
    }
    p.V[(gi - j0) + (size_t)c * m] = v;
  }
  cl.sync();
  if (crank == 0) {
    // R's upper triangle (rows j0..jend-1 live in the first CTAs; beta on the diagonal)
    for (int e = tid; e < nbk * nbk; e += nt) {
      const int a = e % nbk, b = e / nbk;  // row j0+a, column j0+b
      if (a > b) continue;
      const int gi = j0 + a;
      const int o = (gi - j0) / rows_per;
      double v;
      if (a == b) v = s_beta[b];
      else {
        const float2 t = *cl.map_shared_rank(&pan[(gi - j0 - o * rows_per) + b * rows_per], o);
        v = df_to_double(t.x, t.y);
      }
      A[gi + (size_t)(j0 + b) * lda] = v;
    }
    // cluster totals of the Gram entries in FP64, stored in place (each entry read by
    // every rank's sum, then overwritten by the one thread that owns it)
    for (int e = tid; e < nbk * nbk; e += nt) {
      const int a = e % nbk, b = e / nbk;
      if (a >= b) continue;
      double t = 0.0;
      for (int q = 0; q < C; ++q) t += cl.map_shared_rank(&s_gram[0][0], q)[a * (QR_NB + 1) + b];
      s_gram[a][b] = t;
    }
    for (int e = tid; e < QR_NB * QR_NB; e += nt) s_tf[e % QR_NB][e / QR_NB] = 0.0;
    __syncthreads();
    for (int b = 0; b < nbk; ++b) {
      if (tid == 0) s_tf[b][b] = s_tau[b];
      if (tid < b) {
        const int a = tid;
        double t = 0.0;
        for (int c = a; c < b; ++c) t += s_tf[a][c] * s_gram[c][b];
        s_tf[a][b] = -s_tau[b] * t;
      }
      __syncthreads();
    }
    for (int e = tid; e < QR_NB * QR_NB; e += nt) p.Tf[e] = s_tf[e % QR_NB][e / QR_NB];
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
}

// Apply (I - V Tf V^T)^T = I - V Tf^T V^T to A[j0:m, jend:n] in 32-column tiles.
template <typename R>
__global__ void __launch_bounds__(256) k_qr_update(const QrP<R>* __restrict__ P, int j0) {
  const QrP<R> p = P[blockIdx.y];
  if (j0 >= p.kf) return;
  const int m = p.m, n = p.n, tid = threadIdx.x;
  const int jend = min(j0 + QR_NB, p.kf), nbk = jend - j0;
  const int c0 = jend + blockIdx.x * 32;
  if (c0 >= n) return;
  const int nc = min(32, n - c0);
  R* A = p.A;
  const size_t lda = p.lda;
  const R* V = p.V;
  __shared__ R Vs[64][QR_NB + 1];
  __shared__ R As[64][32 + 1];
  __shared__ R Ws[QR_NB][32 + 1];
  __shared__ R W2[QR_NB][32 + 1];
  // each thread owns 4 (jj, cc) outputs: jj = tid & 31, cc = (tid >> 5) + 8*q
  const int ojj = tid & 31, occ = tid >> 5;
  R acc[4] = {R(0), R(0), R(0), R(0)};
  for (int r0 = j0; r0 < m; r0 += 64) {
    for (int e = tid; e < 64 * QR_NB; e += 256) {
      const int i = e & 63, jj = e >> 6;
      const int gi = r0 + i;
      Vs[i][jj] = (gi < m && jj < nbk) ? V[(gi - j0) + (size_t)jj * m] : R(0);
    }
    for (int e = tid; e < 64 * 32; e += 256) {
      const int i = e & 63, cc = e >> 6;
      const int gi = r0 + i;
      As[i][cc] = (gi < m && cc < nc) ? A[gi + (size_t)(c0 + cc) * lda] : R(0);
    }
    __syncthreads();
    for (int i = 0; i < 64; ++i) {
      const R v = Vs[i][ojj];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] += v * As[i][occ + 8 * q];
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) Ws[ojj][occ + 8 * q] = acc[q];
  __syncthreads();
  // W2 = Tf^T W  (Tf upper triangular): W2[jj] = sum_{t<=jj} Tf[t, jj] W[t]
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int cc = occ + 8 * q;
    R t = R(0);
    if (ojj < nbk)
      for (int a = 0; a <= ojj; ++a) t += p.Tf[a + ojj * QR_NB] * Ws[a][cc];
    W2[ojj][cc] = t;
  }
  __syncthreads();
  // A -= V W2
  for (int r0 = j0; r0 < m; r0 += 64) {
    for (int e = tid; e < 64 * QR_NB; e += 256) {
      const int i = e & 63, jj = e >> 6;
      const int gi = r0 + i;
      Vs[i][jj] = (gi < m && jj < nbk) ? V[(gi - j0) + (size_t)jj * m] : R(0);
    }
    __syncthreads();
    for (int e = tid; e < 64 * 32; e += 256) {
      const int i = e & 63, cc = e >> 6;
      const int gi = r0 + i;
      if (gi < m && cc < nc) {
        R t = R(0);
        for (int jj = 0; jj < nbk; ++jj) t += Vs[i][jj] * W2[jj][cc];
        A[gi + (size_t)(c0 + cc) * lda] -= t;
      }
    }
    __syncthreads();
  }
}

// Shared-memory operands of the double-float trailing update, stored in the form the
// f32x2 products take them, so the inner loops issue one 64-bit load per operand and no
// register moves.  A 32-row chunk of V is kept as the broadcast pairs (vh, vh),
// (-vh, -vh), (-vl, -vl); the odd row stride (33 pairs) keeps both the row-wise and the
// column-wise reads free of bank conflicts.  A 32 x 32 tile X of A (or of W2) is kept as
// 16 column pairs per row: pair p = c + 8 u (c < 8, u < 2) holds columns (c + 16 u,
// c + 16 u + 8), the two columns one thread owns together.
struct DfVChunk {
  f32x2 b[32][33], bn[32][33], bl[32][33];
};
struct DfXTile {
  f32x2 h[32][17], l[32][17];
};
// float slot of column cc within a row of a DfXTile
__device__ __forceinline__ int dfx_slot(int cc) { return 2 * ((cc & 7) + 8 * (cc >> 4)) + ((cc >> 3) & 1); }
__device__ __forceinline__ void dfx_put(DfXTile& X, int i, int cc, float h, float l) {
  reinterpret_cast<float*>(X.h[i])[dfx_slot(cc)] = h;
  reinterpret_cast<float*>(X.l[i])[dfx_slot(cc)] = l;
}
// rows r0 .. r0+31 of V (rows past re and columns past nbk read as zero)
__device__ __forceinline__ void dfv_stage(DfVChunk& S, const double* __restrict__ V, int m, int j0, int r0, int re,
                                          int nbk, int tid) {
  for (int e = tid; e < 32 * 32; e += 256) {
    const int i = e & 31, jj = e >> 5;
    const int gi = r0 + i;
    float h, l;
    split_d2f((gi < re && jj < nbk) ? V[(gi - j0) + (size_t)jj * m] : 0.0, h, l);
    S.b[i][jj] = x2_pack(h, h);
    S.bn[i][jj] = x2_pack(-h, -h);
    S.bl[i][jj] = x2_pack(-l, -l);
  }
}

// k_qr_update in double-float arithmetic for FP64 problems: W = V^T A,
// W2 = Tf^T W and A -= V W2 for one 32-column tile, with every product on the
// FP32 pipes (rows of V are the broadcast operand, column pairs of A / W2 the
// f32x2 operand).  32-row chunks keep the static shared memory under 48 KB.
__global__ void __launch_bounds__(256) k_qr_update_df(const QrP<double>* __restrict__ P, int j0) {
  const QrP<double> p = P[blockIdx.y];
  if (j0 >= p.kf) return;
  const int m = p.m, n = p.n, tid = threadIdx.x;
  const int jend = min(j0 + QR_NB, p.kf), nbk = jend - j0;
  const int c0 = jend + blockIdx.x * 32;
  if (c0 >= n) return;
  const int nc = min(32, n - c0);
  double* A = p.A;
  const size_t lda = p.lda;
  const double* V = p.V;
  __shared__ DfVChunk Vc;
  __shared__ DfXTile X;  // A chunk in phase 1, W2 in phase 3
  __shared__ float Wh[32][33], Wl[32][33];
  const int lo5 = tid & 31, hi3 = tid >> 5;
  // phase 1: thread owns W[jj = lo5][cc in {hi3, hi3+8} and {hi3+16, hi3+24}]
  f32x2 sh[2] = {0ULL, 0ULL}, sl[2] = {0ULL, 0ULL};
  for (int r0 = j0; r0 < m; r0 += 32) {
    dfv_stage(Vc, V, m, j0, r0, m, nbk, tid);
    for (int e = tid; e < 32 * 32; e += 256) {
      const int i = e & 31, cc = e >> 5;
      const int gi = r0 + i;
      float h, l;
      split_d2f((gi < m && cc < nc) ? A[gi + (size_t)(c0 + cc) * lda] : 0.0, h, l);
      dfx_put(X, i, cc, h, l);
    }
    __syncthreads();
#pragma unroll 4
    for (int i = 0; i < 32; ++i) {
      const f32x2 b2 = Vc.b[i][lo5], bn2 = Vc.bn[i][lo5], bl2 = Vc.bl[i][lo5];
#pragma unroll
      for (int u = 0; u < 2; ++u)
        df_madd_x2(sh[u], sl[u], X.h[i][hi3 + 8 * u], X.l[i][hi3 + 8 * u], b2, bn2, bl2);
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {  // renormalise once per chunk
      const f32x2 h = x2_add(sh[u], sl[u]);
      sl[u] = x2_sub(sl[u], x2_sub(h, sh[u]));
      sh[u] = h;
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    float h0, h1, l0, l1;
    x2_unpack(sh[u], h0, h1);
    x2_unpack(sl[u], l0, l1);
    const int ca = hi3 + 16 * u, cb = ca + 8;
    Wh[lo5][ca] = h0; Wl[lo5][ca] = l0;
    Wh[lo5][cb] = h1; Wl[lo5][cb] = l1;
  }
  __syncthreads();
  // phase 2: W2[jj][cc] = sum_{a <= jj} Tf[a, jj] W[a][cc]  (Tf upper triangular)
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int cc = hi3 + 8 * q;
    float th = 0.f, tl = 0.f;
    if (lo5 < nbk)
      for (int a = 0; a <= lo5; ++a) {
        float fh, fl;
        split_d2f(p.Tf[a + lo5 * QR_NB], fh, fl);
        df_madd(th, tl, Wh[a][cc], Wl[a][cc], fh, fl);
      }
    dfx_put(X, lo5, cc, th, tl);  // W2 (the A chunk is no longer needed)
  }
  __syncthreads();
  // phase 3: A -= V W2; thread owns rows i = lo5 of the chunk, columns as in phase 1
  for (int r0 = j0; r0 < m; r0 += 32) {
    dfv_stage(Vc, V, m, j0, r0, m, nbk, tid);
    __syncthreads();
    f32x2 ah[2] = {0ULL, 0ULL}, al[2] = {0ULL, 0ULL};
    for (int jj = 0; jj < nbk; ++jj) {
      const f32x2 b2 = Vc.b[lo5][jj], bn2 = Vc.bn[lo5][jj], bl2 = Vc.bl[lo5][jj];
#pragma unroll
      for (int u = 0; u < 2; ++u)
        df_madd_x2(ah[u], al[u], X.h[jj][hi3 + 8 * u], X.l[jj][hi3 + 8 * u], b2, bn2, bl2);
    }
    const int gi = r0 + lo5;
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const f32x2 h = x2_add(ah[u], al[u]);
      const f32x2 l = x2_sub(al[u], x2_sub(h, ah[u]));
      float h2[2], l2[2];
      x2_unpack(h, h2[0], h2[1]);
      x2_unpack(l, l2[0], l2[1]);
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int cc = hi3 + 16 * u + 8 * v;
        if (gi >= m || cc >= nc) continue;
        double* c = A + gi + (size_t)(c0 + cc) * lda;
        float xh, xl;
        split_d2f(*c, xh, xl);
        df_add(xh, xl, -h2[v], -l2[v]);
        *c = df_to_double(xh, xl);
      }
    }
    __syncthreads();
  }
}

// The same trailing update with the rows split over several CTAs (the top levels of a tree
// have a few tall problems: one CTA per 32 columns leaves most SMs idle).
// k_qr_wpart_df: CTA (x, y, z) forms the partial W = V^T A(rows of slice y, its 32 columns);
// k_qr_apply_df: every CTA adds the slices' partials in slice order, forms W2 = Tf^T W and
// updates its own rows.  The sums are fixed-order, so results do not depend on timing.
__device__ __forceinline__ void qr_rows(int m, int j0, int rs, int y, int& rb, int& re) {
  const int per = (((m - j0) + rs - 1) / rs + 31) & ~31;
  rb = j0 + y * per;
  re = min(m, rb + per);
}

__global__ void __launch_bounds__(256) k_qr_wpart_df(const QrP<double>* __restrict__ P, int j0, int rs,
                                                     float2* __restrict__ wpart) {
  const QrP<double> p = P[blockIdx.z];
  if (j0 >= p.kf) return;
  const int m = p.m, n = p.n, tid = threadIdx.x;
  const int jend = min(j0 + QR_NB, p.kf), nbk = jend - j0;
  const int c0 = jend + blockIdx.x * 32;
  if (c0 >= n) return;
  const int nc = min(32, n - c0);
  int rb, re;
  qr_rows(m, j0, rs, blockIdx.y, rb, re);
  const double* A = p.A;
  const size_t lda = p.lda;
  const double* V = p.V;
  __shared__ DfVChunk Vc;
  __shared__ DfXTile X;
  const int lo5 = tid & 31, hi3 = tid >> 5;
  f32x2 sh[2] = {0ULL, 0ULL}, sl[2] = {0ULL, 0ULL};
  for (int r0 = rb; r0 < re; r0 += 32) {
    dfv_stage(Vc, V, m, j0, r0, re, nbk, tid);
    for (int e = tid; e < 32 * 32; e += 256) {
      const int i = e & 31, cc = e >> 5;
      const int gi = r0 + i;
      float h, l;
      split_d2f((gi < re && cc < nc) ? A[gi + (size_t)(c0 + cc) * lda] : 0.0, h, l);
      dfx_put(X, i, cc, h, l);
    }
    __syncthreads();
#pragma unroll 4
    for (int i = 0; i < 32; ++i) {
      const f32x2 b2 = Vc.b[i][lo5], bn2 = Vc.bn[i][lo5], bl2 = Vc.bl[i][lo5];
#pragma unroll
      for (int u = 0; u < 2; ++u)
        df_madd_x2(sh[u], sl[u], X.h[i][hi3 + 8 * u], X.l[i][hi3 + 8 * u], b2, bn2, bl2);
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const f32x2 h = x2_add(sh[u], sl[u]);
      sl[u] = x2_sub(sl[u], x2_sub(h, sh[u]));
      sh[u] = h;
    }
    __syncthreads();
  }
  float2* wp = wpart + (((size_t)blockIdx.z * gridDim.x + blockIdx.x) * rs + blockIdx.y) * 1024;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    float h0, h1, l0, l1;
    x2_unpack(sh[u], h0, h1);
    x2_unpack(sl[u], l0, l1);
    const int ca = hi3 + 16 * u, cb = ca + 8;
    wp[lo5 * 32 + ca] = make_float2(h0, l0);
    wp[lo5 * 32 + cb] = make_float2(h1, l1);
  }
}

__global__ void __launch_bounds__(256) k_qr_apply_df(const QrP<double>* __restrict__ P, int j0, int rs,
                                                     const float2* __restrict__ wpart) {
  const QrP<double> p = P[blockIdx.z];
  if (j0 >= p.kf) return;
  const int m = p.m, n = p.n, tid = threadIdx.x;
  const int jend = min(j0 + QR_NB, p.kf), nbk = jend - j0;
  const int c0 = jend + blockIdx.x * 32;
  if (c0 >= n) return;
  const int nc = min(32, n - c0);
  int rb, re;
  qr_rows(m, j0, rs, blockIdx.y, rb, re);
  double* A = p.A;
  const size_t lda = p.lda;
  const double* V = p.V;
  __shared__ DfVChunk Vc;
  __shared__ DfXTile X;  // W2
  __shared__ float Wh[32][33], Wl[32][33];
  const int lo5 = tid & 31, hi3 = tid >> 5;
  // W = the slices' partials, added in slice order
  const float2* wp = wpart + ((size_t)blockIdx.z * gridDim.x + blockIdx.x) * rs * 1024;
  for (int e = tid; e < 1024; e += 256) {
    float h = 0.f, l = 0.f;
    for (int y = 0; y < rs; ++y) {
      const float2 v = wp[(size_t)y * 1024 + e];
      df_add(h, l, v.x, v.y);
    }
    Wh[e >> 5][e & 31] = h;
    Wl[e >> 5][e & 31] = l;
  }
  __syncthreads();
  // W2[jj][cc] = sum_{a <= jj} Tf[a, jj] W[a][cc]  (Tf upper triangular)
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int cc = hi3 + 8 * q;
    float th = 0.f, tl = 0.f;
    if (lo5 < nbk)
      for (int a = 0; a <= lo5; ++a) {
        float fh, fl;
        split_d2f(p.Tf[a + lo5 * QR_NB], fh, fl);
        df_madd(th, tl, Wh[a][cc], Wl[a][cc], fh, fl);
      }
    dfx_put(X, lo5, cc, th, tl);
  }
  __syncthreads();
  for (int r0 = rb; r0 < re; r0 += 32) {
    dfv_stage(Vc, V, m, j0, r0, re, nbk, tid);
    __syncthreads();
    f32x2 ah[2] = {0ULL, 0ULL}, al[2] = {0ULL, 0ULL};
    for (int jj = 0; jj < nbk; ++jj) {
      const f32x2 b2 = Vc.b[lo5][jj], bn2 = Vc.bn[lo5][jj], bl2 = Vc.bl[lo5][jj];
#pragma unroll
      for (int u = 0; u < 2; ++u)
        df_madd_x2(ah[u], al[u], X.h[jj][hi3 + 8 * u], X.l[jj][hi3 + 8 * u], b2, bn2, bl2);
    }
    const int gi = r0 + lo5;
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const f32x2 h = x2_add(ah[u], al[u]);
      const f32x2 l = x2_sub(al[u], x2_sub(h, ah[u]));
      float h2[2], l2[2];
      x2_unpack(h, h2[0], h2[1]);
      x2_unpack(l, l2[0], l2[1]);
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int cc = hi3 + 16 * u + 8 * v;
        if (gi >= re || cc >= nc) continue;
        double* c = A + gi + (size_t)(c0 + cc) * lda;
        float xh, xl;
        split_d2f(*c, xh, xl);
        df_add(xh, xl, -h2[v], -l2[v]);
        *c = df_to_double(xh, xl);
      }
    }
    __syncthreads();
  }
}

// One back-substitution block step: solve R[b0:b1,b0:b1] X[b0:b1, tile] =
// C[b0:b1, tile] (C = A[0:kf, kf:n], already updated by the blocks below) and
// update C[rows of this CTA's chunk of 0:b0, tile] -= R[.., b0:b1] X.  Every
// CTA of a column tile solves the small block redundantly; blockIdx.y == 0
// stores it into X, so no CTA reads rows another one writes.
template <typename R>
__global__ void __launch_bounds__(256) k_trsm_step(const QrP<R>* __restrict__ P, int blk) {
  const QrP<R> p = P[blockIdx.z];
  const int kf = p.kf, ncol = p.n - p.kf;
  const int b0 = blk * 32;
  if (b0 >= kf) return;
  const int b1 = min(b0 + 32, kf), nb = b1 - b0;
  const int c0 = blockIdx.x * 32;
  if (c0 >= ncol) return;
  const int rc0 = blockIdx.y * 256;
  if (blockIdx.y > 0 && rc0 >= b0) return;
  const int nc = min(32, ncol - c0);
  R* A = p.A;
  const size_t lda = p.lda;
  R* C = A + (size_t)kf * lda;
  __shared__ R Rs[32][33];
  __shared__ R Xs[32][33];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int e = tid; e < 32 * 32; e += 256) {
    const int i = e & 31, j = e >> 5;
    Rs[i][j] = (i < nb && j < nb) ? A[(b0 + i) + (size_t)(b0 + j) * lda] : R(0);
    Xs[i][j] = (i < nb && j < nc) ? C[(b0 + i) + (size_t)(c0 + j) * lda] : R(0);
  }
  __syncthreads();
  for (int q = 0; q < 4; ++q) {
    const int cc = w + 8 * q;
    R x = Xs[lane][cc];
    for (int r = nb - 1; r >= 0; --r) {
      R xr = __shfl_sync(0xffffffffu, x, r);
      xr = xr / Rs[r][r];
      if (lane == r) x = xr;
      if (lane < r) x -= Rs[lane][r] * xr;
    }
    Xs[lane][cc] = x;
  }
  __syncthreads();
  if (blockIdx.y == 0) {
    for (int e = tid; e < 32 * 32; e += 256) {
      const int i = e & 31, j = e >> 5;
      if (i < nb && j < nc) p.X[(b0 + i) + (size_t)(c0 + j) * p.ldx] = Xs[i][j];
    }
  }
  const int rend = min(b0, rc0 + 256);
  for (int i = rc0 + tid; i < rend; i += 256) {
    R rr[32];
#pragma unroll
    for (int t = 0; t < 32; ++t) rr[t] = (t < nb) ? A[i + (size_t)(b0 + t) * lda] : R(0);
    for (int j = 0; j < nc; ++j) {
      R sacc = R(0);
#pragma unroll
      for (int t = 0; t < 32; ++t) sacc += rr[t] * Xs[t][j];
      C[i + (size_t)(c0 + j) * lda] -= sacc;
    }
  }
}

// k_trsm_step in double-float arithmetic, for the FP64 problems of the double-float modes.
// The 32 x 32 block solve runs on float pairs: the diagonal's reciprocals are formed once in
// FP64 (32 lanes, one division each) and split, and every warp carries its four columns
// through the 32 back-substitution steps together.  The update of the rows above,
// C(rows, cols) -= R(rows, b0:b1) X, uses the tiling of the least-squares trailing update
// (R's rows as broadcast pairs, X as column pairs, paired-FP32 products) and adds the result
// into C in double-float.  ~2^-48 relative, every sum in a fixed order.
__global__ void __launch_bounds__(256) k_trsm_step_df(const QrP<double>* __restrict__ P, int blk) {
  const QrP<double> p = P[blockIdx.z];
  const int kf = p.kf, ncol = p.n - p.kf;
  const int b0 = blk * 32;
  if (b0 >= kf) return;
  const int b1 = min(b0 + 32, kf), nb = b1 - b0;
  const int c0 = blockIdx.x * 32;
  if (c0 >= ncol) return;
  const int rc0 = blockIdx.y * 256;
  if (blockIdx.y > 0 && rc0 >= b0) return;
  const int nc = min(32, ncol - c0);
  double* A = p.A;
  const size_t lda = p.lda;
  double* C = A + (size_t)kf * lda;
  __shared__ float Rh[32][33], Rl[32][33];  // the diagonal block
  __shared__ float Dh[32], Dl[32];          // 1 / R(r, r)
  __shared__ DfXTile X;                      // the block's solution, 32 rows x 32 columns
  __shared__ DfVChunk Vc;                    // 32 rows of R(rows above, b0:b1)
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, lo5 = lane, hi3 = w;
  for (int e = tid; e < 32 * 32; e += 256) {
    const int i = e & 31, j = e >> 5;
    float h = 0.f, l = 0.f;
    if (i < nb && j < nb) split_d2f(A[(b0 + i) + (size_t)(b0 + j) * lda], h, l);
    Rh[i][j] = h;
    Rl[i][j] = l;
  }
  if (tid < 32) {
    const double d = (tid < nb) ? A[(b0 + tid) + (size_t)(b0 + tid) * lda] : 1.0;
    split_d2f(1.0 / d, Dh[tid], Dl[tid]);
  }
  // each warp's four columns cc = w + 8 q, row `lane` in registers
  float xh[4], xl[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int cc = w + 8 * q;
    xh[q] = 0.f;
    xl[q] = 0.f;
    if (lane < nb && cc < nc) split_d2f(C[(b0 + lane) + (size_t)(c0 + cc) * lda], xh[q], xl[q]);
  }
  __syncthreads();
  for (int r = nb - 1; r >= 0; --r) {
    const float dh = Dh[r], dl = Dl[r];
    const float nrh = -Rh[lane][r], nrl = -Rl[lane][r];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float yh = __shfl_sync(0xffffffffu, xh[q], r), yl = __shfl_sync(0xffffffffu, xl[q], r);
      df_mul(yh, yl, dh, dl);
      if (lane == r) {
        xh[q] = yh;
        xl[q] = yl;
      } else if (lane < r) {
        df_madd(xh[q], xl[q], nrh, nrl, yh, yl);  // x(lane) -= R(lane, r) x(r)
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int cc = w + 8 * q;
    dfx_put(X, lane, cc, xh[q], xl[q]);
    if (blockIdx.y == 0 && lane < nb && cc < nc)
      p.X[(b0 + lane) + (size_t)(c0 + cc) * p.ldx] = df_to_double(xh[q], xl[q]);
  }
  __syncthreads();
  // rows above the block: thread owns row lo5 of each 32-row chunk and the columns
  // {hi3, hi3 + 8} and {hi3 + 16, hi3 + 24} of the tile
  const int rend = min(b0, rc0 + 256);
  for (int r0 = rc0; r0 < rend; r0 += 32) {
    dfv_stage(Vc, A + (size_t)b0 * lda, (int)lda, 0, r0, rend, nb, tid);
    __syncthreads();
    f32x2 ah[2] = {0ULL, 0ULL}, al[2] = {0ULL, 0ULL};
    for (int jj = 0; jj < nb; ++jj) {
      const f32x2 b2 = Vc.b[lo5][jj], bn2 = Vc.bn[lo5][jj], bl2 = Vc.bl[lo5][jj];
#pragma unroll
      for (int u = 0; u < 2; ++u)
        df_madd_x2(ah[u], al[u], X.h[jj][hi3 + 8 * u], X.l[jj][hi3 + 8 * u], b2, bn2, bl2);
    }
    const int gi = r0 + lo5;
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const f32x2 h = x2_add(ah[u], al[u]);
      const f32x2 l = x2_sub(al[u], x2_sub(h, ah[u]));
      float h2[2], l2[2];
      x2_unpack(h, h2[0], h2[1]);
      x2_unpack(l, l2[0], l2[1]);
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int cc = hi3 + 16 * u + 8 * v;
        if (gi >= rend || cc >= nc) continue;
        double* c = C + gi + (size_t)(c0 + cc) * lda;
        float ch, cl;
        split_d2f(*c, ch, cl);
        df_add(ch, cl, -h2[v], -l2[v]);
        *c = df_to_double(ch, cl);
      }
    }
    __syncthreads();
  }
}

template <typename R>
void lstsq_batched(const QrP<R>* dP, int batch, int maxm, int maxn, int maxkf, cudaStream_t s, bool df, bool solve) {
  if (batch <= 0 || maxkf <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "lstsq batch too large");
  int C = 1;
  if (batch < 152 && maxm > 256)
    while (C < 8 && (maxm + C - 1) / C > 256) C *= 2;
  while ((size_t)((maxm + C - 1) / C) * QR_NB * sizeof(R) > 200 * 1024 && C < 16) C *= 2;
  const int cap = (maxm + C - 1) / C;
  const size_t smem = (size_t)cap * QR_NB * sizeof(R);
  HSS_REQUIRE(smem <= 200 * 1024, HSS_ERR_ARG, "least-squares panel too tall for the cluster (m > 12800)");
  static PerDeviceOnce attr_once;  // per R instantiation; attributes are per device
  attr_once.run([] {
    HSS_CUDA(cudaFuncSetAttribute(k_qr_panel_cl<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    HSS_CUDA(cudaFuncSetAttribute(k_qr_panel_cl<R>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  });
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(batch * C, 1, 1);
  cfg.blockDim = dim3(QR_THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  require_cluster_fits(k_qr_panel_cl<R>, cfg, C);
  if constexpr (std::is_same<R, double>::value) {
    if (df) {
      static PerDeviceOnce attr_once_df;
      attr_once_df.run([] {
        HSS_CUDA(cudaFuncSetAttribute(k_qr_panel_cl_df, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        HSS_CUDA(cudaFuncSetAttribute(k_qr_panel_cl_df, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      });
      require_cluster_fits(k_qr_panel_cl_df, cfg, C);
    }
  }
  DevBuf<double> wpart;  // row-split partial W of the double-float update (float pairs)
  for (int j0 = 0; j0 < maxkf; j0 += QR_NB) {
    bool panel_done = false;
    if constexpr (std::is_same<R, double>::value) {
      if (df) {
        HSS_CUDA(cudaLaunchKernelEx(&cfg, k_qr_panel_cl_df, dP, j0));
        panel_done = true;
      }
    }
    if (!panel_done) HSS_CUDA(cudaLaunchKernelEx(&cfg, k_qr_panel_cl<R>, dP, j0, cap));
    const int jend = std::min(j0 + QR_NB, maxkf);
    const int ncols = maxn - jend;
    if (ncols > 0) {
      if constexpr (std::is_same<R, double>::value) {
        if (df) {
          const int cb = ceil_div(ncols, 32);
          // rows split over CTAs when the problems are too few to fill the GPU twice
          const int rs = std::max(1, std::min(std::min(16, std::max(1, (maxm - j0) / 512)),
                                              ceil_div(2 * 4 * 152, (long long)cb * batch)));
          if (rs == 1) {
            k_qr_update_df<<<dim3(cb, batch), 256, 0, s>>>(dP, j0);
            check_launch("k_qr_update_df");
          } else {
            wpart.ensure((size_t)batch * cb * rs * 1024 * 2);
            k_qr_wpart_df<<<dim3(cb, rs, batch), 256, 0, s>>>(dP, j0, rs, reinterpret_cast<float2*>(wpart.p));
            check_launch("k_qr_wpart_df");
            k_qr_apply_df<<<dim3(cb, rs, batch), 256, 0, s>>>(dP, j0, rs, reinterpret_cast<const float2*>(wpart.p));
            check_launch("k_qr_apply_df");
          }
          continue;
        }
      }
      k_qr_update<R><<<dim3(ceil_div(ncols, 32), batch), 256, 0, s>>>(dP, j0);
      check_launch("k_qr_update");
    }
  }
  if (!solve) return;  // factor only: R11 and (Q^T A(:, kf:n))(0:kf, :) in the top kf rows
  const int nblk = ceil_div(maxkf, 32);
  for (int blk = nblk - 1; blk >= 0; --blk) {
    const int rows_above = blk * 32;
    dim3 g(ceil_div(maxn, 32), std::max(1, ceil_div(rows_above, 256)), batch);
    if constexpr (std::is_same<R, double>::value) {
      if (df) {
        k_trsm_step_df<<<g, 256, 0, s>>>(dP, blk);
        check_launch("k_trsm_step_df");
        continue;
      }
    }
    k_trsm_step<R><<<g, 256, 0, s>>>(dP, blk);
    check_launch("k_trsm_step");
  }
}

// ---------------------------------------------------------------------------
// Pivoted-QR interpolative decomposition (one block per problem, FP64).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double rng_uniform(unsigned long long seed, unsigned long long stream,
                                              unsigned long long i) {
  unsigned long long z = seed ^ (stream * 0xD1B54A32D192ED03ULL);
  z += (i + 1ULL) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double)(z >> 11) * 0x1.0p-53;
}

// Householder scalars of one QR step: beta = -sign(alpha) sqrt(alpha^2 + xn2),
// tau = (beta - alpha) / beta, scal = 1 / (alpha - beta) (tau = scal = 0, beta = alpha when
// the column below the diagonal is zero).  Formed once by thread 0 and shared through s3,
// so the block pays one FP64 square root and two divisions per step instead of 256.
__device__ __forceinline__ void householder_scalars(double alpha, double xn2, double* s3, double& tau,
                                                    double& beta, double& scal) {
  if (threadIdx.x == 0) {
    double t = 0.0, b = alpha, sc = 0.0;
    if (xn2 != 0.0) {
      b = -copysign(sqrt(alpha * alpha + xn2), alpha);
      t = (b - alpha) / b;
      sc = 1.0 / (alpha - b);
    }
    s3[0] = t;
    s3[1] = b;
    s3[2] = sc;
  }
  __syncthreads();
  tau = s3[0];
  beta = s3[1];
  scal = s3[2];
}

// T(0:k, 0:n-k) = R(0:k,0:k) \ R(0:k, k:n); T has leading dimension n.
// Back substitution R(0:r0+1, 0:r0+1) x = b for one column held by a warp in
// registers (tv[q] = row lane + 32 q, rows < 128).  Same operations in the same
// order as the shared-column form below, so both give the same bits.
__device__ __forceinline__ void warp_backsolve128(const double* W, int m, int r0, double (&tv)[4]) {
  const int lane = threadIdx.x & 31;
  for (int r = r0; r >= 0; --r) {
    const int s = r >> 5;
    const double v = (s == 0) ? tv[0] : (s == 1) ? tv[1] : (s == 2) ? tv[2] : tv[3];
    const double xr = __shfl_sync(0xffffffffu, v, r & 31) / W[r + (size_t)r * m];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = lane + 32 * q;
      if (i < r) tv[q] -= W[i + (size_t)r * m] * xr;
      else if (i == r) tv[q] = xr;
    }
  }
}

__device__ void id_trisolve(const double* W, int m, int n, int k, double* T) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (k <= 128) {
    for (int c = k + w; c < n; c += 8) {
      double tv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = lane + 32 * q;
        tv[q] = (i < k) ? W[i + (size_t)c * m] : 0.0;
      }
      warp_backsolve128(W, m, k - 1, tv);
      double* t = T + (size_t)(c - k) * n;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = lane + 32 * q;
        if (i < k) t[i] = tv[q];
      }
    }
    return;
  }
  for (int c = k + w; c < n; c += 8) {
    double* t = T + (size_t)(c - k) * n;
    for (int i = lane; i < k; i += 32) t[i] = W[i + (size_t)c * m];
    __syncwarp();
    for (int r = k - 1; r >= 0; --r) {
      const double xr = t[r] / W[r + (size_t)r * m];
      __syncwarp();
      if (lane == 0) t[r] = xr;
      for (int i = lane; i < r; i += 32) t[i] -= W[i + (size_t)r * m] * xr;
      __syncwarp();
    }
  }
}

// sqrt(||y||) estimators of Common/ID.m:68-86 on the original block A.
__device__ double id_rand_norm(const IdP& p, int k, const double* x, double* y, double* sh) {
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const double* A = p.A;
  // y = A_rs x
  for (int i = tid; i < m; i += 256) {
    double t = 0.0;
    for (int c = k; c < n; ++c) t += A[i + (size_t)p.perm[c] * m] * x[c - k];
    y[i] = t;
  }
  __syncthreads();
  // z = A_rs^T y ; accumulate ||z||^2
  double part = 0.0;
  for (int c = k + w; c < n; c += 8) {
    double d = 0.0;
    for (int i = lane; i < m; i += 32) d += A[i + (size_t)p.perm[c] * m] * y[i];
    d = warp_sum(d);
    if (lane == 0) part += d * d;
  }
  const double z2 = block_sum256(part, sh);
  return sqrt(sqrt(z2));
}

__device__ double id_rand_error(const IdP& p, int k, const double* T, const double* x, double* y,
                                double* t1, double* sh) {
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const double* A = p.A;
  // t1 = T x (k)
  for (int i = tid; i < k; i += 256) {
    double t = 0.0;
    for (int c = 0; c < n - k; ++c) t += T[i + (size_t)c * n] * x[c];
    t1[i] = t;
  }
  __syncthreads();
  // y = A_sk t1 - A_rs x
  for (int i = tid; i < m; i += 256) {
    double a = 0.0, b = 0.0;
    for (int c = 0; c < k; ++c) a += A[i + (size_t)p.perm[c] * m] * t1[c];
    for (int c = k; c < n; ++c) b += A[i + (size_t)p.perm[c] * m] * x[c - k];
    y[i] = a - b;
  }
  __syncthreads();
  // u = A_sk^T y (k) into t1
  for (int c = w; c < k; c += 8) {
    double d = 0.0;
    for (int i = lane; i < m; i += 32) d += A[i + (size_t)p.perm[c] * m] * y[i];
    d = warp_sum(d);
    if (lane == 0) t1[c] = d;
  }
  __syncthreads();
  // z = T^T u - A_rs^T y, ||z||^2
  double part = 0.0;
  for (int c = k + w; c < n; c += 8) {
    double d = 0.0;
    for (int i = lane; i < m; i += 32) d += A[i + (size_t)p.perm[c] * m] * y[i];
    d = warp_sum(d);
    double e = 0.0;
    for (int i = lane; i < k; i += 32) e += T[i + (size_t)(c - k) * n] * t1[i];
    e = warp_sum(e);
    if (lane == 0) { const double z = e - d; part += z * z; }
  }
  const double z2 = block_sum256(part, sh);
  __syncthreads();
  return sqrt(sqrt(z2));
}

// Rank, interpolation matrix and randomized check of the ID (Common/ID.m:40-86) once the
// pivoted QR has left R in W (FP64); jdone = QR steps done, l = min(m, n).
__device__ void id_finish(const IdP& p, double acc, int l, int jdone, double* sh, int* shi) {
  const unsigned long long seed = p.seed;
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  double* W = p.W;
  if (p.steps_hint == ID_QR_ONLY) {  // pivoted QR for a fixed-rank ID of the caller
    if (tid == 0) {
      *p.rank = l;
      if (p.stat) { p.stat[0] = 0; p.stat[1] = l; }
    }
    return;
  }
  // rank detection (Common/ID.m:51-52) over the computed diagonal
  double Rmx = (l > 0) ? fabs(W[0]) * acc : 0.0;
  auto count_rank = [&](double thr) {
    int cnt = 0;
    for (int i = tid; i < jdone; i += 256) cnt += (fabs(W[i + (size_t)i * m]) > thr) ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    __syncthreads();
    if (lane == 0) shi[w] = cnt;
    __syncthreads();
    int t = 0;
    for (int i = 0; i < 8; ++i) t += shi[i];
    __syncthreads();
    return t;
  };
  int k = (l > 0) ? count_rank(Rmx) : 0;
  id_trisolve(W, m, n, k, p.T);
  __syncthreads();
  int draw = 0;
  double* x = p.x;
  double* y = p.y;
  double* t1 = p.y + m;
  while (k < l) {
    const int r = n - k;
    const unsigned long long st0 = ((unsigned long long)p.problem << 8) | (unsigned)(draw & 0xFF);
    const unsigned long long st1 = ((unsigned long long)p.problem << 8) | (unsigned)((draw + 1) & 0xFF);
    // two unit random vectors: x[0:r] for the error, x[n:n+r] for the norm; entry i is
    // drawn at the residual column's own index, independent of the residual order
    double pa = 0.0, pb = 0.0;
    for (int i = tid; i < r; i += 256) {
      const int c = p.perm[k + i];
      const double a = rng_uniform(seed, st0, c), b = rng_uniform(seed, st1, c);
      x[i] = a; x[n + i] = b;
      pa += a * a; pb += b * b;
    }
    const double na = sqrt(block_sum256(pa, sh));
    const double nb = sqrt(block_sum256(pb, sh));
    for (int i = tid; i < r; i += 256) { x[i] /= na; x[n + i] /= nb; }
    __syncthreads();
    draw += 2;
    const double e = id_rand_error(p, k, p.T, x, y, t1, sh);
    const double nr = id_rand_norm(p, k, x + n, y, sh);
    if (!(e > nr * acc)) break;
    Rmx = 0.75 * Rmx;
    if (jdone < l && !(fabs(W[(size_t)(jdone - 1) * (m + 1)]) <= Rmx)) {
      // the relaxed threshold reaches past the truncated factorization: rerun in full
      if (tid == 0 && p.stat) p.stat[0] = 2;
      if (tid == 0) *p.rank = k;
      return;
    }
    k = count_rank(Rmx);
    id_trisolve(W, m, n, k, p.T);
    __syncthreads();
    if (draw > 250) break;
  }
  if (tid == 0) {
    *p.rank = k;
    if (p.stat) {
      p.stat[0] = (jdone < l) ? 1 : 0;
      p.stat[1] = jdone;
    }
  }
}


constexpr double ID_TOL3Z = 1.4901161193847656e-08;  // sqrt(DBL_EPSILON), xLAQP2's threshold

__global__ void __launch_bounds__(256) k_id_adaptive(const IdP* __restrict__ P, double acc) {
  const IdP p = P[blockIdx.x];
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int l = min(m, n);
  double* W = p.W;
  extern __shared__ double s_dyn[];
  double* norms = s_dyn;  // n: trailing norms (squared), downdated
  // n: each column's norm at its last exact computation, in the random-vector workspace
  // (x is read only once the QR is done)
  double* nref = p.x;
  __shared__ double sh[8];
  __shared__ double hs3[3];
  __shared__ double shv[8];
  __shared__ int shi[8];
  for (long long e = tid; e < (long long)m * n; e += 256) W[e] = p.A[e];
  for (int c = tid; c < n; c += 256) p.perm[c] = c;
  __syncthreads();
  for (int c = w; c < n; c += 8) {
    double d = 0.0;
    for (int i = lane; i < m; i += 32) { const double v = W[i + (size_t)c * m]; d += v * v; }
    d = warp_sum(d);
    if (lane == 0) norms[c] = nref[c] = d;
  }
  __syncthreads();
  // Learned-rank mode: at step steps_hint, stop if |R_jj| is already below the
  // rank threshold with room for two relaxations of the randomized check; if not,
  // look again after another half as many steps.  Pivoted QR with exact column
  // norms has non-increasing |R_jj|, so the rank count, the first k pivots and T
  // equal those of the full factorization.
  const bool every = (p.steps_hint == ID_EVERY_STEP);
  int s_hint = every ? 1 : (p.steps_hint > 0) ? min(p.steps_hint, l) : l;
  int jdone = l;
  for (int j = 0; j < l; ++j) {
    if (j == s_hint && j > 0) {
      if (fabs(W[(size_t)(j - 1) * (m + 1)]) <= fabs(W[0]) * acc * 0.5625) {
        jdone = j;
        break;
      }
      s_hint = every ? j + 1 : min(l, j + max(4, j / 2));
    }
    double best = -1.0;
    int bi = INT_MAX;
    for (int c = j + tid; c < n; c += 256) {
      const double v = norms[c];
      if (v > best) { best = v; bi = c; }
    }
    block_argmax256(best, bi, shv, shi);
    if (bi == INT_MAX) bi = j;
    if (bi != j) {
      for (int i = tid; i < m; i += 256) {
        const double t = W[i + (size_t)j * m];
        W[i + (size_t)j * m] = W[i + (size_t)bi * m];
        W[i + (size_t)bi * m] = t;
      }
      if (tid == 0) {
        const int t = p.perm[j]; p.perm[j] = p.perm[bi]; p.perm[bi] = t;
        const double u = norms[j]; norms[j] = norms[bi]; norms[bi] = u;
        const double v = nref[j]; nref[j] = nref[bi]; nref[bi] = v;
      }
    }
    __syncthreads();
    double part = 0.0;
    for (int i = j + 1 + tid; i < m; i += 256) { const double v = W[i + (size_t)j * m]; part += v * v; }
    const double xn2 = block_sum256(part, sh);
    double tau, beta, scal;
    householder_scalars(W[j + (size_t)j * m], xn2, hs3, tau, beta, scal);
    for (int i = j + 1 + tid; i < m; i += 256) W[i + (size_t)j * m] *= scal;
    __syncthreads();
    if (tid == 0) W[j + (size_t)j * m] = beta;
    for (int c = j + 1 + w; c < n; c += 8) {
      const double wjc = W[j + (size_t)c * m];
      double d = wjc * (lane == 0 ? 1.0 : 0.0);
      for (int i = j + 1 + lane; i < m; i += 32) d += W[i + (size_t)j * m] * W[i + (size_t)c * m];
      d = warp_sum(d) * tau;
      // downdate the column's trailing norm by its new row-j entry (LAPACK xLAQP2's rule,
      // without divisions): recompute it exactly when the cancellation leaves less than
      // sqrt(eps) of the norm last computed exactly.  Every lane takes the same decision
      // from the same values.
      const double nc = norms[c], r = wjc - d;
      bool redo = false;
      double nd = nc;
      if (nc != 0.0) {
        nd = fmax(0.0, __dadd_rn(nc, -__dmul_rn(r, r)));
        redo = nd <= __dmul_rn(ID_TOL3Z, nref[c]);
      }
      __syncwarp();
      if (lane == 0) W[j + (size_t)c * m] = r;
      double nn = 0.0;
      for (int i = j + 1 + lane; i < m; i += 32) {
        const double v = W[i + (size_t)c * m] - d * W[i + (size_t)j * m];
        W[i + (size_t)c * m] = v;
        if (redo) nn += v * v;
      }
      if (redo) {
        nn = warp_sum(nn);
        if (lane == 0) norms[c] = nref[c] = nn;
      } else if (lane == 0) {
        norms[c] = nd;
      }
    }
    __syncthreads();
  }
  id_finish(p, acc, l, jdone, sh, shi);
}

// The ID of a complex block through its real 2 x 2 embedding E(A) (m = 2 x rows, n = 2 x
// columns, column pairs (2c, 2c + 1) = complex column c): the pivoted QR moves the pair whose
// first column has the largest exact trailing norm to the front (the lowest pair within a
// factor 1 - 2^-14 of the largest: ties of mirror-symmetric boxes resolve by index, not by
// rounding) and reflects both columns.  The two columns of a pair are a and i a, orthogonal and of equal
// norm, so the pivot order over pairs, the rank counted in pairs (|R_{2t,2t}| = |R_tt| of the
// complex QR) and T = R11 \ R12 = E(T) are those of the complex ID (Common/ID.m:40-65 on a
// complex A).  perm is the real column permutation (pairs kept together), *rank is in real
// columns (twice the complex rank).  The randomized posterior check draws its real unit
// vectors over complex columns (entry of complex column c at counter c), which E maps to
// (x_c, 0) pairs.
__device__ void id_finish_pairs(const IdP& p, double acc, int lp, double* sh, int* shi) {
  const unsigned long long seed = p.seed;
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  double* W = p.W;
  double Rmx = (lp > 0) ? fabs(W[0]) * acc : 0.0;
  auto count_pairs = [&](double thr) {
    int cnt = 0;
    for (int t = tid; t < lp; t += 256) cnt += (fabs(W[2 * t + (size_t)(2 * t) * m]) > thr) ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    __syncthreads();
    if (lane == 0) shi[w] = cnt;
    __syncthreads();
    int t = 0;
    for (int i = 0; i < 8; ++i) t += shi[i];
    __syncthreads();
    return t;
  };
  int kc = (lp > 0) ? count_pairs(Rmx) : 0;
  id_trisolve(W, m, n, 2 * kc, p.T);
  __syncthreads();
  int draw = 0;
  double* x = p.x;
  double* y = p.y;
  double* t1 = p.y + m;
  while (kc < lp) {
    const int k = 2 * kc, r = n - k;
    const unsigned long long st0 = ((unsigned long long)p.problem << 8) | (unsigned)(draw & 0xFF);
    const unsigned long long st1 = ((unsigned long long)p.problem << 8) | (unsigned)((draw + 1) & 0xFF);
    double pa = 0.0, pb = 0.0;
    for (int i = tid; i < r; i += 256) {
      double a = 0.0, b = 0.0;
      if ((i & 1) == 0) {
        const int c = p.perm[k + i] >> 1;
        a = rng_uniform(seed, st0, c);
        b = rng_uniform(seed, st1, c);
      }
      x[i] = a; x[n + i] = b;
      pa += a * a; pb += b * b;
    }
    const double na = sqrt(block_sum256(pa, sh));
    const double nb = sqrt(block_sum256(pb, sh));
    for (int i = tid; i < r; i += 256) { x[i] /= na; x[n + i] /= nb; }
    __syncthreads();
    draw += 2;
    const double e = id_rand_error(p, k, p.T, x, y, t1, sh);
    const double nr = id_rand_norm(p, k, x + n, y, sh);
    if (!(e > nr * acc)) break;
    Rmx = 0.75 * Rmx;
    kc = count_pairs(Rmx);
    id_trisolve(W, m, n, 2 * kc, p.T);
    __syncthreads();
    if (draw > 250) break;
  }
  if (tid == 0) {
    *p.rank = 2 * kc;
    if (p.stat) {
      p.stat[0] = 0;
      p.stat[1] = 2 * lp;
    }
  }
}

__global__ void __launch_bounds__(256) k_id_pairs(const IdP* __restrict__ P, double acc) {
  const IdP p = P[blockIdx.x];
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int lp = min(m, n) / 2;
  double* W = p.W;
  extern __shared__ double s_dyn[];
  double* norms = s_dyn;  // n: trailing norms (squared), downdated
  // n: each column's norm at its last exact computation, in the random-vector workspace
  // (x is read only once the QR is done)
  double* nref = p.x;
  __shared__ double sh[8];
  __shared__ double hs3[3];
  __shared__ double shv[8];
  __shared__ int shi[8];
  for (long long e = tid; e < (long long)m * n; e += 256) W[e] = p.A[e];
  for (int c = tid; c < n; c += 256) p.perm[c] = c;
  __syncthreads();
  for (int c = w; c < n; c += 8) {
    double d = 0.0;
    for (int i = lane; i < m; i += 32) { const double v = W[i + (size_t)c * m]; d += v * v; }
    d = warp_sum(d);
    if (lane == 0) norms[c] = d;
  }
  __syncthreads();
  for (int t = 0; t < lp; ++t) {
    double best = -1.0;
    int bi = INT_MAX;
    for (int q = t + tid; q < n / 2; q += 256) {
      const double v = norms[2 * q];
      if (v > best) { best = v; bi = q; }
    }
    block_argmax256(best, bi, shv, shi);
    // pivot ties: the lowest pair whose norm is within a factor 1 - 2^-14 of the largest
    // (mirror-symmetric boxes have pairs of equal norm up to rounding)
    const double thr = __dadd_rn(best, -__dmul_rn(best, 0x1.0p-14));
    double cand = -1.0;
    int ci = INT_MAX;
    for (int q = t + tid; q < n / 2; q += 256)
      if (norms[2 * q] >= thr) { cand = 1.0; ci = q; break; }
    block_argmax256(cand, ci, shv, shi);
    bi = (ci == INT_MAX) ? t : ci;
    if (bi != t) {
      for (int e = tid; e < 2 * m; e += 256) {
        const int i = e % m, h = e / m;
        const size_t a = i + (size_t)(2 * t + h) * m, b = i + (size_t)(2 * bi + h) * m;
        const double u = W[a];
        W[a] = W[b];
        W[b] = u;
      }
      if (tid < 2) {
        const int a = 2 * t + tid, b = 2 * bi + tid;
        const int u = p.perm[a]; p.perm[a] = p.perm[b]; p.perm[b] = u;
        const double v = norms[a]; norms[a] = norms[b]; norms[b] = v;
      }
    }
    __syncthreads();
    for (int j = 2 * t; j < 2 * t + 2; ++j) {
      double part = 0.0;
      for (int i = j + 1 + tid; i < m; i += 256) { const double v = W[i + (size_t)j * m]; part += v * v; }
      const double xn2 = block_sum256(part, sh);
      double tau, beta, scal;
      householder_scalars(W[j + (size_t)j * m], xn2, hs3, tau, beta, scal);
      for (int i = j + 1 + tid; i < m; i += 256) W[i + (size_t)j * m] *= scal;
      __syncthreads();
      if (tid == 0) W[j + (size_t)j * m] = beta;
      for (int c = j + 1 + w; c < n; c += 8) {
        double d = W[j + (size_t)c * m] * (lane == 0 ? 1.0 : 0.0);
        for (int i = j + 1 + lane; i < m; i += 32) d += W[i + (size_t)j * m] * W[i + (size_t)c * m];
        d = warp_sum(d) * tau;
        if (lane == 0) W[j + (size_t)c * m] -= d;
        double nn = 0.0;
        for (int i = j + 1 + lane; i < m; i += 32) {
          const double v = W[i + (size_t)c * m] - d * W[i + (size_t)j * m];
          W[i + (size_t)c * m] = v;
          nn += v * v;
        }
        nn = warp_sum(nn);
        if (lane == 0) norms[c] = nn;
      }
      __syncthreads();
    }
  }
  id_finish_pairs(p, acc, lp, sh, shi);
}

// Sum of a double-float value over a 256-thread block (xor butterfly, then the eight
// warp sums in order); every thread gets the same (h, l).
__device__ __forceinline__ void block_sum256_df(float& h, float& l, float* shh, float* shl) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, h, o), ol = __shfl_xor_sync(0xffffffffu, l, o);
    df_add(h, l, oh, ol);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) { shh[w] = h; shl[w] = l; }
  __syncthreads();
  h = shh[0];
  l = shl[0];
#pragma unroll
  for (int i = 1; i < 8; ++i) df_add(h, l, shh[i], shl[i]);
  __syncthreads();
}

__device__ __forceinline__ double df_val(float2 v) { return (double)v.x + (double)v.y; }

// The ID with its pivoted QR in double-float arithmetic (FP64 data held as float pairs in
// W's own storage, every product and sum on the FP32 pipes, ~2^-48 relative): the same
// pivot rule (exact trailing column norms), Householder steps and learned-rank stop as
// k_id_adaptive.  The per-step Householder scalars are formed in FP64.  R is then
// widened to FP64 in place and the rank, T and the randomized check run as in FP64.
__global__ void __launch_bounds__(256) k_id_adaptive_df(const IdP* __restrict__ P, double acc) {
  const IdP p = P[blockIdx.x];
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int l = min(m, n);
  float2* W = reinterpret_cast<float2*>(p.W);
  extern __shared__ double s_dyn[];
  float2* norms = reinterpret_cast<float2*>(s_dyn);  // n
  __shared__ double sh[8];
  __shared__ int shi[8];
  __shared__ float shh[8], shl[8];
  __shared__ float hsf[6];
  for (long long e = tid; e < (long long)m * n; e += 256) {
    float h, lo;
    split_d2f(p.A[e], h, lo);
    W[e] = make_float2(h, lo);
  }
  for (int c = tid; c < n; c += 256) p.perm[c] = c;
  __syncthreads();
  for (int c = w; c < n; c += 8) {
    float nh = 0.f, nl = 0.f;
    for (int i = lane; i < m; i += 32) { const float2 v = W[i + (size_t)c * m]; df_madd(nh, nl, v.x, v.y, v.x, v.y); }
    warp_sum_df(nh, nl);
    if (lane == 0) norms[c] = make_float2(nh, nl);
  }
  __syncthreads();
  const bool every = (p.steps_hint == ID_EVERY_STEP);
  int s_hint = every ? 1 : (p.steps_hint > 0) ? min(p.steps_hint, l) : l;
  int jdone = l;
  for (int j = 0; j < l; ++j) {
    if (j == s_hint && j > 0) {
      if (fabs(df_val(W[(size_t)(j - 1) * (m + 1)])) <= fabs(df_val(W[0])) * acc * 0.5625) {
        jdone = j;
        break;
      }
      s_hint = every ? j + 1 : min(l, j + max(4, j / 2));
    }
    // arg-max of the normalised float-pair norms (hi, then lo), lowest index among equals
    float bh = -1.f, bl = 0.f;
    int bi = INT_MAX;
    for (int c = j + tid; c < n; c += 256) {
      const float2 v = norms[c];
      if (v.x > bh || (v.x == bh && v.y > bl)) { bh = v.x; bl = v.y; bi = c; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, bh, o), ol = __shfl_xor_sync(0xffffffffu, bl, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (oh > bh || (oh == bh && (ol > bl || (ol == bl && oi < bi)))) { bh = oh; bl = ol; bi = oi; }
    }
    __syncthreads();
    if (lane == 0) { shh[w] = bh; shl[w] = bl; shi[w] = bi; }
    __syncthreads();
    bh = shh[0]; bl = shl[0]; bi = shi[0];
#pragma unroll
    for (int q = 1; q < 8; ++q)
      if (shh[q] > bh || (shh[q] == bh && (shl[q] > bl || (shl[q] == bl && shi[q] < bi)))) {
        bh = shh[q]; bl = shl[q]; bi = shi[q];
      }
    __syncthreads();
    if (bi == INT_MAX) bi = j;
    if (bi != j) {
      for (int i = tid; i < m; i += 256) {
        const float2 t = W[i + (size_t)j * m];
        W[i + (size_t)j * m] = W[i + (size_t)bi * m];
        W[i + (size_t)bi * m] = t;
      }
      if (tid == 0) {
        const int t = p.perm[j]; p.perm[j] = p.perm[bi]; p.perm[bi] = t;
        const float2 u = norms[j]; norms[j] = norms[bi]; norms[bi] = u;
      }
    }
    __syncthreads();
    float xh = 0.f, xl = 0.f;
    for (int i = j + 1 + tid; i < m; i += 256) { const float2 v = W[i + (size_t)j * m]; df_madd(xh, xl, v.x, v.y, v.x, v.y); }
    block_sum256_df(xh, xl, shh, shl);
    // the step's scalars in FP64 by thread 0, shared as float pairs
    if (tid == 0) {
      const double xn2 = (double)xh + (double)xl;
      const double alpha = df_val(W[j + (size_t)j * m]);
      double tau = 0.0, beta = alpha, scal = 0.0;
      if (xn2 != 0.0) {
        beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
        tau = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      split_d2f(scal, hsf[0], hsf[1]);
      split_d2f(tau, hsf[2], hsf[3]);
      split_d2f(beta, hsf[4], hsf[5]);
    }
    __syncthreads();
    const float sch = hsf[0], scl = hsf[1], tah = hsf[2], tal = hsf[3];
    for (int i = j + 1 + tid; i < m; i += 256) {
      float2 v = W[i + (size_t)j * m];
      df_mul(v.x, v.y, sch, scl);
      W[i + (size_t)j * m] = v;
    }
    __syncthreads();
    if (tid == 0) W[j + (size_t)j * m] = make_float2(hsf[4], hsf[5]);
    for (int c = j + 1 + w; c < n; c += 8) {
      float dh = 0.f, dl = 0.f;
      if (lane == 0) { const float2 v = W[j + (size_t)c * m]; dh = v.x; dl = v.y; }
      for (int i = j + 1 + lane; i < m; i += 32) {
        const float2 v = W[i + (size_t)j * m], a = W[i + (size_t)c * m];
        df_madd(dh, dl, v.x, v.y, a.x, a.y);
      }
      warp_sum_df(dh, dl);
      df_mul(dh, dl, tah, tal);
      if (lane == 0) {
        float2 v = W[j + (size_t)c * m];
        df_add(v.x, v.y, -dh, -dl);
        W[j + (size_t)c * m] = v;
      }
      float nh = 0.f, nl = 0.f;
      for (int i = j + 1 + lane; i < m; i += 32) {
        const float2 v = W[i + (size_t)j * m];
        float2 a = W[i + (size_t)c * m];
        df_madd(a.x, a.y, -dh, -dl, v.x, v.y);
        W[i + (size_t)c * m] = a;
        df_madd(nh, nl, a.x, a.y, a.x, a.y);
      }
      warp_sum_df(nh, nl);
      if (lane == 0) norms[c] = make_float2(nh, nl);
    }
    __syncthreads();
  }
  // widen R (and the reflectors) to FP64 in place: element e's float pair and its double
  // share the same 8 bytes
  double* Wd = p.W;
  for (long long e = tid; e < (long long)m * n; e += 256) {
    const float2 v = W[e];
    Wd[e] = df_to_double(v.x, v.y);
  }
  __syncthreads();
  id_finish(p, acc, l, jdone, sh, shi);
}

void id_adaptive_batched(const IdP* dP, int batch, double acc, cudaStream_t s, bool df) {
  if (batch <= 0) return;
  // dynamic shared memory: norms (n doubles or float pairs); the host guarantees n <= 4096
  if (df) {
    k_id_adaptive_df<<<batch, 256, 4096 * sizeof(double), s>>>(dP, acc);
    check_launch("k_id_adaptive_df");
    return;
  }
  k_id_adaptive<<<batch, 256, 4096 * sizeof(double), s>>>(dP, acc);
  check_launch("k_id_adaptive");
}

// Fixed-rank ID reusing the pivoted QR in W: T = V_q diag(1/s_q) U_q^T R12 over
// the singular triplets of R11 = W(0:k,0:k) with s > 1e-12 (skel_col_fixed,
// Common/ID.m:106-113).  When every singular value is provably above the cut --
// 1/||R11^-1||_F <= s_min -- the pseudo-inverse is the inverse and T = R11 \ R12
// by back substitution; otherwise a one-sided Jacobi SVD applies the cut.
__global__ void __launch_bounds__(256) k_id_fixed(const IdP* __restrict__ P) {
  const IdP p = P[blockIdx.x];
  const int k = p.force_k;
  if (k < 0) return;
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const double* Wq = p.W;
  __shared__ double sh[8];
  if (k >= 1 && k <= 128) {
    double part = 0.0;
    for (int c = w; c < k; c += 8) {  // column c of R11^-1 (zero below row c)
      double tv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) tv[q] = (lane + 32 * q == c) ? 1.0 : 0.0;
      warp_backsolve128(Wq, m, c, tv);
      double ss = 0.0;
#pragma unroll
      for (int q = 0; q < 4; ++q) ss += tv[q] * tv[q];
      ss = warp_sum(ss);
      if (lane == 0) part += ss;
    }
    const double fro2 = block_sum256(part, sh);
    if (1.0 / sqrt(fro2) > 2e-12) {  // factor-2 margin over rounding in the computed inverse
      id_trisolve(Wq, m, n, k, p.T);
      if (tid == 0) *p.rank = k;
      return;
    }
  }
  // One-sided Jacobi on X = R11^T (R11 comes from a column-pivoted QR, which
  // makes the columns of its transpose nearly orthogonal: few sweeps, as in
  // Drmac & Veselic, "New fast and accurate Jacobi SVD algorithm", SIMAX 2008).
  // X V = M with orthogonal columns M_q = s_q u_q, so R11 = V S U^T and
  // pinv(R11) = sum_q M_q V_q^T / s_q^2.
  double* U = p.svdW;  // k x k, ld k: X, rotated into M
  double* V = p.svdV;  // k x k, ld k
  __shared__ int s_rot;
  for (int e = tid; e < k * k; e += 256) {
    const int i = e % k, j = e / k;
    U[e] = (j <= i) ? Wq[j + (size_t)i * m] : 0.0;
    V[e] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  const int K2 = (k % 2 == 0) ? k : k + 1;
  for (int sweep = 0; sweep < 60 && k > 1; ++sweep) {
    if (tid == 0) s_rot = 0;
    __syncthreads();
    for (int rnd = 0; rnd < K2 - 1; ++rnd) {
      for (int pi = w; pi < K2 / 2; pi += 8) {
        int a, b;
        if (pi == 0) { a = K2 - 1; b = rnd; }
        else { a = (rnd + pi) % (K2 - 1); b = (rnd - pi + K2 - 1) % (K2 - 1); }
        if (a >= k || b >= k) continue;
        if (a > b) { const int t = a; a = b; b = t; }
        double al = 0.0, be = 0.0, ga = 0.0;
        for (int i = lane; i < k; i += 32) {
          const double u = U[i + (size_t)a * k], v = U[i + (size_t)b * k];
          al += u * u; be += v * v; ga += u * v;
        }
        al = warp_sum(al); be = warp_sum(be); ga = warp_sum(ga);
        // the rotation is formed by lane 0 and broadcast (its FP64 square roots and
        // divisions would otherwise run in all 32 lanes and outweigh the update itself)
        double c = 1.0, s = 0.0;
        int rot = 0;
        if (lane == 0 && ga != 0.0 && fabs(ga) > 1e-15 * sqrt(al * be)) {
          const double zeta = (be - al) / (2.0 * ga);
          const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          c = 1.0 / sqrt(1.0 + t * t);
          s = c * t;
          rot = 1;
        }
        rot = __shfl_sync(0xffffffffu, rot, 0);
        if (rot) {
          c = __shfl_sync(0xffffffffu, c, 0);
          s = __shfl_sync(0xffffffffu, s, 0);
          for (int i = lane; i < k; i += 32) {
            const double u = U[i + (size_t)a * k], v = U[i + (size_t)b * k];
            U[i + (size_t)a * k] = c * u - s * v;
            U[i + (size_t)b * k] = s * u + c * v;
            const double x = V[i + (size_t)a * k], y = V[i + (size_t)b * k];
            V[i + (size_t)a * k] = c * x - s * y;
            V[i + (size_t)b * k] = s * x + c * y;
          }
          if (lane == 0) s_rot = 1;
        }
      }
      __syncthreads();
    }
    const int rot = s_rot;
    __syncthreads();
    if (!rot) break;
  }
  // sigma_i^2 into x[0:k]
  double* s2 = p.x;
  for (int c = w; c < k; c += 8) {
    double d = 0.0;
    for (int i = lane; i < k; i += 32) { const double u = U[i + (size_t)c * k]; d += u * u; }
    d = warp_sum(d);
    if (lane == 0) s2[c] = d;
  }
  __syncthreads();
  // T(:, c) = sum_{q: s_q > 1e-12} M_q (V_q . R12(:,c)) / s_q^2
  for (int c = k + w; c < n; c += 8) {
    double* t = p.T + (size_t)(c - k) * n;
    for (int i = lane; i < k; i += 32) t[i] = 0.0;
    __syncwarp();
    for (int q = 0; q < k; ++q) {
      if (!(sqrt(s2[q]) > 1e-12)) continue;
      double d = 0.0;
      for (int i = lane; i < k; i += 32) d += V[i + (size_t)q * k] * Wq[i + (size_t)c * m];
      d = warp_sum(d) / s2[q];
      for (int i = lane; i < k; i += 32) t[i] += U[i + (size_t)q * k] * d;
      __syncwarp();
    }
  }
  if (tid == 0) *p.rank = k;
}

// Pivoted Householder QR with the explicit thin Q (QR_findrank's [Q,R,~] = qr(Y,0),
// Common/QR_findrank.m:50-70): the pivot rule, reflectors and norms of k_id_adaptive,
// then Q = H_0 ... H_{l-1} [I; 0] accumulated backwards (LAPACK dorg2r order).
__global__ void __launch_bounds__(256) k_pqr_q(const PqrP* __restrict__ P) {
  const PqrP p = P[blockIdx.x];
  const int m = p.m, n = p.l, ld = p.ldw, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int l = min(m, n);
  double* W = p.W;
  extern __shared__ double s_dyn[];
  double* norms = s_dyn;  // n
  __shared__ double hs3[3];
  __shared__ double sh[8];
  __shared__ double shv[8];
  __shared__ int shi[8];
  for (int c = w; c < n; c += 8) {
    double d = 0.0;
    for (int i = lane; i < m; i += 32) { const double v = W[i + (size_t)c * ld]; d += v * v; }
    d = warp_sum(d);
    if (lane == 0) norms[c] = d;
  }
  __syncthreads();
  for (int j = 0; j < l; ++j) {
    double best = -1.0;
    int bi = INT_MAX;
    for (int c = j + tid; c < n; c += 256) {
      const double v = norms[c];
      if (v > best) { best = v; bi = c; }
    }
    block_argmax256(best, bi, shv, shi);
    if (bi == INT_MAX) bi = j;
    if (bi != j) {
      for (int i = tid; i < m; i += 256) {
        const double t = W[i + (size_t)j * ld];
        W[i + (size_t)j * ld] = W[i + (size_t)bi * ld];
        W[i + (size_t)bi * ld] = t;
      }
      if (tid == 0) { const double u = norms[j]; norms[j] = norms[bi]; norms[bi] = u; }
    }
    __syncthreads();
    double part = 0.0;
    for (int i = j + 1 + tid; i < m; i += 256) { const double v = W[i + (size_t)j * ld]; part += v * v; }
    const double xn2 = block_sum256(part, sh);
    double tau, beta, scal;
    householder_scalars(W[j + (size_t)j * ld], xn2, hs3, tau, beta, scal);
    for (int i = j + 1 + tid; i < m; i += 256) W[i + (size_t)j * ld] *= scal;
    __syncthreads();
    if (tid == 0) {
      W[j + (size_t)j * ld] = beta;
      p.tau[j] = tau;
      p.D[j] = fabs(beta);
    }
    for (int c = j + 1 + w; c < n; c += 8) {
      double d = W[j + (size_t)c * ld] * (lane == 0 ? 1.0 : 0.0);
      for (int i = j + 1 + lane; i < m; i += 32) d += W[i + (size_t)j * ld] * W[i + (size_t)c * ld];
      d = warp_sum(d) * tau;
      if (lane == 0) W[j + (size_t)c * ld] -= d;
      double nn = 0.0;
      for (int i = j + 1 + lane; i < m; i += 32) {
        const double v = W[i + (size_t)c * ld] - d * W[i + (size_t)j * ld];
        W[i + (size_t)c * ld] = v;
        nn += v * v;
      }
      nn = warp_sum(nn);
      if (lane == 0) norms[c] = nn;
    }
    __syncthreads();
  }
  // Q = [I; 0], then H_j from j = l-1 down to 0 on columns c >= j (the others are e_c)
  for (long long e = tid; e < (long long)m * l; e += 256) {
    const int i = (int)(e % m), c = (int)(e / m);
    p.Q[i + (size_t)c * p.ldq] = (i == c) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int j = l - 1; j >= 0; --j) {
    const double tau = p.tau[j];
    if (tau != 0.0) {
      for (int c = j + w; c < l; c += 8) {
        double* q = p.Q + (size_t)c * p.ldq;
        double d = (lane == 0) ? q[j] : 0.0;
        for (int i = j + 1 + lane; i < m; i += 32) d += W[i + (size_t)j * ld] * q[i];
        d = warp_sum(d) * tau;
        if (lane == 0) q[j] -= d;
        for (int i = j + 1 + lane; i < m; i += 32) q[i] -= d * W[i + (size_t)j * ld];
      }
    }
    __syncthreads();
  }
}

void pqr_q_batched(const PqrP* dP, int batch, cudaStream_t s) {
  if (batch <= 0) return;
  // dynamic shared memory: column norms (l doubles); the host guarantees l <= 4096
  k_pqr_q<<<batch, 256, 4096 * sizeof(double), s>>>(dP);
  check_launch("k_pqr_q");
}

__global__ void k_gauss(const GaussP* __restrict__ P, long long maxEntries) {
  const GaussP g = P[blockIdx.y];
  const long long cnt = (long long)g.m * g.l;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt && e < maxEntries;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % g.m), j = (int)(e / g.m);
    const unsigned long long c0 = 12ULL * (unsigned long long)e;
    double v = rng_uniform(g.seed, g.stream, c0);
    for (int t = 1; t < 12; ++t) v = __dadd_rn(v, rng_uniform(g.seed, g.stream, c0 + t));
    g.G[i + (size_t)j * g.ldg] = __dadd_rn(v, -6.0);
  }
}

void gauss_batched(const GaussP* dP, int batch, long long maxEntries, cudaStream_t s) {
  if (batch <= 0 || maxEntries <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "gauss batch too large");
  const int gx = std::min(ceil_div(maxEntries, 256), 1024);
  k_gauss<<<dim3(gx, batch), 256, 0, s>>>(dP, maxEntries);
  check_launch("k_gauss");
}

void id_pairs_batched(const IdP* dP, int batch, int maxn, double acc, cudaStream_t s) {
  if (batch <= 0) return;
  HSS_REQUIRE(maxn <= 4096 && maxn % 2 == 0, HSS_ERR_ARG, "pair ID: at most 4096 real columns, even");
  k_id_pairs<<<batch, 256, 4096 * sizeof(double), s>>>(dP, acc);
  check_launch("k_id_pairs");
}

void id_fixed_batched(const IdP* dP, int batch, cudaStream_t s) {
  if (batch <= 0) return;
  k_id_fixed<<<batch, 256, 0, s>>>(dP);
  check_launch("k_id_fixed");
}

// ---------------------------------------------------------------------------
// Explicit instantiations
// ---------------------------------------------------------------------------
#define HSS_INST(R)                                                                          \
  template void gemm_batched<R>(const GemmP<R>*, int, int, int, bool, bool, R, R, cudaStream_t); \
  template void gemm_skinny<R>(const GemmP<R>*, int, int, R, R, cudaStream_t);               \
  template void gemm_skinny_split<R>(const GemmP<R>*, int, int, int, R, R, int, R*, cudaStream_t); \
  template int skinny_ksplit<R>(int, int, int);                                              \
  template void invert_batched<R>(const InvP<R>*, int, int, cudaStream_t, bool);             \
  template void lstsq_batched<R>(const QrP<R>*, int, int, int, int, cudaStream_t, bool, bool);
HSS_INST(double)
HSS_INST(float)
#undef HSS_INST

}  // namespace hss
