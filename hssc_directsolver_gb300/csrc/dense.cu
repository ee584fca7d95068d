// Batched dense linear algebra kernels (FP64 and FP32) for the HSS levels.
#include "dense.cuh"

#include <cfloat>
#include <cmath>

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
// One block = 32 rows; the 8 warps take interleaved K indices; fixed-order
// cross-warp reduction.
// ---------------------------------------------------------------------------
constexpr int SKINNY_NR = 8;

template <typename R>
__global__ void __launch_bounds__(256) k_gemm_skinny(const GemmP<R>* __restrict__ P, R alpha, R beta) {
  const GemmP<R> p = P[blockIdx.y];
  const int row0 = blockIdx.x * 32;
  if (row0 >= p.M) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int row = row0 + lane;
  const bool live = row < p.M;
  const int N = p.N;
  R acc[SKINNY_NR];
#pragma unroll
  for (int c = 0; c < SKINNY_NR; ++c) acc[c] = R(0);
  const R* __restrict__ A = p.A + (live ? row : 0);
  const R* __restrict__ B = p.B;
  int k = w;
  for (; k + 24 < p.K; k += 32) {
    R a0 = live ? __ldg(A + (size_t)k * p.lda) : R(0);
    R a1 = live ? __ldg(A + (size_t)(k + 8) * p.lda) : R(0);
    R a2 = live ? __ldg(A + (size_t)(k + 16) * p.lda) : R(0);
    R a3 = live ? __ldg(A + (size_t)(k + 24) * p.lda) : R(0);
#pragma unroll
    for (int c = 0; c < SKINNY_NR; ++c) {
      if (c < N) {
        const R* bc = B + (size_t)c * p.ldb;
        acc[c] += a0 * __ldg(bc + k);
        acc[c] += a1 * __ldg(bc + k + 8);
        acc[c] += a2 * __ldg(bc + k + 16);
        acc[c] += a3 * __ldg(bc + k + 24);
      }
    }
  }
  for (; k < p.K; k += 8) {
    R a0 = live ? __ldg(A + (size_t)k * p.lda) : R(0);
#pragma unroll
    for (int c = 0; c < SKINNY_NR; ++c)
      if (c < N) acc[c] += a0 * __ldg(B + (size_t)c * p.ldb + k);
  }
  __shared__ R red[8][SKINNY_NR][32];
#pragma unroll
  for (int c = 0; c < SKINNY_NR; ++c) red[w][c][lane] = acc[c];
  __syncthreads();
  if (w == 0 && live) {
#pragma unroll
    for (int c = 0; c < SKINNY_NR; ++c) {
      if (c >= N) break;
      R t = red[0][c][lane];
#pragma unroll
      for (int q = 1; q < 8; ++q) t += red[q][c][lane];
      R* cp = p.C + row + (size_t)c * p.ldc;
      *cp = (beta == R(0)) ? alpha * t : alpha * t + beta * (*cp);
    }
  }
}

template <typename R>
void gemm_skinny(const GemmP<R>* dP, int batch, int maxM, R alpha, R beta, cudaStream_t s) {
  if (batch <= 0 || maxM <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "skinny gemm batch too large");
  dim3 grid(ceil_div(maxM, 32), batch);
  k_gemm_skinny<R><<<grid, 256, 0, s>>>(dP, alpha, beta);
  check_launch("k_gemm_skinny");
}

// ---------------------------------------------------------------------------
// Blocked Gauss-Jordan inversion with partial pivoting.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_gj_panel(const InvP<R>* __restrict__ P, int j0) {
  const InvP<R> p = P[blockIdx.x];
  const int n = p.n;
  if (j0 >= n) return;
  if (*p.info != 0) return;
  const int tid = threadIdx.x;
  const int jend = min(j0 + GJ_NB, n), nbk = jend - j0;
  R* A = p.A;
  const size_t lda = p.lda;
  __shared__ R s_row[GJ_NB];
  __shared__ R shv[8];
  __shared__ int shi[8];
  for (int j = j0; j < jend; ++j) {
    R best = R(-1);
    int bi = INT_MAX;
    for (int i = j + tid; i < n; i += 256) {
      const R v = fabs(A[i + j * lda]);
      if (v > best) { best = v; bi = i; }
    }
    block_argmax256(best, bi, shv, shi);
    if (bi == INT_MAX || !(best > R(0)) || !isfinite(best)) {
      if (tid == 0) *p.info = (best == R(0)) ? (j + 1) : -1;
      return;
    }
    if (tid == 0) p.ipiv[j] = bi;
    if (bi != j) {
      for (int c = tid; c < n; c += 256) {
        const R t = A[j + c * lda];
        A[j + c * lda] = A[bi + c * lda];
        A[bi + c * lda] = t;
      }
    }
    __syncthreads();
    const R piv = A[j + j * lda];
    const R rp = R(1) / piv;
    if (tid < nbk) {
      const int c = j0 + tid;
      s_row[tid] = (c == j) ? rp : A[j + c * lda] * rp;
    }
    __syncthreads();
    for (int i = tid; i < n; i += 256) {
      if (i == j) continue;
      const R aij = A[i + j * lda];
      for (int cc = 0; cc < nbk; ++cc) {
        const int c = j0 + cc;
        if (c == j) continue;
        A[i + c * lda] -= aij * s_row[cc];
      }
      A[i + j * lda] = -aij * rp;
    }
    __syncthreads();
    if (tid < nbk) A[j + (j0 + tid) * lda] = s_row[tid];
    __syncthreads();
  }
  // Save the pivot rows of every column for the delayed update.
  for (int e = tid; e < nbk * n; e += 256) {
    const int r = e % nbk, c = e / nbk;
    p.W[r + (size_t)c * GJ_NB] = A[j0 + r + c * lda];
  }
}

// A[:, c] = mask(A[:, c]) + A[:, panel] * W[:, c] for every c outside the panel,
// mask zeroing the panel rows.
template <typename R>
__global__ void __launch_bounds__(256) k_gj_update(const InvP<R>* __restrict__ P, int j0) {
  const InvP<R> p = P[blockIdx.z];
  const int n = p.n;
  if (j0 >= n) return;
  if (*p.info != 0) return;
  const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  if (m0 >= n || n0 >= n) return;
  const int jend = min(j0 + GJ_NB, n), nbk = jend - j0;
  if (n0 >= j0 && n0 + 64 <= jend) return;
  __shared__ R Ps[GJ_NB][64 + 1];
  __shared__ R Ws[GJ_NB][64 + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  R* A = p.A;
  const size_t lda = p.lda;
  for (int e = tid; e < 64 * GJ_NB; e += 256) {
    const int i = e & 63, r = e >> 6;
    const int gi = m0 + i;
    Ps[r][i] = (gi < n && r < nbk) ? A[gi + (size_t)(j0 + r) * lda] : R(0);
  }
  for (int e = tid; e < 64 * GJ_NB; e += 256) {
    const int r = e % GJ_NB, j = e / GJ_NB;
    const int gj = n0 + j;
    Ws[r][j] = (gj < n && r < nbk) ? p.W[r + (size_t)gj * GJ_NB] : R(0);
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
      const int gi = m0 + tx + 16 * i;
      if (gi >= n) continue;
      R* c = A + gi + (size_t)gj * lda;
      const bool prow = (gi >= j0 && gi < jend);
      *c = prow ? acc[i][j] : (*c + acc[i][j]);
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
__global__ void __launch_bounds__(256) k_gj_gather(const InvP<R>* __restrict__ P) {
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
void invert_batched(const InvP<R>* dP, int batch, int maxn, cudaStream_t s) {
  if (batch <= 0 || maxn <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "invert batch too large");
  for (int j0 = 0; j0 < maxn; j0 += GJ_NB) {
    k_gj_panel<R><<<batch, 256, 0, s>>>(dP, j0);
    check_launch("k_gj_panel");
    dim3 g(ceil_div(maxn, 64), ceil_div(maxn, 64), batch);
    k_gj_update<R><<<g, 256, 0, s>>>(dP, j0);
    check_launch("k_gj_update");
  }
  k_gj_perm<R><<<batch, 32, 0, s>>>(dP);
  check_launch("k_gj_perm");
  const int gx = std::max(1, std::min(ceil_div((long long)maxn * maxn, 256), 1024));
  k_gj_gather<R><<<dim3(gx, batch), 256, 0, s>>>(dP);
  check_launch("k_gj_gather");
  k_gj_copyback<R><<<dim3(gx, batch), 256, 0, s>>>(dP);
  check_launch("k_gj_copyback");
}


// ---------------------------------------------------------------------------
// Blocked Householder least squares.
// ---------------------------------------------------------------------------
// Unblocked Householder on the panel A[j0:m, j0:jend] (one block per problem);
// writes the explicit reflectors to V (rows j0..m-1, ld m) and the compact-WY
// factor Tf (ld QR_NB).
template <typename R>
__global__ void __launch_bounds__(256) k_qr_panel(const QrP<R>* __restrict__ P, int j0) {
  const QrP<R> p = P[blockIdx.x];
  if (j0 >= p.kf) return;
  const int m = p.m, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int jend = min(j0 + QR_NB, p.kf), nbk = jend - j0;
  R* A = p.A;
  const size_t lda = p.lda;
  R* V = p.V;
  __shared__ R s_tau[QR_NB];
  __shared__ R sh[8];
  __shared__ R s_z[QR_NB][QR_NB];
  // zero V panel
  for (long long e = tid; e < (long long)(m - j0) * QR_NB; e += 256) {
    const int i = (int)(e % (m - j0)), c = (int)(e / (m - j0));
    V[i + (size_t)c * m] = R(0);
  }
  __syncthreads();
  for (int j = j0; j < jend; ++j) {
    const int jj = j - j0;
    R part = R(0);
    for (int i = j + 1 + tid; i < m; i += 256) {
      const R v = A[i + j * lda];
      part += v * v;
    }
    const R xn2 = block_sum256(part, sh);
    const R alpha = A[j + j * lda];
    R tau, beta, scal;
    if (xn2 == R(0)) {
      tau = R(0); beta = alpha; scal = R(0);
    } else {
      beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
      tau = (beta - alpha) / beta;
      scal = R(1) / (alpha - beta);
    }
    for (int i = j + tid; i < m; i += 256) {
      R v;
      if (i == j) v = R(1);
      else v = A[i + j * lda] * scal;
      V[(i - j0) + (size_t)jj * m] = v;
    }
    if (tid == 0) {
      s_tau[jj] = tau;
      p.diag[j] = fabs(beta);
    }
    __syncthreads();
    if (tid == 0) A[j + j * lda] = beta;
    // apply H_j to the remaining panel columns, one warp per column
    for (int c = j + 1 + w; c < jend; c += 8) {
      R d = R(0);
      for (int i = j + lane; i < m; i += 32) d += V[(i - j0) + (size_t)jj * m] * A[i + c * lda];
      d = warp_sum(d) * tau;
      for (int i = j + lane; i < m; i += 32) A[i + c * lda] -= d * V[(i - j0) + (size_t)jj * m];
    }
    __syncthreads();
  }
  // Gram matrix Z = V^T V (lower part needed), then the T recurrence.
  for (int pr = w; pr < nbk * nbk; pr += 8) {
    const int a = pr % nbk, b = pr / nbk;
    if (a >= b) continue;
    R d = R(0);
    for (int i = j0 + b + lane; i < m; i += 32) d += V[(i - j0) + (size_t)a * m] * V[(i - j0) + (size_t)b * m];
    d = warp_sum(d);
    if (lane == 0) s_z[a][b] = d;
  }
  __syncthreads();
  if (tid == 0) {
    R* Tf = p.Tf;
    for (int b = 0; b < QR_NB; ++b)
      for (int a = 0; a < QR_NB; ++a) Tf[a + b * QR_NB] = R(0);
    for (int b = 0; b < nbk; ++b) {
      Tf[b + b * QR_NB] = s_tau[b];
      for (int a = 0; a < b; ++a) {
        R t = R(0);
        for (int c = a; c < b; ++c) t += Tf[a + c * QR_NB] * s_z[c][b];
        Tf[a + b * QR_NB] = -s_tau[b] * t;
      }
    }
  }
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

// One back-substitution block step: solve R[b0:b1,b0:b1] X = C[b0:b1, tile]
// and update C[0:b0, tile] -= R[0:b0, b0:b1] X, where C = A[0:kf, kf:n].
template <typename R>
__global__ void __launch_bounds__(256) k_trsm_step(const QrP<R>* __restrict__ P, int blk) {
  const QrP<R> p = P[blockIdx.y];
  const int kf = p.kf, ncol = p.n - p.kf;
  const int b0 = blk * 32;
  if (b0 >= kf) return;
  const int b1 = min(b0 + 32, kf), nb = b1 - b0;
  const int c0 = blockIdx.x * 32;
  if (c0 >= ncol) return;
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
  // each warp solves 4 columns; lane = row
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
  for (int e = tid; e < 32 * 32; e += 256) {
    const int i = e & 31, j = e >> 5;
    if (i < nb && j < nc) C[(b0 + i) + (size_t)(c0 + j) * lda] = Xs[i][j];
  }
  // update rows above
  for (int i = tid; i < b0; i += 256) {
    R rr[32];
#pragma unroll
    for (int t = 0; t < 32; ++t) rr[t] = (t < nb) ? A[i + (size_t)(b0 + t) * lda] : R(0);
    for (int j = 0; j < nc; ++j) {
      R s = R(0);
#pragma unroll
      for (int t = 0; t < 32; ++t) s += rr[t] * Xs[t][j];
      C[i + (size_t)(c0 + j) * lda] -= s;
    }
  }
}

template <typename R>
void lstsq_batched(const QrP<R>* dP, int batch, int maxm, int maxn, int maxkf, cudaStream_t s) {
  if (batch <= 0 || maxkf <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "lstsq batch too large");
  for (int j0 = 0; j0 < maxkf; j0 += QR_NB) {
    k_qr_panel<R><<<batch, 256, 0, s>>>(dP, j0);
    check_launch("k_qr_panel");
    const int jend = std::min(j0 + QR_NB, maxkf);
    const int ncols = maxn - jend;
    if (ncols > 0) {
      k_qr_update<R><<<dim3(ceil_div(ncols, 32), batch), 256, 0, s>>>(dP, j0);
      check_launch("k_qr_update");
    }
  }
  const int nrhs = maxn - 0;  // upper bound of n - kf over the batch
  const int nblk = ceil_div(maxkf, 32);
  for (int blk = nblk - 1; blk >= 0; --blk) {
    k_trsm_step<R><<<dim3(ceil_div(nrhs, 32), batch), 256, 0, s>>>(dP, blk);
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

// T(0:k, 0:n-k) = R(0:k,0:k) \ R(0:k, k:n); T has leading dimension n.
__device__ void id_trisolve(const double* W, int m, int n, int k, double* T) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
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

__global__ void __launch_bounds__(256) k_id_adaptive(const IdP* __restrict__ P, double acc,
                                                     unsigned long long seed) {
  const IdP p = P[blockIdx.x];
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int l = min(m, n);
  double* W = p.W;
  extern __shared__ double s_dyn[];
  double* norms = s_dyn;  // n
  __shared__ double sh[8];
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
        const double t = W[i + (size_t)j * m];
        W[i + (size_t)j * m] = W[i + (size_t)bi * m];
        W[i + (size_t)bi * m] = t;
      }
      if (tid == 0) {
        const int t = p.perm[j]; p.perm[j] = p.perm[bi]; p.perm[bi] = t;
        const double u = norms[j]; norms[j] = norms[bi]; norms[bi] = u;
      }
    }
    __syncthreads();
    double part = 0.0;
    for (int i = j + 1 + tid; i < m; i += 256) { const double v = W[i + (size_t)j * m]; part += v * v; }
    const double xn2 = block_sum256(part, sh);
    const double alpha = W[j + (size_t)j * m];
    double tau = 0.0, beta = alpha, scal = 0.0;
    if (xn2 != 0.0) {
      beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
      tau = (beta - alpha) / beta;
      scal = 1.0 / (alpha - beta);
    }
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
  // rank detection (Common/ID.m:51-52)
  double Rmx = (l > 0) ? fabs(W[0]) * acc : 0.0;
  auto count_rank = [&](double thr) {
    int cnt = 0;
    for (int i = tid; i < l; i += 256) cnt += (fabs(W[i + (size_t)i * m]) > thr) ? 1 : 0;
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
    // two unit random vectors: x[0:r] for the error, x[n:n+r] for the norm
    double pa = 0.0, pb = 0.0;
    for (int i = tid; i < r; i += 256) {
      const double a = rng_uniform(seed, st0, i), b = rng_uniform(seed, st1, i);
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
    k = count_rank(Rmx);
    id_trisolve(W, m, n, k, p.T);
    __syncthreads();
    if (draw > 250) break;
  }
  if (tid == 0) *p.rank = k;
}

void id_adaptive_batched(const IdP* dP, int batch, double acc, unsigned long long seed, cudaStream_t s) {
  if (batch <= 0) return;
  // dynamic shared memory: norms (n doubles); the host guarantees n <= 4096
  k_id_adaptive<<<batch, 256, 4096 * sizeof(double), s>>>(dP, acc, seed);
  check_launch("k_id_adaptive");
}

// Fixed-rank ID reusing the pivoted QR in W: one-sided Jacobi SVD of
// R11 = W(0:k,0:k), then T = V_q diag(1/s_q) U_q^T R12 with s > 1e-12
// (skel_col_fixed, Common/ID.m:106-113).
__global__ void __launch_bounds__(256) k_id_fixed(const IdP* __restrict__ P) {
  const IdP p = P[blockIdx.x];
  const int k = p.force_k;
  if (k < 0) return;
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const double* Wq = p.W;
  double* U = p.svdW;  // k x k, ld k
  double* V = p.svdV;  // k x k, ld k
  __shared__ int s_rot;
  for (int e = tid; e < k * k; e += 256) {
    const int i = e % k, j = e / k;
    U[e] = (i <= j) ? Wq[i + (size_t)j * m] : 0.0;
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
        if (ga != 0.0 && fabs(ga) > 1e-15 * sqrt(al * be)) {
          const double zeta = (be - al) / (2.0 * ga);
          const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
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
  // T(:, c) = sum_{i: s_i > 1e-12} v_i (w_i . R12(:,c)) / s_i^2
  for (int c = k + w; c < n; c += 8) {
    double* t = p.T + (size_t)(c - k) * n;
    for (int i = lane; i < k; i += 32) t[i] = 0.0;
    __syncwarp();
    for (int q = 0; q < k; ++q) {
      if (!(sqrt(s2[q]) > 1e-12)) continue;
      double d = 0.0;
      for (int i = lane; i < k; i += 32) d += U[i + (size_t)q * k] * Wq[i + (size_t)c * m];
      d = warp_sum(d) / s2[q];
      for (int i = lane; i < k; i += 32) t[i] += V[i + (size_t)q * k] * d;
      __syncwarp();
    }
  }
  if (tid == 0) *p.rank = k;
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
  template void invert_batched<R>(const InvP<R>*, int, int, cudaStream_t);                   \
  template void lstsq_batched<R>(const QrP<R>*, int, int, int, int, cudaStream_t);
HSS_INST(double)
HSS_INST(float)
#undef HSS_INST

}  // namespace hss
