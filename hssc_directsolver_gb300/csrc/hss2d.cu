// HSS2D dense-block ("HSS-D") solver on the GPU.
//
//  build_tree : host geometry (hss2d_tree.cpp) + level-batched least squares
//               T = K(Xp,X_sk) \ K(Xp,X_rs)   (interpolation_operator.m:57-77)
//  compress   : Bself, B12, B21 kernel blocks (HSS2D_compress_nsym.m:81-107)
//  invert     : per level, FI = inv([E1 B12; B21 E2]) and E = inv(R FI L)
//               (HSS2D_invert_nsym.m:70-155, build_Finv_nsym.m:92-100,
//               build_E_nsym.m:43-51), stored in the precomputed form
//                 U = E R FI (k x n),  G = FI L (n x k),  GE = G E (n x k)
//               so the inverse apply of HSS2D_applyinv_nsym.m:74-243 becomes
//                 up:   phi_up = U q
//                 down: phi    = FI q - G phi_up + GE phi_dn
//               (algebraically identical: R FI q = tmp, E tmp = phi_up,
//               lam = q - L phi_up, eta = L E phi_dn, phi = FI (eta + lam)).
//  apply      : forward telescoping product (HSS2D_apply_nsym.m:74-218), FP64.
//  solve      : inverse apply + iterative refinement against the FP64 forward
//               operator (Iterative_Refinement.m:20-35).
#include "hss2d.h"

#include <cstdlib>

#include <algorithm>
#include <chrono>
#include <cmath>

namespace hss {

// Size limit of the single-launch block inversion and least squares (the cluster panels);
// larger blocks take the two-level inversion and the row-blocked least squares.  The
// environment variable HSS2D_PANEL_LIMIT (>= 256) lowers it, so that tests reach those
// paths at small sizes.
static int panel_limit(int def) {
  const char* e = std::getenv("HSS2D_PANEL_LIMIT");
  if (!e) return def;
  const int v = std::atoi(e);
  return (v >= 256 && v < def) ? v : def;
}


// ---------------------------------------------------------------------------
// small batched kernels
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_assemble_F(int nb, int n, int kc, int leaf, int ti, const double* __restrict__ Bself,
                             const double* __restrict__ B12, const double* __restrict__ B21,
                             const R* __restrict__ Ech, R* __restrict__ F) {
  const long long per = (long long)n * n;
  const long long tot = per * nb;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int b = (int)(e / per);
    const long long r = e - (long long)b * per;
    const int i = (int)(r % n), j = (int)(r / n);
    R v;
    if (leaf) {
      v = (R)Bself[e];
    } else {
      const int bi = i >= kc, bj = j >= kc;
      const int ii = i - bi * kc, jj = j - bj * kc;
      const long long o = ii + (long long)jj * kc;
      const long long kk = (long long)kc * kc;
      const long long e1 = ti ? 0 : 2LL * b, e2 = ti ? 0 : 2LL * b + 1;
      if (!bi && !bj) v = Ech[e1 * kk + o];
      else if (!bi && bj) v = (R)B12[(long long)b * kk + o];
      else if (bi && !bj) v = (R)B21[(long long)b * kk + o];
      else v = Ech[e2 * kk + o];
    }
    F[e] = v;
  }
}

// dst_b[i + c*ldd] = src_b[J_b[i] + c*lds]  (row gather), rows i < n, cols c < ncol
template <typename R>
__global__ void k_gather_rows(int nb, int n, int ncol, const int* __restrict__ J, const R* __restrict__ src,
                              long long sstride, int lds, R* __restrict__ dst, long long dstride, int ldd) {
  const long long per = (long long)n * ncol, tot = per * nb;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int b = (int)(e / per);
    const long long r = e - (long long)b * per;
    const int i = (int)(r % n), c = (int)(r / n);
    dst[b * dstride + i + (long long)c * ldd] = src[b * sstride + J[(long long)b * n + i] + (long long)c * lds];
  }
}

// dst_b[i + c*ldd] = src_b[i + J_b[c]*lds]  (column gather), rows i < nrow, cols c < n
template <typename R>
__global__ void k_gather_cols(int nb, int nrow, int n, const int* __restrict__ J, const R* __restrict__ src,
                              long long sstride, int lds, R* __restrict__ dst, long long dstride, int ldd) {
  const long long per = (long long)nrow * n, tot = per * nb;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int b = (int)(e / per);
    const long long r = e - (long long)b * per;
    const int i = (int)(r % nrow), c = (int)(r / nrow);
    dst[b * dstride + i + (long long)c * ldd] = src[b * sstride + i + (long long)J[(long long)b * n + c] * lds];
  }
}

// strided batched copy with conversion: dst_b(0:m,0:n) = src_b(0:m,0:n)
template <typename S, typename D>
__global__ void k_copy2d(int nb, int m, int n, const S* __restrict__ src, long long sstride, int lds,
                         D* __restrict__ dst, long long dstride, int ldd) {
  const long long per = (long long)m * n, tot = per * nb;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int b = (int)(e / per);
    const long long r = e - (long long)b * per;
    const int i = (int)(r % m), j = (int)(r / m);
    dst[b * dstride + i + (long long)j * ldd] = (D)src[b * sstride + i + (long long)j * lds];
  }
}

// Tikhonov rows of a damped interpolation least squares (one block per problem): below the p
// proxy rows of [K11 | K21] the k x n block [lam I | 0], lam = 2^-40 ||K11||_F (K11 = the
// first k columns; the embedding of a complex tree doubles the squared Frobenius norm).
struct TikP {
  double* A;
  int p, n, k, ld;
  double sq;  // ||K11||_F^2 per sum of squares of the block (1/2 for an embedded complex block)
};
__global__ void k_tikhonov_rows(const TikP* __restrict__ P) {
  const TikP q = P[blockIdx.x];
  __shared__ double sh[256];
  double ss = 0.0;
  for (long long e = threadIdx.x; e < (long long)q.p * q.k; e += 256) {
    const double v = q.A[(e % q.p) + (size_t)(e / q.p) * q.ld];
    ss += v * v;
  }
  sh[threadIdx.x] = ss;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  const double lam = 0x1.0p-40 * sqrt(q.sq * sh[0]);
  for (long long e = threadIdx.x; e < (long long)q.k * q.n; e += 256) {
    const int r = (int)(e % q.k), c = (int)(e / q.k);
    q.A[q.p + r + (size_t)c * q.ld] = (c == r) ? lam : 0.0;
  }
}

// One stacking step of a row-blocked least squares (TSQR): in W (ld ldw) the top k rows keep
// the previous block's R11 | Q^T B (the reflectors below R11's diagonal are cleared) and the
// rows below take `count` rows of A starting at row `from` (clean = 0: W starts empty and
// takes the rows from its top).
struct TsqrP {
  const double* A;
  int lda;
  double* W;
  int ldw, k, n, from, count, clean;
};
__global__ void k_tsqr_fill(const TsqrP* __restrict__ P) {
  const TsqrP q = P[blockIdx.y];
  const int top = q.clean ? q.k : 0;
  const long long tot = (long long)(top + q.count) * q.n;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int r = (int)(e % (top + q.count)), c = (int)(e / (top + q.count));
    double* w = q.W + r + (size_t)c * q.ldw;
    if (r < top) {
      if (c < q.k && r > c) *w = 0.0;
    } else {
      *w = q.A[(q.from + r - top) + (size_t)c * q.lda];
    }
  }
}

// transpose copy: dst_b(j, i) = src_b(i, j), src m x n
__global__ void k_transpose(int nb, int m, int n, const double* __restrict__ src, long long sstride, int lds,
                            double* __restrict__ dst, long long dstride, int ldd) {
  const long long per = (long long)m * n, tot = per * nb;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int b = (int)(e / per);
    const long long r = e - (long long)b * per;
    const int j = (int)(r % n), i = (int)(r / n);
    dst[b * dstride + j + (long long)i * ldd] = src[b * sstride + i + (long long)j * lds];
  }
}

// Row map of box i, local row q (J order) into the level's input / output:
//   leaf  : global point IsrcJ[i*n+q]            (vector ld = N)
//   parent: children stack row 2i*kc + J[i*n+q]   (vector ld = 2*nb*kc)
__device__ __forceinline__ long long rowmap(int leaf, const int* J, const int* IsrcJ, int i, int n, int kc,
                                            int q) {
  const long long o = (long long)i * n + q;
  return leaf ? (long long)IsrcJ[o] : (long long)(2 * i) * kc + J[o];
}

// forward apply gather: q in J order -> [phi_up (k rows) | rs (n-k rows)]
__global__ void k_fwd_gather(int nb, int n, int k, int kc, int leaf, int r, const int* __restrict__ J,
                             const int* __restrict__ IsrcJ, const double* __restrict__ src, long long lds,
                             double* __restrict__ up, long long ldu, double* __restrict__ rs, long long ldr) {
  const long long tot = (long long)nb * n * r;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int c = (int)(e / ((long long)nb * n));
    const long long t = e - (long long)c * nb * n;
    const int i = (int)(t / n), q = (int)(t % n);
    const double v = src[rowmap(leaf, J, IsrcJ, i, n, kc, q) + c * lds];
    if (q < k) up[(long long)i * k + q + c * ldu] = v;
    else rs[(long long)i * (n - k) + (q - k) + c * ldr] = v;
  }
}

// forward apply scatter-add: phi[J[q]] += q < k ? dn[q] : tmp[q-k]
__global__ void k_fwd_scatter(int nb, int n, int k, int kc, int leaf, int r, const int* __restrict__ J,
                              const int* __restrict__ IsrcJ, double* __restrict__ dst, long long ldd,
                              const double* __restrict__ dn, long long ldn, const double* __restrict__ tmp,
                              long long ldt) {
  const long long tot = (long long)nb * n * r;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int c = (int)(e / ((long long)nb * n));
    const long long t = e - (long long)c * nb * n;
    const int i = (int)(t / n), q = (int)(t % n);
    const double v = (q < k) ? dn[(long long)i * k + q + c * ldn] : tmp[(long long)i * (n - k) + (q - k) + c * ldt];
    dst[rowmap(leaf, J, IsrcJ, i, n, kc, q) + c * ldd] += v;
  }
}

template <typename S, typename D>
__global__ void k_convert(long long cnt, const S* __restrict__ a, D* __restrict__ b) {
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < cnt; e += (long long)gridDim.x * 256) b[e] = (D)a[e];
}

// res = f - y (column-major N x r), and per-column squared norms of res and f
__global__ void k_residual(long long N, int r, const double* __restrict__ f, long long ldf,
                           const double* __restrict__ y, long long ldy, double* __restrict__ res,
                           long long ldr, double* __restrict__ part /* gridDim.x x r x 2 */) {
  __shared__ double sr[8], sf[8];
  for (int c = 0; c < r; ++c) {
    double a = 0.0, b = 0.0;
    for (long long i = blockIdx.x * 256LL + threadIdx.x; i < N; i += (long long)gridDim.x * 256) {
      const double fv = f[i + c * ldf];
      const double rv = fv - y[i + c * ldy];
      res[i + c * ldr] = rv;
      a += rv * rv;
      b += fv * fv;
    }
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) { sr[threadIdx.x >> 5] = a; sf[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double ta = 0.0, tb = 0.0;
      for (int w = 0; w < 8; ++w) { ta += sr[w]; tb += sf[w]; }
      part[((long long)blockIdx.x * r + c) * 2] = ta;
      part[((long long)blockIdx.x * r + c) * 2 + 1] = tb;
    }
    __syncthreads();
  }
}

__global__ void k_axpy(long long N, int r, const double* __restrict__ dx, long long ldd, double* __restrict__ x,
                       long long ldx) {
  const long long tot = N * r;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const long long i = e % N, c = e / N;
    x[i + c * ldx] += dx[i + c * ldd];
  }
}

static int grid_for(long long tot) { return std::max(1, std::min(ceil_div(tot, 256), 4096)); }

// ---------------------------------------------------------------------------
// descriptor helpers
// ---------------------------------------------------------------------------
template <typename R>
static void run_gemm(std::vector<GemmP<R>>& P, bool tA, bool tB, R alpha, R beta, cudaStream_t s,
                     DevBuf<GemmP<R>>& scratch, bool df = false) {
  if (P.empty()) return;
  int maxM = 0, maxN = 0;
  for (auto& p : P) { maxM = std::max(maxM, p.M); maxN = std::max(maxN, p.N); }
  scratch.alloc(P.size());
  HSS_CUDA(cudaMemcpyAsync(scratch.p, P.data(), P.size() * sizeof(GemmP<R>), cudaMemcpyHostToDevice, s));
  if constexpr (std::is_same<R, double>::value) {
    if (df) {
      gemm_batched_df(scratch.p, (int)P.size(), maxM, maxN, tA, tB, alpha, beta, s);
      HSS_CUDA(cudaStreamSynchronize(s));
      return;
    }
  }
  gemm_batched<R>(scratch.p, (int)P.size(), maxM, maxN, tA, tB, alpha, beta, s);
  HSS_CUDA(cudaStreamSynchronize(s));
}

template <typename R>
void SolvePlan<R>::add(const std::vector<GemmP<R>>& P, R alpha, R beta, cudaStream_t s) {
  Step st;
  st.batch = (int)P.size();
  st.maxM = 0;
  int maxK = 0;
  for (auto& p : P) { st.maxM = std::max(st.maxM, p.M); st.maxN = std::max(st.maxN, p.N); maxK = std::max(maxK, p.K); }
  st.alpha = alpha;
  st.beta = beta;
  st.maxK = maxK;
  st.ksplit = df ? skinny_ksplit_df(st.batch, st.maxM, maxK) : skinny_ksplit<R>(st.batch, st.maxM, maxK);
  if (st.ksplit > 1) st.part.alloc((size_t)st.batch * st.ksplit * st.maxM * 8);
  st.d.alloc(P.size());
  HSS_CUDA(cudaMemcpyAsync(st.d.p, P.data(), P.size() * sizeof(GemmP<R>), cudaMemcpyHostToDevice, s));
  steps.push_back(std::move(st));
}

template <typename R>
void SolvePlan<R>::add_seg(const std::vector<SegGemmP>& P, R alpha, R beta, cudaStream_t s) {
  HSS_REQUIRE(df, HSS_ERR_STATE, "segmented plan steps need double-float operands");
  Step st;
  st.batch = (int)P.size();
  int maxK = 0;
  for (auto& p : P) {
    st.maxM = std::max(st.maxM, p.M);
    st.maxN = std::max(st.maxN, p.N);
    maxK = std::max(maxK, p.K[0] + p.K[1] + p.K[2]);
  }
  st.alpha = alpha;
  st.beta = beta;
  st.maxK = maxK;
  st.ksplit = skinny_ksplit_df(st.batch, st.maxM, maxK);
  if (st.ksplit > 1) st.part.alloc((size_t)st.batch * st.ksplit * st.maxM * 8);
  st.dseg.alloc(P.size());
  HSS_CUDA(cudaMemcpyAsync(st.dseg.p, P.data(), P.size() * sizeof(SegGemmP), cudaMemcpyHostToDevice, s));
  steps.push_back(std::move(st));
}

template <typename R>
void SolvePlan<R>::run_step(const Step& st, cudaStream_t s) const {
  if constexpr (std::is_same<R, double>::value) {
    if (df && st.dseg.p) {
      gemm_skinny_split_df(st.dseg.p, st.batch, st.maxM, st.maxN, st.alpha, st.beta, st.ksplit, st.part.p, s);
      return;
    }
    if (df) {
      gemm_skinny_split_df(st.d.p, st.batch, st.maxM, st.maxN, st.alpha, st.beta, st.ksplit, st.part.p, s);
      return;
    }
  }
  gemm_skinny_split<R>(st.d.p, st.batch, st.maxM, st.maxN, st.alpha, st.beta, st.ksplit, st.part.p, s);
}

template <typename R>
void SolvePlan<R>::run(cudaStream_t s) const {
  if (!streams) {
    for (auto& st : steps) run_step(st, s);
  } else {
    // fork both streams from s, issue every step after the steps it depends on, join
    // both back into s (under graph capture the events become graph edges)
    PlanStreams& S = *streams;
    S.fork_from(s);
    for (size_t i = 0; i < steps.size(); ++i) {
      const Step& st = steps[i];
      cudaStream_t q = st.side ? S.side : S.crit;
      for (int d : st.deps) HSS_CUDA(cudaStreamWaitEvent(q, S.ev[d], 0));
      run_step(st, q);
      if (st.rec) HSS_CUDA(cudaEventRecord(S.ev[i], q));
    }
    S.join_into(s);
  }
  for (auto& st : tc_steps) st.run(s);
}

// The steps run on the plan's own buffers: a step's output is rewritten by the next real
// apply before anything reads it (accumulating steps follow an overwriting one), so the
// timing runs leave no trace.
template <typename R>
void SolvePlan<R>::tune(cudaStream_t s) {
  cudaEvent_t e0, e1;
  HSS_CUDA(cudaEventCreate(&e0));
  HSS_CUDA(cudaEventCreate(&e1));
  try {
    for (auto& st : steps) {
      const int cap = std::max(1, std::min(32, st.maxK / 64));
      if (st.maxK < 128 || cap <= 1) continue;
      std::vector<int> cand;
      const int around[4] = {st.ksplit, st.ksplit / 2, st.ksplit * 2, st.ksplit * 4};
      for (int c : around) {
        const int cc = std::max(1, std::min(cap, c));
        if (std::find(cand.begin(), cand.end(), cc) == cand.end()) cand.push_back(cc);
      }
      if (cand.size() <= 1) continue;
      const int kmax = *std::max_element(cand.begin(), cand.end());
      if (kmax > 1) st.part.ensure((size_t)st.batch * kmax * st.maxM * 8);
      float best = 0.f;
      int bestc = cand[0];
      for (size_t i = 0; i < cand.size(); ++i) {
        st.ksplit = cand[i];
        run_step(st, s);
        HSS_CUDA(cudaEventRecord(e0, s));
        for (int rep = 0; rep < 3; ++rep) run_step(st, s);
        HSS_CUDA(cudaEventRecord(e1, s));
        HSS_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        HSS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (i == 0 || ms < 0.98f * best) {
          best = ms;
          bestc = cand[i];
        }
      }
      st.ksplit = bestc;
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
}

template struct SolvePlan<double>;
template struct SolvePlan<float>;

// ---------------------------------------------------------------------------
// build_tree
// ---------------------------------------------------------------------------
// The ID step of a kh > 0 tree level (LOCAL_Non_Preset_Skeleton_Info,
// HSS2D_build_tree_nsym.m:614-627): per box, the complex ID of K(proxies, box) at tolerance acc
// through the pair-pivoted QR of its real embedding, problem 2 box of the shared random
// stream.  Returns the complex column order and the rank per box; the raw T of each box
// (2k x 2(n - k) real, the embedding of the complex T) is kept in id_T[lev].
void HSS2D::id_level(int lev, const std::vector<std::vector<int>>& boxes, const std::vector<std::vector<double>>& px,
                     const std::vector<std::vector<double>>& py, std::vector<std::vector<int>>& perm_out,
                     std::vector<int>& k_out) {
  const int nb = (int)boxes.size();
  const int n = (int)boxes[0].size(), n2 = 2 * n;
  HSS_REQUIRE(n2 <= 4096, HSS_ERR_ARG, "ID level: more than 2048 points in a box");
  // temporary point table: per box its sources, then its proxies; each point twice (the two
  // components of the embedding)
  std::vector<long long> soff(nb + 1, 0), qoff(nb + 1, 0);
  long long npt = 0;
  for (int i = 0; i < nb; ++i) {
    HSS_REQUIRE((int)boxes[i].size() == n, HSS_ERR_ARG, "ID level: non-uniform box sizes");
    HSS_REQUIRE((int)px[i].size() >= 1, HSS_ERR_ARG, "ID level: box without proxies");
    soff[i] = npt;
    npt += n;
    qoff[i] = npt;
    npt += (long long)px[i].size();
  }
  HSS_REQUIRE(2 * npt < (1LL << 31), HSS_ERR_ARG, "ID level: point table exceeds 2^31 entries");
  std::vector<double> hx(2 * npt), hy(2 * npt), zero(2 * npt, 0.0);
  std::vector<int> ti, si;
  std::vector<long long> aoff(nb + 1, 0);
  for (int i = 0; i < nb; ++i) {
    for (int j = 0; j < n; ++j)
      for (int a = 0; a < 2; ++a) {
        const size_t e = 2 * (size_t)(soff[i] + j) + a;
        hx[e] = geo.X[2 * (size_t)boxes[i][j]];
        hy[e] = geo.X[2 * (size_t)boxes[i][j] + 1];
      }
    const int p = (int)px[i].size();
    for (int q = 0; q < p; ++q)
      for (int a = 0; a < 2; ++a) {
        const size_t e = 2 * (size_t)(qoff[i] + q) + a;
        hx[e] = px[i][q];
        hy[e] = py[i][q];
      }
    aoff[i + 1] = aoff[i] + (long long)(2 * p) * n2;
  }
  // index arrays: rows (proxies) then columns (sources) per box, in embedded entries
  std::vector<long long> ioff(nb + 1, 0);
  std::vector<int> idx;
  for (int i = 0; i < nb; ++i) {
    ioff[i] = (long long)idx.size();
    for (long long q = 0; q < (long long)px[i].size(); ++q)
      for (int a = 0; a < 2; ++a) idx.push_back((int)(2 * (qoff[i] + q) + a));
    for (int j = 0; j < n; ++j)
      for (int a = 0; a < 2; ++a) idx.push_back((int)(2 * (soff[i] + j) + a));
  }
  PointTable tp;
  tp.upload(hx, hy, zero, zero, zero, zero, prm.kp, stream);
  DevBuf<int> didx;
  didx.upload(idx, stream);
  DevBuf<double> A(aoff[nb]), W(aoff[nb]);
  std::vector<KgenP<double>> kg(nb);
  long long maxe = 0;
  int maxm = 0;
  for (int i = 0; i < nb; ++i) {
    const int m2 = 2 * (int)px[i].size();
    kg[i] = KgenP<double>{didx.p + ioff[i], didx.p + ioff[i] + m2, m2, n2, A.p + aoff[i], m2, 0};
    maxe = std::max(maxe, (long long)m2 * n2);
    maxm = std::max(maxm, m2);
  }
  for (int off = 0; off < nb; off += 65535) {
    const int cnt = std::min(65535, nb - off);
    DevBuf<KgenP<double>> dkg(cnt);
    HSS_CUDA(cudaMemcpyAsync(dkg.p, kg.data() + off, cnt * sizeof(KgenP<double>), cudaMemcpyHostToDevice, stream));
    kgen_batched<double>(dkg.p, cnt, maxe, view(tp), kdev, stream);
    HSS_CUDA(cudaStreamSynchronize(stream));
  }
  // adaptive pair ID of every box
  DevBuf<int> perm((size_t)nb * n2), rank(nb);
  DevBuf<double> T((size_t)nb * n2 * n2), xw((size_t)nb * 2 * n2), yw((size_t)nb * (maxm + n2));
  std::vector<IdP> ip(nb);
  for (int i = 0; i < nb; ++i) {
    IdP q{};
    q.A = A.p + aoff[i];
    q.W = W.p + aoff[i];
    q.m = 2 * (int)px[i].size();
    q.n = n2;
    q.perm = perm.p + (size_t)i * n2;
    q.rank = rank.p + i;
    q.T = T.p + (size_t)i * n2 * n2;
    q.force_k = -1;
    q.x = xw.p + (size_t)i * 2 * n2;
    q.y = yw.p + (size_t)i * (maxm + n2);
    q.problem = 2 * ((1 << lev) - 1 + i);  // 2 * box (heap index) of the shared random stream
    q.steps_hint = 0;
    q.seed = prm.seed;
    ip[i] = q;
  }
  for (int off = 0; off < nb; off += 65535) {
    const int cnt = std::min(65535, nb - off);
    DevBuf<IdP> dip(cnt);
    HSS_CUDA(cudaMemcpyAsync(dip.p, ip.data() + off, cnt * sizeof(IdP), cudaMemcpyHostToDevice, stream));
    id_pairs_batched(dip.p, cnt, n2, prm.acc, stream);
    HSS_CUDA(cudaStreamSynchronize(stream));
  }
  std::vector<int> hr, hp;
  download(hr, rank.p, nb, stream);
  download(hp, perm.p, (size_t)nb * n2, stream);
  std::vector<double> ht;
  download(ht, T.p, (size_t)nb * n2 * n2, stream);
  HSS_CUDA(cudaStreamSynchronize(stream));
  perm_out.assign(nb, std::vector<int>(n));
  k_out.assign(nb, 0);
  // raw T per box (2k x 2(n - k), ld 2k), packed
  std::vector<double>& keep = id_T[lev];
  std::vector<long long>& toff = id_Toff[lev];
  keep.clear();
  toff.assign(nb + 1, 0);
  for (int i = 0; i < nb; ++i) {
    const int k2 = hr[i], nr2 = n2 - k2;
    HSS_REQUIRE(k2 % 2 == 0 && k2 >= 0 && k2 <= n2, HSS_ERR_CUDA, "pair ID: odd rank");
    for (int q = 0; q < n; ++q) {
      const int c = hp[(size_t)i * n2 + 2 * q];
      HSS_REQUIRE(c % 2 == 0 && hp[(size_t)i * n2 + 2 * q + 1] == c + 1, HSS_ERR_CUDA, "pair ID split a pair");
      perm_out[i][q] = c / 2;
    }
    k_out[i] = k2 / 2;
    toff[i + 1] = toff[i] + (long long)k2 * nr2;
    for (int c = 0; c < nr2; ++c)
      for (int r = 0; r < k2; ++r) keep.push_back(ht[(size_t)i * n2 * n2 + r + (size_t)c * n2]);
  }
}

// The real 2 x 2 embedding of a complex tree level: point i becomes the entries 2i, 2i + 1
// (real and imaginary components), so n, k and the proxy counts double and every index
// array interleaves the two components.
static void embed_level(Level2Geom& g) {
  auto dbl = [](std::vector<int>& v) {
    std::vector<int> o(2 * v.size());
    for (size_t q = 0; q < v.size(); ++q) {
      o[2 * q] = 2 * v[q];
      o[2 * q + 1] = 2 * v[q] + 1;
    }
    v.swap(o);
  };
  dbl(g.J);
  dbl(g.Isrc);
  dbl(g.IsrcJ);
  dbl(g.proxy);
  for (auto& o : g.poff) o *= 2;
  g.n *= 2;
  g.k *= 2;
  g.p *= 2;
}

void HSS2D::build_tree() {
  using clk = std::chrono::steady_clock;
  auto t0 = clk::now();
  cplx = (prm.kp.flag == HSS_SL_H_2D);
  kdev = make_kernel_dev(prm.kp);
  if (cplx) {
    HSS_REQUIRE(prm.interform == HSS_INTER_DENSE, HSS_ERR_ARG, "kh > 0: dense interpolation operators only");
    HSS_REQUIRE(prm.transinv == 0, HSS_ERR_ARG, "kh > 0: transinv 0 only");
    HSS_REQUIRE(prm.precision == HSS_PREC_FP64 || prm.precision == HSS_PREC_MIXED, HSS_ERR_ARG,
                "kh > 0: HSS_PREC_FP64 or HSS_PREC_MIXED");
  }
  if (prm.proxy_rule == HSS_PROXY_RAND)
    HSS_REQUIRE(prm.interform == HSS_INTER_DENSE, HSS_ERR_ARG, "'rand' proxies: dense interpolation operators only");
  id_T.clear();
  id_Toff.clear();
  IdLevelFn fn = [this](int lev, const std::vector<std::vector<int>>& b, const std::vector<std::vector<double>>& x,
                        const std::vector<std::vector<double>>& y, std::vector<std::vector<int>>& perm,
                        std::vector<int>& k) { id_level(lev, b, x, y, perm, k); };
  build_tree_geometry(prm, geo, cplx ? fn : IdLevelFn());
  auto t1 = clk::now();
  phase_s[0] = std::chrono::duration<double>(t1 - t0).count();
  const long long N = geo.N;
  const size_t npts = (size_t)N + geo.proxy_x.size();
  const int rep = cplx ? 2 : 1;  // table entries per point
  std::vector<double> hx(rep * npts), hy(rep * npts), zero(rep * npts, 0.0);
  for (size_t i = 0; i < npts; ++i) {
    const double x = i < (size_t)N ? geo.X[2 * i] : geo.proxy_x[i - N];
    const double y = i < (size_t)N ? geo.X[2 * i + 1] : geo.proxy_y[i - N];
    for (int a = 0; a < rep; ++a) {
      hx[rep * i + a] = x;
      hy[rep * i + a] = y;
    }
  }
  if (cplx) {
    for (auto& g : geo.levels) embed_level(g);
    geo.N = 2 * N;
  }
  ng_pts = rep * prm.Ng * prm.Ng;
  pts.upload(hx, hy, zero, zero, zero, zero, prm.kp, stream);
  L.clear();
  L.resize(geo.depth + 1);
  for (int lev = 0; lev <= geo.depth; ++lev) {
    auto& g = geo.levels[lev];
    auto& d = L[lev];
    d.J.upload(g.J, stream);
    d.Isrc.upload(g.Isrc, stream);
    d.IsrcJ.upload(g.IsrcJ, stream);
    d.proxy.upload(g.proxy, stream);
  }
  HSS_CUDA(cudaStreamSynchronize(stream));
  qlev.assign(geo.depth + 1, 0);
  qrank_up.assign(geo.depth + 1, {});
  qrank_dn.assign(geo.depth + 1, {});
  auto t2 = clk::now();
  phase_s[1] = std::chrono::duration<double>(t2 - t1).count();
  for (int lev = geo.depth; lev >= 1; --lev) {
    if (geo.levels[lev].id_level) id_T_level(lev);
    else compute_T(lev);
  }
  HSS_CUDA(cudaStreamSynchronize(stream));
  id_T.clear();
  id_Toff.clear();
  phase_s[2] = std::chrono::duration<double>(clk::now() - t2).count();
  tree_built = true;
}

// T of an ID level: rows and columns of each box's raw ID T in the tree's order (complex
// indices, each an embedded 2 x 2 block; zero rows for promoted points); T_dn = T_up
// (LOCAL_Non_Preset_Skeleton_Info :656).  A complex tree keeps T_dn conjugated, E(conj T_dn)
// (entries of odd row xor odd column negated), as the least squares of the other levels leave
// it: its real transpose is then E(T_dn^T), the plain transpose the HSS formulas apply.
void HSS2D::id_T_level(int lev) {
  auto& g = geo.levels[lev];
  auto& d = L[lev];
  const int nb = g.nb, k = g.k, nr = g.n - g.k, kc = k / 2, nrc = nr / 2;
  d.Tup.alloc((size_t)nb * k * std::max(nr, 1));
  d.Tdn.alloc((size_t)nb * k * std::max(nr, 1));
  d.TdnT.alloc((size_t)nb * k * std::max(nr, 1));
  if (nr == 0 || k == 0) return;
  const std::vector<double>& raw = id_T.at(lev);
  const std::vector<long long>& toff = id_Toff.at(lev);
  std::vector<double> tu((size_t)nb * k * nr), td((size_t)nb * k * nr), tt((size_t)nb * k * nr);
  for (int i = 0; i < nb; ++i) {
    const int* rows = g.id_rows.data() + (size_t)i * kc;
    const int* cols = g.id_cols.data() + (size_t)i * nrc;
    const double* src = raw.data() + toff[i];
    // rows of the raw T: twice the box's own rank (the rows that are not promoted points)
    const int kraw = 2 * (int)std::count_if(rows, rows + kc, [](int v) { return v >= 0; });
    HSS_REQUIRE((long long)kraw * (g.n - kraw) == toff[i + 1] - toff[i], HSS_ERR_ARG, "ID level: raw T size");
    double* dst = tu.data() + (size_t)i * k * nr;
    double* ddn = td.data() + (size_t)i * k * nr;
    double* dtt = tt.data() + (size_t)i * k * nr;
    for (int c = 0; c < nr; ++c)
      for (int r = 0; r < k; ++r) {
        const int rr = rows[r / 2];
        const double v = (rr < 0) ? 0.0 : src[(2 * rr + (r & 1)) + (size_t)(2 * cols[c / 2] + (c & 1)) * kraw];
        const double vc = ((r ^ c) & 1) ? -v : v;  // E(conj T)
        dst[r + (size_t)c * k] = v;
        ddn[r + (size_t)c * k] = vc;
        dtt[c + (size_t)r * nr] = vc;
      }
  }
  HSS_CUDA(cudaMemcpyAsync(d.Tup.p, tu.data(), tu.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
  HSS_CUDA(cudaMemcpyAsync(d.Tdn.p, td.data(), td.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
  HSS_CUDA(cudaMemcpyAsync(d.TdnT.p, tt.data(), tt.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
  HSS_CUDA(cudaStreamSynchronize(stream));
  qlev[lev] = nr;
}

// Least squares taller than the cluster panel's row limit, by row blocks (TSQR): the first
// block is factored, then the k rows of R11 | Q^T B are stacked onto the next rows of A and
// factored again, until every row has been taken; the last step solves with the k x k R11.
// The solution is that of the full problem (orthogonal transformations of row blocks).
void HSS2D::lstsq_tsqr(const std::vector<QrP<double>>& qp, int n, int k) {
  const int batch = (int)qp.size();
  const int ldw = panel_limit(LSTSQ_MAX_ROWS), chunk = ldw - k;
  HSS_REQUIRE(chunk >= 32, HSS_ERR_ARG, "least squares: too many columns for a row-blocked solve");
  DevBuf<double> W((size_t)batch * ldw * n), V((size_t)batch * ldw * QR_NB), Tf((size_t)batch * QR_NB * QR_NB);
  DevBuf<TsqrP> dtp(batch);
  DevBuf<QrP<double>> dqp(batch);
  std::vector<int> done(batch, 0);
  int maxrows = 0;
  for (auto& q : qp) maxrows = std::max(maxrows, q.m);
  auto fill = [&](bool clean, std::vector<QrP<double>>& step) {
    std::vector<TsqrP> tp(batch);
    long long maxe = 1;
    for (int b = 0; b < batch; ++b) {
      const int take = std::min(clean ? chunk : ldw, qp[b].m - done[b]);
      tp[b] = TsqrP{qp[b].A, qp[b].lda, W.p + (size_t)b * ldw * n, ldw, k, n, done[b], take, clean ? 1 : 0};
      step[b] = qp[b];
      step[b].A = tp[b].W;
      step[b].lda = ldw;
      step[b].m = (clean ? k : 0) + take;
      step[b].V = V.p + (size_t)b * ldw * QR_NB;
      step[b].Tf = Tf.p + (size_t)b * QR_NB * QR_NB;
      done[b] += take;
      maxe = std::max(maxe, (long long)step[b].m * n);
    }
    HSS_CUDA(cudaMemcpyAsync(dtp.p, tp.data(), batch * sizeof(TsqrP), cudaMemcpyHostToDevice, stream));
    const int gx = std::max(1, std::min(ceil_div(maxe, 256), 4096));
    k_tsqr_fill<<<dim3(gx, batch), 256, 0, stream>>>(dtp.p);
    check_launch("k_tsqr_fill");
    HSS_CUDA(cudaStreamSynchronize(stream));
  };
  auto run = [&](std::vector<QrP<double>>& step, bool solve) {
    int maxm = 1;
    for (auto& q : step) maxm = std::max(maxm, q.m);
    HSS_CUDA(cudaMemcpyAsync(dqp.p, step.data(), batch * sizeof(QrP<double>), cudaMemcpyHostToDevice, stream));
    lstsq_batched<double>(dqp.p, batch, maxm, n, k, stream, dftree(), solve);
    HSS_CUDA(cudaStreamSynchronize(stream));
  };
  std::vector<QrP<double>> step(batch);
  fill(false, step);
  run(step, false);
  bool more = true;
  while (more) {
    more = false;
    for (int b = 0; b < batch; ++b) more = more || done[b] < qp[b].m;
    fill(true, step);  // with no rows left this only clears the reflectors under R11
    run(step, !more);
  }
}

void HSS2D::compute_T(int lev) {
  auto& g = geo.levels[lev];
  auto& d = L[lev];
  const int nb = nf(g), n = g.n, k = g.k, p = g.p, nr = n - k;
  d.Tup.alloc((size_t)nb * k * std::max(nr, 1));
  d.Tdn.alloc((size_t)nb * k * std::max(nr, 1));
  d.TdnT.alloc((size_t)nb * k * std::max(nr, 1));
  if (nr == 0 || k == 0) return;
  // per factor box: its proxy count (the 'rand' rule samples a different set per box); a
  // complex tree's systems, and those of the sampled and Whitney skeleton rules, carry k
  // Tikhonov rows under the proxy rows (k_tikhonov_rows): their proxy systems are
  // numerically rank deficient
  const int tk = (cplx || prm.skel_rule != HSS_SKEL_BDRY) ? k : 0;
  std::vector<int> pb(nb);
  std::vector<long long> aoff(2 * nb + 1, 0);
  for (int i = 0; i < nb; ++i) {
    pb[i] = g.poff[i + 1] - g.poff[i];
    HSS_REQUIRE(pb[i] >= k, HSS_ERR_ARG, "proxy set smaller than skeleton: least squares is underdetermined");
    aoff[2 * i + 1] = aoff[2 * i] + (long long)(pb[i] + tk) * n;
    aoff[2 * i + 2] = aoff[2 * i + 1] + (long long)(pb[i] + tk) * n;
  }
  const int batch = 2 * nb;
  DevBuf<double> A(aoff[batch]);
  // kernel blocks: problem 2i = [K(Xp, X_sk) | K(Xp, X_rs)], 2i+1 = K(X_src[J], Xp)^T (the real
  // transpose: of a complex tree's embedded blocks E(K)^T = E(K^H), so its T_dn comes out
  // conjugated, E(conj T_dn), whose real transpose is the E(T_dn^T) the HSS formulas use)
  std::vector<KgenP<double>> kg(batch);
  for (int i = 0; i < nb; ++i) {
    const int* pr = d.proxy.p + g.poff[i];
    kg[2 * i] = KgenP<double>{pr, d.IsrcJ.p + (size_t)i * n, pb[i], n, A.p + aoff[2 * i], pb[i] + tk, 0};
    kg[2 * i + 1] = KgenP<double>{d.IsrcJ.p + (size_t)i * n, pr, n, pb[i], A.p + aoff[2 * i + 1], pb[i] + tk, 1};
  }
  DevBuf<KgenP<double>> dkg(batch);
  HSS_CUDA(cudaMemcpyAsync(dkg.p, kg.data(), batch * sizeof(KgenP<double>), cudaMemcpyHostToDevice, stream));
  kgen_batched<double>(dkg.p, batch, (long long)p * n, view(pts), kdev, stream);
  if (tk > 0) {
    std::vector<TikP> tp(batch);
    for (int b = 0; b < batch; ++b) tp[b] = TikP{A.p + aoff[b], pb[b / 2], n, k, pb[b / 2] + tk, cplx ? 0.5 : 1.0};
    DevBuf<TikP> dtp(batch);
    HSS_CUDA(cudaMemcpyAsync(dtp.p, tp.data(), batch * sizeof(TikP), cudaMemcpyHostToDevice, stream));
    k_tikhonov_rows<<<batch, 256, 0, stream>>>(dtp.p);
    check_launch("k_tikhonov_rows");
    HSS_CUDA(cudaStreamSynchronize(stream));
  }
  DevBuf<double> V((size_t)batch * (p + tk) * QR_NB), Tf((size_t)batch * QR_NB * QR_NB), diag((size_t)batch * k);
  if (uses_lowrank(lev)) {
    HSS_REQUIRE(g.p_uniform, HSS_ERR_ARG, "low-rank T needs the same proxy count in every box");
    diag.zero(stream);
    lowrank_T(lev, A.p, V, Tf, diag);
  } else {
    std::vector<QrP<double>> qp(batch);
    for (int b = 0; b < batch; ++b) {
      double* X = ((b & 1) ? d.Tdn.p : d.Tup.p) + (size_t)(b / 2) * k * nr;
      const int pm = pb[b / 2] + tk;
      qp[b] = QrP<double>{A.p + aoff[b], pm, n, k, pm, V.p + (size_t)b * (p + tk) * QR_NB,
                          Tf.p + (size_t)b * QR_NB * QR_NB, diag.p + (size_t)b * k, X, k};
    }
    if (p + tk <= panel_limit(LSTSQ_MAX_ROWS)) {
      DevBuf<QrP<double>> dqp(batch);
      HSS_CUDA(cudaMemcpyAsync(dqp.p, qp.data(), batch * sizeof(QrP<double>), cudaMemcpyHostToDevice, stream));
      lstsq_batched<double>(dqp.p, batch, p + tk, n, k, stream, dftree());
      HSS_CUDA(cudaStreamSynchronize(stream));
    } else {
      lstsq_tsqr(qp, n, k);
    }
    qlev[lev] = nr;  // a dense T.U is k x nr
  }
  // T_up came from the even problems, T_dn from the odd ones
  k_transpose<<<grid_for((long long)nb * k * nr), 256, 0, stream>>>(nb, k, nr, d.Tdn.p, (long long)k * nr, k,
                                                                     d.TdnT.p, (long long)k * nr, nr);
  check_launch("compute_T copies");
  // rank diagnostics: smallest/largest |R_ii| over the level
  std::vector<double> hd;
  download(hd, diag.p, (size_t)batch * k, stream);
  HSS_CUDA(cudaStreamSynchronize(stream));
  double mn = INFINITY, mx = 0.0;
  bool finite = true;
  for (double v : hd) { finite = finite && std::isfinite(v); mn = std::min(mn, v); mx = std::max(mx, v); }
  HSS_REQUIRE(finite, HSS_ERR_NONFINITE, "non-finite value in interpolation least squares");
  d.rdiag_min = mn;
  d.rdiag_max = mx;
}

// ---------------------------------------------------------------------------
// compress
// ---------------------------------------------------------------------------
void HSS2D::compress() {
  HSS_REQUIRE(tree_built, HSS_ERR_STATE, "hss2d_compress before hss2d_build_tree");
  const auto tc0 = std::chrono::steady_clock::now();
  const int depth = geo.depth;
  std::vector<KgenP<double>> kg;
  {
    auto& g = geo.levels[depth];
    auto& d = L[depth];
    d.Bself.alloc((size_t)nf(g) * g.n * g.n);
    for (int i = 0; i < nf(g); ++i)
      kg.push_back(KgenP<double>{d.Isrc.p + (size_t)i * g.n, d.Isrc.p + (size_t)i * g.n, g.n, g.n,
                                 d.Bself.p + fo(i) * g.n * g.n, g.n, 0});
  }
  for (int lev = 0; lev < depth; ++lev) {
    auto& gc = geo.levels[lev + 1];
    auto& dc = L[lev + 1];
    auto& d = L[lev];
    const int nb = nf(geo.levels[lev]), kc = gc.k, nc = gc.n;
    d.B12.alloc((size_t)nb * kc * kc);
    d.B21.alloc((size_t)nb * kc * kc);
    for (int i = 0; i < nb; ++i) {  // nb = factor boxes (1 in translation-invariant mode)
      const int* s1 = dc.IsrcJ.p + (size_t)(2 * i) * nc;
      const int* s2 = dc.IsrcJ.p + (size_t)(2 * i + 1) * nc;
      kg.push_back(KgenP<double>{s1, s2, kc, kc, d.B12.p + fo(i) * kc * kc, kc, 0});
      kg.push_back(KgenP<double>{s2, s1, kc, kc, d.B21.p + fo(i) * kc * kc, kc, 0});
    }
  }
  long long maxe = 0;
  for (auto& q : kg) maxe = std::max(maxe, (long long)q.m * q.n);
  for (size_t off = 0; off < kg.size(); off += 65535) {
    const int cnt = (int)std::min<size_t>(65535, kg.size() - off);
    DevBuf<KgenP<double>> dkg(cnt);
    HSS_CUDA(cudaMemcpyAsync(dkg.p, kg.data() + off, cnt * sizeof(KgenP<double>), cudaMemcpyHostToDevice, stream));
    kgen_batched<double>(dkg.p, cnt, maxe, view(pts), kdev, stream);
    HSS_CUDA(cudaStreamSynchronize(stream));
  }
  if (dfm()) make_df_forward();  // the tensor-core mode's forward apply runs on double-float products
  HSS_CUDA(cudaStreamSynchronize(stream));
  phase_s[3] = std::chrono::duration<double>(std::chrono::steady_clock::now() - tc0).count();
  compressed = true;
  g_fwd.clear();
  fwd_plans.clear();
}

// ---------------------------------------------------------------------------
// invert
// ---------------------------------------------------------------------------
template <typename R>
static R* fac(Level2Dev& d, int which);

template <typename R>
void HSS2D::invert_impl() {
  const int depth = geo.depth;
  DevBuf<GemmP<R>> gscratch;
  for (int lev = depth; lev >= 0; --lev) {
    auto& g = geo.levels[lev];
    auto& d = L[lev];
    const int nb = nf(g), n = g.n, k = g.k, nr = n - k;
    const bool leaf = (lev == depth);
    const int kc = leaf ? 0 : geo.levels[lev + 1].k;
    auto& FIb = d.fac<R>(0);
    FIb.alloc((size_t)nb * n * n);
    R* FI = FIb.p;
    const R* Ech = leaf ? nullptr : L[lev + 1].fac<R>(1).p;
    k_assemble_F<R><<<grid_for((long long)nb * n * n), 256, 0, stream>>>(
        nb, n, kc, leaf ? 1 : 0, prm.transinv ? 1 : 0, leaf ? d.Bself.p : nullptr, leaf ? nullptr : d.B12.p,
        leaf ? nullptr : d.B21.p, Ech, FI);
    check_launch("k_assemble_F");
    invert_level<R>(FI, n, nb);
    if (lev == 0) break;
    // interpolation operators in the factor precision
    DevBuf<R> Tup, Tdn;
    const R* pTup;
    const R* pTdn;
    if (std::is_same<R, double>::value) {
      pTup = reinterpret_cast<const R*>(d.Tup.p);
      pTdn = reinterpret_cast<const R*>(d.Tdn.p);
    } else {
      Tup.alloc((size_t)nb * k * std::max(nr, 1));
      Tdn.alloc((size_t)nb * k * std::max(nr, 1));
      if (nr > 0) {
        k_convert<double, R><<<grid_for((long long)nb * k * nr), 256, 0, stream>>>((long long)nb * k * nr, d.Tup.p, Tup.p);
        k_convert<double, R><<<grid_for((long long)nb * k * nr), 256, 0, stream>>>((long long)nb * k * nr, d.Tdn.p, Tdn.p);
      }
      pTup = Tup.p;
      pTdn = Tdn.p;
    }
    DevBuf<R> W1((size_t)nb * n * n), W2((size_t)nb * k * n);
    // (1) FIJ = FI[J, :]
    k_gather_rows<R><<<grid_for((long long)nb * n * n), 256, 0, stream>>>(nb, n, n, d.J.p, FI, (long long)n * n, n,
                                                                          W1.p, (long long)n * n, n);
    // (2) RFI = FIJ[0:k,:] + Tup * FIJ[k:n,:]   (in place, rows 0..k-1 of W1)
    std::vector<GemmP<R>> P;
    if (nr > 0) {
      P.clear();
      for (int i = 0; i < nb; ++i)
        P.push_back(GemmP<R>{pTup + (size_t)i * k * nr, W1.p + (size_t)i * n * n + k, W1.p + (size_t)i * n * n, k, n,
                             nr, k, n, n});
      run_gemm<R>(P, false, false, R(1), R(1), stream, gscratch, dfgemm());
    }
    // (3) W2 = RFI[:, J]   (k x n, ld k)
    k_gather_cols<R><<<grid_for((long long)nb * k * n), 256, 0, stream>>>(nb, k, n, d.J.p, W1.p, (long long)n * n, n,
                                                                          W2.p, (long long)k * n, k);
    // (4) EI = W2[:,0:k] + W2[:,k:n] * Tdn^T
    if (nr > 0) {
      P.clear();
      for (int i = 0; i < nb; ++i)
        P.push_back(GemmP<R>{W2.p + (size_t)i * k * n + (size_t)k * k, pTdn + (size_t)i * k * nr,
                             W2.p + (size_t)i * k * n, k, k, nr, k, k, k});
      run_gemm<R>(P, false, true, R(1), R(1), stream, gscratch, dfgemm());
    }
    // (5) E = inv(EI)
    auto& Eb = d.fac<R>(1);
    Eb.alloc((size_t)nb * k * k);
    k_copy2d<R, R><<<grid_for((long long)nb * k * k), 256, 0, stream>>>(nb, k, k, W2.p, (long long)k * n, k, Eb.p,
                                                                       (long long)k * k, k);
    invert_level<R>(Eb.p, k, nb);
    // (6) U = E * RFI
    auto& Ub = d.fac<R>(2);
    Ub.alloc((size_t)nb * k * n);
    P.clear();
    for (int i = 0; i < nb; ++i)
      P.push_back(GemmP<R>{Eb.p + (size_t)i * k * k, W1.p + (size_t)i * n * n, Ub.p + (size_t)i * k * n, k, n, k, k,
                           n, k});
    run_gemm<R>(P, false, false, R(1), R(0), stream, gscratch, dfgemm());
    // (7) FIc = FI[:, J]
    k_gather_cols<R><<<grid_for((long long)nb * n * n), 256, 0, stream>>>(nb, n, n, d.J.p, FI, (long long)n * n, n,
                                                                          W1.p, (long long)n * n, n);
    // (8) G = FIc[:,0:k] + FIc[:,k:n] * Tdn^T   (in place, columns 0..k-1)
    if (nr > 0) {
      P.clear();
      for (int i = 0; i < nb; ++i)
        P.push_back(GemmP<R>{W1.p + (size_t)i * n * n + (size_t)k * n, pTdn + (size_t)i * k * nr,
                             W1.p + (size_t)i * n * n, n, k, nr, n, k, n});
      run_gemm<R>(P, false, true, R(1), R(1), stream, gscratch, dfgemm());
    }
    auto& Gb = d.fac<R>(3);
    Gb.alloc((size_t)nb * n * k);
    k_copy2d<R, R><<<grid_for((long long)nb * n * k), 256, 0, stream>>>(nb, n, k, W1.p, (long long)n * n, n, Gb.p,
                                                                       (long long)n * k, n);
    // (10) GE = G * E
    auto& GEb = d.fac<R>(4);
    GEb.alloc((size_t)nb * n * k);
    P.clear();
    for (int i = 0; i < nb; ++i)
      P.push_back(GemmP<R>{Gb.p + (size_t)i * n * k, Eb.p + (size_t)i * k * k, GEb.p + (size_t)i * n * k, n, k, k, n,
                           k, n});
    run_gemm<R>(P, false, false, R(1), R(0), stream, gscratch, dfgemm());
    check_launch("invert level");
    HSS_CUDA(cudaStreamSynchronize(stream));
  }
}

template <typename R>
void HSS2D::invert_level(R* A, int n, int nb) {
  if (n > panel_limit(GJ_MAX_N)) {
    invert_level_schur<R>(A, n, nb);
    return;
  }
  invert_level_ld<R>(A, n, n, nb, (size_t)n * n);
}

// Blocks above the cluster panel's size, by the 2 x 2 block inverse: with the leading n1 x n1
// block A11 and S = A22 - A21 A11^-1 A12,
//   A^-1 = [[A11^-1 + Z Y, -Z], [-S^-1 Y, S^-1]],  Y = A21 A11^-1, Z = A11^-1 A12 S^-1,
// two inversions of half size and six products, in place.  A11 is a diagonal block of the
// HSS system (at the root: the first child's E), inverted with partial pivoting.
template <typename R>
void HSS2D::invert_level_schur(R* A, int n, int nb) {
  const int n1 = (n / 2) & ~1, n2 = n - n1;
  HSS_REQUIRE(n2 <= GJ_MAX_N, HSS_ERR_ARG, "block too large for the two-level inversion");
  HSS_REQUIRE(n1 >= 2, HSS_ERR_ARG, "two-level inversion of a tiny block");
  DevBuf<GemmP<R>> gs;
  DevBuf<R> Ai((size_t)nb * n1 * n1), X((size_t)nb * n1 * n2), Y((size_t)nb * n2 * n1);
  auto blk = [&](int i, int r, int c) { return A + (size_t)i * n * n + r + (size_t)c * n; };
  k_copy2d<R, R><<<grid_for((long long)nb * n1 * n1), 256, 0, stream>>>(nb, n1, n1, A, (long long)n * n, n, Ai.p,
                                                                        (long long)n1 * n1, n1);
  check_launch("schur copy");
  invert_level_ld<R>(Ai.p, n1, n1, nb, (size_t)n1 * n1);
  std::vector<GemmP<R>> P;
  auto gemm = [&](auto mk, R alpha, R beta) {
    P.clear();
    for (int i = 0; i < nb; ++i) P.push_back(mk(i));
    run_gemm<R>(P, false, false, alpha, beta, stream, gs, dfgemm());
  };
  const R* Aip = Ai.p;
  // X = A11^-1 A12, Y = A21 A11^-1
  gemm([&](int i) { return GemmP<R>{Aip + (size_t)i * n1 * n1, blk(i, 0, n1), X.p + (size_t)i * n1 * n2, n1, n2, n1, n1, n, n1}; },
       R(1), R(0));
  gemm([&](int i) { return GemmP<R>{blk(i, n1, 0), Aip + (size_t)i * n1 * n1, Y.p + (size_t)i * n2 * n1, n2, n1, n1, n, n1, n2}; },
       R(1), R(0));
  // S = A22 - A21 X in place, then S^-1 in place
  gemm([&](int i) { return GemmP<R>{blk(i, n1, 0), X.p + (size_t)i * n1 * n2, blk(i, n1, n1), n2, n2, n1, n, n1, n}; },
       R(-1), R(1));
  invert_level_ld<R>(blk(0, n1, n1), n2, n, nb, (size_t)n * n);
  // A12 = -Z = -X S^-1, A21 = -S^-1 Y, A11 = A11^-1 - A12 Y
  gemm([&](int i) { return GemmP<R>{X.p + (size_t)i * n1 * n2, blk(i, n1, n1), blk(i, 0, n1), n1, n2, n2, n1, n, n}; },
       R(-1), R(0));
  gemm([&](int i) { return GemmP<R>{blk(i, n1, n1), Y.p + (size_t)i * n2 * n1, blk(i, n1, 0), n2, n1, n2, n, n2, n}; },
       R(-1), R(0));
  k_copy2d<R, R><<<grid_for((long long)nb * n1 * n1), 256, 0, stream>>>(nb, n1, n1, Ai.p, (long long)n1 * n1, n1, A,
                                                                        (long long)n * n, n);
  check_launch("schur copy");
  gemm([&](int i) { return GemmP<R>{blk(i, 0, n1), Y.p + (size_t)i * n2 * n1, blk(i, 0, 0), n1, n1, n2, n, n2, n}; },
       R(-1), R(1));
  HSS_CUDA(cudaStreamSynchronize(stream));
}

// Gauss-Jordan inversion of nb blocks (n x n, leading dimension lda, block stride bs).
template <typename R>
void HSS2D::invert_level_ld(R* A, int n, int lda, int nb, size_t bs) {
  DevBuf<int> ipiv((size_t)nb * n), info(nb), aux((size_t)nb * GJ_AUX);
  DevBuf<R> W((size_t)nb * 2 * GJ_NB * n), Wf((size_t)nb * n * n);
  info.zero(stream);
  std::vector<InvP<R>> P(nb);
  for (int i = 0; i < nb; ++i)
    P[i] = InvP<R>{A + (size_t)i * bs, n, lda, ipiv.p + (size_t)i * n, W.p + (size_t)i * 2 * GJ_NB * n,
                   Wf.p + (size_t)i * n * n, info.p + i, aux.p + (size_t)i * GJ_AUX};
  DevBuf<InvP<R>> dP(nb);
  HSS_CUDA(cudaMemcpyAsync(dP.p, P.data(), nb * sizeof(InvP<R>), cudaMemcpyHostToDevice, stream));
  invert_batched<R>(dP.p, nb, n, stream, dfinv());
  std::vector<int> hi;
  download(hi, info.p, nb, stream);
  HSS_CUDA(cudaStreamSynchronize(stream));
  for (int v : hi) {
    HSS_REQUIRE(v >= 0, HSS_ERR_NONFINITE, "non-finite pivot in block inversion");
    HSS_REQUIRE(v == 0, HSS_ERR_SINGULAR, "singular diagonal block in inversion");
  }
}

static void split_copy(const DevBuf<double>& src, DevBuf<double>& dst, cudaStream_t s) {
  dst.alloc(std::max<size_t>((src.n + 1) & ~(size_t)1, 2));  // whole (hi, hi, lo, lo) blocks
  split_df(src.p, dst.p, (long long)src.n, s);
}

// Float-pair copies of the forward operator's blocks (T, Bself, B12, B21).
void HSS2D::make_df_forward() {
  for (auto& d : L) {
    split_copy(d.Tup, d.Tup_df, stream);
    split_copy(d.TdnT, d.TdnT_df, stream);
    split_copy(d.Bself, d.Bself_df, stream);
    split_copy(d.B12, d.B12_df, stream);
    split_copy(d.B21, d.B21_df, stream);
  }
  HSS_CUDA(cudaStreamSynchronize(stream));
}

// Float-pair copies of the FP64 inverse factors (FI, E, U, G, GE).
void HSS2D::make_df_inverse() {
  for (auto& d : L)
    for (int i = 0; i < 5; ++i) split_copy(d.fd[i], d.fdf[i], stream);
  HSS_CUDA(cudaStreamSynchronize(stream));
}

// Digit slices of the FP64 inverse factors for the tensor-core inverse apply: per factor
// box, U (k x n) for the upward products and [FI, -G, GE] (n x (n + 2k); FI alone at the
// root) for the downward ones, in the order the solve plan reads them.
void HSS2D::make_tc_inverse() {
  for (int lev = 0; lev <= geo.depth; ++lev) {
    const auto& g = geo.levels[lev];
    auto& d = L[lev];
    const int nbf = nf(g);
    std::vector<TcPackP> P;
    if (lev > 0) {
      d.tcU_box = tc_packed_bytes(g.k, g.n);
      d.tcU.alloc(d.tcU_box * nbf);
      d.tcUe.alloc((size_t)g.k * nbf);
      for (int i = 0; i < nbf; ++i) {
        TcPackP q{};
        q.A[0] = d.fd[2].p + (size_t)i * g.k * g.n;
        q.K[0] = g.n;
        q.lda[0] = g.k;
        q.sign[0] = 1.0;
        q.M = g.k;
        q.out = d.tcU.p + d.tcU_box * i;
        q.rexp = d.tcUe.p + (size_t)i * g.k;
        P.push_back(q);
      }
    }
    const int Kd = (lev > 0) ? g.n + 2 * g.k : g.n;
    d.tcD_box = tc_packed_bytes(g.n, Kd);
    d.tcD.alloc(d.tcD_box * nbf);
    d.tcDe.alloc((size_t)g.n * nbf);
    for (int i = 0; i < nbf; ++i) {
      TcPackP q{};
      q.A[0] = d.fd[0].p + (size_t)i * g.n * g.n;
      q.K[0] = g.n;
      q.lda[0] = g.n;
      q.sign[0] = 1.0;
      if (lev > 0) {
        q.A[1] = d.fd[3].p + (size_t)i * g.n * g.k;
        q.K[1] = g.k;
        q.lda[1] = g.n;
        q.sign[1] = -1.0;
        q.A[2] = d.fd[4].p + (size_t)i * g.n * g.k;
        q.K[2] = g.k;
        q.lda[2] = g.n;
        q.sign[2] = 1.0;
      }
      q.M = g.n;
      q.out = d.tcD.p + d.tcD_box * i;
      q.rexp = d.tcDe.p + (size_t)i * g.n;
      P.push_back(q);
    }
    int maxM = 0, maxK = 0;
    for (auto& q : P) {
      maxM = std::max(maxM, q.M);
      maxK = std::max(maxK, q.K[0] + q.K[1] + q.K[2]);
    }
    DevBuf<TcPackP> dP(P.size());
    HSS_CUDA(cudaMemcpyAsync(dP.p, P.data(), P.size() * sizeof(TcPackP), cudaMemcpyHostToDevice, stream));
    tc_pack(dP.p, (int)P.size(), maxM, maxK, stream);
    HSS_CUDA(cudaStreamSynchronize(stream));
  }
}

void HSS2D::ensure_tc_err() {
  if (tc_err.p) return;
  tc_err.alloc(1);
  tc_err.zero(stream);
  HSS_CUDA(cudaMallocHost(&tc_err_host, sizeof(int)));
  *tc_err_host = 0;
}

void HSS2D::invert() {
  HSS_REQUIRE(compressed, HSS_ERR_STATE, "hss2d_invert before hss2d_compress");
  if (tcm()) ensure_tc_err();
  const auto ti0 = std::chrono::steady_clock::now();
  if (prm.precision == HSS_PREC_MIXED) invert_impl<float>();
  else invert_impl<double>();
  if (tcm()) make_tc_inverse();
  else if (dfm()) make_df_inverse();
  HSS_CUDA(cudaStreamSynchronize(stream));
  phase_s[4] = std::chrono::duration<double>(std::chrono::steady_clock::now() - ti0).count();
  inverted = true;
  g_inv_d.clear();
  g_inv_f.clear();
  inv_plans_d.clear();
  inv_plans_f.clear();
}

// ---------------------------------------------------------------------------
// inverse apply
// ---------------------------------------------------------------------------
template <typename R>
SolvePlan<R>& HSS2D::inv_plan(int r) {
  auto& cache = plan_cache<R>();
  auto it = cache.find(r);
  if (it != cache.end()) return it->second;
  SolvePlan<R>& pl = cache[r];
  const int depth = geo.depth;
  const long long N = geo.N;
  bool use_df = false;
  if constexpr (std::is_same<R, double>::value) use_df = dfm();
  pl.df = use_df;
  auto F = [&](Level2Dev& d, int i) -> const R* {
    if constexpr (std::is_same<R, double>::value) {
      if (use_df) return d.fdf[i].p;
    }
    return d.fac<R>(i).p;
  };
  auto& vin = stage_in<R>();
  auto& vout = stage_out<R>();
  const int NG = ng_pts;
  for (int lev = 0; lev <= depth; ++lev) {
    auto& d = L[lev];
    const auto& g = geo.levels[lev];
    d.vec<R>(0).ensure((size_t)g.nb * g.k * 8);
    d.vec<R>(1).ensure((size_t)g.nb * g.k * 8);
  }
  auto qptr = [&](int lev, int i, const R*& ptr, int& ld) {
    const auto& g = geo.levels[lev];
    if (lev == depth) {
      const int b = (1 << lev) - 1 + i;
      ptr = vin.p + (size_t)NG * geo.leaf_panel[b];
      ld = (int)N;
    } else {
      const auto& gc = geo.levels[lev + 1];
      ptr = L[lev + 1].vec<R>(0).p + (size_t)(2 * i) * gc.k;
      ld = gc.nb * gc.k;
    }
    (void)g;
  };
  if constexpr (std::is_same<R, double>::value) {
    if (tcm()) {
      // tensor-core products over the digit slices; at most 4 columns per product
      auto outptr = [&](int lev, int i, double*& ptr, int& ld) {
        if (lev == depth) {
          const int b = (1 << lev) - 1 + i;
          ptr = vout.p + (size_t)NG * geo.leaf_panel[b];
          ld = (int)N;
        } else {
          const auto& gc = geo.levels[lev + 1];
          ptr = L[lev + 1].vec<double>(1).p + (size_t)(2 * i) * gc.k;
          ld = gc.nb * gc.k;
        }
      };
      std::vector<std::vector<TcProd>> phases;
      for (int lev = depth; lev >= 1; --lev) {
        const auto& g = geo.levels[lev];
        auto& d = L[lev];
        std::vector<TcProd> P;
        for (int c0 = 0; c0 < r; c0 += TC_NR)
          for (int i = 0; i < g.nb; ++i) {
            const double* q;
            int ldq;
            qptr(lev, i, q, ldq);
            TcProd t{};
            t.A = d.tcU.p + d.tcU_box * fo(i);
            t.rexp = d.tcUe.p + (size_t)fo(i) * g.k;
            t.B[0] = q + (size_t)c0 * ldq;
            t.K[0] = g.n;
            t.ldb[0] = ldq;
            t.C = d.vec<double>(0).p + (size_t)i * g.k + (size_t)c0 * g.nb * g.k;
            t.ldc = g.nb * g.k;
            t.M = g.k;
            t.r = std::min(TC_NR, r - c0);
            P.push_back(t);
          }
        phases.push_back(std::move(P));
      }
      for (int lev = 0; lev <= depth; ++lev) {
        const auto& g = geo.levels[lev];
        auto& d = L[lev];
        std::vector<TcProd> P;
        for (int c0 = 0; c0 < r; c0 += TC_NR)
          for (int i = 0; i < g.nb; ++i) {
            const double* q;
            int ldq;
            qptr(lev, i, q, ldq);
            double* out;
            int ldo;
            outptr(lev, i, out, ldo);
            TcProd t{};
            t.A = d.tcD.p + d.tcD_box * fo(i);
            t.rexp = d.tcDe.p + (size_t)fo(i) * g.n;
            t.B[0] = q + (size_t)c0 * ldq;
            t.K[0] = g.n;
            t.ldb[0] = ldq;
            if (lev > 0) {
              t.B[1] = d.vec<double>(0).p + (size_t)i * g.k + (size_t)c0 * g.nb * g.k;
              t.K[1] = g.k;
              t.ldb[1] = g.nb * g.k;
              t.B[2] = d.vec<double>(1).p + (size_t)i * g.k + (size_t)c0 * g.nb * g.k;
              t.K[2] = g.k;
              t.ldb[2] = g.nb * g.k;
            }
            t.C = out + (size_t)c0 * ldo;
            t.ldc = ldo;
            t.M = g.n;
            t.r = std::min(TC_NR, r - c0);
            P.push_back(t);
          }
        phases.push_back(std::move(P));
      }
      // the whole apply, up and down the tree, as one chain of phases (one launch)
      pl.tc_steps.emplace_back();
      pl.tc_steps.back().build(phases, 1.0, 0.0, tc_err.p, stream);
      HSS_CUDA(cudaStreamSynchronize(stream));
      return pl;
    }
  }
  // HSS2D_applyinv_nsym.m:74-243: the upward pass phi_up = U q (q: the right-hand sides
  // at the leaves, the children's phi_up above), then per level out = FI q - G phi_up +
  // GE phi_dn (phi_dn: the parent's output).  FI q needs only the level's input and
  // - G phi_up only the level's own phi_up, so both leave the critical path: they run on a
  // low-priority side stream as soon as the upward pass has produced their operands, while
  // the high-priority stream runs the upward pass, the root and the + GE phi_dn
  // accumulations.  The three parts are added in FP64 storage (beta = 1).
  auto out_of = [&](int lev, int i, R*& out, int& ldo) {
    if (lev == depth) {
      const int b = (1 << lev) - 1 + i;
      out = vout.p + (size_t)NG * geo.leaf_panel[b];
      ldo = (int)N;
    } else {
      const auto& gc = geo.levels[lev + 1];
      out = L[lev + 1].vec<R>(1).p + (size_t)(2 * i) * gc.k;
      ldo = gc.nb * gc.k;
    }
  };
  // part 0: U q (upward); 1: FI q; 2: G phi_up; 3: GE phi_dn
  auto prods = [&](int lev, int part) {
    const auto& g = geo.levels[lev];
    auto& d = L[lev];
    std::vector<GemmP<R>> P;
    for (int i = 0; i < g.nb; ++i) {
      const R* q;
      int ldq;
      qptr(lev, i, q, ldq);
      R* out;
      int ldo;
      out_of(lev, i, out, ldo);
      if (part == 0)
        P.push_back(GemmP<R>{F(d, 2) + fo(i) * g.k * g.n, q, d.vec<R>(0).p + (size_t)i * g.k, g.k, r, g.n, g.k,
                             ldq, g.nb * g.k});
      else if (part == 1)
        P.push_back(GemmP<R>{F(d, 0) + fo(i) * g.n * g.n, q, out, g.n, r, g.n, g.n, ldq, ldo});
      else
        P.push_back(GemmP<R>{F(d, part == 2 ? 3 : 4) + fo(i) * g.n * g.k,
                             d.vec<R>(part == 2 ? 0 : 1).p + (size_t)i * g.k, out, g.n, r, g.k, g.n, g.nb * g.k,
                             ldo});
    }
    return P;
  };
  auto mark = [&](int side, int dep) {
    auto& st = pl.steps.back();
    st.side = side;
    if (dep >= 0) {
      st.deps.push_back(dep);
      pl.steps[dep].rec = true;
    }
    return (int)pl.steps.size() - 1;
  };
  auto push = [&](int lev, int part, R alpha, R beta, int side, int dep) {
    auto P = prods(lev, part);
    pl.add(P, alpha, beta, stream);
    return mark(side, dep);
  };
  // the side stream's product of a level: FI q - G phi_up (one double-float sum with
  // double-float operands), after the level's upward product
  auto push_side = [&](int lev, int dep) {
    if constexpr (std::is_same<R, double>::value) {
      if (use_df) {
        const auto& g = geo.levels[lev];
        auto& d = L[lev];
        std::vector<SegGemmP> PS;
        for (int i = 0; i < g.nb; ++i) {
          const R* q;
          int ldq;
          qptr(lev, i, q, ldq);
          R* out;
          int ldo;
          out_of(lev, i, out, ldo);
          SegGemmP sp{};
          sp.A[0] = F(d, 0) + fo(i) * g.n * g.n;
          sp.B[0] = q;
          sp.K[0] = g.n;
          sp.lda[0] = g.n;
          sp.ldb[0] = ldq;
          sp.sign[0] = 1.0;
          sp.A[1] = F(d, 3) + fo(i) * g.n * g.k;
          sp.B[1] = d.vec<R>(0).p + (size_t)i * g.k;
          sp.K[1] = g.k;
          sp.lda[1] = g.n;
          sp.ldb[1] = g.nb * g.k;
          sp.sign[1] = -1.0;
          sp.C = out;
          sp.M = g.n;
          sp.N = r;
          sp.ldc = ldo;
          PS.push_back(sp);
        }
        pl.add_seg(PS, R(1), R(0), stream);
        return mark(1, dep);
      }
    }
    push(lev, 1, R(1), R(0), 1, dep);
    return push(lev, 2, R(-1), R(1), 1, -1);
  };
  // Issue order.  The side stream takes the lower half of the levels in the order the
  // upward pass completes them (bottom up, overlapping the upward pass), then the upper
  // half top down, which is the order the downward accumulations need them: the side
  // product of level l + 1 overlaps the accumulation of level l.
  const int mid = depth / 2;
  std::vector<int> up(depth + 1, -1), side(depth + 1, -1);
  for (int lev = depth; lev >= 1; --lev) {
    up[lev] = push(lev, 0, R(1), R(0), 0, -1);
    if (lev > mid) side[lev] = push_side(lev, up[lev]);
  }
  push(0, 1, R(1), R(0), 0, -1);  // the root: FI q, after the whole upward pass
  for (int lev = 1; lev <= depth; ++lev) {
    if (lev <= mid) side[lev] = push_side(lev, up[lev]);
    push(lev, 3, R(1), R(1), 0, side[lev]);
  }
  if (depth >= 1) pl.streams = std::make_shared<PlanStreams>(pl.steps.size());
  HSS_CUDA(cudaStreamSynchronize(stream));
  if (autotune) pl.tune(stream);
  return pl;
}

void HSS2D::set_autotune(bool on) {
  autotune = on;
  g_inv_d.clear();
  g_inv_f.clear();
  g_fwd.clear();
  inv_plans_d.clear();
  inv_plans_f.clear();
  fwd_plans.clear();
}

template <typename R>
void HSS2D::applyinv_stage(int r) {
  // vin (N x r, ld N) -> vout; the plan is built (and synchronised) before capture
  SolvePlan<R>& pl = inv_plan<R>(r);
  run_graph(inv_graphs<R>(), r, stream, use_graphs, [&] { pl.run(stream); });
}

void HSS2D::ensure_stage() {
  const size_t cnt = (size_t)geo.N * 8;
  Xd.ensure(cnt);
  Yd.ensure(cnt);
  if (prm.precision == HSS_PREC_MIXED) { Xf.ensure(cnt); Yf.ensure(cnt); }
}

void HSS2D::applyinv_device(const double* dX, double* dY, int nrhs, cudaStream_t user) {
  HSS_REQUIRE(inverted, HSS_ERR_STATE, "hss2d_applyinv before hss2d_invert");
  HSS_REQUIRE(nrhs >= 1, HSS_ERR_ARG, "nrhs must be >= 1");
  ensure_stage();
  sync_from(user);
  const long long N = geo.N;
  for (int c0 = 0; c0 < nrhs; c0 += 8) {
    const int r = std::min(8, nrhs - c0);
    if (prm.precision == HSS_PREC_MIXED) {
      k_convert<double, float><<<grid_for(N * r), 256, 0, stream>>>(N * r, dX + (size_t)c0 * N, Xf.p);
      applyinv_stage<float>(r);
      k_convert<float, double><<<grid_for(N * r), 256, 0, stream>>>(N * r, Yf.p, dY + (size_t)c0 * N);
    } else {
      HSS_CUDA(cudaMemcpyAsync(Xd.p, dX + (size_t)c0 * N, (size_t)N * r * sizeof(double), cudaMemcpyDeviceToDevice, stream));
      applyinv_stage<double>(r);
      HSS_CUDA(cudaMemcpyAsync(dY + (size_t)c0 * N, Yd.p, (size_t)N * r * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    }
    check_launch("applyinv");
  }
  sync_to(user);
}

// ---------------------------------------------------------------------------
// forward apply (FP64)
// ---------------------------------------------------------------------------
void HSS2D::fwd_prepare(int r) {
  if (fwd_plans.count(r)) return;
  FwdPlan& fp = fwd_plans[r];
  const int depth = geo.depth;
  const long long N = geo.N;
  const int NG = ng_pts;
  for (int lev = 0; lev <= depth; ++lev) {
    const auto& g = geo.levels[lev];
    auto& d = L[lev];
    d.upF.ensure((size_t)g.nb * g.k * 8);
    d.dnF.ensure((size_t)g.nb * g.k * 8);
    d.rsF.ensure((size_t)g.nb * std::max(g.n - g.k, 1) * 8);
    d.tmF.ensure((size_t)g.nb * std::max(g.n - g.k, 1) * 8);
  }
  fp.up.resize(depth + 1);
  fp.lam.resize(depth + 1);
  fp.eta.resize(depth + 1);
  const bool df = dfm();
  for (int lev = 0; lev <= depth; ++lev) fp.up[lev].df = fp.lam[lev].df = fp.eta[lev].df = df;
  auto pick = [&](DevBuf<double>& a, DevBuf<double>& b) -> const double* { return df ? b.p : a.p; };
  for (int lev = depth; lev >= 1; --lev) {
    const auto& g = geo.levels[lev];
    auto& d = L[lev];
    const int nr = g.n - g.k;
    if (nr > 0) {
      std::vector<GemmP<double>> P;
      for (int i = 0; i < g.nb; ++i)
        P.push_back(GemmP<double>{pick(d.Tup, d.Tup_df) + fo(i) * g.k * nr, d.rsF.p + (size_t)i * nr,
                                  d.upF.p + (size_t)i * g.k, g.k, r, nr, g.k, g.nb * nr, g.nb * g.k});
      fp.up[lev].add(P, 1.0, 1.0, stream);
    }
  }
  // the sibling products of level lev (the leaves' self products at lev = depth) read the
  // upward pass of level lev + 1 (the input at the leaves): fp.lam[lev] runs on a side
  // stream once that level is done; the downward pass then runs eta and the scatters,
  // which add onto what lam wrote
  for (int lev = 0; lev <= depth; ++lev) {
    const auto& g = geo.levels[lev];
    auto& d = L[lev];
    std::vector<GemmP<double>> P;
    for (int i = 0; i < g.nb; ++i) {
      double* out;
      int ldo;
      if (lev == depth) {
        const int b = (1 << lev) - 1 + i;
        out = Yd.p + (size_t)NG * geo.leaf_panel[b];
        ldo = (int)N;
        P.push_back(GemmP<double>{pick(d.Bself, d.Bself_df) + fo(i) * g.n * g.n, Xd.p + (size_t)NG * geo.leaf_panel[b], out, g.n,
                                  r, g.n, g.n, (int)N, ldo});
      } else {
        const auto& gc = geo.levels[lev + 1];
        auto& dc = L[lev + 1];
        out = dc.dnF.p + (size_t)(2 * i) * gc.k;
        ldo = gc.nb * gc.k;
        const int kc = gc.k;
        P.push_back(GemmP<double>{pick(d.B12, d.B12_df) + fo(i) * kc * kc, dc.upF.p + (size_t)(2 * i + 1) * kc, out, kc, r, kc,
                                  kc, gc.nb * kc, ldo});
        P.push_back(GemmP<double>{pick(d.B21, d.B21_df) + fo(i) * kc * kc, dc.upF.p + (size_t)(2 * i) * kc, out + kc, kc, r, kc,
                                  kc, gc.nb * kc, ldo});
      }
    }
    const int nr = g.n - g.k;
    if (lev > 0 && nr > 0) {
      std::vector<GemmP<double>> Q;
      for (int i = 0; i < g.nb; ++i)
        Q.push_back(GemmP<double>{pick(d.TdnT, d.TdnT_df) + fo(i) * g.k * nr, d.dnF.p + (size_t)i * g.k,
                                  d.tmF.p + (size_t)i * nr, nr, r, g.k, nr, g.nb * g.k, g.nb * nr});
      fp.eta[lev].add(Q, 1.0, 0.0, stream);
    }
    fp.lam[lev].add(P, 1.0, 0.0, stream);
  }
  fp.streams = std::make_shared<PlanStreams>(2 * (size_t)(depth + 1));
  HSS_CUDA(cudaStreamSynchronize(stream));
  if (autotune)
    for (int lev = 0; lev <= depth; ++lev) {
      fp.up[lev].tune(stream);
      fp.lam[lev].tune(stream);
      fp.eta[lev].tune(stream);
    }
}

void HSS2D::apply_stage(int r) {
  // Xd (N x r) -> Yd
  fwd_prepare(r);
  run_graph(g_fwd, r, stream, use_graphs, [&] { apply_stage_body(r); });
}

void HSS2D::apply_stage_body(int r) {
  FwdPlan& fp = fwd_plans[r];
  const int depth = geo.depth;
  const long long N = geo.N;
  // HSS2D_apply_nsym.m:74-218 on two streams: the upward pass, then per level the
  // downward evaluation and scatter on a high-priority stream; each level's sibling
  // products (the leaves' self products) on a low-priority stream as soon as the upward
  // pass has produced their operands
  PlanStreams& S = *fp.streams;
  cudaStream_t cs = S.crit, ss = S.side;
  auto ev_up = [&](int lev) { return S.ev[lev]; };
  auto ev_lam = [&](int lev) { return S.ev[depth + 1 + lev]; };
  S.fork_from(stream);
  fp.lam[depth].run(ss);  // the leaves' self products: the input only
  HSS_CUDA(cudaEventRecord(ev_lam(depth), ss));
  for (int lev = depth; lev >= 1; --lev) {
    const auto& g = geo.levels[lev];
    auto& d = L[lev];
    const bool leaf = (lev == depth);
    const int kc = leaf ? 0 : geo.levels[lev + 1].k;
    const double* src = leaf ? Xd.p : L[lev + 1].upF.p;
    const long long lds = leaf ? N : (long long)geo.levels[lev + 1].nb * kc;
    const int nr = g.n - g.k;
    k_fwd_gather<<<grid_for((long long)g.nb * g.n * r), 256, 0, cs>>>(
        g.nb, g.n, g.k, kc, leaf ? 1 : 0, r, d.J.p, d.IsrcJ.p, src, lds, d.upF.p, (long long)g.nb * g.k, d.rsF.p,
        (long long)g.nb * std::max(nr, 1));
    fp.up[lev].run(cs);
    HSS_CUDA(cudaEventRecord(ev_up(lev), cs));
    HSS_CUDA(cudaStreamWaitEvent(ss, ev_up(lev), 0));
    fp.lam[lev - 1].run(ss);  // the siblings of level lev - 1: this level's upward values
    HSS_CUDA(cudaEventRecord(ev_lam(lev - 1), ss));
  }
  for (int lev = 1; lev <= depth; ++lev) {
    const auto& g = geo.levels[lev];
    auto& d = L[lev];
    const bool leaf = (lev == depth);
    const int kc = leaf ? 0 : geo.levels[lev + 1].k;
    double* dst = leaf ? Yd.p : L[lev + 1].dnF.p;
    const long long ldd = leaf ? N : (long long)geo.levels[lev + 1].nb * kc;
    const int nr = g.n - g.k;
    HSS_CUDA(cudaStreamWaitEvent(cs, ev_lam(lev - 1), 0));  // this level's downward input
    fp.eta[lev].run(cs);
    HSS_CUDA(cudaStreamWaitEvent(cs, ev_lam(lev), 0));  // the scatter adds onto lam's output
    k_fwd_scatter<<<grid_for((long long)g.nb * g.n * r), 256, 0, cs>>>(
        g.nb, g.n, g.k, kc, leaf ? 1 : 0, r, d.J.p, d.IsrcJ.p, dst, ldd, d.dnF.p, (long long)g.nb * g.k, d.tmF.p,
        (long long)g.nb * std::max(nr, 1));
  }
  S.join_into(stream);
  check_launch("apply");
}

void HSS2D::apply_device(const double* dX, double* dY, int nrhs, cudaStream_t user) {
  HSS_REQUIRE(compressed, HSS_ERR_STATE, "hss2d_apply before hss2d_compress");
  HSS_REQUIRE(nrhs >= 1, HSS_ERR_ARG, "nrhs must be >= 1");
  ensure_stage();
  sync_from(user);
  const long long N = geo.N;
  for (int c0 = 0; c0 < nrhs; c0 += 8) {
    const int r = std::min(8, nrhs - c0);
    HSS_CUDA(cudaMemcpyAsync(Xd.p, dX + (size_t)c0 * N, (size_t)N * r * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    apply_stage(r);
    HSS_CUDA(cudaMemcpyAsync(dY + (size_t)c0 * N, Yd.p, (size_t)N * r * sizeof(double), cudaMemcpyDeviceToDevice, stream));
  }
  sync_to(user);
}

// ---------------------------------------------------------------------------
// solve with iterative refinement
// ---------------------------------------------------------------------------
void HSS2D::solve_device(const double* df, double* dx, int nrhs, double tol, int maxit, double* relres,
                         int* iters, cudaStream_t user) {
  HSS_REQUIRE(inverted, HSS_ERR_STATE, "hss2d_solve before hss2d_invert");
  HSS_REQUIRE(nrhs >= 1 && maxit >= 1, HSS_ERR_ARG, "nrhs and maxit must be >= 1");
  ensure_stage();
  sync_from(user);
  const long long N = geo.N;
  Rd.ensure((size_t)N * 8);
  Dd.ensure((size_t)N * 8);
  const int gx = 256;
  ir_part.ensure((size_t)gx * 8 * 2);
  ir_host.ensure((size_t)gx * 8 * 2);
  double* part_d = ir_part.p;
  const double* hp = ir_host.p;
  double worst_all = 0.0;
  int used_all = 0;
  for (int c0 = 0; c0 < nrhs; c0 += 8) {
    const int r = std::min(8, nrhs - c0);
    const double* f = df + (size_t)c0 * N;
    double* x = dx + (size_t)c0 * N;
    // x = A^-1 f
    solve_once(f, x, r);
    int used = 1;
    double worst = 0.0;
    while (true) {
      // res = f - A x
      HSS_CUDA(cudaMemcpyAsync(Xd.p, x, (size_t)N * r * sizeof(double), cudaMemcpyDeviceToDevice, stream));
      apply_stage(r);
      k_residual<<<gx, 256, 0, stream>>>(N, r, f, N, Yd.p, N, Rd.p, N, part_d);
      HSS_CUDA(cudaMemcpyAsync(ir_host.p, part_d, (size_t)gx * r * 2 * sizeof(double), cudaMemcpyDeviceToHost,
                               stream));
      if (tcm()) HSS_CUDA(cudaMemcpyAsync(tc_err_host, tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
      HSS_CUDA(cudaStreamSynchronize(stream));
      HSS_REQUIRE(!tcm() || *tc_err_host == 0, HSS_ERR_CUDA,
                  "tensor-core product: a pipeline wait timed out (results invalid)");
      worst = 0.0;
      for (int c = 0; c < r; ++c) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < gx; ++q) { a += hp[((size_t)q * r + c) * 2]; b += hp[((size_t)q * r + c) * 2 + 1]; }
        const double rel = (b > 0.0) ? std::sqrt(a / b) : std::sqrt(a);
        HSS_REQUIRE(std::isfinite(rel), HSS_ERR_NONFINITE, "non-finite residual in refinement");
        worst = std::max(worst, rel);
      }
      if (worst <= tol || used >= maxit) break;
      solve_once(Rd.p, Dd.p, r);
      k_axpy<<<grid_for(N * r), 256, 0, stream>>>(N, r, Dd.p, N, x, N);
      ++used;
    }
    worst_all = std::max(worst_all, worst);
    used_all = std::max(used_all, used);
  }
  if (relres) *relres = worst_all;
  if (iters) *iters = used_all;
  sync_to(user);
}

void HSS2D::solve_once(const double* f, double* x, int r) {
  const long long N = geo.N;
  if (prm.precision == HSS_PREC_MIXED) {
    k_convert<double, float><<<grid_for(N * r), 256, 0, stream>>>(N * r, f, Xf.p);
    applyinv_stage<float>(r);
    k_convert<float, double><<<grid_for(N * r), 256, 0, stream>>>(N * r, Yf.p, x);
  } else {
    HSS_CUDA(cudaMemcpyAsync(Xd.p, f, (size_t)N * r * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    applyinv_stage<double>(r);
    HSS_CUDA(cudaMemcpyAsync(x, Yd.p, (size_t)N * r * sizeof(double), cudaMemcpyDeviceToDevice, stream));
  }
  check_launch("solve_once");
}

// ---------------------------------------------------------------------------
// stream ordering with a caller stream
// ---------------------------------------------------------------------------
void HSS2D::sync_from(cudaStream_t user) {
  if (user == nullptr || user == stream) return;
  HSS_CUDA(cudaEventRecord(ev, user));
  HSS_CUDA(cudaStreamWaitEvent(stream, ev, 0));
}

void HSS2D::sync_to(cudaStream_t user) {
  if (user == nullptr) {
    HSS_CUDA(cudaStreamSynchronize(stream));
    return;
  }
  if (user == stream) return;
  HSS_CUDA(cudaEventRecord(ev, stream));
  HSS_CUDA(cudaStreamWaitEvent(user, ev, 0));
}

HSS2D::HSS2D(const hss2d_params& p) : prm(p) {
  HSS_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  HSS_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
}

HSS2D::~HSS2D() {
  g_inv_d.clear();
  g_inv_f.clear();
  g_fwd.clear();
  L.clear();
  if (tc_err_host) cudaFreeHost(tc_err_host);
  if (ev) cudaEventDestroy(ev);
  if (stream) cudaStreamDestroy(stream);
}

long long HSS2D::solve_bytes() const {
  const size_t es = (prm.precision == HSS_PREC_MIXED) ? sizeof(float) : sizeof(double);
  long long b = 0;
  for (int lev = 0; lev <= geo.depth; ++lev) {
    const auto& g = geo.levels[lev];
    long long per = (long long)g.n * g.n;
    if (lev > 0) per += 3LL * g.n * g.k;
    b += per * g.nb;
  }
  return b * (long long)es;
}

// Kernels of one solve with one residual check: inverse apply (skinny steps and
// split-K reductions of the cached plan), forward apply (gather, products,
// scatter per level) and the residual kernel; conversions in mixed precision.
int HSS2D::solve_launches(int nrhs) const {
  int total = 0;
  for (int c0 = 0; c0 < nrhs; c0 += 8) {
    const int r = std::min(8, nrhs - c0);
    int inv = 0;
    if (prm.precision == HSS_PREC_MIXED) {
      auto it = inv_plans_f.find(r);
      inv = (it != inv_plans_f.end()) ? it->second.launches() : (geo.depth + 1 + 3 * geo.depth);
      inv += 2;  // FP64 <-> FP32 conversions
    } else {
      auto it = inv_plans_d.find(r);
      inv = (it != inv_plans_d.end()) ? it->second.launches() : (geo.depth + 1 + 3 * geo.depth);
    }
    int fwd = 2 * geo.depth;  // gather and scatter per level
    auto f = fwd_plans.find(r);
    if (f != fwd_plans.end()) {
      for (auto& pl : f->second.up) fwd += pl.launches();
      for (auto& pl : f->second.lam) fwd += pl.launches();
      for (auto& pl : f->second.eta) fwd += pl.launches();
    } else {
      fwd += 3 * geo.depth + 1;
    }
    total += inv + fwd + 1;
  }
  return total;
}

}  // namespace hss
