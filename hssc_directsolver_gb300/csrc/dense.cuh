// Batched dense linear algebra for the HSS levels (declarations).
//
// Every routine works on a batch of independent column-major problems whose
// descriptors live in device memory, so one launch covers every box of a tree
// level (and every problem of a batch).  Sizes may differ per problem; a
// problem whose size is already finished simply idles in that launch.
#pragma once

#include "common.cuh"

namespace hss {

// C_b = alpha * op(A_b) * op(B_b) + beta * C_b
template <typename R>
struct GemmP {
  const R* A;
  const R* B;
  R* C;
  int M, N, K;
  int lda, ldb, ldc;
};

// C = sum_s sign_s A_s B_s over up to three K segments (A_s: M x K_s, ld lda_s; B_s:
// K_s x N, ld ldb_s): one launch for a sum of products that share their rows, e.g.
// FI q - G phi_up + GE phi_dn of the inverse apply's downward pass.
struct SegGemmP {
  const double* A[3];
  const double* B[3];
  double* C;
  int K[3];
  int lda[3], ldb[3];
  double sign[3];
  int M, N, ldc;
};

// Double-float ("FP64 x FP32 pairs") skinny product: A holds every FP64 element
// as a float pair (hi, lo) with hi + lo equal to it to 2^-48 (same 8 bytes per
// element), B and C are FP64.  Each multiply-add runs on the FP32 pipes: an exact
// product (FMA error term) plus the cross terms, added into a (hi, lo) float
// accumulator with TwoSum and a Fast2Sum renormalisation.  GB300 issues FP32 at
// 64x its FP64 rate, so this outruns native FP64 for matrix-vector products.
void gemm_skinny_split_df(const GemmP<double>* dP, int batch, int maxM, int maxN, double alpha, double beta,
                          int ksplit, double* part, cudaStream_t s);
// the segmented form (A_s as float pairs; C = alpha * sum + beta * C)
void gemm_skinny_split_df(const SegGemmP* dP, int batch, int maxM, int maxN, double alpha, double beta,
                          int ksplit, double* part, cudaStream_t s);
// gemm_batched in double-float arithmetic (FP64 in and out, ~2^-47 per product)
void gemm_batched_df(const GemmP<double>* dP, int batch, int maxM, int maxN, bool tA, bool tB, double alpha,
                     double beta, cudaStream_t s);
// K slices for gemm_skinny_split_df: enough CTAs for several waves on 152 SMs
// (the double-float kernel does ~15x the arithmetic per byte of the FP64 one)
int skinny_ksplit_df(int batch, int maxM, int maxK);
// FP64 -> pair-interleaved float pairs (hi, hi, lo, lo per element pair); dst holds
// n rounded up to even elements and starts on a 16-byte boundary
void split_df(const double* src, double* dst, long long n, cudaStream_t s);

template <typename R>
void gemm_batched(const GemmP<R>* dP, int batch, int maxM, int maxN, bool tA, bool tB,
                  R alpha, R beta, cudaStream_t s);

// Same product for skinny outputs (N <= 8 columns, the right-hand sides of a
// solve): one warp per 32 rows, K split over the warps of a block; the result
// is deterministic (fixed summation order).
template <typename R>
void gemm_skinny(const GemmP<R>* dP, int batch, int maxM, R alpha, R beta, cudaStream_t s);
// split-K variant: ksplit CTAs per row tile write partial sums to `part`
// (batch * ksplit * maxM * 8 entries), added in a fixed order by a second pass
template <typename R>
void gemm_skinny_split(const GemmP<R>* dP, int batch, int maxM, int maxN, R alpha, R beta, int ksplit, R* part,
                       cudaStream_t s);
template <typename R>
int skinny_ksplit(int batch, int maxM, int maxK);

// In-place inversion by blocked Gauss-Jordan with partial (row) pivoting.
template <typename R>
struct InvP {
  R* A;
  int n, lda;
  int* ipiv;  // n entries
  R* W;       // 2*GJ_NB x n workspace (pivot rows, then displaced rows)
  R* Wfull;   // n x n workspace (final column permutation)
  int* info;  // 0 ok, j+1 if pivot j was exactly zero, -1 non-finite
  int* aux;   // GJ_AUX ints: row-permutation bookkeeping of the current panel
};
constexpr int GJ_NB = 32;
constexpr int GJ_MAX_N = 12800;  // the cluster panel's size limit of invert_batched
constexpr int GJ_AUX = 4 * GJ_NB + 4;

template <typename R>
// df (FP64 only): the rank-32 trailing updates in double-float arithmetic
void invert_batched(const InvP<R>* dP, int batch, int maxn, cudaStream_t s, bool df = false);

// Least squares X = A(:, 0:kf) \ A(:, kf:n) for tall full-rank problems, by
// blocked Householder QR of the first kf columns applied to the remaining
// ones, then a blocked back substitution into X (A is overwritten).  diag
// receives |R_ii| (kf entries) for rank diagnostics.
template <typename R>
struct QrP {
  R* A;
  int m, n, kf, lda;
  R* V;     // m x QR_NB workspace (explicit reflectors)
  R* Tf;    // QR_NB x QR_NB workspace (compact-WY factor)
  R* diag;  // kf entries
  R* X;     // output: kf x (n - kf) solution, leading dimension ldx
  int ldx;
};
constexpr int QR_NB = 32;

template <typename R>
// df (FP64 only): the compact-WY trailing updates in double-float arithmetic
// solve = false: the QR only; the top kf rows then hold R11 (upper triangle; the reflectors
// below it) and the first kf rows of Q^T A(:, kf:n), the data a row-blocked (TSQR) solve
// stacks onto the next block of rows.
void lstsq_batched(const QrP<R>* dP, int batch, int maxm, int maxn, int maxkf, cudaStream_t s, bool df = false,
                   bool solve = true);
// the cluster panel's row limit of lstsq_batched
constexpr int LSTSQ_MAX_ROWS = 12800;

// Interpolative decomposition of one m x n block per problem (the pivoted-QR
// rank detection of the reference ID, with its randomized posterior check).
struct IdP {
  const double* A;  // original block, column-major m x n, ld = m
  double* W;        // m x n workspace: overwritten by the pivoted QR (R on top)
  int m, n;
  int* perm;        // n: column permutation (0-based)
  int* rank;        // output rank k
  double* T;        // output k x (n-k) interpolation matrix (ld = n)
  int force_k;      // >= 0: fixed-rank mode on an already factored W
  double* svdW;     // n x n workspace (fixed-rank mode)
  double* svdV;     // n x n workspace (fixed-rank mode)
  double* x;        // 2*n workspace (random vectors)
  double* y;        // m+n workspace
  int problem;      // id for the random stream (2*box + side, box local to its tree)
  int steps_hint;   // > 0: stop the pivoted QR after this many steps if the rank is resolved;
                    // ID_QR_ONLY: the full pivoted QR only (rank = min(m, n), T untouched)
  unsigned long long seed;  // key of the random stream (one per independent problem)
  int* stat;        // out (may be null): [0] 0 full / 1 truncated / 2 needs a full rerun, [1] QR steps done
};

constexpr int ID_QR_ONLY = -2;
// steps_hint = ID_EVERY_STEP: the truncation test of the learned-rank mode at every step (the
// plain per-step threshold rule, no model)
constexpr int ID_EVERY_STEP = -3;

// df: the pivoted QR in double-float arithmetic (k_id_adaptive_df), rank / T / check in FP64
void id_adaptive_batched(const IdP* dP, int batch, double acc, cudaStream_t s, bool df = false);
void id_fixed_batched(const IdP* dP, int batch, cudaStream_t s);
// The complex ID through the real 2 x 2 embedding (m, n real, pairs of columns pivoted
// together; *rank and T in real columns); maxn <= 4096 real columns.
void id_pairs_batched(const IdP* dP, int batch, int maxn, double acc, cudaStream_t s);

// Householder QR with column pivoting of W (m x l, ld ldw; overwritten) and the
// explicit thin Q (m x min(m,l), ld ldq); D = |diag R|.  Same pivots and
// reflectors as the ID's pivoted QR.  One block per problem; l <= 4096.
struct PqrP {
  double* W;
  int m, l, ldw;
  double* tau;  // min(m,l) workspace
  double* Q;
  int ldq;
  double* D;    // min(m,l)
};
void pqr_q_batched(const PqrP* dP, int batch, cudaStream_t s);

// Gaussian test matrix G (m x l, ld ldg): entry (i, j) is the Irwin-Hall sum of the
// 12 uniforms u(seed, stream, 12*(i + m*j) + t), t = 0..11, added in order, minus 6.
struct GaussP {
  double* G;
  int m, l, ldg;
  unsigned long long seed, stream;
};
void gauss_batched(const GaussP* dP, int batch, long long maxEntries, cudaStream_t s);

}  // namespace hss
