/*
 * hssgpu.h -- C ABI of the GB300 HSS direct-solver library (libhssgpu.so).
 *
 * Drop-in boundary for the MATLAB-level entry points of
 * EduardoCorona84/HSSC_DirectSolver.  Each function below names the reference
 * function it replaces (file:line of the reference project).  Conventions:
 *
 *  - Every entry point returns an int status (HSS_OK = 0); the reference
 *    raises MATLAB errors instead.  hss_last_error() gives a message.
 *  - Dense arrays are column-major (MATLAB layout).  Index arrays exported by
 *    this library are 0-based; the MEX shim adds 1.
 *  - Handles own their device memory and one CUDA stream; a handle is not
 *    thread-safe, distinct handles are.
 *  - Host-pointer calls copy inputs to the device and results back; the
 *    *_device variants take device pointers and a cudaStream_t (as void*).
 *  - Plain types only: no C++ or torch types cross this boundary.
 */
#ifndef HSSGPU_H
#define HSSGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define HSS_OK 0
#define HSS_ERR_ARG 1       /* invalid argument / size */
#define HSS_ERR_CUDA 2      /* CUDA runtime failure or no device */
#define HSS_ERR_SINGULAR 3  /* exact zero pivot in a block inversion */
#define HSS_ERR_NONFINITE 4 /* NaN/Inf met in inputs or factors */
#define HSS_ERR_RANK 5      /* rank / buffer capacity exceeded */
#define HSS_ERR_STATE 6     /* call out of order (e.g. applyinv before invert) */
#define HSS_ERR_NOMEM 7     /* device allocation failed */

/* ---- kernels (Common/Kernel_Eval.m) ------------------------------------ */
#define HSS_SL_L_2D 0 /* Kernel_Eval.m:60-61, (den==0) + h^2/2 b(x) log(den) c(y) */
#define HSS_DL_L_2D 1 /* custom-kernel slot Kernel_Eval.m:75-79: Laplace double layer */
#define HSS_SL_H_2D 2 /* Kernel_Eval.m:44-53, complex: w (den==0) + h^2 kh^2 (i/4) b(x) H0(kh r) c(y),
                         w = 1 + kh^2 (i/4) dr (dr = the order-4 Duan-Rokhlin weight; 0 = order 0).
                         Evaluated by hss_kernel_eval and solved by HSS2D (complex vectors:
                         interleaved (re, im) doubles); HSS1D takes the real kernels. */

/* modulation forms of b(x) / c(y) (hss_kernel_params.b_kind / c_kind) */
#define HSS_MOD_GAUSS 0     /* 1 + alpha exp(-isig |p - p0|^2); alpha = 0: 1 (b_func, Kernel_Eval.m:99-108) */
#define HSS_MOD_BUMP 1      /* Bump_function option 4 called without h (Common/Bump_function.m:53-63,
                               shift 0): the nonsymmetric Lippmann-Schwinger b, Kernel_Eval.m:115-119 */
#define HSS_MOD_SQRT_BUMP 2 /* sqrt(Bump_function option 4 with shift 4h): the symmetric
                               Lippmann-Schwinger b and c, Kernel_Eval.m:129-140 */
#define HSS_MOD_GAUSS0 3    /* alpha exp(-isig |p - p0|^2) without the constant: a Gaussian
                               contrast taken symmetrically (b = c = its square root, isig halved) */

/* HSS2D skeleton rules (params.skel_rule, HSS2D_build_tree_nsym.m:399-412, :668-730); every
 * box of a level then holds the level's largest count (residual points nearest the box
 * boundary promoted) */
#define HSS_SKEL_BDRY 0 /* the points within layers h of the box boundary */
#define HSS_SKEL_RAND 1 /* a random sample of the box's points (LOCAL_random_sampler until
                           ceil(2/3 n) or ceil(3/4 n) / 1.1 are kept) */
#define HSS_SKEL_ID 2   /* the ID of K(proxies, box) on every level (kh > 0 trees) */
#define HSS_SKEL_WDEC 3 /* a Whitney decomposition of the box (Common/Whitney_decomposition.m):
                           boundary layers plus sampled lines at dyadic distances */

/* HSS2D box proxies (params.proxy_rule, HSS2D_build_tree_nsym.m:870-961) */
#define HSS_PROXY_BDRY 0 /* every point of the box's proxy layers (build_box_proxy.m:52-88) */
#define HSS_PROXY_RAND 1 /* the layers sampled with probability 2^(-lambda l) by dyadic distance
                            band l until ceil(2/3 n) (even levels) or ceil(3/4 n) points remain
                            (LOCAL_Build_Proxy :883-905, LOCAL_random_sampler :964-1001) */
#define HSS_PROXY_WDEC 2 /* the points of twice the proxy layers kept by a Whitney decomposition
                            of the box boundary (LOCAL_Build_Proxy :877-881 over
                            Common/Whitney_decomposition_1Dcurve.m) */

/* precision modes */
#define HSS_PREC_FP64 0  /* plain FP64 everywhere */
#define HSS_PREC_MIXED 1 /* FP32 inverse factors; the least squares (panels, updates, back
                            substitution) and the refinement's forward products in double-float;
                            FP64 refinement residual */
#define HSS_PREC_DFLOAT 2 /* FP64 inversion; the interpolation least squares (panels, trailing
                             updates, back substitution) and the solve products in paired FP32
                             arithmetic (~2^-48); FP64 refinement against the forward operator */
#define HSS_PREC_DFLOAT_INV 3 /* HSS_PREC_DFLOAT plus the inversion's and the least squares'
                                 trailing updates and products in paired FP32 (factors ~5 bits
                                 short of FP64; refinement restores the residual) */
#define HSS_PREC_TC 4 /* HSS_PREC_DFLOAT's FP64 inversion and forward products; the inverse apply's
                         products on the tensor cores (tcgen05): each FP64 inverse factor is cut
                         once into 6 bf16 fixed-point digit slices per row (12 bytes per entry),
                         the right-hand sides likewise per column, and the exact digit products
                         are summed in integers (~2^-48 of the row and column maxima) */

/* HSS2D interpolation-operator storage (params.INTERform) */
#define HSS_INTER_DENSE 0
#define HSS_INTER_LOWRANK 1

/* b(x) = 1 + b_alpha*exp(-b_isig*|x-(b_x0,b_y0)|^2), c(y) likewise; alpha = 0
 * switches a modulation off (LOCAL_get_bc, Kernel_Eval.m:98-159).  b_kind / c_kind
 * select the Lippmann-Schwinger bump forms instead (HSS_MOD_*; 0 for the Laplace kernels). */
typedef struct hss_kernel_params {
  int32_t flag;
  int32_t pad_;
  double h;
  double b_alpha, b_x0, b_y0, b_isig;
  double c_alpha, c_x0, c_y0, c_isig;
  double kh;           /* wavenumber (params.kh) of HSS_SL_H_2D */
  double dr_re, dr_im; /* params.dr_weights (order 4) of HSS_SL_H_2D */
  int32_t b_kind, c_kind; /* HSS_MOD_* */
} hss_kernel_params;

/* A = Kernel_Eval(X1, X2, params) (Common/Kernel_Eval.m:1-96) on the device, host
 * buffers.  X1: m targets, X2: n sources, each column-major (x column, then y column).
 * A: m x n column-major, doubles for HSS_SL_L_2D, interleaved (re, im) pairs for
 * HSS_SL_H_2D (2 m n doubles).  HSS_DL_L_2D needs normals and weights and is not
 * evaluated here (HSS_ERR_ARG). */
int hss_kernel_eval(const hss_kernel_params* kp, const double* X1, int64_t m, const double* X2, int64_t n,
                    double* A);
/* the same on device buffers (d_A: m n or 2 m n doubles); returns after the stream's work */
int hss_kernel_eval_device(const hss_kernel_params* kp, const double* d_X1, int64_t m, const double* d_X2, int64_t n,
                           double* d_A, void* stream);

/* Duan-Rokhlin corrections of the punctured trapezoidal rule for H0(k |x|) on the grid
 * h Z^2, host computation (the corr0 and corr1 lines of Common/FORTRAN_get_DR_weights.f,
 * corr_hank :85-): corr = {Re corr0, Im corr0, Re corr1, Im corr1}.  |k| h < 2 pi. */
int hss_dr_corrections(double h, double k_re, double k_im, double* corr);
/* [J, dr_weights, iistencil] = DR_stencil(h, rk, n, order) (Common/DR_stencil.m:1-53) for
 * order 0, 4 and 6 (8 and 10 need corr2..corr5: HSS_ERR_ARG).  *count entries (<= 5):
 * J[e] (offset i2 + n i1), w[2e], w[2e+1] (complex weight), stencil[3e..3e+2] (the
 * column of iistencil). */
int hss_dr_stencil(double h, double k_re, double k_im, int64_t n, int32_t order, int32_t* count, int64_t* J,
                   double* w, int32_t* stencil);

const char* hss_last_error(void);
int hss_version(void);
/* number of CUDA devices visible (0 on a machine without GPU) */
int hss_device_count(int* count);

/* ---- HSS1D (curves) ---------------------------------------------------- */
typedef struct hss1d_matrix hss1d_matrix;

/* K_HSS = HSS1D_compress_nsym('green', X, TREE, acc, knl_params)
 *   HSS1D/HSS1D_compress_nsym.m:1 (tree :277-334, skeletons :84-216,
 *   self/sibling blocks :220-271).
 * X: N x 6 column-major [x y nx ny w kappa] (ldx >= N); leaf = nbox_max.
 * seed: key of the counter RNG drawing the rank-check vectors (ID.m:68-86).
 * HSS_SL_H_2D (also in hss1d_compress_batch): the complex Helmholtz matrix, with the proxy
 *   ring of min(max(50, round(4 kh 1.75 R + 30)), N) points (:111-114) and complex IDs; its
 *   vectors are N x nrhs complex, interleaved (re, im) doubles (2 N doubles per column), and
 *   hss1d_info / hss1d_export_box report points and complex T (hss1d_is_complex); with
 *   hss1d_compress_fsym the matrix is taken as complex symmetric (K.' = K, plain transposes).
 *   Not with the rank predictor or the double-float ID; hss1d_transpose, hss1d_sum,
 *   hss1d_dense_matrix and the submatrix applies reject complex handles. */
int hss1d_compress(hss1d_matrix** out, const double* X, int64_t N, int64_t ldx, int32_t leaf,
                   double acc, const hss_kernel_params* kp, uint64_t seed);
/* K_HSS = HSS1D_compress_fsym('green', X, TREE, acc, knl_params), HSS1D/HSS1D_compress_fsym.m:98-248:
 * one ID per box (incoming skeletons = outgoing, T_DN = T_UP) and M_SIB{c2} = M_SIB{c1}.'.
 * hss1d_invert / hss1d_apply / hss1d_applyinv then act as HSS1D_invert_fsym (with its E fix at
 * :79), HSS1D_apply_fsym and HSS1D_applyinv_fsym. */
int hss1d_compress_fsym(hss1d_matrix** out, const double* X, int64_t N, int64_t ldx, int32_t leaf,
                        double acc, const hss_kernel_params* kp, uint64_t seed);
/* Batched HSS1D: nprob independent curves of uneven N compressed as one forest, every level of
 * every tree in the same launches.  X[p] is N[p] x 6 column-major (ld ldx[p]); seeds[p] keys
 * the rank-check stream of problem p (NULL: all 0).  No reference counterpart for the batching
 * itself: each tree is HSS1D_compress_nsym (HSS1D/HSS1D_compress_nsym.m:1).  Vectors passed to
 * the apply calls are the problems' vectors stacked (sum of N rows). */
int hss1d_compress_batch(hss1d_matrix** out, int32_t nprob, const int64_t* N, const double* const* X,
                         const int64_t* ldx, int32_t leaf, double acc, const hss_kernel_params* kp,
                         const uint64_t* seeds);
/* problems of a forest: count, total points, root box and first stacked row of each (NULL ok) */
int hss1d_forest_info(const hss1d_matrix* H, int32_t* nprob, int64_t* Ntot, int32_t* root, int64_t* pbase);
/* 1 when the handle holds a complex (HSS_SL_H_2D) matrix, else 0 */
int hss1d_is_complex(const hss1d_matrix* H, int32_t* is_complex);
/* tree and skeleton sizes over the forest's global box ids: arrays of nboxes entries (NULL ok);
 * off is the global (stacked) first point of a box */
int hss1d_info(const hss1d_matrix* H, int32_t* nboxes, int32_t* level, int32_t* parent,
               int32_t* c1, int32_t* c2, int32_t* off, int32_t* cnt, int32_t* nskel,
               int32_t* kskel);
/* K_HSS{I_SKUP,I_SKDN,J_UP,J_DN,T_UP,T_DN} of one box (box_constants.m:33-52);
 * T_* are k x (n-k) column-major (complex handles: interleaved (re, im), 2 k (n-k) doubles);
 * any pointer may be NULL. */
int hss1d_export_box(const hss1d_matrix* H, int32_t box, int32_t* I_skup, int32_t* I_skdn,
                     int32_t* J_up, int32_t* J_dn, double* T_up, double* T_dn);
/* K_HSS = HSS1D_compress_rectangular_nsym('green', Xin, Xout, TREE, acc, params)
 *   HSS1D/HSS1D_compress_rectangular_nsym.m:1 (trees :70-88 with LOCAL_get_tree_in :325-356,
 *   neighbour lists :397-462, skeletons :112-236, self/sibling blocks :238-266): the M x N
 *   matrix K(Xin, Xout).  Xin: M x 6 and Xout: N x 6 column-major [x y nx ny w kappa].  The
 *   columns follow the halving tree over Xout (leaf = nbox_max), the rows a tree of the same
 *   shape over Xin (each of its boxes must keep at least one point).  Outgoing and incoming
 *   ranks are independent.  hss1d_apply then computes uu (M x nrhs) = K qq (qq: N x nrhs),
 *   HSS1D/HSS1D_apply_rect_nsym.m:1; hss1d_info gives the column tree, hss1d_rect_info the
 *   row side, and hss1d_export_box returns I_SKDN as row indices into Xin.  invert,
 *   applyinv, solve, transforminv, transpose, dense_matrix and apply_submatrix return
 *   HSS_ERR_ARG on such a handle. */
int hss1d_compress_rect(hss1d_matrix** out, const double* Xin, int64_t M, int64_t ldin, const double* Xout,
                        int64_t N, int64_t ldout, int32_t leaf, double acc, const hss_kernel_params* kp,
                        uint64_t seed);
/* row side of a handle (K_HSS rows 16:19): M, and per box the first row and row count in
 * Xin and the incoming skeleton sizes (a square handle reports its column side) */
int hss1d_rect_info(const hss1d_matrix* H, int64_t* M, int32_t* off_in, int32_t* cnt_in, int32_t* nskel_in,
                    int32_t* kskel_in);
/* C_HSS = HSS1D_sum_nsym(A_HSS, B_HSS, acc), HSS1D/HSS1D_sum_nsym.m:1: a new handle holding
 * A + B, for two square handles on one tree (the same curves, leaf size and forest).  Each
 * box re-skeletonizes the stacked bases of A and B by the ID at tolerance acc (rank raised
 * to max(k_out, k_in) as in the compress); sibling blocks are projected, self blocks added.
 * The result is an ordinary handle (invert, apply, solve ...); fsym operands are accepted
 * and give an nsym result. */
int hss1d_sum(const hss1d_matrix* A, const hss1d_matrix* B, double acc, hss1d_matrix** C);
/* A_NEW = HSS1D_recompress_nsym(A, acc) (HSS1D/HSS1D_recompress_nsym.m:1): a new handle
 *   holding A with its ranks reduced to what acc needs (after sums and low-rank updates):
 *   top down, SVD truncation (absolute acc) of the sons' sibling blocks stacked with their
 *   parent's far-field factors (:30-146, one-sided Jacobi SVDs on the GPU); bottom up, the
 *   full-rank ID of each box's reduced bases (:148-246).  Real square handles; not inverted. */
int hss1d_recompress(const hss1d_matrix* A, double acc, hss1d_matrix** out);
/* K_HSS = HSS1D_compressLR_nsym(U, V, TREE, acc), HSS1D/HSS1D_compressLR_nsym.m:1: the N x N
 * matrix U V^T (U, V: N x r column-major, ld ldu / ldv) on the halving tree with leaf size
 * `leaf`; every box IDs V(out,:).' and U(in,:).' at tolerance acc (seed keys the rank check).
 * With hss1d_sum this forms low-rank updates of a compressed matrix. */
int hss1d_compress_lr(hss1d_matrix** out, const double* U, const double* V, int64_t N, int32_t r, int64_t ldu,
                      int64_t ldv, int32_t leaf, double acc, uint64_t seed);
/* [HSSinv, FTinv] = HSS1D_invert_nsym(K_HSS, acc), HSS1D/HSS1D_invert_nsym.m:44-91 */
int hss1d_invert(hss1d_matrix* H);
/* Kinv_HSS = HSS1D_transforminv_nsym(K_HSS, HSSinv, FTinv),
 * HSS1D/HSS1D_transforminv_nsym.m:38-161: a new handle holding the inverse in compressed
 * format (same tree and skeleton sets, J_UP/J_DN swapped), so hss1d_apply on *out applies
 * the inverse.  H must be inverted. */
int hss1d_transforminv(hss1d_matrix* H, hss1d_matrix** out);
/* uu = HSS1D_apply_nsym(K_HSS, qq), HSS1D/HSS1D_apply_nsym.m:38-100 */
int hss1d_apply(hss1d_matrix* H, const double* qq, double* uu, int32_t nrhs);
/* xx = HSS1D_applyinv_nsym(K_HSS, HSSinv, FTinv, ff), HSS1D/HSS1D_applyinv_nsym.m:43-86 */
int hss1d_applyinv(hss1d_matrix* H, const double* ff, double* xx, int32_t nrhs);
int hss1d_applyinv_device(hss1d_matrix* H, const double* d_ff, double* d_xx, int32_t nrhs,
                          void* stream);
/* inverse apply with iterative refinement against the FP64 HSS1D forward operator
 * (Common/Iterative_Refinement.m:20-35); relres = final max column ||f - A x|| / ||f|| over the
 * (stacked) vectors, iters = inverse applies used (either may be NULL) */
int hss1d_solve(hss1d_matrix* H, const double* f, double* x, int32_t nrhs, double tol, int32_t maxit,
                double* relres, int32_t* iters);
int hss1d_solve_device(hss1d_matrix* H, const double* d_f, double* d_x, int32_t nrhs, double tol,
                       int32_t maxit, double* relres, int32_t* iters, void* stream);
/* the same residual against the kernel matrix of each curve of the handle (block diagonal over
 * a forest; stacked vectors); handles from hss1d_compress* only (HSS_ERR_ARG otherwise) */
int hss1d_kernel_residual(hss1d_matrix* H, const double* f, const double* x, int32_t nrhs, double* relres);
/* At_HSS = HSS1D_transpose(A_HSS) (HSS1D/HSS1D_transpose.m:1): a new handle holding the
 * transpose in compressed form (up/down skeletons and T swapped, M_SELF transposed, sibling
 * blocks swapped and transposed); not inverted. */
int hss1d_transpose(const hss1d_matrix* A, hss1d_matrix** At);
/* A = HSS1D_scalarmult(c, A) (HSS1D/HSS1D_scalarmult.m:1), in place: M_SELF and M_SIB are
 * scaled by c; the handle's inverse is dropped (invert again before applyinv). */
int hss1d_scalarmult(hss1d_matrix* A, double c);
/* Kd = HSS1D_dense_matrix(K_HSS) (HSS1D/HSS1D_dense_matrix.m:1) for problem prob of the
 * handle: N_p x N_p column-major host array (N_p from hss1d_forest_info). */
int hss1d_dense_matrix(hss1d_matrix* A, int32_t prob, double* Kd);
/* uu = HSS1D_apply_submatrix_nsym(K_HSS, Box_dn, Box_up, I_dn, I_up, qq)
 * (HSS1D/HSS1D_apply_submatrix_nsym.m:1, _fsym likewise): uu = K(I_dn, I_up) qq(I_up).
 * I_dn, I_up: N flags (0/1) over the handle's (stacked) points; qq: N x nrhs; uu:
 * (count of I_dn) x nrhs, column-major.  The box masks are not needed here. */
int hss1d_apply_submatrix(hss1d_matrix* K, const uint8_t* I_dn, const uint8_t* I_up, const double* qq, int32_t nrhs,
                          double* uu);
/* [Box_dn, Box_up] = HSS1D_apply_submatrix_boxes(TREE, I_dn, I_up)
 * (HSS1D/HSS1D_apply_submatrix_boxes.m:1): per box (hss1d_info numbering), 1 if it holds
 * rows (Box_dn) / columns (Box_up) of the submatrix. */
int hss1d_apply_submatrix_boxes(const hss1d_matrix* K, const uint8_t* I_dn, const uint8_t* I_up, uint8_t* Box_dn,
                                uint8_t* Box_up);
/* arithmetic of the solve products: HSS_PREC_FP64 (default), HSS_PREC_DFLOAT (float-pair
 * copies of the FP64 operators, products on the FP32 pipes, ~2^-48 per product) or
 * HSS_PREC_DFLOAT_INV (also the following hss1d_invert's updates and products) */
int hss1d_set_precision(hss1d_matrix* H, int32_t precision);
int hss1d_destroy(hss1d_matrix* H);

/* ---- learned ranks (HSS1D) ---------------------------------------------- */
/* A small MLP (nin -> 32 -> 32 -> 1, ReLU, sigmoid) predicting the ID rank fraction k/n of a
 * box from features known before its ID.  It replaces the reference's hand-fitted rank table
 * (HSS2D/predict_rank.m:5-23): the learned compress below uses the prediction only to stop
 * the pivoted QR early, so ranks, skeletons and T equal those of the plain compress; a box
 * whose rank check reaches past the truncated factorization is redone in full.
 * Parameters: one float32 vector [W1 (32 x nin row-major), b1, W2 (32 x 32), b2, W3, b3]. */
typedef struct hss_mlp hss_mlp;
int hss_mlp_create(hss_mlp** out, int32_t nin, int32_t hidden, uint64_t seed);
int hss_mlp_nparams(const hss_mlp* M, int32_t* nparams);
int hss_mlp_get_params(const hss_mlp* M, float* params);
int hss_mlp_set_params(hss_mlp* M, const float* params);
/* gradient of 0.5*mean((y - t)^2) over B samples (X: B x nin row-major, host buffers);
 * grad: nparams floats (NULL ok); loss may be NULL */
int hss_mlp_grad(hss_mlp* M, const float* X, const float* t, int32_t B, float* grad, float* loss);
/* Adam (lr, 0.9, 0.999, 1e-8) over `epochs` passes of minibatches of `batch` samples in order;
 * loss = final full-batch loss (NULL ok) */
int hss_mlp_train(hss_mlp* M, const float* X, const float* t, int32_t B, int32_t epochs,
                  int32_t batch, float lr, float* loss);
int hss_mlp_predict(hss_mlp* M, const float* X, int32_t B, float* y);
int hss_mlp_destroy(hss_mlp* M);
/* per-box rank features of the last compress (nboxes x 8 row-major floats; roots are 0):
 * log2 n, -log10(acc)/10, log2(1+near in-skeletons), log2(1+near out-skeletons),
 * radius / arc length, max|curvature| * radius, level / 16, kernel flag.
 * rank_frac[b] = k/n of the box's plain ID (NULL ok). */
int hss1d_features(const hss1d_matrix* H, float* feat, float* rank_frac);
/* QR steps done by the last compress, steps a full factorization takes, boxes redone in full */
int hss1d_id_stats(const hss1d_matrix* H, int64_t* qr_steps, int64_t* qr_steps_full,
                   int32_t* reruns);
/* host wall seconds of the last compress by phase (6 entries): setup (trees, neighbour lists,
 * point upload), per-level geometry, per-level uploads and launches, per-level GPU work up to
 * its sync, per-level bookkeeping, final blocks (the reference's tic/toc reports) */
int hss1d_phase_times(const hss1d_matrix* H, double* seconds);
/* hss1d_compress_batch with a rank predictor (M: 8 inputs) bounding each ID's QR steps */
int hss1d_compress_batch_learned(hss1d_matrix** out, int32_t nprob, const int64_t* N,
                                 const double* const* X, const int64_t* ldx, int32_t leaf,
                                 double acc, const hss_kernel_params* kp, const uint64_t* seeds,
                                 hss_mlp* M);
/* hss1d_compress_batch with options: M (NULL or a rank predictor as in
 * hss1d_compress_batch_learned) and the arithmetic of the IDs' pivoted QR: HSS_PREC_FP64
 * (the reference's ID, exact-rank parity) or HSS_PREC_DFLOAT (double-float QR on the FP32
 * pipes, ~2^-48 per operation; rank, T and the randomized check stay FP64).
 * id_precision | HSS_ID_STEP_TEST (M NULL): the model-free baseline of the learned mode,
 * every pivoted QR testing the same stop rule at every step. */
#define HSS_ID_STEP_TEST 256
int hss1d_compress_batch_ex(hss1d_matrix** out, int32_t nprob, const int64_t* N, const double* const* X,
                            const int64_t* ldx, int32_t leaf, double acc, const hss_kernel_params* kp,
                            const uint64_t* seeds, hss_mlp* M, int32_t id_precision);

/* ---- HSS2D (planar volumes) -------------------------------------------- */
typedef struct hss2d_matrix hss2d_matrix;

/* the params fields of Common/HSS_tree_parameters.m:108-139 the dense path uses */
typedef struct hss2d_params {
  int32_t Ng;        /* points per panel side */
  int32_t npan;      /* panels per domain side (power of two) */
  int32_t layers;    /* boundary layers of the preset skeletons */
  int32_t interform; /* HSS_INTER_DENSE or HSS_INTER_LOWRANK (the reference default) */
  int32_t transinv;  /* 0: NTI (per-box operators) */
  int32_t sym;       /* 0: nsym */
  int32_t precision; /* HSS_PREC_FP64, HSS_PREC_MIXED, HSS_PREC_DFLOAT or HSS_PREC_DFLOAT_INV */
  int32_t pad_;
  double acc;
  hss_kernel_params kp;
  int32_t k_cut;     /* low-rank T only where k < k_cut (0: 2500) */
  int32_t pad2_;
  uint64_t seed;     /* key of the randomized ID's Gaussian samples */
  int32_t proxy_rule; /* HSS_PROXY_BDRY, HSS_PROXY_RAND or HSS_PROXY_WDEC (params.proxy_rule) */
  int32_t pad3_;
  double lambda;      /* params.lambda of the 'rand' rules (0: 2) */
  int32_t skel_rule;  /* HSS_SKEL_BDRY, HSS_SKEL_RAND, HSS_SKEL_ID or HSS_SKEL_WDEC (params.skel_rule) */
  int32_t pad4_;
} hss2d_params;

/* INFO_TREE = HSS2D_build_tree_nsym(params), HSS2D/HSS2D_build_tree_nsym.m:80-610
 * ('uniform' tree, 'bdry' preset skeletons, 'bdry' or 'rand' proxies, dense T).
 * HSS_SL_H_2D (kh > 0, the Lippmann-Schwinger operator): the skeletons of the two finest
 * levels come from the interpolative decomposition of K(proxies, box) (:399-412, :614-657),
 * every box of such a level at the level's largest rank (boxes below it take the fixed-rank
 * ID's next pivots), T_dn = T_up = the ID's T; complex arithmetic runs as the real 2 x 2
 * embedding [[Re, -Im], [Im, Re]] of every block.  Vectors of a complex tree are N complex
 * entries per column, interleaved (re, im); hss2d_info reports N complex rows.
 * Dense T only (HSS_INTER_DENSE), transinv 0. */
int hss2d_build_tree(hss2d_matrix** out, const hss2d_params* p);
/* A_HSS = HSS2D_compress_nsym(INFO_TREE, params) dense blocks, HSS2D/HSS2D_compress_nsym.m:67-125 */
int hss2d_compress(hss2d_matrix* H);
/* A_HSS = HSS2D_invert_nsym(INFO_TREE, params), Fopts = 'dense',
 * HSS2D/HSS2D_invert_nsym.m:70-155 with HSS2D_build_Finv_nsym.m:92-100 and
 * HSS2D_build_E_nsym.m:43-51 */
int hss2d_invert(hss2d_matrix* H);
/* Y = HSS2D_apply_nsym(INFO_TREE, A_HSS, X, params), HSS2D/HSS2D_apply_nsym.m:74-218 */
int hss2d_apply(hss2d_matrix* H, const double* X, double* Y, int32_t nrhs);
int hss2d_apply_device(hss2d_matrix* H, const double* d_X, double* d_Y, int32_t nrhs, void* stream);
/* Y = HSS2D_applyinv_nsym(INFO_TREE, A_HSS, X, params), HSS2D/HSS2D_applyinv_nsym.m:74-243 */
int hss2d_applyinv(hss2d_matrix* H, const double* X, double* Y, int32_t nrhs);
int hss2d_applyinv_device(hss2d_matrix* H, const double* d_X, double* d_Y, int32_t nrhs,
                          void* stream);
/* solve with iterative refinement (Common/Iterative_Refinement.m:20-35): x = A^-1 f,
 * then x += A^-1 (f - A x) until max_col ||f - A x||/||f|| <= tol or maxit solves.
 * A is the FP64 forward HSS operator, as the reference test uses it
 * (HSS2D/Test/Test_HSS2D_InverseCompression.m:281-298).  relres (may be NULL)
 * receives the final max column relative residual, iters the solves used. */
int hss2d_solve(hss2d_matrix* H, const double* f, double* x, int32_t nrhs, double tol,
                int32_t maxit, double* relres, int32_t* iters);
int hss2d_solve_device(hss2d_matrix* H, const double* d_f, double* d_x, int32_t nrhs, double tol,
                       int32_t maxit, double* relres, int32_t* iters, void* stream);
/* relres = max over columns of ||f - K x|| / ||f|| with K the kernel matrix itself
 * (Kernel_Eval over the grid, never formed: each entry is generated in FP64 and applied on
 * the fly).  The reference measures this residual against the dense matrix
 * (HSS2D/Test/Test_HSS2D_InverseCompression.m:300-324; Common/Iterative_Refinement.m:20-35
 * forms f - A x); hss2d_solve's relres is against the compressed operator.  f, x: host
 * N x nrhs column-major.  O(N^2) work per column. */
int hss2d_kernel_residual(hss2d_matrix* H, const double* f, const double* x, int32_t nrhs, double* relres);
/* tree sizes: depth, box count, N */
/* on != 0: when a solve plan is built (first apply / inverse apply per column count), time
 * every batched product at K-split counts around the built-in heuristic's and keep the
 * fastest (2% hysteresis).  Solves then replay the tuned plan; results are reproducible
 * within a plan but may differ in the last bits between tuned and untuned plans.  No
 * reference counterpart (a GPU launch-shape choice). */
int hss2d_set_autotune(hss2d_matrix* H, int32_t on);
/* [x,flag,relres,iter] = bicgstab(Mapp, f, tol, maxit, Iapp) of the reference's iterative
 * solution (HSS2D/Test/Test_HSS2D_InverseCompression.m:201-228): Mapp = forward apply of
 * the compressed operator A, Iapp = inverse apply of the inverted handle M (e.g. a
 * translation-invariant tree of the constant-coefficient kernel); M may be NULL.
 * f, x host N x nrhs column-major; relres = max column true residual; iters = iterations. */
int hss2d_bicgstab(hss2d_matrix* A, hss2d_matrix* M, const double* f, double* x, int32_t nrhs,
                   double tol, int32_t maxit, double* relres, int32_t* iters);
/* x = A^-1 f by restarted GMRES(restart) with right preconditioner M^-1 (the inverse apply
 * of the inverted handle M, e.g. A itself in HSS_PREC_MIXED: the FP32 "complex64" inverse),
 * A the FP64 forward operator; complex for HSS_SL_H_2D trees (complex128 arithmetic,
 * interleaved vectors).  Each column iterates on its own Krylov space until its relative
 * residual ||f - A x|| / ||f|| <= tol; all columns share the operator applies.  f, x host
 * N x nrhs; relres = max column residual of the returned x; iters = Arnoldi steps.
 * The reference's Krylov use: HSS2D/Test/Test_HSS2D_InverseCompression.m:201-228. */
int hss2d_gmres(hss2d_matrix* A, hss2d_matrix* M, const double* f, double* x, int32_t nrhs, double tol,
                int32_t restart, int32_t maxit, double* relres, int32_t* iters);
/* relres = max over columns of ||f - K x|| / ||f|| over the target rows [row0, row0 + nrows)
 * only (complex rows for a complex tree): the kernel-matrix residual on a row sample when
 * the full O(N^2) product is too long.  f: those rows of the right-hand sides (nrows x nrhs),
 * x: the full solution (N x nrhs). */
int hss2d_kernel_residual_rows(hss2d_matrix* H, int64_t row0, int64_t nrows, const double* f, const double* x,
                               int32_t nrhs, double* relres);
/* LOCAL_Build_Proxy of one box (host computation, HSS2D_build_tree_nsym.m:870-961): the
 * proxy points of box `box` (heap numbering, 0-based) on level lev of the tree p describes,
 * for a box of n_src sources; rule and lambda from p.  xy receives x then y columns
 * (2 cap doubles), *count the number of points (HSS_ERR_ARG if above cap). */
int hss2d_proxy_points(const hss2d_params* p, int32_t box, int32_t n_src, double* xy, int32_t cap,
                       int32_t* count);
int hss2d_info(const hss2d_matrix* H, int32_t* depth, int32_t* nboxes, int64_t* N);
/* 1 when the tree holds a complex (HSS_SL_H_2D) matrix, else 0 */
int hss2d_is_complex(const hss2d_matrix* H, int32_t* is_complex);
/* per-box sizes: n (|I_src|), k (|I_sk|), proxy count; arrays of nboxes (NULL ok) */
int hss2d_box_sizes(const hss2d_matrix* H, int32_t* n, int32_t* k, int32_t* nproxy);
/* INFO_TREE.BOX(b).{I_src, J, T_up, T_dn} (T_* k x (n-k) column-major); NULL ok */
int hss2d_export_box(const hss2d_matrix* H, int32_t box, int32_t* I_src, int32_t* J,
                     double* T_up, double* T_dn);
/* A_HSS(b).FI (n x n) and .E (k x k), FP64 copies; NULL ok */
int hss2d_export_inverse(const hss2d_matrix* H, int32_t box, double* FI, double* E);
/* host wall seconds of the last build/compress/invert by phase (5 entries): tree geometry,
 * point and index uploads, interpolation operators, compress, invert */
int hss2d_phase_times(const hss2d_matrix* H, double* seconds);
/* ranks of the low-rank interpolation operators T_up = T.U T.V^T and T_dn per box
 * (nboxes entries each; -1 where T is dense: the root, the two finest levels, k >= k_cut) */
int hss2d_interp_ranks(const hss2d_matrix* H, int32_t* q_up, int32_t* q_dn);
/* bytes of factor storage read by one inverse apply (roofline accounting) */
int hss2d_solve_bytes(const hss2d_matrix* H, int64_t* bytes);
/* kernels launched by one solve of nrhs columns with one residual check: the inverse
 * apply, the forward apply and the residual (counted by the host from the cached plans) */
int hss2d_solve_launches(const hss2d_matrix* H, int32_t nrhs, int32_t* launches);
int hss2d_destroy(hss2d_matrix* H);

/* ---- batched dense primitives (exposed for parity tests and benches) ---- */
/* In-place inversion of `batch` n x n column-major matrices stored back to back
 * (device pointer), blocked Gauss-Jordan with partial pivoting; info[b] = 0 ok. */
int hss_batched_inverse_device(double* d_A, int32_t n, int32_t batch, int32_t* d_info,
                               void* stream);
int hss_batched_inverse_device_f32(float* d_A, int32_t n, int32_t batch, int32_t* d_info,
                                   void* stream);
/* Same inversion without any device allocation, for callers that cannot call
 * cudaMalloc/cudaFree while running (device memory owned by their own pool
 * allocator, or latency-bound loops where allocation would synchronise the
 * device).  No counterpart in the reference (MATLAB allocates freely).  All
 * scratch comes from one fixed 16 MiB array in device global memory (held by
 * every GPU that loads the library): batch <= 256 and
 * batch*(n*n + 64*n)*8 + batch*(n + 132)*4 bytes plus descriptors must fit, else
 * HSS_ERR_ARG.  The first call on a device resolves the array's address there
 * (make it before any stream capture); a cudaDeviceReset invalidates that address.
 * Calls share the array: overlapping calls on the GPU race and must be ordered
 * by the caller.  d_info is cleared by each call. */
int hss_batched_inverse_noalloc_device(double* d_A, int32_t n, int32_t batch, int32_t* d_info,
                                       void* stream);
/* Least squares X_b = A_b(:,0:kf) \ A_b(:,kf:n) for `batch` m x n blocks back to
 * back (device); X overwrites A_b(0:kf, kf:n). */
int hss_batched_lstsq_device(double* d_A, int32_t m, int32_t n, int32_t kf, int32_t batch,
                             void* stream);
/* hss_batched_lstsq_device with the arithmetic chosen: HSS_PREC_FP64 (as
 * hss_batched_lstsq_device) or HSS_PREC_DFLOAT (the Householder panels, the compact-WY
 * trailing updates and the back substitution in paired FP32, ~2^-48 relative; the least
 * squares of the interpolation operators, T = K(Xp,X_sk) \ K(Xp,X_rs), in the tree's
 * double-float and mixed modes).  Any other precision: HSS_ERR_ARG. */
int hss_batched_lstsq_device_ex(double* d_A, int32_t m, int32_t n, int32_t kf, int32_t batch,
                                int32_t precision, void* stream);
/* Interpolative decomposition of `batch` m x n blocks (device, back to back):
 * rank[b], perm[b*n..], T[b*n*n..] (k x (n-k), ld n).  force_k < 0: adaptive
 * (ID.m:40-65), else fixed rank (ID.m:106-113). */
int hss_batched_id_device(const double* d_A, int32_t m, int32_t n, int32_t batch, double acc,
                          uint64_t seed, int32_t force_k, int32_t* d_rank, int32_t* d_perm,
                          double* d_T, void* stream);
/* C = A*B for `batch` column-major blocks back to back (device), FP64. */
int hss_batched_gemm_device(const double* d_A, const double* d_B, double* d_C, int32_t M,
                            int32_t N, int32_t K, int32_t batch, void* stream);
/* C = A*B for `batch` column-major blocks back to back (device, FP64 in and out, N <= 4
 * columns) on the tensor cores: each A is cut into 6 bf16 fixed-point digit slices per row,
 * B likewise per column, and the exact digit products are summed in integers (error
 * ~2^-47 of max_k |A(i,k)| * max_k |B(k,j)| per term).  The skinny products of the inverse
 * apply of HSS2D_applyinv_nsym (HSS2D/HSS2D_applyinv_nsym.m:74-243, HSS2D_applyFinv_nsym.m:30-31)
 * in the HSS_PREC_TC mode run on this kernel. */
int hss_batched_gemv_tc_device(const double* d_A, const double* d_B, double* d_C, int32_t M,
                               int32_t N, int32_t K, int32_t batch, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HSSGPU_H */
