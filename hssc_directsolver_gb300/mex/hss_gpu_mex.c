/*
 * hss_gpu_mex.c -- MATLAB MEX binding of libhssgpu.so (the C ABI in include/hssgpu.h).
 *
 * Build next to the reference's .m files:
 *   mex -R2018a hss_gpu_mex.c -I<repo>/include -L<repo>/hssc_directsolver_gb300 -lhssgpu
 *
 * Every operation takes and returns the reference's own MATLAB data structures, so the
 * reference scripts keep their call sites (a one-line wrapper per function forwards to
 * this MEX file):
 *
 *   INFO_TREE = hss_gpu_mex('HSS2D_build_tree_nsym', params)
 *       params: the struct of Common/HSS_tree_parameters.m:108-175 (Ng, flag_pot, kh, acc,
 *       layers, h, INTERform, transinv, sym, k_cut, X_source; np follows from X_source).
 *       Optional GPU fields: precision ('fp64' | 'mixed' | 'dfloat' | 'dfloat_inv' | 'tc'),
 *       seed, and b_alpha/b_x0/b_y0/b_isig, c_alpha/c_x0/c_y0/c_isig to set b(x), c(y)
 *       (the custom-kernel slot of Common/Kernel_Eval.m:75-79; otherwise LOCAL_get_bc's
 *       choice, Kernel_Eval.m:111-159).
 *       INFO_TREE: the fields of HSS2D/HSS2D_build_tree_nsym.m:600-609 (numlev, depth,
 *       leaves, box_numbers) and BOX(b).{I_src, J, k, n_skel, levbox, parent, child,
 *       T_up, T_dn} (T_* as .U / .V with V = I for dense interpolation operators, indices
 *       1-based), plus .gpu, the device handle.
 *   A_HSS = hss_gpu_mex('HSS2D_compress_nsym', INFO_TREE, params)
 *   A_HSS = hss_gpu_mex('HSS2D_invert_nsym', INFO_TREE, params)
 *       A_HSS(b).{FI, E} (HSS2D/HSS2D_invert_nsym.m:70-155), FP64 copies of the device factors.
 *   Y = hss_gpu_mex('HSS2D_apply_nsym', INFO_TREE, A_HSS, X, params)
 *   Y = hss_gpu_mex('HSS2D_applyinv_nsym', INFO_TREE, A_HSS, X, params)
 *   [X, relres, iters] = hss_gpu_mex('Iterative_Refinement', INFO_TREE, B, acc, maxit)
 *   hss_gpu_mex('HSS2D_destroy', INFO_TREE)
 *
 *   K_HSS = hss_gpu_mex('HSS1D_compress_nsym', 'green', X, TREE, acc, knl_params)
 *       X: N x 6 [x y nx ny w kappa]; knl_params.flag_pot 'DL_L_2D' (the custom double layer)
 *       or 'SL_L_2D'.  K_HSS: cell(50, nboxes) with the rows of Common/box_constants.m:33-52
 *       (LEVEL, PARENT, C1, C2, END1, END2, NSKEL, KSKEL, I_SKUP, I_SKDN, T_UP, J_UP, T_DN,
 *       J_DN; 1-based) and the device handle in K_HSS{50, 1}.
 *   [HSSinv, FTinv] = hss_gpu_mex('HSS1D_invert_nsym', K_HSS, acc)
 *       the inverse stays on the device: HSSinv is the handle, FTinv is [].
 *   uu = hss_gpu_mex('HSS1D_apply_nsym', K_HSS, qq)
 *   xx = hss_gpu_mex('HSS1D_applyinv_nsym', K_HSS, HSSinv, FTinv, ff)
 *   hss_gpu_mex('HSS1D_destroy', K_HSS)
 *
 *   A = hss_gpu_mex('Kernel_Eval', X1, X2, params)   (SL_L_2D, Common/Kernel_Eval.m:1-96)
 *
 * Errors: a non-zero status becomes mexErrMsgIdAndTxt("hss:gpu", ...) with
 * hss_last_error(), as MATLAB errors are the reference's failure mode.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "hssgpu.h"
#include "mex.h"

#define BOX_ROWS 50
#define BOX_LEVEL 2
#define BOX_PARENT 3
#define BOX_C1 4
#define BOX_C2 5
#define BOX_END1 6
#define BOX_END2 7
#define BOX_NSKEL 8
#define BOX_KSKEL 9
#define BOX_I_SKUP 20
#define BOX_I_SKDN 22
#define BOX_T_UP 30
#define BOX_J_UP 31
#define BOX_T_DN 32
#define BOX_J_DN 33
#define BOX_GPU 50

static void check(int st) {
  if (st != HSS_OK) mexErrMsgIdAndTxt("hss:gpu", "%s (status %d)", hss_last_error(), st);
}

static void* xmalloc(size_t n) {
  void* p = malloc(n ? n : 1);
  if (!p) mexErrMsgIdAndTxt("hss:gpu", "host allocation of %zu bytes failed", n);
  return p;
}

static mxArray* handle_out(void* h) {
  mxArray* a = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
  *(uint64_t*)mxGetData(a) = (uint64_t)(uintptr_t)h;
  return a;
}
static void* handle_in(const mxArray* a) {
  if (!a || mxGetClassID(a) != mxUINT64_CLASS) mexErrMsgIdAndTxt("hss:gpu", "expected a device handle");
  return (void*)(uintptr_t)(*(const uint64_t*)mxGetData(a));
}

static double field_or(const mxArray* s, const char* name, double dflt) {
  const mxArray* f = mxGetField(s, 0, name);
  return (f && mxGetNumberOfElements(f) > 0) ? mxGetScalar(f) : dflt;
}
static int field_str(const mxArray* s, const char* name, char* buf, size_t len) {
  const mxArray* f = mxGetField(s, 0, name);
  if (!f || !mxIsChar(f)) return 0;
  return mxGetString(f, buf, (mwSize)len) == 0;
}

/* 0-based int indices -> 1 x n double row (MATLAB's 1-based index vectors) */
static mxArray* index_row(const int32_t* v, int n) {
  mxArray* a = mxCreateDoubleMatrix(1, (mwSize)n, mxREAL);
  double* d = mxGetDoubles(a);
  for (int i = 0; i < n; ++i) d[i] = (double)v[i] + 1.0;
  return a;
}
static mxArray* scalar(double v) { return mxCreateDoubleScalar(v); }

/* ---- kernel parameters ---------------------------------------------------- */
static int flag_of(const mxArray* params) {
  char pot[32] = "SL_L_2D";
  field_str(params, "flag_pot", pot, sizeof pot);
  if (!strcmp(pot, "SL_L_2D")) return HSS_SL_L_2D;
  if (!strcmp(pot, "DL_L_2D")) return HSS_DL_L_2D;
  if (!strcmp(pot, "SL_H_2D")) return HSS_SL_H_2D;
  mexErrMsgIdAndTxt("hss:gpu", "flag_pot '%s' is not one of SL_L_2D, DL_L_2D, SL_H_2D", pot);
  return -1;
}

/* b(x), c(y): explicit fields (b_kind / c_kind: HSS_MOD_*), else the choice of LOCAL_get_bc
 * (Kernel_Eval.m:111-159) from params.sym, .transinv, .proxy (default 0) and .kh */
static void modulations(const mxArray* params, hss_kernel_params* kp) {
  const int sym = (int)field_or(params, "sym", 0), ti = (int)field_or(params, "transinv", 0);
  const int proxy = (int)field_or(params, "proxy", 0);
  if (mxGetField(params, 0, "b_alpha") || mxGetField(params, 0, "c_alpha") || mxGetField(params, 0, "b_kind") ||
      mxGetField(params, 0, "c_kind")) {
    kp->b_alpha = field_or(params, "b_alpha", 0.0);
    kp->b_x0 = field_or(params, "b_x0", 0.0);
    kp->b_y0 = field_or(params, "b_y0", 0.0);
    kp->b_isig = field_or(params, "b_isig", 1.0);
    kp->c_alpha = field_or(params, "c_alpha", 0.0);
    kp->c_x0 = field_or(params, "c_x0", 0.0);
    kp->c_y0 = field_or(params, "c_y0", 0.0);
    kp->c_isig = field_or(params, "c_isig", 1.0);
    kp->b_kind = (int32_t)field_or(params, "b_kind", HSS_MOD_GAUSS);
    kp->c_kind = (int32_t)field_or(params, "c_kind", HSS_MOD_GAUSS);
    return;
  }
  kp->b_isig = kp->c_isig = 1.0;
  if (sym == 0 && kp->kh > 0) {  /* nonsymmetric Lippmann-Schwinger (:113-125) */
    if (proxy <= 0) kp->b_kind = HSS_MOD_BUMP;
    return;
  }
  if (ti) return;
  if (kp->kh > 0) {  /* symmetric Lippmann-Schwinger (:129-140) */
    if (proxy <= 0) kp->b_kind = HSS_MOD_SQRT_BUMP;
    if (proxy >= 0) kp->c_kind = HSS_MOD_SQRT_BUMP;
    return;
  }
  if (proxy <= 0) {
    kp->b_alpha = 0.25;
    kp->b_x0 = 0.3;
    kp->b_y0 = 0.6;
  }
  if (proxy >= 0) {
    kp->c_alpha = 0.25;
    kp->c_x0 = sym ? 0.3 : 0.2;
    kp->c_y0 = sym ? 0.6 : -0.6;
  }
}

static void kernel_params(const mxArray* params, hss_kernel_params* kp) {
  memset(kp, 0, sizeof *kp);
  kp->flag = flag_of(params);
  kp->h = field_or(params, "h", 1.0);
  kp->kh = field_or(params, "kh", 0.0);
  if (kp->flag != HSS_DL_L_2D) modulations(params, kp);
  if (kp->flag == HSS_SL_H_2D) {  /* params.dr_weights: the complex diagonal weight */
    const mxArray* dr = mxGetField(params, 0, "dr_weights");
    if (dr && mxIsComplex(dr)) {
      kp->dr_re = mxGetComplexDoubles(dr)[0].real;
      kp->dr_im = mxGetComplexDoubles(dr)[0].imag;
    } else if (dr) {
      kp->dr_re = mxGetScalar(dr);
    }
  }
}

/* A double matrix's data in the library's layout: interleaved (re, im) pairs for a complex
 * handle (a real X is widened into *tmp), plain doubles otherwise */
static const double* vec_in(const mxArray* X, int cplx, mxArray** tmp) {
  if (!mxIsDouble(X)) mexErrMsgIdAndTxt("hss:gpu", "vectors must be double");
  if (!cplx) {
    if (mxIsComplex(X)) mexErrMsgIdAndTxt("hss:gpu", "a complex vector for a real matrix");
    return mxGetDoubles(X);
  }
  if (mxIsComplex(X)) return (const double*)mxGetComplexDoubles(X);
  const size_t n = mxGetNumberOfElements(X);
  *tmp = mxCreateDoubleMatrix(mxGetM(X), mxGetN(X), mxCOMPLEX);
  mxComplexDouble* d = mxGetComplexDoubles(*tmp);
  const double* s = mxGetDoubles(X);
  for (size_t i = 0; i < n; ++i) { d[i].real = s[i]; d[i].imag = 0.0; }
  return (const double*)d;
}

static mxArray* vec_out(mwSize m, mwSize n, int cplx, double** data) {
  mxArray* a = mxCreateDoubleMatrix(m, n, cplx ? mxCOMPLEX : mxREAL);
  *data = cplx ? (double*)mxGetComplexDoubles(a) : mxGetDoubles(a);
  return a;
}

static int tree_complex(hss2d_matrix* H) {
  int32_t c = 0;
  check(hss2d_is_complex(H, &c));
  return c;
}

static int khss_complex(hss1d_matrix* H) {
  int32_t c = 0;
  check(hss1d_is_complex(H, &c));
  return c;
}

static void hss2d_params_of(const mxArray* params, hss2d_params* p) {
  char buf[32];
  memset(p, 0, sizeof *p);
  if (!mxIsStruct(params)) mexErrMsgIdAndTxt("hss:gpu", "params must be the struct of HSS_tree_parameters");
  p->Ng = (int32_t)field_or(params, "Ng", 0);
  const mxArray* X = mxGetField(params, 0, "X_source");
  if (!X || p->Ng <= 0) mexErrMsgIdAndTxt("hss:gpu", "params needs Ng and X_source");
  const double np = sqrt((double)mxGetM(X)) / p->Ng;
  p->npan = (int32_t)lround(np);
  p->layers = (int32_t)field_or(params, "layers", 2);
  p->acc = field_or(params, "acc", 1e-10);
  p->transinv = (int32_t)field_or(params, "transinv", 0);
  p->sym = (int32_t)field_or(params, "sym", 0);
  p->k_cut = (int32_t)field_or(params, "k_cut", 2500);
  p->seed = (uint64_t)field_or(params, "seed", 0);
  p->interform = HSS_INTER_LOWRANK;
  if (field_str(params, "INTERform", buf, sizeof buf) && !strcmp(buf, "dense")) p->interform = HSS_INTER_DENSE;
  p->precision = HSS_PREC_FP64;
  if (field_str(params, "precision", buf, sizeof buf)) {
    if (!strcmp(buf, "mixed")) p->precision = HSS_PREC_MIXED;
    else if (!strcmp(buf, "dfloat")) p->precision = HSS_PREC_DFLOAT;
    else if (!strcmp(buf, "dfloat_inv")) p->precision = HSS_PREC_DFLOAT_INV;
    else if (!strcmp(buf, "tc")) p->precision = HSS_PREC_TC;
  }
  p->proxy_rule = HSS_PROXY_BDRY;
  if (field_str(params, "proxy_rule", buf, sizeof buf)) {
    if (!strcmp(buf, "rand")) p->proxy_rule = HSS_PROXY_RAND;
    else if (!strcmp(buf, "wdec")) p->proxy_rule = HSS_PROXY_WDEC;
  }
  p->skel_rule = HSS_SKEL_BDRY;
  if (field_str(params, "skel_rule", buf, sizeof buf)) {
    if (!strcmp(buf, "rand")) p->skel_rule = HSS_SKEL_RAND;
    else if (!strcmp(buf, "ID")) p->skel_rule = HSS_SKEL_ID;
    else if (!strcmp(buf, "wdec")) p->skel_rule = HSS_SKEL_WDEC;
  }
  p->lambda = field_or(params, "lambda", 2.0);
  kernel_params(params, &p->kp);
}

/* ---- HSS2D -------------------------------------------------------------- */
static hss2d_matrix* tree_handle(const mxArray* info) {
  if (!mxIsStruct(info)) mexErrMsgIdAndTxt("hss:gpu", "expected INFO_TREE");
  return (hss2d_matrix*)handle_in(mxGetField(info, 0, "gpu"));
}

static mxArray* identity(int n) {
  mxArray* a = mxCreateDoubleMatrix((mwSize)n, (mwSize)n, mxREAL);
  double* d = mxGetDoubles(a);
  for (int i = 0; i < n; ++i) d[i + (size_t)i * n] = 1.0;
  return a;
}

static mxArray* tstruct(mxArray* U, int nr) {
  const char* f[] = {"U", "V"};
  mxArray* t = mxCreateStructMatrix(1, 1, 2, f);
  mxSetField(t, 0, "U", U);
  mxSetField(t, 0, "V", identity(nr));
  return t;
}

static mxArray* info_tree(hss2d_matrix* H) {
  int32_t depth = 0, nb = 0;
  int64_t N = 0;
  check(hss2d_info(H, &depth, &nb, &N));
  int32_t* n = (int32_t*)xmalloc(sizeof(int32_t) * nb);
  int32_t* k = (int32_t*)xmalloc(sizeof(int32_t) * nb);
  int32_t* px = (int32_t*)xmalloc(sizeof(int32_t) * nb);
  check(hss2d_box_sizes(H, n, k, px));
  const char* bf[] = {"levbox", "parent", "child", "n_skel", "k", "I_src", "J", "T_up", "T_dn"};
  mxArray* box = mxCreateStructMatrix((mwSize)nb, 1, 9, bf);
  const int cx = tree_complex(H), w = cx ? 2 : 1;  /* complex trees export complex T */
  int32_t* isrc = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)N);
  int32_t* J = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)N);
  for (int b = 0; b < nb; ++b) {
    int lev = 0;
    while ((2 << lev) - 1 <= b) ++lev;  /* BFS numbering: level l holds boxes 2^l - 1 .. 2^(l+1) - 2 */
    const int nr = n[b] - k[b];
    double* Tu = (double*)xmalloc(sizeof(double) * w * (size_t)k[b] * (nr > 0 ? nr : 1));
    double* Td = (double*)xmalloc(sizeof(double) * w * (size_t)k[b] * (nr > 0 ? nr : 1));
    check(hss2d_export_box(H, b, isrc, J, b > 0 ? Tu : NULL, b > 0 ? Td : NULL));
    mxSetField(box, b, "levbox", scalar(lev));
    mxSetField(box, b, "parent", scalar(b > 0 ? (b - 1) / 2 + 1 : 0));
    mxArray* ch = mxCreateDoubleMatrix(1, 2, mxREAL);
    if (lev < depth) {
      mxGetDoubles(ch)[0] = 2 * b + 2;
      mxGetDoubles(ch)[1] = 2 * b + 3;
    }
    mxSetField(box, b, "child", ch);
    mxSetField(box, b, "n_skel", scalar(n[b]));
    mxSetField(box, b, "k", scalar(k[b]));
    mxSetField(box, b, "I_src", index_row(isrc, n[b]));
    mxSetField(box, b, "J", index_row(J, n[b]));
    if (b > 0 && nr > 0) {
      double* d = NULL;
      mxArray* U = vec_out((mwSize)k[b], (mwSize)nr, cx, &d);
      memcpy(d, Tu, sizeof(double) * w * (size_t)k[b] * nr);
      mxSetField(box, b, "T_up", tstruct(U, nr));
      U = vec_out((mwSize)k[b], (mwSize)nr, cx, &d);
      memcpy(d, Td, sizeof(double) * w * (size_t)k[b] * nr);
      mxSetField(box, b, "T_dn", tstruct(U, nr));
    }
    free(Tu);
    free(Td);
  }
  const char* tf[] = {"BOX", "numlev", "depth", "leaves", "box_numbers", "gpu"};
  mxArray* t = mxCreateStructMatrix(1, 1, 6, tf);
  mxSetField(t, 0, "BOX", box);
  mxSetField(t, 0, "numlev", scalar(depth + 1));
  mxSetField(t, 0, "depth", scalar(depth));
  const int nleaf = 1 << depth;
  mxArray* lv = mxCreateDoubleMatrix(1, (mwSize)nleaf, mxREAL);
  for (int i = 0; i < nleaf; ++i) mxGetDoubles(lv)[i] = nleaf + i;  /* boxes 2^d .. 2^(d+1)-1, 1-based */
  mxSetField(t, 0, "leaves", lv);
  mxArray* bn = mxCreateDoubleMatrix(1, (mwSize)nb, mxREAL);
  for (int i = 0; i < nb; ++i) mxGetDoubles(bn)[i] = i + 1;
  mxSetField(t, 0, "box_numbers", bn);
  mxSetField(t, 0, "gpu", handle_out(H));
  free(n);
  free(k);
  free(px);
  free(isrc);
  free(J);
  return t;
}

static mxArray* a_hss(hss2d_matrix* H, int inverted) {
  int32_t depth = 0, nb = 0;
  int64_t N = 0;
  check(hss2d_info(H, &depth, &nb, &N));
  const char* af[] = {"FI", "E", "gpu"};
  mxArray* a = mxCreateStructMatrix((mwSize)nb, 1, 3, af);
  mxSetField(a, 0, "gpu", handle_out(H));
  if (!inverted) return a;
  int32_t* n = (int32_t*)xmalloc(sizeof(int32_t) * nb);
  int32_t* k = (int32_t*)xmalloc(sizeof(int32_t) * nb);
  check(hss2d_box_sizes(H, n, k, NULL));
  const int cx = tree_complex(H);
  for (int b = 0; b < nb; ++b) {
    double *fi = NULL, *e = NULL;
    mxArray* FI = vec_out((mwSize)n[b], (mwSize)n[b], cx, &fi);
    mxArray* E = (b > 0) ? vec_out((mwSize)k[b], (mwSize)k[b], cx, &e) : NULL;
    check(hss2d_export_inverse(H, b, fi, e));
    mxSetField(a, b, "FI", FI);
    if (E) mxSetField(a, b, "E", E);
  }
  free(n);
  free(k);
  return a;
}

/* ---- HSS1D -------------------------------------------------------------- */
static hss1d_matrix* khss_handle(const mxArray* K) {
  if (!K || mxGetClassID(K) != mxCELL_CLASS || mxGetM(K) < BOX_ROWS)
    mexErrMsgIdAndTxt("hss:gpu", "expected K_HSS (cell(50, nboxes) from HSS1D_compress_nsym)");
  return (hss1d_matrix*)handle_in(mxGetCell(K, BOX_GPU - 1));
}

static void set_row(mxArray* K, int row, int box, mxArray* v) {
  mxSetCell(K, (mwIndex)box * BOX_ROWS + (row - 1), v);
}

static mxArray* k_hss(hss1d_matrix* H) {
  int32_t nb = 0;
  check(hss1d_info(H, &nb, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL));
  int32_t* lv = (int32_t*)xmalloc(sizeof(int32_t) * nb * 8);
  int32_t *par = lv + nb, *c1 = lv + 2 * nb, *c2 = lv + 3 * nb, *off = lv + 4 * nb, *cnt = lv + 5 * nb,
          *ns = lv + 6 * nb, *ks = lv + 7 * nb;
  check(hss1d_info(H, &nb, lv, par, c1, c2, off, cnt, ns, ks));
  mxArray* K = mxCreateCellMatrix(BOX_ROWS, (mwSize)nb);
  const int cx = khss_complex(H);
  for (int b = 0; b < nb; ++b) {
    set_row(K, BOX_LEVEL, b, scalar(lv[b]));
    set_row(K, BOX_PARENT, b, scalar(par[b] >= 0 ? par[b] + 1 : 0));
    set_row(K, BOX_C1, b, scalar(c1[b] >= 0 ? c1[b] + 1 : 0));
    set_row(K, BOX_C2, b, scalar(c2[b] >= 0 ? c2[b] + 1 : 0));
    set_row(K, BOX_END1, b, scalar(off[b] + 1));
    set_row(K, BOX_END2, b, scalar(off[b] + cnt[b]));
    set_row(K, BOX_NSKEL, b, scalar(ns[b]));
    set_row(K, BOX_KSKEL, b, scalar(ks[b]));
    if (par[b] < 0) continue;  /* roots carry no skeletons */
    const int n = ns[b], k = ks[b], nr = n - k;
    int32_t* iu = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)(2 * k + 2 * n));
    int32_t *id = iu + k, *ju = iu + 2 * k, *jd = ju + n;
    double *tu = NULL, *td = NULL;
    mxArray* Tu = vec_out((mwSize)k, (mwSize)(nr > 0 ? nr : 0), cx, &tu);  /* complex for a complex handle */
    mxArray* Td = vec_out((mwSize)k, (mwSize)(nr > 0 ? nr : 0), cx, &td);
    check(hss1d_export_box(H, b, iu, id, ju, jd, tu, td));
    set_row(K, BOX_I_SKUP, b, index_row(iu, k));
    set_row(K, BOX_I_SKDN, b, index_row(id, k));
    set_row(K, BOX_J_UP, b, index_row(ju, n));
    set_row(K, BOX_J_DN, b, index_row(jd, n));
    set_row(K, BOX_T_UP, b, Tu);
    set_row(K, BOX_T_DN, b, Td);
    free(iu);
  }
  set_row(K, BOX_GPU, 0, handle_out(H));
  free(lv);
  return K;
}

static int64_t hss1d_rows(hss1d_matrix* H) {
  int64_t M = 0;
  check(hss1d_rect_info(H, &M, NULL, NULL, NULL, NULL));
  return M;
}

/* ---- entry -------------------------------------------------------------- */
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  char op[64];
  if (nrhs < 1 || !mxIsChar(prhs[0]) || mxGetString(prhs[0], op, sizeof op))
    mexErrMsgIdAndTxt("hss:gpu", "first argument: operation name");
#define NEED(k) \
  if (nrhs < (k)) mexErrMsgIdAndTxt("hss:gpu", "%s needs %d arguments", op, (k) - 1)
  if (!strcmp(op, "HSS2D_build_tree_nsym")) {
    NEED(2);
    hss2d_params p;
    hss2d_params_of(prhs[1], &p);
    hss2d_matrix* H = NULL;
    check(hss2d_build_tree(&H, &p));
    plhs[0] = info_tree(H);
  } else if (!strcmp(op, "HSS2D_compress_nsym")) {
    NEED(2);
    hss2d_matrix* H = tree_handle(prhs[1]);
    check(hss2d_compress(H));
    plhs[0] = a_hss(H, 0);
  } else if (!strcmp(op, "HSS2D_invert_nsym")) {
    NEED(2);
    hss2d_matrix* H = tree_handle(prhs[1]);
    check(hss2d_invert(H));
    plhs[0] = a_hss(H, 1);
  } else if (!strcmp(op, "HSS2D_apply_nsym") || !strcmp(op, "HSS2D_applyinv_nsym")) {
    NEED(4);
    hss2d_matrix* H = tree_handle(prhs[1]);
    const mxArray* X = prhs[3];
    const int cx = tree_complex(H);
    mxArray* tmp = NULL;
    const double* x = vec_in(X, cx, &tmp);
    const mwSize N = mxGetM(X), r = mxGetN(X);
    double* y = NULL;
    plhs[0] = vec_out(N, r, cx, &y);
    if (!strcmp(op, "HSS2D_applyinv_nsym")) check(hss2d_applyinv(H, x, y, (int32_t)r));
    else check(hss2d_apply(H, x, y, (int32_t)r));
  } else if (!strcmp(op, "Iterative_Refinement")) {
    NEED(5);
    hss2d_matrix* H = tree_handle(prhs[1]);
    const mwSize N = mxGetM(prhs[2]), r = mxGetN(prhs[2]);
    double relres = 0.0;
    int32_t iters = 0;
    const int cx = tree_complex(H);
    mxArray* tmp = NULL;
    const double* f = vec_in(prhs[2], cx, &tmp);
    double* x = NULL;
    plhs[0] = vec_out(N, r, cx, &x);
    check(hss2d_solve(H, f, x, (int32_t)r, mxGetScalar(prhs[3]), (int32_t)mxGetScalar(prhs[4]), &relres, &iters));
    if (nlhs > 1) plhs[1] = scalar(relres);
    if (nlhs > 2) plhs[2] = scalar(iters);
  } else if (!strcmp(op, "HSS2D_destroy")) {
    NEED(2);
    check(hss2d_destroy(tree_handle(prhs[1])));
  } else if (!strcmp(op, "HSS1D_compress_nsym")) {
    NEED(6);
    char type[16];
    if (!mxIsChar(prhs[1]) || mxGetString(prhs[1], type, sizeof type) || strcmp(type, "green"))
      mexErrMsgIdAndTxt("hss:gpu", "HSS1D_compress_nsym: type 'green' (the proxy compression)");
    const mxArray* X = prhs[2];
    if (!mxIsDouble(X) || mxGetN(X) < 6) mexErrMsgIdAndTxt("hss:gpu", "X must be N x 6 [x y nx ny w kappa]");
    hss_kernel_params kp;
    kernel_params(prhs[5], &kp);
    hss1d_matrix* K = NULL;
    check(hss1d_compress(&K, mxGetDoubles(X), (int64_t)mxGetM(X), (int64_t)mxGetM(X),
                         (int32_t)mxGetScalar(prhs[3]), mxGetScalar(prhs[4]), &kp,
                         (uint64_t)field_or(prhs[5], "seed", 0)));
    plhs[0] = k_hss(K);
  } else if (!strcmp(op, "HSS1D_invert_nsym")) {
    NEED(2);
    hss1d_matrix* K = khss_handle(prhs[1]);
    check(hss1d_invert(K));
    plhs[0] = handle_out(K);
    if (nlhs > 1) plhs[1] = mxCreateDoubleMatrix(0, 0, mxREAL);
  } else if (!strcmp(op, "HSS1D_apply_nsym")) {
    NEED(3);
    hss1d_matrix* K = khss_handle(prhs[1]);
    const int cx = khss_complex(K);
    mxArray* tmp = NULL;
    const double* q = vec_in(prhs[2], cx, &tmp);
    double* u = NULL;
    plhs[0] = vec_out((mwSize)hss1d_rows(K), mxGetN(prhs[2]), cx, &u);
    check(hss1d_apply(K, q, u, (int32_t)mxGetN(prhs[2])));
  } else if (!strcmp(op, "HSS1D_applyinv_nsym")) {
    NEED(5);
    hss1d_matrix* K = khss_handle(prhs[1]);
    const mwSize N = mxGetM(prhs[4]), r = mxGetN(prhs[4]);
    const int cx = khss_complex(K);
    mxArray* tmp = NULL;
    const double* f = vec_in(prhs[4], cx, &tmp);
    double* x = NULL;
    plhs[0] = vec_out(N, r, cx, &x);
    check(hss1d_applyinv(K, f, x, (int32_t)r));
  } else if (!strcmp(op, "HSS1D_destroy")) {
    NEED(2);
    check(hss1d_destroy(khss_handle(prhs[1])));
  } else if (!strcmp(op, "Kernel_Eval")) {
    NEED(4);
    hss_kernel_params kp;
    kernel_params(prhs[3], &kp);
    const mwSize m = mxGetM(prhs[1]), n = mxGetM(prhs[2]);
    double* A = NULL;
    plhs[0] = vec_out(m, n, kp.flag == HSS_SL_H_2D, &A);  /* complex for the Helmholtz kernel */
    check(hss_kernel_eval(&kp, mxGetDoubles(prhs[1]), (int64_t)m, mxGetDoubles(prhs[2]), (int64_t)n, A));
  } else {
    mexErrMsgIdAndTxt("hss:gpu", "unknown operation %s", op);
  }
#undef NEED
}
