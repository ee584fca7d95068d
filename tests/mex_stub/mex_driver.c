/*
 * Runs the MEX shim (hssc_directsolver_gb300/mex/hss_gpu_mex.c) through the host-side
 * stand-ins of mex_stub.c, as the reference's scripts would call it from MATLAB:
 *   params -> HSS2D_build_tree_nsym -> HSS2D_compress_nsym -> HSS2D_invert_nsym ->
 *   HSS2D_applyinv_nsym, then HSS1D_compress_nsym -> HSS1D_invert_nsym -> HSS1D_applyinv_nsym,
 *   then the same HSS1D sequence with the complex Helmholtz kernel (SL_H_2D, complex
 *   right-hand side) and Kernel_Eval of it.
 * usage: mex_driver DIR   (DIR holds sizes.txt "N npan M", x_source.bin (N x 2), rhs.bin
 * (N x 2), curve.bin (M x 6), column-major doubles).  Writes y2d.bin, y1d.bin, y1c.bin,
 * ke.bin, info.txt.
 * Exit 0 on success, 3 when the shim raised a MATLAB error (printed as "MEXERR: ...").
 */
#include <setjmp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"

extern jmp_buf mex_stub_jmp;
extern char mex_stub_msg[1024];
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);

static char dir[512];

static double* read_doubles(const char* name, size_t n) {
  char path[600];
  snprintf(path, sizeof path, "%s/%s", dir, name);
  FILE* f = fopen(path, "rb");
  if (!f) { perror(path); exit(2); }
  double* v = (double*)malloc(n * sizeof(double));
  if (fread(v, sizeof(double), n, f) != n) { fprintf(stderr, "short read %s\n", path); exit(2); }
  fclose(f);
  return v;
}
static void write_doubles(const char* name, const double* v, size_t n) {
  char path[600];
  snprintf(path, sizeof path, "%s/%s", dir, name);
  FILE* f = fopen(path, "wb");
  fwrite(v, sizeof(double), n, f);
  fclose(f);
}
static mxArray* matrix(const double* v, size_t m, size_t n) {
  mxArray* a = mxCreateDoubleMatrix(m, n, mxREAL);
  memcpy(mxGetDoubles(a), v, m * n * sizeof(double));
  return a;
}
static mxArray* call(const char* op, int nlhs, mxArray** out, int nin, mxArray** in) {
  mxArray* args[8];
  args[0] = mxCreateString(op);
  for (int i = 0; i < nin; ++i) args[i + 1] = in[i];
  mxArray* res[4] = {0, 0, 0, 0};
  mexFunction(nlhs, res, nin + 1, (const mxArray**)args);
  if (out)
    for (int i = 0; i < nlhs; ++i) out[i] = res[i];
  return res[0];
}

int main(int argc, char** argv) {
  if (argc != 2) { fprintf(stderr, "usage: mex_driver DIR\n"); return 2; }
  snprintf(dir, sizeof dir, "%s", argv[1]);
  char path[600];
  snprintf(path, sizeof path, "%s/sizes.txt", dir);
  FILE* fs = fopen(path, "r");
  long N = 0, npan = 0, M = 0;
  if (!fs || fscanf(fs, "%ld %ld %ld", &N, &npan, &M) != 3) { fprintf(stderr, "bad sizes.txt\n"); return 2; }
  fclose(fs);
  double* xs = read_doubles("x_source.bin", (size_t)N * 2);
  double* rhs = read_doubles("rhs.bin", (size_t)N * 2);
  double* curve = read_doubles("curve.bin", (size_t)M * 6);
  if (setjmp(mex_stub_jmp)) {
    printf("MEXERR: %s\n", mex_stub_msg);
    return 3;
  }
  /* params as Common/HSS_tree_parameters.m builds it, with the workload's c(y) */
  const char* names[] = {"Ng", "X_source", "layers", "acc", "flag_pot", "h", "INTERform", "sym", "transinv",
                         "b_alpha", "c_alpha", "c_x0", "c_y0", "c_isig", "precision"};
  mxArray* prm = mxCreateStructMatrix(1, 1, 15, names);
  mxSetField(prm, 0, "Ng", mxCreateDoubleScalar(8));
  mxSetField(prm, 0, "X_source", matrix(xs, (size_t)N, 2));
  mxSetField(prm, 0, "layers", mxCreateDoubleScalar(2));
  mxSetField(prm, 0, "acc", mxCreateDoubleScalar(1e-10));
  mxSetField(prm, 0, "flag_pot", mxCreateString("SL_L_2D"));
  mxSetField(prm, 0, "h", mxCreateDoubleScalar(2.0 / (8.0 * npan)));
  mxSetField(prm, 0, "INTERform", mxCreateString("dense"));
  mxSetField(prm, 0, "sym", mxCreateDoubleScalar(0));
  mxSetField(prm, 0, "transinv", mxCreateDoubleScalar(0));
  mxSetField(prm, 0, "b_alpha", mxCreateDoubleScalar(0));
  mxSetField(prm, 0, "c_alpha", mxCreateDoubleScalar(0.5));
  mxSetField(prm, 0, "c_x0", mxCreateDoubleScalar(0));
  mxSetField(prm, 0, "c_y0", mxCreateDoubleScalar(0));
  mxSetField(prm, 0, "c_isig", mxCreateDoubleScalar(20));
  mxSetField(prm, 0, "precision", mxCreateString("fp64"));
  mxArray* in[5];
  in[0] = prm;
  mxArray* info = call("HSS2D_build_tree_nsym", 1, NULL, 1, in);
  in[0] = info;
  in[1] = prm;
  call("HSS2D_compress_nsym", 1, NULL, 2, in);
  mxArray* ahss = call("HSS2D_invert_nsym", 1, NULL, 2, in);
  in[0] = info;
  in[1] = ahss;
  in[2] = matrix(rhs, (size_t)N, 2);
  in[3] = prm;
  mxArray* Y = call("HSS2D_applyinv_nsym", 1, NULL, 4, in);
  write_doubles("y2d.bin", mxGetDoubles(Y), (size_t)N * 2);
  snprintf(path, sizeof path, "%s/info.txt", dir);
  FILE* fo = fopen(path, "w");
  mxArray* box = mxGetField(info, 0, "BOX");
  const size_t nb = mxGetNumberOfElements(box);
  fprintf(fo, "%g %zu\n", mxGetScalar(mxGetField(info, 0, "depth")), nb);
  for (size_t b = 0; b < nb; ++b) fprintf(fo, "%g ", mxGetScalar(mxGetField(box, b, "k")));
  fprintf(fo, "\n");
  mxArray* J1 = mxGetField(box, 1, "J");
  for (size_t i = 0; i < mxGetNumberOfElements(J1); ++i) fprintf(fo, "%g ", mxGetDoubles(J1)[i]);
  fprintf(fo, "\n");
  mxArray* FI0 = mxGetField(ahss, 0, "FI");
  fprintf(fo, "%zu %.17g\n", mxGetM(FI0), mxGetDoubles(FI0)[0]);
  /* HSS1D: the double-layer curve */
  const char* kn[] = {"flag_pot"};
  mxArray* knl = mxCreateStructMatrix(1, 1, 1, kn);
  mxSetField(knl, 0, "flag_pot", mxCreateString("DL_L_2D"));
  in[0] = mxCreateString("green");
  in[1] = matrix(curve, (size_t)M, 6);
  in[2] = mxCreateDoubleScalar(64);
  in[3] = mxCreateDoubleScalar(1e-10);
  in[4] = knl;
  mxArray* K = call("HSS1D_compress_nsym", 1, NULL, 5, in);
  mxArray* inv[2];
  in[0] = K;
  in[1] = mxCreateDoubleScalar(1e-10);
  call("HSS1D_invert_nsym", 2, inv, 2, in);
  in[0] = K;
  in[1] = inv[0];
  in[2] = inv[1];
  in[3] = matrix(rhs, (size_t)M, 1);
  mxArray* x1 = call("HSS1D_applyinv_nsym", 1, NULL, 4, in);
  write_doubles("y1d.bin", mxGetDoubles(x1), (size_t)M);
  const size_t nb1 = mxGetN(K);
  fprintf(fo, "%zu\n", nb1);
  for (size_t b = 0; b < nb1; ++b) fprintf(fo, "%g ", mxGetScalar(mxGetCell(K, b * 50 + 8)));  /* KSKEL */
  fprintf(fo, "\n");
  mxArray* isk = mxGetCell(K, 1 * 50 + 19);  /* I_SKUP of box 2 */
  for (size_t i = 0; i < mxGetNumberOfElements(isk); ++i) fprintf(fo, "%g ", mxGetDoubles(isk)[i]);
  fprintf(fo, "\n");
  fclose(fo);
  /* the complex Helmholtz curve: SL_H_2D, kh = 20, h = 0.05, dr_weights 0.3 + 0.1i, explicit
   * Gaussian b and c; the right-hand side rhs(:, 1) + i rhs(:, 2) */
  const char* hn[] = {"flag_pot", "kh", "h", "dr_weights", "b_alpha", "b_x0", "b_y0", "b_isig",
                      "c_alpha", "c_x0", "c_y0", "c_isig"};
  mxArray* hk = mxCreateStructMatrix(1, 1, 12, hn);
  mxSetField(hk, 0, "flag_pot", mxCreateString("SL_H_2D"));
  mxSetField(hk, 0, "kh", mxCreateDoubleScalar(20));
  mxSetField(hk, 0, "h", mxCreateDoubleScalar(0.05));
  mxArray* dr = mxCreateDoubleMatrix(1, 1, mxCOMPLEX);
  mxGetComplexDoubles(dr)[0].real = 0.3;
  mxGetComplexDoubles(dr)[0].imag = 0.1;
  mxSetField(hk, 0, "dr_weights", dr);
  mxSetField(hk, 0, "b_alpha", mxCreateDoubleScalar(0.5));
  mxSetField(hk, 0, "b_x0", mxCreateDoubleScalar(0.3));
  mxSetField(hk, 0, "b_y0", mxCreateDoubleScalar(0));
  mxSetField(hk, 0, "b_isig", mxCreateDoubleScalar(2));
  mxSetField(hk, 0, "c_alpha", mxCreateDoubleScalar(-0.3));
  mxSetField(hk, 0, "c_x0", mxCreateDoubleScalar(0));
  mxSetField(hk, 0, "c_y0", mxCreateDoubleScalar(-0.2));
  mxSetField(hk, 0, "c_isig", mxCreateDoubleScalar(3));
  in[0] = mxCreateString("green");
  in[1] = matrix(curve, (size_t)M, 6);
  in[2] = mxCreateDoubleScalar(64);
  in[3] = mxCreateDoubleScalar(1e-10);
  in[4] = hk;
  mxArray* Kc = call("HSS1D_compress_nsym", 1, NULL, 5, in);
  in[0] = Kc;
  in[1] = mxCreateDoubleScalar(1e-10);
  call("HSS1D_invert_nsym", 2, inv, 2, in);
  mxArray* fc = mxCreateDoubleMatrix((size_t)M, 1, mxCOMPLEX);
  for (long i = 0; i < M; ++i) {
    mxGetComplexDoubles(fc)[i].real = rhs[i];
    mxGetComplexDoubles(fc)[i].imag = rhs[N + i];
  }
  in[0] = Kc;
  in[1] = inv[0];
  in[2] = inv[1];
  in[3] = fc;
  mxArray* xc = call("HSS1D_applyinv_nsym", 1, NULL, 4, in);
  if (!mxIsComplex(xc)) { printf("MEXERR: complex handle returned a real vector\n"); return 3; }
  write_doubles("y1c.bin", (const double*)mxGetComplexDoubles(xc), (size_t)M * 2);
  in[0] = matrix(curve, 8, 2);  /* Kernel_Eval(X(1:8, 1:2), X(1:8, 1:2), params): rows 1..8 */
  {
    double* q = mxGetDoubles(in[0]);
    for (int i = 0; i < 8; ++i) { q[i] = curve[i]; q[8 + i] = curve[M + i]; }
  }
  in[1] = in[0];
  in[2] = hk;
  mxArray* ke = call("Kernel_Eval", 1, NULL, 3, in);
  if (!mxIsComplex(ke)) { printf("MEXERR: Kernel_Eval of SL_H_2D is not complex\n"); return 3; }
  write_doubles("ke.bin", (const double*)mxGetComplexDoubles(ke), 64 * 2);
  in[0] = Kc;
  call("HSS1D_destroy", 0, NULL, 1, in);
  in[0] = info;
  call("HSS2D_destroy", 0, NULL, 1, in);
  in[0] = K;
  call("HSS1D_destroy", 0, NULL, 1, in);
  printf("MEXOK\n");
  return 0;
}
