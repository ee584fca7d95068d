/*
 * Host-side stand-ins for the MATLAB matrix / MEX API declared in mex.h: doubles, uint64
 * scalars, strings, structs and cells in plain heap memory, so a test can call the MEX
 * shim's mexFunction without MATLAB.  mexErrMsgIdAndTxt records the message and jumps back
 * to the caller's mex_stub_try point (MATLAB unwinds to the prompt the same way).
 */
#define _POSIX_C_SOURCE 200809L  /* strdup */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"

struct mxArray_tag {
  mxClassID cls;
  mwSize m, n;
  int cplx;             /* complex double: (re, im) pairs in data (the interleaved API) */
  void* data;           /* numeric / char payload */
  int nfields;
  char** names;         /* struct field names */
  mxArray** items;      /* struct: m*n*nfields values; cell: m*n values */
};

jmp_buf mex_stub_jmp;
char mex_stub_msg[1024];

static mxArray* alloc_array(mxClassID cls, mwSize m, mwSize n) {
  mxArray* a = (mxArray*)calloc(1, sizeof(mxArray));
  a->cls = cls;
  a->m = m;
  a->n = n;
  return a;
}

mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) {
  mxArray* a = alloc_array(mxDOUBLE_CLASS, m, n);
  a->cplx = (c == mxCOMPLEX);
  a->data = calloc((m * n) > 0 ? m * n * (a->cplx ? 2 : 1) : 1, sizeof(double));
  return a;
}
mxArray* mxCreateDoubleScalar(double v) {
  mxArray* a = mxCreateDoubleMatrix(1, 1, mxREAL);
  *(double*)a->data = v;
  return a;
}
mxArray* mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity c) {
  (void)c;
  mxArray* a = alloc_array(cls, m, n);
  a->data = calloc((m * n) > 0 ? m * n : 1, 8);
  return a;
}
mxArray* mxCreateCellMatrix(mwSize m, mwSize n) {
  mxArray* a = alloc_array(mxCELL_CLASS, m, n);
  a->items = (mxArray**)calloc((m * n) > 0 ? m * n : 1, sizeof(mxArray*));
  return a;
}
mxArray* mxCreateStructMatrix(mwSize m, mwSize n, int nfields, const char** names) {
  mxArray* a = alloc_array(mxSTRUCT_CLASS, m, n);
  a->nfields = nfields;
  a->names = (char**)calloc(nfields ? nfields : 1, sizeof(char*));
  for (int f = 0; f < nfields; ++f) a->names[f] = strdup(names[f]);
  a->items = (mxArray**)calloc((m * n * nfields) > 0 ? m * n * nfields : 1, sizeof(mxArray*));
  return a;
}
mxArray* mxCreateString(const char* s) {
  mxArray* a = alloc_array(mxCHAR_CLASS, 1, strlen(s));
  a->data = strdup(s);
  return a;
}
void mxSetCell(mxArray* cell, mwIndex i, mxArray* v) { cell->items[i] = v; }
mxArray* mxGetCell(const mxArray* cell, mwIndex i) { return cell->items[i]; }
static int field_index(const mxArray* s, const char* name) {
  for (int f = 0; f < s->nfields; ++f)
    if (!strcmp(s->names[f], name)) return f;
  return -1;
}
void mxSetField(mxArray* s, mwIndex i, const char* name, mxArray* v) {
  int f = field_index(s, name);
  if (f < 0) {  /* MATLAB adds the field; the stand-in grows the name table */
    f = s->nfields++;
    s->names = (char**)realloc(s->names, s->nfields * sizeof(char*));
    s->names[f] = strdup(name);
    mxArray** it = (mxArray**)calloc(s->m * s->n * s->nfields, sizeof(mxArray*));
    for (mwSize e = 0; e < s->m * s->n; ++e)
      for (int g = 0; g < f; ++g) it[e * s->nfields + g] = s->items[e * f + g];
    free(s->items);
    s->items = it;
  }
  s->items[i * s->nfields + f] = v;
}
mxArray* mxGetField(const mxArray* s, mwIndex i, const char* name) {
  if (!s || s->cls != mxSTRUCT_CLASS) return NULL;
  const int f = field_index(s, name);
  return f < 0 ? NULL : s->items[i * s->nfields + f];
}
mxDouble* mxGetDoubles(const mxArray* a) { return (a->cls == mxDOUBLE_CLASS && !a->cplx) ? (double*)a->data : NULL; }
mxComplexDouble* mxGetComplexDoubles(const mxArray* a) {
  return (a->cls == mxDOUBLE_CLASS && a->cplx) ? (mxComplexDouble*)a->data : NULL;
}
int mxIsComplex(const mxArray* a) { return a && a->cplx; }
void* mxGetData(const mxArray* a) { return a->data; }
double mxGetScalar(const mxArray* a) {
  if (a->cls == mxDOUBLE_CLASS) return *(double*)a->data;
  if (a->cls == mxUINT64_CLASS) return (double)*(unsigned long long*)a->data;
  return 0.0;
}
int mxGetString(const mxArray* a, char* buf, mwSize len) {
  if (a->cls != mxCHAR_CLASS || len == 0) return 1;
  strncpy(buf, (const char*)a->data, len - 1);
  buf[len - 1] = 0;
  return strlen((const char*)a->data) >= len;
}
mwSize mxGetM(const mxArray* a) { return a->m; }
mwSize mxGetN(const mxArray* a) { return a->n; }
mwSize mxGetNumberOfElements(const mxArray* a) { return a->m * a->n; }
int mxIsStruct(const mxArray* a) { return a && a->cls == mxSTRUCT_CLASS; }
int mxIsDouble(const mxArray* a) { return a && a->cls == mxDOUBLE_CLASS; }
int mxIsChar(const mxArray* a) { return a && a->cls == mxCHAR_CLASS; }
mxClassID mxGetClassID(const mxArray* a) { return a->cls; }
void mxDestroyArray(mxArray* a) { (void)a; /* the stand-in keeps everything until exit */ }

void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  int n = snprintf(mex_stub_msg, sizeof mex_stub_msg, "%s: ", id);
  vsnprintf(mex_stub_msg + n, sizeof mex_stub_msg - n, fmt, ap);
  va_end(ap);
  longjmp(mex_stub_jmp, 1);
}
