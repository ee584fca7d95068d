/*
 * Minimal declarations of the MATLAB C matrix / MEX API (the subset hss_gpu_mex.c uses),
 * for compile and link checks of the shim where MATLAB is not installed.  Signatures
 * follow the interleaved-complex API (mex -R2018a).  The definitions in mex_stub.c are
 * host-side stand-ins: they hold doubles, structs and cells in plain heap memory so a test
 * can call mexFunction without MATLAB.
 */
#ifndef HSS_TEST_MEX_STUB_H
#define HSS_TEST_MEX_STUB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef size_t mwSize;
typedef size_t mwIndex;
typedef struct mxArray_tag mxArray;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef enum {
  mxUNKNOWN_CLASS = 0, mxCELL_CLASS, mxSTRUCT_CLASS, mxLOGICAL_CLASS, mxCHAR_CLASS, mxVOID_CLASS,
  mxDOUBLE_CLASS, mxSINGLE_CLASS, mxINT8_CLASS, mxUINT8_CLASS, mxINT16_CLASS, mxUINT16_CLASS,
  mxINT32_CLASS, mxUINT32_CLASS, mxINT64_CLASS, mxUINT64_CLASS
} mxClassID;
typedef double mxDouble;
typedef struct { double real, imag; } mxComplexDouble;

mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
mxArray* mxCreateDoubleScalar(double v);
mxArray* mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity c);
mxArray* mxCreateCellMatrix(mwSize m, mwSize n);
mxArray* mxCreateStructMatrix(mwSize m, mwSize n, int nfields, const char** names);
mxArray* mxCreateString(const char* s);
void mxSetCell(mxArray* cell, mwIndex i, mxArray* v);
mxArray* mxGetCell(const mxArray* cell, mwIndex i);
void mxSetField(mxArray* s, mwIndex i, const char* name, mxArray* v);
mxArray* mxGetField(const mxArray* s, mwIndex i, const char* name);
mxDouble* mxGetDoubles(const mxArray* a);
mxComplexDouble* mxGetComplexDoubles(const mxArray* a);
int mxIsComplex(const mxArray* a);
void* mxGetData(const mxArray* a);
double mxGetScalar(const mxArray* a);
int mxGetString(const mxArray* a, char* buf, mwSize len);
mwSize mxGetM(const mxArray* a);
mwSize mxGetN(const mxArray* a);
mwSize mxGetNumberOfElements(const mxArray* a);
int mxIsStruct(const mxArray* a);
int mxIsDouble(const mxArray* a);
int mxIsChar(const mxArray* a);
mxClassID mxGetClassID(const mxArray* a);
void mxDestroyArray(mxArray* a);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);

#ifdef __cplusplus
}
#endif

#endif
