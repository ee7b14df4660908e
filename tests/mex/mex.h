/* Minimal stand-in for MATLAB's mex.h / matrix.h: just the part of the C
 * Matrix API that mnad_mex.c uses, implemented by fake_mx.c so the gateway
 * can be compiled and driven from the test suite without MATLAB.  Test
 * infrastructure only. */
#ifndef FAKE_MEX_H
#define FAKE_MEX_H
#include <stddef.h>
#include <stdint.h>

typedef struct mxArray_tag mxArray;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

double* mxGetPr(const mxArray* a);
size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
size_t mxGetNumberOfElements(const mxArray* a);
int mxIsDouble(const mxArray* a);
int mxIsComplex(const mxArray* a);
int mxIsCell(const mxArray* a);
int mxIsChar(const mxArray* a);
double mxGetScalar(const mxArray* a);
mxArray* mxGetCell(const mxArray* a, size_t i);
void mxSetCell(mxArray* a, size_t i, mxArray* v);
mxArray* mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c);
mxArray* mxCreateDoubleScalar(double x);
mxArray* mxCreateCellMatrix(size_t m, size_t n);
char* mxArrayToString(const mxArray* a);
void mxFree(void* p);
void mxDestroyArray(mxArray* a);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
int mexAtExit(void (*fn)(void));

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);
#endif
