/* Fake MATLAB C Matrix API for driving mnad_mex.c from Python (ctypes).
 * Test infrastructure only.  Arrays are real doubles, cells or strings;
 * mexErrMsgIdAndTxt unwinds to fmx_call with longjmp, as MATLAB unwinds a
 * MEX call on error. */
#define _POSIX_C_SOURCE 200809L   /* strdup */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"

struct mxArray_tag {
    int kind;            /* 0: double, 1: cell, 2: char */
    size_t m, n;
    double* pr;
    mxArray** cells;
    char* str;
};

static jmp_buf g_jmp;
static char g_id[64], g_msg[512];
static void (*g_exit)(void) = NULL;

static mxArray* make(int kind, size_t m, size_t n)
{
    mxArray* a = (mxArray*)calloc(1, sizeof(mxArray));
    a->kind = kind;
    a->m = m;
    a->n = n;
    const size_t count = (m * n > 0) ? m * n : 1;
    if (kind == 0) a->pr = (double*)calloc(count, sizeof(double));
    if (kind == 1) a->cells = (mxArray**)calloc(count, sizeof(mxArray*));
    return a;
}

double* mxGetPr(const mxArray* a) { return a->pr; }
size_t mxGetM(const mxArray* a) { return a->m; }
size_t mxGetN(const mxArray* a) { return a->n; }
size_t mxGetNumberOfElements(const mxArray* a) { return a->m * a->n; }
int mxIsDouble(const mxArray* a) { return a->kind == 0; }
int mxIsComplex(const mxArray* a) { (void)a; return 0; }
int mxIsCell(const mxArray* a) { return a->kind == 1; }
int mxIsChar(const mxArray* a) { return a->kind == 2; }
double mxGetScalar(const mxArray* a) { return (a->kind == 0 && a->m * a->n > 0) ? a->pr[0] : 0.0; }
mxArray* mxGetCell(const mxArray* a, size_t i) { return a->cells[i]; }
void mxSetCell(mxArray* a, size_t i, mxArray* v) { a->cells[i] = v; }
mxArray* mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c) { (void)c; return make(0, m, n); }
mxArray* mxCreateDoubleScalar(double x)
{
    mxArray* a = make(0, 1, 1);
    a->pr[0] = x;
    return a;
}
mxArray* mxCreateCellMatrix(size_t m, size_t n) { return make(1, m, n); }
char* mxArrayToString(const mxArray* a) { return a->kind == 2 ? strdup(a->str) : NULL; }
void mxFree(void* p) { free(p); }
void mxDestroyArray(mxArray* a)
{
    if (!a) return;
    if (a->kind == 1)
        for (size_t i = 0; i < a->m * a->n; ++i) mxDestroyArray(a->cells[i]);
    free(a->pr);
    free(a->cells);
    free(a->str);
    free(a);
}
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...)
{
    va_list ap;
    snprintf(g_id, sizeof g_id, "%s", id);
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, ap);
    va_end(ap);
    longjmp(g_jmp, 1);
}
int mexAtExit(void (*fn)(void))
{
    g_exit = fn;
    return 0;
}

/* ---- entry points for the test driver ---------------------------------- */
mxArray* fmx_double(size_t m, size_t n, const double* data)
{
    mxArray* a = make(0, m, n);
    if (data) memcpy(a->pr, data, m * n * sizeof(double));
    return a;
}
mxArray* fmx_string(const char* s)
{
    mxArray* a = make(2, 1, strlen(s));
    a->str = strdup(s);
    return a;
}
mxArray* fmx_cell1(mxArray* v)
{
    mxArray* a = make(1, 1, 1);
    a->cells[0] = v;
    return a;
}
int fmx_kind(const mxArray* a) { return a->kind; }
/* Calls mexFunction; returns 0, or 1 after an error (fmx_error_id / _msg). */
int fmx_call(int nlhs, mxArray** plhs, int nrhs, const mxArray** prhs)
{
    if (setjmp(g_jmp)) return 1;
    g_id[0] = g_msg[0] = '\0';
    mexFunction(nlhs, plhs, nrhs, prhs);
    return 0;
}
const char* fmx_error_id(void) { return g_id; }
const char* fmx_error_msg(void) { return g_msg; }
void fmx_exit(void)
{
    if (g_exit) g_exit();
    g_exit = NULL;
}
