/*
 * mnad_mex.c -- MATLAB MEX gateway of libmnad.so (include/mnad.h).
 *
 * One gateway, called through the two .m shims in this directory that keep
 * the reference signatures of SRC/MNAD/fwd_PDE_exact_MNAD.m:1 and
 * SRC/migration/Born_adj_MNAD.m:1, so the reference drivers
 * (SRC/migration/main_Acoustic_RTM.m, SRC/modeling/main_Acoustic_Data.m and
 * the examples) run unchanged once this directory precedes SRC/MNAD and
 * SRC/migration on the MATLAB path.
 *
 *   data = mnad_mex('fwd', dx,xs,xr,dz,zs,zr,v,dt,nt,w,d_pml,ss,indx)   1x1 cell {nt x nr}
 *   Im   = mnad_mex('adj', dx,dz,nt,dt,v,xr,zr,data,d_pml,ss)           Nint x 1
 *   tf   = mnad_mex('has', ss)                  source wavefield of ss stored on the GPU?
 *   [UU, illum] = mnad_mex('export', ss)        the UU_<ss>.mat / illum_<ss>.mat contents
 *   mnad_mex('import', ss, nz, nx, d_pml, nt, T, UU[, illum])
 *   mnad_mex('release', ss)
 *   data = mnad_mex('noalloc', dx,xs,xr,dz,zs,zr,v,dt,nt,w,d_pml)      forward, no device allocation
 *   mnad_mex('reset')                           frees the GPU context of this MATLAB process
 *
 * Each MATLAB process (a parfor worker is a process) holds one context on
 * GPU 0, created on first use and destroyed by mexAtExit.  A non-zero status
 * of the library becomes mexErrMsgIdAndTxt("mnad:<code>", message), the
 * error-identifier style of the reference (e.g. SRC/MNAD/acquisi.m:66-67).
 *
 * Build inside MATLAB:  mex -R2017b mnad_mex.c -I<repo>/include -L<lib dir> -lmnad
 */
#include <stdio.h>
#include <string.h>

#include "mex.h"
#include "mnad.h"

static mnad_context* g_ctx = NULL;

static const char* code_name(int rc)
{
    switch (rc) {
    case MNAD_E_ARG: return "arg";
    case MNAD_E_OOM: return "oom";
    case MNAD_E_CUDA: return "cuda";
    case MNAD_E_TIMEOUT: return "timeout";
    case MNAD_E_NOTFOUND: return "notfound";
    case MNAD_E_NUMERIC: return "numeric";
    case MNAD_E_BUDGET: return "budget";
    case MNAD_E_STATE: return "state";
    default: return "unknown";
    }
}

static void check(int rc)
{
    if (rc != MNAD_OK) {
        char id[32];
        snprintf(id, sizeof id, "mnad:%s", code_name(rc));
        mexErrMsgIdAndTxt(id, "%s", mnad_last_error());
    }
}

static void fail(const char* msg) { mexErrMsgIdAndTxt("mnad:arg", "%s", msg); }

static void at_exit(void)
{
    if (g_ctx) mnad_context_destroy(g_ctx);
    g_ctx = NULL;
}

static mnad_context* context(void)
{
    if (!g_ctx) {
        check(mnad_context_create(0, 0, &g_ctx));
        mexAtExit(at_exit);
    }
    return g_ctx;
}

/* A real double array argument (numeric checks only; sizes are checked by the library). */
static const double* dbl(const mxArray* a, const char* what)
{
    if (!mxIsDouble(a) || mxIsComplex(a)) {
        char msg[96];
        snprintf(msg, sizeof msg, "%s must be a real double array", what);
        fail(msg);
    }
    return mxGetPr(a);
}

static double scalar(const mxArray* a, const char* what)
{
    if (!mxIsDouble(a) || mxGetNumberOfElements(a) != 1) {
        char msg[96];
        snprintf(msg, sizeof msg, "%s must be a double scalar", what);
        fail(msg);
    }
    return mxGetScalar(a);
}

static void nargs(int nrhs, int lo, int hi, const char* cmd)
{
    if (nrhs < lo || nrhs > hi) {
        char msg[96];
        snprintf(msg, sizeof msg, "mnad_mex('%s', ...): wrong number of arguments", cmd);
        fail(msg);
    }
}

/* 'fwd' / 'noalloc': prhs = dx,xs,xr,dz,zs,zr,v,dt,nt,w,d_pml[,ss,indx] */
static void do_fwd(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[], int noalloc)
{
    const double dx = scalar(prhs[0], "dx"), xs = scalar(prhs[1], "xs");
    const double* xr = dbl(prhs[2], "xr");
    const double dz = scalar(prhs[3], "dz"), zs = scalar(prhs[4], "zs");
    const double* zr = dbl(prhs[5], "zr");
    const double* v = dbl(prhs[6], "v");
    const double dt = scalar(prhs[7], "dt");
    const int nt = (int)scalar(prhs[8], "nt");
    const double* w = dbl(prhs[9], "w");
    const int d_pml = (int)scalar(prhs[10], "d_pml");
    const int nr = (int)mxGetNumberOfElements(prhs[2]);
    const int nz = (int)mxGetM(prhs[6]), nx = (int)mxGetN(prhs[6]);
    if ((int)mxGetNumberOfElements(prhs[5]) != nr) fail("xr and zr differ in length");
    if ((int)mxGetNumberOfElements(prhs[9]) < nt) fail("w has fewer than nt samples");
    mxArray* datau = mxCreateDoubleMatrix((size_t)nt, (size_t)nr, mxREAL);
    if (noalloc) {
        check(mnad_fwd_pde_exact_noalloc(0, dx, xs, xr, nr, dz, zs, zr, v, nz, nx, dt, nt, w, d_pml,
                                         mxGetPr(datau)));
    } else {
        const int ss = nrhs > 11 ? (int)scalar(prhs[11], "ss") : 0;
        const int indx = nrhs > 12 && mxGetNumberOfElements(prhs[12]) > 0 ? (int)scalar(prhs[12], "indx") : 0;
        check(mnad_fwd_pde_exact(context(), dx, xs, xr, nr, dz, zs, zr, v, nz, nx, dt, nt, w, d_pml, ss, indx,
                                 mxGetPr(datau), NULL, NULL));
    }
    /* data = cell(1,1); data{1} = datau  (fwd_PDE_exact_MNAD.m:166) */
    plhs[0] = mxCreateCellMatrix(1, 1);
    mxSetCell(plhs[0], 0, datau);
    (void)nlhs;
}

/* 'adj': prhs = dx,dz,nt,dt,v,xr,zr,data,d_pml,ss */
static void do_adj(mxArray* plhs[], const mxArray* prhs[])
{
    const double dx = scalar(prhs[0], "dx"), dz = scalar(prhs[1], "dz");
    const int nt = (int)scalar(prhs[2], "nt");
    const double dt = scalar(prhs[3], "dt");
    const double* v = dbl(prhs[4], "v");
    const double* xr = dbl(prhs[5], "xr");
    const double* zr = dbl(prhs[6], "zr");
    const mxArray* data = prhs[7];
    const int d_pml = (int)scalar(prhs[8], "d_pml");
    const int ss = (int)scalar(prhs[9], "ss");
    const int nz = (int)mxGetM(prhs[4]), nx = (int)mxGetN(prhs[4]);
    const int nr = (int)mxGetNumberOfElements(prhs[5]);
    /* datau = data{1} (Born_adj_MNAD.m:50), or the matrix itself (the driver's call, D2) */
    if (mxIsCell(data)) {
        if (mxGetNumberOfElements(data) < 1 || !mxGetCell(data, 0)) fail("data is an empty cell");
        data = mxGetCell(data, 0);
    }
    const double* d = dbl(data, "data");
    if ((int)mxGetNumberOfElements(prhs[6]) != nr) fail("xr and zr differ in length");
    if (mxGetM(data) != (size_t)nt || mxGetN(data) != (size_t)nr) fail("data must be nt x nr");
    if (nz <= 2 * d_pml || nx <= 2 * d_pml) fail("v is not larger than its CPML");
    const size_t nint = (size_t)(nz - 2 * d_pml) * (size_t)(nx - 2 * d_pml);
    plhs[0] = mxCreateDoubleMatrix(nint, 1, mxREAL);
    check(mnad_born_adj(context(), dx, dz, nt, dt, v, nz, nx, xr, zr, nr, d, d_pml, ss, mxGetPr(plhs[0])));
}

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[])
{
    if (nrhs < 1 || !mxIsChar(prhs[0])) fail("first argument must be a command string");
    char* cmd = mxArrayToString(prhs[0]);
    if (!cmd) fail("bad command string");
    char c[16];
    strncpy(c, cmd, sizeof c - 1);
    c[sizeof c - 1] = '\0';
    mxFree(cmd);
    const int n = nrhs - 1;
    const mxArray** a = prhs + 1;
    if (!strcmp(c, "fwd")) {
        nargs(n, 11, 13, c);
        do_fwd(nlhs, plhs, n, a, 0);
    } else if (!strcmp(c, "noalloc")) {
        nargs(n, 11, 11, c);
        do_fwd(nlhs, plhs, n, a, 1);
    } else if (!strcmp(c, "adj")) {
        nargs(n, 10, 10, c);
        do_adj(plhs, a);
    } else if (!strcmp(c, "has")) {
        nargs(n, 1, 1, c);
        int64_t nint;
        int ncols, nsnap, T;
        const int rc = mnad_wavefield_info(context(), (int)scalar(a[0], "ss"), &nint, &ncols, &nsnap, &T);
        if (rc != MNAD_OK && rc != MNAD_E_NOTFOUND) check(rc);
        plhs[0] = mxCreateDoubleScalar(rc == MNAD_OK ? 1.0 : 0.0);
    } else if (!strcmp(c, "export")) {
        nargs(n, 1, 1, c);
        const int ss = (int)scalar(a[0], "ss");
        int64_t nint;
        int ncols, nsnap, T;
        check(mnad_wavefield_info(context(), ss, &nint, &ncols, &nsnap, &T));
        plhs[0] = mxCreateDoubleMatrix((size_t)nint, (size_t)ncols, mxREAL);
        mxArray* il = mxCreateDoubleMatrix((size_t)nint, 1, mxREAL);
        check(mnad_wavefield_export(context(), ss, mxGetPr(plhs[0]), mxGetPr(il)));
        if (nlhs > 1) plhs[1] = il;
        else mxDestroyArray(il);
    } else if (!strcmp(c, "import")) {
        nargs(n, 7, 8, c);
        const mxArray* UU = a[6];
        const double* il = n > 7 ? dbl(a[7], "illum") : NULL;
        const int nt = (int)scalar(a[4], "nt"), T = (int)scalar(a[5], "T");
        const int ncols = (int)mxGetN(UU);
        const int nsnap = T > 0 ? (nt / T < ncols ? nt / T : ncols) : 0;
        check(mnad_wavefield_import(context(), (int)scalar(a[0], "ss"), (int)scalar(a[1], "nz"),
                                    (int)scalar(a[2], "nx"), (int)scalar(a[3], "d_pml"), nt, T, ncols, nsnap,
                                    dbl(UU, "UU"), il));
    } else if (!strcmp(c, "release")) {
        nargs(n, 1, 1, c);
        check(mnad_wavefield_release(context(), (int)scalar(a[0], "ss")));
    } else if (!strcmp(c, "reset")) {
        at_exit();
    } else {
        fail("unknown command");
    }
}
