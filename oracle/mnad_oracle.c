/*
 * FP64 matrix-free CPU oracle for the MNAD modeling / RTM hot path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker (and the timed CPU port),
 * never the product.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline legs load it.  The CUDA library behind include/mnad.h never
 * links or calls it.
 *
 * It restates, independently of oracle/mnad_oracle.py (which assembles the
 * sparse operators), the reference MATLAB code Ahmadreza205/MNAD-Modeling-RTM:
 *   - the 63 stencil coefficients of SRC/MNAD/A??_gen.m, evaluated per
 *     destination point from v(j,i) (out-of-grid neighbours are omitted, as
 *     the reference's index ranges omit them);
 *   - the CPML coefficients of SRC/MNAD/C_cof.m and the memory recurrences of
 *     SRC/MNAD/Ux123_gen.m / Uz123_gen.m;
 *   - the forward loop of SRC/MNAD/fwd_PDE_exact_MNAD.m:92-157 and the
 *     adjoint loop of SRC/migration/Born_adj_MNAD.m:85-138 (with U_r read as
 *     U, Born_adj_MNAD.m:105-106).
 * Pinned to the reference: it reproduces, to 1e-12, the outputs of the
 * reference's own .m sources run under the MATLAB-subset interpreter
 * oracle/mlite.py (fixtures tests/golden/golden_ref_*.npz; no MATLAB or
 * Octave is available).
 *
 * Layout: column-major, z fastest: F[j + i*nz], j in [0,nz), i in [0,nx).
 * Indices passed in are 1-based, like the MATLAB call signature.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define MNAD_ORACLE_EXPORT __attribute__((visibility("default")))

typedef struct {
    int nz, nx, d;
    double dx, dz, dt;
    int adjoint;              /* 1: V2dt2 = (v*dt)^2 (Born_adj_MNAD.m:36) */
} og_t;

/* Per-point stencil coefficients (one set per destination point). */
typedef struct {
    /* nU row */
    double uu_zm, uu_xm, uu_c, uu_xp, uu_zp, uu_d;
    double uv_xm, uv_xp, uv_dm, uv_dp, uv_x2m, uv_x2p;
    double uw_zp, uw_zm, uw_dm, uw_dp, uw_z2p, uw_z2m;
    /* nV row */
    double vu_xm, vu_xp, vu_dm, vu_dp;
    double vv_z, vv_x, vv_c, vv_d;
    double vw_a, vw_b;
    /* nW row */
    double wu_zm, wu_zp, wu_dm, wu_dp;
    double wv_a, wv_b;
    double ww_z, ww_x, ww_c, ww_d;
} coef_t;

static void coefs(double a, double dx, double dz, double dt, coef_t* c)
{
    /* Expressions as in SRC/MNAD/A??_gen.m (same operation order). */
    double a2 = a * a, a4 = a2 * a2;
    double dt2 = dt * dt, dt4 = dt2 * dt2;
    double dx2 = dx * dx, dz2 = dz * dz;
    double dx3 = dx2 * dx, dz3 = dz2 * dz;
    double dx4 = dx2 * dx2, dz4 = dz2 * dz2;
    double dx5 = dx4 * dx, dz5 = dz4 * dz;
    /* Auu_gen.m:30,37,44,65 */
    c->uu_zm = (24.0/11)*a2*dt2/dz2 - a4*dt4*(15/(11*dz4) + 1/(dx2*dz2));
    c->uu_zp = c->uu_zm;
    c->uu_xm = (24.0/11)*a2*dt2/dx2 - a4*dt4*(15/(11*dx4) + 1/(dx2*dz2));
    c->uu_xp = c->uu_xm;
    c->uu_c = 2 - (48.0/11)*a2*dt2*(1/dx2 + 1/dz2) + (30.0/11)*a4*dt4*(1/dx4 + 1/dz4 + 11/(15*dx2*dz2));
    c->uu_d = a4*dt4/(2*dx2*dz2);
    /* Auv_gen.m:29,36,43,57,71,78 */
    c->uv_xm = (-20.0/33)*a2*dt2/dx + a4*dt4*(47/(66*dx3) + 1/(6*dx*dz2));
    c->uv_xp = (20.0/33)*a2*dt2/dx - a4*dt4*(47/(66*dx3) + 1/(6*dx*dz2));
    c->uv_dm = -a4*dt4/(12*dx*dz2);         /* neighbours at i-1 */
    c->uv_dp = a4*dt4/(12*dx*dz2);          /* neighbours at i+1 */
    c->uv_x2m = (1.0/132)*a2*dt2/dx - (1.0/66)*a4*dt4/dx3;
    c->uv_x2p = (-1.0/132)*a2*dt2/dx + (1.0/66)*a4*dt4/dx3;
    /* Auw_gen.m:29,36,43,50,71,78 */
    c->uw_zp = (20.0/33)*a2*dt2/dz - a4*dt4*(47/(66*dz3) + 1/(6*dz*dx2));
    c->uw_zm = (-20.0/33)*a2*dt2/dz + a4*dt4*(47/(66*dz3) + 1/(6*dz*dx2));
    c->uw_dm = -a4*dt4/(12*dz*dx2);         /* neighbours at j-1 */
    c->uw_dp = a4*dt4/(12*dz*dx2);          /* neighbours at j+1 */
    c->uw_z2p = (-1.0/132)*a2*dt2/dz + (1.0/66)*a4*dt4/dz3;
    c->uw_z2m = (1.0/132)*a2*dt2/dz - (1.0/66)*a4*dt4/dz3;
    /* Avu_gen.m:30,37,44,58 */
    c->vu_xm = -a4*dt4*(15/(2*dx5) - 1/(dx*dz4) + 5/(2*dx3*dz2)) + a2*dt2*(15/(2*dx3) - 1/(dx*dz2));
    c->vu_xp = a4*dt4*(15/(2*dx5) - 1/(dx*dz4) + 5/(2*dx3*dz2)) - a2*dt2*(15/(2*dx3) - 1/(dx*dz2));
    c->vu_dm = a4*dt4*(5/(4*dx3*dz2) - 1/(2*dx*dz4)) + a2*dt2/(2*dx*dz2);
    c->vu_dp = -a4*dt4*(5/(4*dx3*dz2) - 1/(2*dx*dz4)) - a2*dt2/(2*dx*dz2);
    /* Avv_gen.m:29,36,43,64 */
    c->vv_z = a2*dt2/dz2 - 2*a4*dt4/(dx2*dz2);
    c->vv_x = -(3.0/2)*a2*dt2/dx2 + a4*dt4*(5/(2*dx4) + 1/(2*dx2*dz2));
    c->vv_c = 2 - a2*dt2*(12/dx2 + 2/dz2) + a4*dt4*(10/dx4 + 4/(dx2*dz2));
    c->vv_d = -a4*dt4/(4*dx2*dz2);
    /* Avw_gen.m:29,36: a on (j-1,i-1),(j+1,i+1); b on (j+1,i-1),(j-1,i+1) */
    c->vw_a = a4*dt4/(4*dz3*dx) - a2*dt2/(4*dz*dx);
    c->vw_b = -a4*dt4/(4*dz3*dx) + a2*dt2/(4*dz*dx);
    /* Awu_gen.m:29,36,44,51 */
    c->wu_zm = -a4*dt4*(15/(2*dz5) - 1/(dz*dx4) + 5/(2*dz3*dx2)) + a2*dt2*(15/(2*dz3) - 1/(dz*dx2));
    c->wu_zp = a4*dt4*(15/(2*dz5) - 1/(dz*dx4) + 5/(2*dz3*dx2)) - a2*dt2*(15/(2*dz3) - 1/(dz*dx2));
    c->wu_dm = a4*dt4*(5/(4*dz3*dx2) - 1/(2*dz*dx4)) + a2*dt2*(1/(2*dz*dx2));    /* j-1 */
    c->wu_dp = -a4*dt4*(5/(4*dz3*dx2) - 1/(2*dz*dx4)) - a2*dt2*(1/(2*dz*dx2));   /* j+1 */
    /* Awv_gen.m:31,38 */
    c->wv_a = a4*dt4/(4*dx3*dz) - a2*dt2/(4*dz*dx);
    c->wv_b = -a4*dt4/(4*dx3*dz) + a2*dt2/(4*dz*dx);
    /* Aww_gen.m:31,38,45,66 */
    c->ww_z = -(3.0/2)*a2*dt2/dz2 + a4*dt4*(5/(2*dz4) + 1/(2*dx2*dz2));
    c->ww_x = a2*dt2/dx2 - 2*a4*dt4/(dz2*dx2);
    c->ww_c = 2 - a2*dt2*(12/dz2 + 2/dx2) + a4*dt4*(10/dz4 + 4/(dx2*dz2));
    c->ww_d = -a4*dt4/(4*dx2*dz2);
}

/* Neighbour read with the reference's zero (omitted) halo. */
static inline double at(const double* F, int nz, int nx, int j, int i)
{
    if (j < 0 || j >= nz || i < 0 || i >= nx) return 0.0;
    return F[j + (size_t)i * nz];
}

/* One MNAD update at (j,i): nF = sum_G A_FG*G - pF - r*(cp) */
static void mnad_point(const og_t* g, const double* v, const double* U, const double* V,
                       const double* W, int j, int i, double out[3])
{
    const int nz = g->nz, nx = g->nx;
    coef_t c;
    coefs(v[j + (size_t)i * nz], g->dx, g->dz, g->dt, &c);
#define Q(F, dj, di) at(F, nz, nx, j + (dj), i + (di))
    double uu = c.uu_zm*Q(U,-1,0) + c.uu_xm*Q(U,0,-1) + c.uu_c*Q(U,0,0) + c.uu_xp*Q(U,0,1) + c.uu_zp*Q(U,1,0)
              + c.uu_d*(Q(U,-1,-1) + Q(U,1,-1) + Q(U,-1,1) + Q(U,1,1));
    double uv = c.uv_xm*Q(V,0,-1) + c.uv_xp*Q(V,0,1) + c.uv_dm*(Q(V,-1,-1) + Q(V,1,-1))
              + c.uv_dp*(Q(V,-1,1) + Q(V,1,1)) + c.uv_x2m*Q(V,0,-2) + c.uv_x2p*Q(V,0,2);
    double uw = c.uw_zp*Q(W,1,0) + c.uw_zm*Q(W,-1,0) + c.uw_dm*(Q(W,-1,-1) + Q(W,-1,1))
              + c.uw_dp*(Q(W,1,-1) + Q(W,1,1)) + c.uw_z2p*Q(W,2,0) + c.uw_z2m*Q(W,-2,0);
    double vv = c.vv_z*(Q(V,-1,0) + Q(V,1,0)) + c.vv_x*(Q(V,0,-1) + Q(V,0,1)) + c.vv_c*Q(V,0,0)
              + c.vv_d*(Q(V,-1,-1) + Q(V,1,-1) + Q(V,-1,1) + Q(V,1,1));
    double vu = c.vu_xm*Q(U,0,-1) + c.vu_xp*Q(U,0,1) + c.vu_dm*(Q(U,-1,-1) + Q(U,1,-1))
              + c.vu_dp*(Q(U,-1,1) + Q(U,1,1));
    double vw = c.vw_a*(Q(W,-1,-1) + Q(W,1,1)) + c.vw_b*(Q(W,1,-1) + Q(W,-1,1));
    double ww = c.ww_z*(Q(W,-1,0) + Q(W,1,0)) + c.ww_x*(Q(W,0,-1) + Q(W,0,1)) + c.ww_c*Q(W,0,0)
              + c.ww_d*(Q(W,-1,-1) + Q(W,1,-1) + Q(W,-1,1) + Q(W,1,1));
    double wu = c.wu_zm*Q(U,-1,0) + c.wu_zp*Q(U,1,0) + c.wu_dm*(Q(U,-1,-1) + Q(U,-1,1))
              + c.wu_dp*(Q(U,1,-1) + Q(U,1,1));
    double wv = c.wv_a*(Q(V,-1,-1) + Q(V,1,1)) + c.wv_b*(Q(V,1,-1) + Q(V,-1,1));
#undef Q
    out[0] = uu + uv + uw;
    out[1] = vv + vu + vw;
    out[2] = ww + wu + wv;
}

/* CPML state: 3 fields x {x,z} x {1,2,3} memory variables, full grid (zero
 * outside the strips, as in the reference). */
typedef struct {
    double* m;  /* [field 3][dir 2][var 3][N] */
    size_t N;
} mem_t;

static inline double* MEM(mem_t* M, int f, int dir, int var) { return M->m + (((size_t)f * 2 + dir) * 3 + var) * M->N; }

/* C_cof.m for one point: side coefficient triple for direction dir (0: x, 1: z).
 * Returns 0 when the point is outside both strips of that direction. */
static int cpml_coef(const og_t* g, double vv, int j, int i, int dir, double* c1, double* c2, double* c3, int* sgn)
{
    const double R = 1e-4;                       /* fwd_PDE_exact_MNAD.m:88 */
    int n = dir == 0 ? g->nx : g->nz;
    int k = dir == 0 ? i : j;
    double h = dir == 0 ? g->dx : g->dz;
    int d = g->d;
    double D = d * h;
    double X;
    if (k < d) { X = D - h * k; *sgn = 1; }            /* left / top: D:-h:h */
    else if (k >= n - d) { X = h * (k - (n - d) + 1); *sgn = -1; }   /* right / bottom */
    else return 0;
    double sig0 = ((3 * log(1 / R)) / (2 * D * D * D)) * vv;
    double sig = sig0 * (X * X);
    double dsig = 2 * sig0 * X;
    double den = 1 + sig * (g->dt / 2);
    *c1 = (1 - sig * (g->dt / 2)) / den;
    *c2 = (dsig * g->dt) / den;
    *c3 = (sig * g->dt) / den;
    return 1;
}

/* Ux123_gen.m / Uz123_gen.m at one point for field F; returns F1 (x or z). */
static double cpml_point(const og_t* g, const double* v, const double* F, mem_t* M, int f, int dir, int j, int i)
{
    double c1, c2, c3;
    int sgn;
    size_t p = j + (size_t)i * g->nz;
    if (!cpml_coef(g, v[p], j, i, dir, &c1, &c2, &c3, &sgn)) return 0.0;
    double Fa, Fd, h;
    if (dir == 0) { Fa = at(F, g->nz, g->nx, j, i + 1); Fd = at(F, g->nz, g->nx, j, i - 1); h = g->dx; }
    else          { Fa = at(F, g->nz, g->nx, j + 1, i); Fd = at(F, g->nz, g->nx, j - 1, i); h = g->dz; }
    double F0 = F[p];
    double gr, lap;
    if (sgn > 0) { gr = Fd - Fa; lap = Fd - 2 * F0 + Fa; }
    else         { gr = Fa - Fd; lap = Fa - 2 * F0 + Fd; }
    double* m1 = MEM(M, f, dir, 0);
    double* m2 = MEM(M, f, dir, 1);
    double* m3 = MEM(M, f, dir, 2);
    m3[p] = c1 * m3[p] + (c2 / (2 * h)) * gr;
    m2[p] = c1 * m2[p] + (c2 / h) * gr + c3 * (lap / (h * h) - m3[p]);
    m1[p] = c1 * m1[p] + (c2 / (2 * h)) * gr + c3 * (2 * lap / (h * h) - m2[p]);
    return m1[p];
}

typedef struct {
    double *pU, *U, *pV, *V, *pW, *W, *nU, *nV, *nW;
    double *cpU, *cpV, *cpW;   /* F1_x + F1_z per field */
    double* r;                 /* V2dt2 */
    mem_t M;
} state_t;

static int state_alloc(state_t* s, const og_t* g, const double* v)
{
    size_t N = (size_t)g->nz * g->nx;
    memset(s, 0, sizeof(*s));
    double** ptrs[] = {&s->pU, &s->U, &s->pV, &s->V, &s->pW, &s->W, &s->nU, &s->nV, &s->nW,
                       &s->cpU, &s->cpV, &s->cpW, &s->r};
    for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); ++k) {
        *ptrs[k] = (double*)calloc(N, sizeof(double));
        if (!*ptrs[k]) return -1;
    }
    s->M.N = N;
    s->M.m = (double*)calloc(N * 18, sizeof(double));
    if (!s->M.m) return -1;
    for (size_t p = 0; p < N; ++p)
        s->r[p] = g->adjoint ? (v[p] * g->dt) * (v[p] * g->dt) : (v[p] * v[p]) * (g->dt * g->dt);
    return 0;
}

static void state_free(state_t* s)
{
    double* ptrs[] = {s->pU, s->U, s->pV, s->V, s->pW, s->W, s->nU, s->nV, s->nW, s->cpU, s->cpV, s->cpW, s->r, s->M.m};
    for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); ++k) free(ptrs[k]);
}

/* CPML memory update for all strip points (uses the fields as they are now). */
static void cpml_all(const og_t* g, const double* v, state_t* s)
{
    const int nz = g->nz, nx = g->nx, d = g->d;
    const double* F[3] = {s->U, s->V, s->W};
    double* cp[3] = {s->cpU, s->cpV, s->cpW};
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < nz; ++j) {
            int strip = (i < d || i >= nx - d || j < d || j >= nz - d);
            if (!strip) continue;
            for (int f = 0; f < 3; ++f) {
                double ax = cpml_point(g, v, F[f], &s->M, f, 0, j, i);
                double az = cpml_point(g, v, F[f], &s->M, f, 1, j, i);
                cp[f][j + (size_t)i * nz] = ax + az;
            }
        }
    }
}

static void stencil_all(const og_t* g, const double* v, state_t* s)
{
    const int nz = g->nz, nx = g->nx;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < nz; ++j) {
            size_t p = j + (size_t)i * nz;
            double o[3];
            mnad_point(g, v, s->U, s->V, s->W, j, i, o);
            s->nU[p] = o[0] - s->pU[p] - s->r[p] * s->cpU[p];
            s->nV[p] = o[1] - s->pV[p] - s->r[p] * s->cpV[p];
            s->nW[p] = o[2] - s->pW[p] - s->r[p] * s->cpW[p];
        }
    }
}

static void rotate(state_t* s)
{
    double* t;
    t = s->pU; s->pU = s->U; s->U = s->nU; s->nU = t;
    t = s->pV; s->pV = s->V; s->V = s->nV; s->nV = t;
    t = s->pW; s->pW = s->W; s->W = s->nW; s->nW = t;
}

/*
 * Forward modeling of one shot (fwd_PDE_exact_MNAD.m:39-168).
 *   v: nz*nx, column-major; zs,xs,zr,xr: 1-based padded indices.
 *   datau/datav/dataw: nt*nr column-major (datav/dataw may be NULL).
 *   indx==1: T>=1 required; UU: nint*ncols (zero-filled here, first k
 *   columns written), illum: nint (multiplied by T, :162).  May be NULL.
 *   keep: optional list of nkeep 1-based steps; keep_out receives
 *   nkeep*3*N values (nU,nV,nW after each listed step).
 * Returns 0, or -1 on bad arguments / allocation failure.
 */
MNAD_ORACLE_EXPORT int mnad_oracle_fwd(int nz, int nx, double dz, double dx, double dt, int d_pml,
    const double* v, int zs, int xs, int nr, const int* zr, const int* xr,
    int nt, const double* w, int indx, int T, int ncols,
    double* datau, double* datav, double* dataw, double* UU, double* illum,
    int nkeep, const int* keep, double* keep_out)
{
    og_t g = {nz, nx, d_pml, dx, dz, dt, 0};
    if (nz < 1 || nx < 1 || nt < 0 || zs < 1 || zs > nz || xs < 1 || xs > nx) return -1;
    for (int r = 0; r < nr; ++r)
        if (zr[r] < 1 || zr[r] > nz || xr[r] < 1 || xr[r] > nx) return -1;
    if (indx == 1 && T < 1) return -1;
    state_t s;
    if (state_alloc(&s, &g, v)) { state_free(&s); return -1; }
    const size_t N = (size_t)nz * nx;
    const int d = d_pml;
    const int niz = nz - 2 * d, nix = nx - 2 * d;
    const size_t nint = (indx == 1) ? (size_t)niz * nix : 0;
    if (indx == 1) {
        if (UU) memset(UU, 0, sizeof(double) * nint * (size_t)ncols);
        if (illum) memset(illum, 0, sizeof(double) * nint);
    }
    const size_t ps = (zs - 1) + (size_t)(xs - 1) * nz;
    int ttt = 0;
    for (int tt = 1; tt <= nt; ++tt) {
        cpml_all(&g, v, &s);                                  /* :95-108  */
        s.U[ps] = s.U[ps] + s.r[ps] * w[tt - 1];              /* :111     */
        stencil_all(&g, v, &s);                               /* :114-116 */
        for (int r = 0; r < nr; ++r) {                        /* :119-123 */
            size_t q = (zr[r] - 1) + (size_t)(xr[r] - 1) * nz;
            datau[(tt - 1) + (size_t)r * nt] = s.U[q];
            if (datav) datav[(tt - 1) + (size_t)r * nt] = s.V[q];
            if (dataw) dataw[(tt - 1) + (size_t)r * nt] = s.W[q];
        }
        if (indx == 1 && tt % T == 0) {                       /* :126-143 */
            for (int i = 0; i < nix; ++i)
                for (int j = 0; j < niz; ++j) {
                    size_t p = (j + d) + (size_t)(i + d) * nz;
                    double d2u;
                    if (tt == 1) d2u = s.nU[p] / (dt * dt);
                    else if (tt == 2) d2u = (s.nU[p] - 2 * s.U[p]) / (dt * dt);
                    else d2u = (s.nU[p] - 2 * s.U[p] + s.pU[p]) / (dt * dt);
                    size_t q = j + (size_t)i * niz;
                    if (UU && ttt < ncols) UU[q + (size_t)ttt * nint] = d2u;
                    if (illum) illum[q] += d2u * d2u;
                }
            ++ttt;
        }
        for (int k = 0; k < nkeep; ++k)
            if (keep[k] == tt) {
                memcpy(keep_out + ((size_t)k * 3 + 0) * N, s.nU, N * sizeof(double));
                memcpy(keep_out + ((size_t)k * 3 + 1) * N, s.nV, N * sizeof(double));
                memcpy(keep_out + ((size_t)k * 3 + 2) * N, s.nW, N * sizeof(double));
            }
        rotate(&s);                                           /* :146-153 */
    }
    if (indx == 1 && illum)
        for (size_t q = 0; q < nint; ++q) illum[q] = T * illum[q];   /* :162 */
    state_free(&s);
    return 0;
}

/*
 * Adjoint propagation + imaging of one shot (Born_adj_MNAD.m:33-138).
 *   data: nt*nr column-major residual; UU: nint*ncols forward snapshots.
 *   pairing 0: reference (column ncols-ttt+1, Born_adj_MNAD.m:128);
 *   pairing 1: aligned (column k-ttt+1, k = floor(nt/T)).
 *   Im: nint output (already multiplied by T, :138).
 */
MNAD_ORACLE_EXPORT int mnad_oracle_adj(int nz, int nx, double dz, double dx, double dt, int d_pml,
    const double* v, int nr, const int* zr, const int* xr, int nt, const double* data,
    const double* UU, int ncols, int T, int pairing, double* Im)
{
    og_t g = {nz, nx, d_pml, dx, dz, dt, 1};
    if (nz < 1 || nx < 1 || nt < 0 || T < 1) return -1;
    for (int r = 0; r < nr; ++r)
        if (zr[r] < 1 || zr[r] > nz || xr[r] < 1 || xr[r] > nx) return -1;
    state_t s;
    if (state_alloc(&s, &g, v)) { state_free(&s); return -1; }
    const int d = d_pml;
    const int niz = nz - 2 * d, nix = nx - 2 * d;
    const size_t nint = (size_t)niz * nix;
    const int k = nt / T;
    memset(Im, 0, sizeof(double) * nint);
    int ttt = 0;
    for (int tt = nt; tt >= 1; --tt) {
        cpml_all(&g, v, &s);                                  /* :88-101  */
        stencil_all(&g, v, &s);                               /* :104-106 */
        for (int r = 0; r < nr; ++r) {                        /* :109-111 */
            size_t q = (zr[r] - 1) + (size_t)(xr[r] - 1) * nz;
            s.U[q] = s.U[q] + s.r[q] * data[(tt - 1) + (size_t)r * nt];
        }
        rotate(&s);                                           /* :116-123 */
        if (tt % T == 0) {                                    /* :127-134 */
            int col = pairing == 0 ? ncols - ttt : k - ttt;   /* 1-based */
            if (col >= 1 && col <= ncols) {
                const double* US = UU + (size_t)(col - 1) * nint;
                #pragma omp parallel for schedule(static)
                for (int i = 0; i < nix; ++i)
                    for (int j = 0; j < niz; ++j) {
                        size_t q = j + (size_t)i * niz;
                        Im[q] = Im[q] + US[q] * s.U[(j + d) + (size_t)(i + d) * nz];
                    }
            }
            ++ttt;
        }
    }
    for (size_t q = 0; q < nint; ++q) Im[q] = T * Im[q];     /* :138 */
    state_free(&s);
    return 0;
}

MNAD_ORACLE_EXPORT int mnad_oracle_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* The nine-operator stencil alone, Sigma_G A_FG*G for F in {U,V,W}, applied
 * to given fields (no pF, no CPML): the matrix-free counterpart of the
 * sparse products in fwd_PDE_exact_MNAD.m:114-116.  For operator tests. */
MNAD_ORACLE_EXPORT void mnad_oracle_apply(int nz, int nx, double dz, double dx, double dt,
    const double* v, const double* U, const double* V, const double* W,
    double* oU, double* oV, double* oW)
{
    og_t g = {nz, nx, 0, dx, dz, dt, 0};
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
            double o[3];
            mnad_point(&g, v, U, V, W, j, i, o);
            size_t p = j + (size_t)i * nz;
            oU[p] = o[0]; oV[p] = o[1]; oW[p] = o[2];
        }
}
