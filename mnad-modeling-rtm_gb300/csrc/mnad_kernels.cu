// MNAD time-step kernels and their small helpers.
//
// step_direct: one fused kernel per time step for a whole batch of
// propagations.  Per point it reads U,V,W (3x3 box, plus x+-2 for V and z+-2
// for W, through the read-only cache), pU,pV,pW and r, and writes nU,nV,nW
// over pU,pV,pW (in-place leapfrog).  In the CPML strips it also updates the
// memory variables of Ux123_gen.m / Uz123_gen.m; the source, the receivers,
// the d2u snapshots + illumination (forward) and the imaging condition
// (adjoint) are fused in as well, so one step is one launch.
#include "mnad_device.cuh"
#include "mnad_kernels.h"

namespace mnad {

// Copy the propagation descriptor of this block into shared memory.
__device__ __forceinline__ void load_desc(PropDesc& dst, const PropDesc* src)
{
    static_assert(sizeof(PropDesc) % 8 == 0, "descriptor copy uses 8-byte words");
    const int n = sizeof(PropDesc) / 8;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nth = blockDim.x * blockDim.y;
    for (int k = tid; k < n; k += nth)
        reinterpret_cast<unsigned long long*>(&dst)[k] = __ldg(reinterpret_cast<const unsigned long long*>(src) + k);
}

// Current time index of a propagation at global step s (1-based tt), or 0
// when it has no work at this step.
__device__ __forceinline__ int step_tt(const PropDesc& P, int s)
{
    if (s >= P.nt) return 0;
    return P.mode == MODE_FWD ? s + 1 : P.nt - s;
}

// CPML contribution (F1_x + F1_z) for the three fields at a strip point.
// u-values are pre-injection (the caller removes the source amount).
__device__ __forceinline__ void cpml_point(const PropDesc& P, int j, int i, float r,
    float u0, float uxm, float uxp, float uzm, float uzp,
    float v0, float vxm, float vxp, float vzm, float vzp,
    float w0, float wxm, float wxp, float wzm, float wzp,
    float& cu, float& cv, float& cw)
{
    const int d = P.d;
    const float vel = sqrtf(r) * P.inv_dt;
    cu = cv = cw = 0.0f;
    if (i < d || i >= P.nx - d) {
        const int side = i < d ? 0 : 1;
        const int k = side ? i - (P.nx - d) : i;
        const float X = side ? float(k + 1) * P.dx : float(d - i) * P.dx;
        float c1, c2, c3;
        cpml_coefs(P.kx, vel, X, P.dt, c1, c2, c3);
        const float inv_h = 1.0f / P.dx;
        const size_t vs = (size_t)d * P.ld;
        float* m = P.mx + ((size_t)(side * 9) * d + k) * P.ld + j;
        const float Fa[3] = {uxp, vxp, wxp}, Fd[3] = {uxm, vxm, wxm}, F0[3] = {u0, v0, w0};
        float out[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            float* mf = m + (size_t)(f * 3) * vs;
            float m1 = mf[0], m2 = mf[vs], m3 = mf[2 * vs];
            const float gr = side ? Fa[f] - Fd[f] : Fd[f] - Fa[f];
            const float lap = (Fd[f] + Fa[f]) - 2.0f * F0[f];
            out[f] = cpml_mem(c1, c2, c3, inv_h, gr, lap, m1, m2, m3);
            mf[0] = m1; mf[vs] = m2; mf[2 * vs] = m3;
        }
        cu += out[0]; cv += out[1]; cw += out[2];
    }
    if (j < d || j >= P.nz - d) {
        const int side = j < d ? 0 : 1;
        const int k = side ? j - (P.nz - d) : j;
        const float X = side ? float(k + 1) * P.dz : float(d - j) * P.dz;
        float c1, c2, c3;
        cpml_coefs(P.kz, vel, X, P.dt, c1, c2, c3);
        const float inv_h = 1.0f / P.dz;
        const size_t vs = (size_t)P.nx * P.dpz;
        float* m = P.mz + ((size_t)(side * 9) * P.nx + i) * P.dpz + k;
        const float Fa[3] = {uzp, vzp, wzp}, Fd[3] = {uzm, vzm, wzm}, F0[3] = {u0, v0, w0};
        float out[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            float* mf = m + (size_t)(f * 3) * vs;
            float m1 = mf[0], m2 = mf[vs], m3 = mf[2 * vs];
            const float gr = side ? Fa[f] - Fd[f] : Fd[f] - Fa[f];
            const float lap = (Fd[f] + Fa[f]) - 2.0f * F0[f];
            out[f] = cpml_mem(c1, c2, c3, inv_h, gr, lap, m1, m2, m3);
            mf[0] = m1; mf[vs] = m2; mf[2 * vs] = m3;
        }
        cu += out[0]; cv += out[1]; cw += out[2];
    }
}

// Everything after the stencil for one point: CPML, source, receivers,
// snapshot/illumination or imaging, store.  Shared by all step kernels.
__device__ __forceinline__ void finish_point(const PropDesc& P, int tt, int tl, int j, int i, size_t p,
    float r, const Hood& h, float su, float sv, float sw,
    float* __restrict__ nU, float* __restrict__ nV, float* __restrict__ nW,
    float pu, float pv, float pw)
{
    const int d = P.d;
    const bool strip = (i < d) | (i >= P.nx - d) | (j < d) | (j >= P.nz - d);
    if (strip) {
        // The CPML sees U before this step's source injection
        // (fwd_PDE_exact_MNAD.m:95-111): the stored U already holds it.
        float u0 = h.u00, uxm = h.uxm, uxp = h.uxp, uzm = h.uzm, uzp = h.uzp;
        if (P.mode == MODE_FWD && P.src >= 0) {
            const float a = P.src_amp[tt - 1];
            const long long ds = (long long)P.src - (long long)p;
            if (ds == 0) u0 -= a;
            else if (ds == -(long long)P.ld) uxm -= a;
            else if (ds == (long long)P.ld) uxp -= a;
            else if (ds == -1) uzm -= a;
            else if (ds == 1) uzp -= a;
        }
        float cu, cv, cw;
        cpml_point(P, j, i, r, u0, uxm, uxp, uzm, uzp,
                   h.v00, h.vxm, h.vxp, h.vzm, h.vzp, h.w00, h.wxm, h.wxp, h.wzm, h.wzp, cu, cv, cw);
        su = fmaf(-r, cu, su);
        sv = fmaf(-r, cv, sv);
        sw = fmaf(-r, cw, sw);
    }
    // nF = F + ((F - pF) + sF): one rounding at the field's magnitude.
    float xu = h.u00 + ((h.u00 - pu) + su);
    const float xv = h.v00 + ((h.v00 - pv) + sv);
    const float xw = h.w00 + ((h.w00 - pw) + sw);
    const bool interior = (i >= d) & (i < P.nx - d) & (j >= d) & (j < P.nz - d);
    const int niz = P.nz - 2 * d;
    if (P.mode == MODE_FWD) {
        if (P.T > 0 && tt % P.T == 0 && interior) {
            // fwd_PDE_exact_MNAD.m:128-141 with nU - 2U + pU = su exactly:
            // tt == 1 keeps nU (= 2U - pU + su), tt == 2 keeps nU - 2U.
            float d2u = su;
            if (tt == 1) d2u = fmaf(2.0f, h.u00, su - pu);
            else if (tt == 2) d2u = su - pu;
            d2u *= P.inv_dt2;
            const size_t q = (size_t)(j - d) + (size_t)(i - d) * niz;
            const size_t nint = (size_t)niz * (P.nx - 2 * d);
            const size_t o = (size_t)(tt / P.T - 1) * nint + q;
            if (P.codec == CODEC_BF16) static_cast<__nv_bfloat16*>(P.snap)[o] = __float2bfloat16_rn(d2u);
            else if (P.codec == CODEC_F16) {
                const float e = d2u * (1.0f / P.snap_scale[tt / P.T - 1]);   // power of two: exact
                if (!(fabsf(e) <= 65504.0f)) atomicOr(P.status, ST_F16_RANGE);
                static_cast<__half*>(P.snap)[o] = __float2half_rn(e);
            } else static_cast<float*>(P.snap)[o] = d2u;
            P.illum[q] = fma((double)d2u, (double)d2u, P.illum[q]);
        }
        if ((long long)p == P.src && tt < P.nt) xu += P.src_amp[tt];   // next step's injection
    } else {
        // Born_adj_MNAD.m:109-111: the residual injected at step tt+1 entered
        // U after that step's update; it reaches this step through -pU.
        if (tt < P.nt) {
            const int beg = __ldg(P.tile_rec + tl), end = __ldg(P.tile_rec + tl + 1);
            for (int k = beg; k < end; ++k)
                if (__ldg(P.rec_pt + k) == (int)p) {
                    const int rr = __ldg(P.rec_id + k);
                    xu -= (float)(__ldg(P.rec_r + k) * __ldg(P.data + (size_t)rr * P.nt + tt));
                }
        }
        if (P.T > 0 && tt % P.T == 0 && interior) {
            // Born_adj_MNAD.m:127-134: pairs column ncols-ttt+1 of UU.
            const int ttt = P.img_steps - tt / P.T;              // 0-based imaging count
            const int col = (P.pairing == PAIR_REFERENCE ? P.ncols : P.nsnap) - ttt;   // 1-based
            if (col >= 1 && col <= P.nsnap) {
                const size_t q = (size_t)(j - d) + (size_t)(i - d) * niz;
                const size_t nint = (size_t)niz * (P.nx - 2 * d);
                const float sc = P.codec == CODEC_F16 ? P.snap_scale[col - 1] : 1.0f;
                const float us = snap_decode(P.snap, P.codec, (size_t)(col - 1) * nint + q, sc);
                P.image[q] = fma((double)us, (double)xu, P.image[q]);
            }
        }
    }
    nU[p] = xu;
    nV[p] = xv;
    nW[p] = xw;
}

// Forward receivers: datau(tt,rr) = U(zr,xr) after the injection and before
// the update (fwd_PDE_exact_MNAD.m:119-123).  Stored U holds exactly that.
__device__ __forceinline__ void record_receivers(const PropDesc& P, int tt, int tl,
    const float* U, const float* V, const float* W)
{
    const int beg = __ldg(P.tile_rec + tl), end = __ldg(P.tile_rec + tl + 1);
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nth = blockDim.x * blockDim.y;
    for (int k = beg + tid; k < end; k += nth) {
        const int pt = __ldg(P.rec_pt + k);
        const size_t o = (size_t)__ldg(P.rec_id + k) * P.nt + (tt - 1);
        const float u = U[pt];
        if (!isfinite(u)) atomicOr(P.status, ST_NONFINITE);
        P.data[o] = u;
        if (P.datav) P.datav[o] = V[pt];
        if (P.dataw) P.dataw[o] = W[pt];
    }
}

__global__ void __launch_bounds__(DIRECT_TZ * DIRECT_TX)
step_direct(const PropDesc* __restrict__ props, const int* __restrict__ tile_prop, int s)
{
    __shared__ __align__(16) PropDesc P;
    const int pi = __ldg(tile_prop + blockIdx.x);
    load_desc(P, props + pi);
    __syncthreads();
    const int tt = step_tt(P, s);
    if (tt == 0) return;
    const int tl = blockIdx.x - P.tile_base;
    const int tz = tl % P.ntz, tx = tl / P.ntz;
    const int j = tz * DIRECT_TZ + threadIdx.x;
    const int i = tx * DIRECT_TX + threadIdx.y;
    const int cur = s & 1;
    const float* __restrict__ U = P.fld[cur][0];
    const float* __restrict__ V = P.fld[cur][1];
    const float* __restrict__ W = P.fld[cur][2];
    float* nU = P.fld[cur ^ 1][0];
    float* nV = P.fld[cur ^ 1][1];
    float* nW = P.fld[cur ^ 1][2];
    if (P.mode == MODE_FWD && P.nr > 0) record_receivers(P, tt, tl, U, V, W);
    if (j >= P.nz || i >= P.nx) return;
    const int ld = P.ld;
    const size_t p = (size_t)(i + HX) * ld + (j + HZ);
    Hood h;
#define LD(F, dj, di) __ldg(F + p + (long long)(di) * ld + (dj))
    h.u00 = LD(U, 0, 0); h.uzm = LD(U, -1, 0); h.uzp = LD(U, 1, 0); h.uxm = LD(U, 0, -1); h.uxp = LD(U, 0, 1);
    h.umm = LD(U, -1, -1); h.upm = LD(U, 1, -1); h.ump = LD(U, -1, 1); h.upp = LD(U, 1, 1);
    h.v00 = LD(V, 0, 0); h.vzm = LD(V, -1, 0); h.vzp = LD(V, 1, 0); h.vxm = LD(V, 0, -1); h.vxp = LD(V, 0, 1);
    h.vmm = LD(V, -1, -1); h.vpm = LD(V, 1, -1); h.vmp = LD(V, -1, 1); h.vpp = LD(V, 1, 1);
    h.vxm2 = LD(V, 0, -2); h.vxp2 = LD(V, 0, 2);
    h.w00 = LD(W, 0, 0); h.wzm = LD(W, -1, 0); h.wzp = LD(W, 1, 0); h.wxm = LD(W, 0, -1); h.wxp = LD(W, 0, 1);
    h.wmm = LD(W, -1, -1); h.wpm = LD(W, 1, -1); h.wmp = LD(W, -1, 1); h.wpp = LD(W, 1, 1);
    h.wzm2 = LD(W, -2, 0); h.wzp2 = LD(W, 2, 0);
#undef LD
    const float r = __ldg(P.r + p);
    const float pu = nU[p], pv = nV[p], pw = nW[p];
    float su, sv, sw;
    mnad_update(P, r, h, su, sv, sw);
    finish_point(P, tt, tl, j, i, p, r, h, su, sv, sw, nU, nV, nW, pu, pv, pw);
}

// r = v^2 dt^2 into padded storage (forward: v.^2.*(dt^2),
// fwd_PDE_exact_MNAD.m:39; adjoint: (v.*dt).^2, Born_adj_MNAD.m:36).
__global__ void build_r(const double* __restrict__ v, int nz, int nx, double dt, int adjoint,
                        float* __restrict__ r, int ld)
{
    const size_t n = (size_t)nz * nx;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(k % nz), i = (int)(k / nz);
        const double a = v[k];
        const double rr = adjoint ? (a * dt) * (a * dt) : (a * a) * (dt * dt);
        r[(size_t)(i + HX) * ld + (j + HZ)] = (float)rr;
    }
}

// U(zs,xs) of the first step holds r_src*w(1) (the injection of tt=1).
__global__ void seed_sources(const PropDesc* __restrict__ props, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const PropDesc& P = props[k];
    if (P.mode == MODE_FWD && P.src >= 0 && P.nt > 0) P.fld[0][0][P.src] = P.src_amp[0];
}

// Snapshot matrix in the reference's layout (Nint x ncols FP64, columns past
// nsnap zero) from the device codec.
__global__ void snap_export(const void* __restrict__ snap, int codec, const float* __restrict__ scale,
                            size_t nint, int nsnap, int ncols, double* __restrict__ out)
{
    const size_t n = nint * (size_t)ncols;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(k / nint);
        double val = 0.0;
        if (c < nsnap) {
            const float sc = (codec == CODEC_F16) ? scale[c] : 1.0f;
            val = (double)snap_decode(snap, codec, k, sc);
        }
        out[k] = val;
    }
}

// Encode FP64 snapshots (the reference's UU matrix) into the device codec.
__global__ void snap_import(const double* __restrict__ in, int codec, const float* __restrict__ scale,
                            size_t nint, int nsnap, void* __restrict__ snap)
{
    const size_t n = nint * (size_t)nsnap;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const float x = (float)in[k];
        if (codec == CODEC_BF16) static_cast<__nv_bfloat16*>(snap)[k] = __float2bfloat16_rn(x);
        else if (codec == CODEC_F16) static_cast<__half*>(snap)[k] = __float2half_rn(x * (1.0f / scale[k / nint]));
        else static_cast<float*>(snap)[k] = x;
    }
}

// Dense FP64 copy (column-major nz x nx) of one field in padded storage;
// `fix` is subtracted at offset `fix_at` (the stored U at the source point
// already holds the next step's injection, which the reference's nU does not).
__global__ void field_export(const float* __restrict__ F, int nz, int nx, int ld, int fix_at, float fix,
                             double* __restrict__ out)
{
    const size_t n = (size_t)nz * nx;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(k % nz), i = (int)(k / nz);
        const int o = (i + HX) * ld + (j + HZ);
        float x = F[o];
        if (o == fix_at) x -= fix;
        out[k] = (double)x;
    }
}

// out[k] = scale * in[k]  (image and illumination carry the factor T of
// Born_adj_MNAD.m:138 and fwd_PDE_exact_MNAD.m:162).
__global__ void scale_f64(const double* __restrict__ in, double s, size_t n, double* __restrict__ out)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        out[k] = s * in[k];
}

}  // namespace mnad

namespace mnad {

// Scattered data of the RTM workflow: data_sct = data - datas
// (main_Acoustic_RTM.m:225), formed on the device.
__global__ void residual_f64(const double* __restrict__ a, const double* __restrict__ b, size_t n,
                             double* __restrict__ out)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        out[k] = a[k] - b[k];
}

}  // namespace mnad
