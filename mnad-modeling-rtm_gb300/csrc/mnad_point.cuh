// Per-point pieces shared by the step kernels (descriptor staging, CPML,
// source/receivers, snapshots and imaging).
#pragma once
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
// when it has no work at this step (outside its window [s_begin, s_end) or
// its nt steps).  The local step is s - s_off; s_off is even, so the time
// level s & 1 is the same for every propagation of a launch.
__device__ __forceinline__ int step_tt(const PropDesc& P, int s)
{
    if (s < P.s_begin || s >= P.s_end) return 0;
    s -= P.s_off;
    if (s < 0 || s >= P.nt) return 0;
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
        // every load before the first store (the stores could alias them as
        // far as the compiler knows, which would serialise the three fields)
        float mv[9];
#pragma unroll
        for (int v = 0; v < 9; ++v) mv[v] = m[(size_t)v * vs];
        float out[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            float* mf = m + (size_t)(f * 3) * vs;
            float m1 = mv[3 * f], m2 = mv[3 * f + 1], m3 = mv[3 * f + 2];
            const float gr = side ? Fa[f] - Fd[f] : Fd[f] - Fa[f];
            const float lap = (Fd[f] + Fa[f]) - 2.0f * F0[f];
            out[f] = cpml_mem(c1, c2, c3, inv_h, gr, lap, m1, m2, m3);
            mf[0] = m1; mf[vs] = m2; mf[2 * vs] = m3;
        }
        cu += out[0]; cv += out[1]; cw += out[2];
    }
    if (j < d || j >= P.nz - d) {
        const int side = j < d ? 0 : 1;
        const int k = side ? j - P.zb0 : j;      // storage slot (zb0 is nz - d rounded down to 4)
        const float X = side ? float(j - (P.nz - d) + 1) * P.dz : float(d - j) * P.dz;
        float c1, c2, c3;
        cpml_coefs(P.kz, vel, X, P.dt, c1, c2, c3);
        const float inv_h = 1.0f / P.dz;
        const size_t vs = (size_t)P.nx * P.dpz;
        float* m = P.mz + ((size_t)(side * 9) * P.nx + i) * P.dpz + k;
        const float Fa[3] = {uzp, vzp, wzp}, Fd[3] = {uzm, vzm, wzm}, F0[3] = {u0, v0, w0};
        // every load before the first store (the stores could alias them as
        // far as the compiler knows, which would serialise the three fields)
        float mv[9];
#pragma unroll
        for (int v = 0; v < 9; ++v) mv[v] = m[(size_t)v * vs];
        float out[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            float* mf = m + (size_t)(f * 3) * vs;
            float m1 = mv[3 * f], m2 = mv[3 * f + 1], m3 = mv[3 * f + 2];
            const float gr = side ? Fa[f] - Fd[f] : Fd[f] - Fa[f];
            const float lap = (Fd[f] + Fa[f]) - 2.0f * F0[f];
            out[f] = cpml_mem(c1, c2, c3, inv_h, gr, lap, m1, m2, m3);
            mf[0] = m1; mf[vs] = m2; mf[2 * vs] = m3;
        }
        cu += out[0]; cv += out[1]; cw += out[2];
    }
}

// Everything after the stencil for one point: CPML, source, receiver
// injection, snapshot/illumination or imaging.  Shared by all step kernels.
// `inj` is the adjoint's receiver injection of step tt+1 at this point.
// Returns the new values in xu, xv, xw (the caller stores them).
__device__ __forceinline__ void finish_point(const PropDesc& P, int tt, int j, int i, size_t p,
    float r, const Hood& h, float su, float sv, float sw, float pu, float pv, float pw, float inj,
    float& xu_out, float& xv_out, float& xw_out)
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
            const int slot = P.snap_stage ? 0 : tt / P.T - 1 - P.snap_col0;
            if ((P.snap_flags & SNAP_WRITE) && slot >= 0 && slot < P.snap_cols) {
                const size_t o = (size_t)slot * nint + q;
                if (P.codec == CODEC_BF16) static_cast<__nv_bfloat16*>(P.snap)[o] = __float2bfloat16_rn(d2u);
                else static_cast<float*>(P.snap)[o] = d2u;   // FP32, or the FP16 codec's staging slot
            }
            if (P.snap_flags & SNAP_ILLUM) accumulate_product(&P.illum[q], d2u, d2u);
        }
        if ((long long)p == P.src && tt < P.nt) xu += P.src_amp[tt];   // next step's injection
    } else {
        // Born_adj_MNAD.m:109-111: the residual injected at step tt+1 entered
        // U after that step's update; it reaches this step through -pU.
        xu -= inj;
        if (P.T > 0 && tt % P.T == 0 && interior) {
            // Born_adj_MNAD.m:127-134: pairs column ncols-ttt+1 of UU.
            const int ttt = P.img_steps - tt / P.T;              // 0-based imaging count
            const int col = (P.pairing == PAIR_REFERENCE ? P.ncols : P.nsnap) - ttt;   // 1-based
            const int slot = col - 1 - P.snap_col0;
            if (col >= 1 && col <= P.nsnap && slot >= 0 && slot < P.snap_cols) {
                const size_t q = (size_t)(j - d) + (size_t)(i - d) * niz;
                const size_t nint = (size_t)niz * (P.nx - 2 * d);
                const float sc = P.codec == CODEC_F16 ? P.snap_scale[col - 1] : 1.0f;
                const float us = snap_decode(P.snap, P.codec, (size_t)slot * nint + q, sc);
                accumulate_product(&P.image[q], us, xu);
            }
        }
    }
    xu_out = xu;
    xv_out = xv;
    xw_out = xw;
}

// Forward receivers: datau(tt,rr) = U(zr,xr) after the injection and before
// the update (fwd_PDE_exact_MNAD.m:119-123).  Stored U holds exactly that.
// The block records the entries of the DIRECT_TX bucket columns from `cb`
// whose row lies in its DIRECT_TZ rows from j0.
__device__ __forceinline__ void record_receivers(const PropDesc& P, int tt, int cb, int j0,
    const float* U, const float* V, const float* W)
{
    const int beg = __ldg(P.col_rec + cb), end = __ldg(P.col_rec + cb + DIRECT_TX);
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nth = blockDim.x * blockDim.y;
    for (int k = beg + tid; k < end; k += nth) {
        const int pt = __ldg(P.rec_pt + k);
        const int row = pt % P.ld - HZ;
        if (row < j0 || row >= j0 + DIRECT_TZ) continue;
        const size_t o = (size_t)__ldg(P.rec_id + k) * P.nt + (tt - 1);
        const float u = U[pt];
        if (!isfinite(u)) atomicOr(P.status, ST_NONFINITE);
        P.data[o] = u;
        if (P.datav) P.datav[o] = V[pt];
        if (P.dataw) P.dataw[o] = W[pt];
    }
}

// Adjoint receiver injection r*data(tt+1) summed over the entries of bucket
// column `c` that sit at storage offset p (duplicated receivers add up).
__device__ __forceinline__ float adjoint_injection(const PropDesc& P, int tt, int c, size_t p)
{
    float inj = 0.0f;
    if (P.mode != MODE_ADJ || tt >= P.nt) return inj;
    const int beg = __ldg(P.col_rec + c), end = __ldg(P.col_rec + c + 1);
    const float* row = P.inj + (size_t)tt * P.nr;
    for (int k = beg; k < end; ++k)
        if (__ldg(P.rec_pt + k) == (int)p) inj += __ldg(row + k);
    return inj;
}

}  // namespace mnad
