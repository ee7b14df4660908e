// Pieces shared by the persistent, TMA-fed step kernels (step_tma: one time
// step per pass; step_tma2: two time steps per pass).
//
// Staged fields live in shared memory as columns of BZ = TMA_TZ + 8 rows
// (a tile column plus a 4-row halo above and below): element (row r, column
// c) of field f of a buffer is base[f * FS + c * BZ + r], FS being the
// buffer's field stride.  A thread owns TMA_PZ consecutive rows of one
// column; the helpers below read its register window, evaluate the stencil
// in packed FP32x2 arithmetic, and update the CPML memory variables of those
// points (SRC/MNAD/Ux123_gen.m, Uz123_gen.m).
#pragma once
#include <cuda.h>

#include "mnad_kernels.h"
#include "mnad_point.cuh"

namespace mnad {
namespace tile {

constexpr int BZ = TMA_TZ + 8;     // rows of a staged column (z)
static_assert(TMA_PZ == 4, "a thread covers two z-pairs");
static_assert(TMA_TZY == 16 || TMA_TZY == 32, "a warp spans whole tile columns");
static_assert((BZ * 4) % 16 == 0 && (TMA_TZ * 4) % 16 == 0, "box inner extents must be multiples of 16 bytes");

// ---- mbarrier / bulk-copy primitives (inline PTX) -------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) writes to the same bytes.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// The same test without waiting (returns at once).
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, unsigned parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_addr(dst)), "l"(map), "r"(c0), "r"(c1), "r"(smem_addr(bar))
        : "memory");
}

// A 3-D box: coordinates (c0 innermost, c1, c2).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_addr(dst)), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Bounded wait of at most `limit` polls; gives up early once another thread
// has aborted.  Callers pass the kernel parameter StepArgs::spin_limit itself,
// which stays a constant-bank operand instead of a register held across the
// tile loop.
__device__ __forceinline__ bool wait_bounded(uint64_t* bar, unsigned parity, const volatile int* abort_flag,
                                             const unsigned& limit)
{
    // The first poll does not wait (mbarrier.try_wait may itself wait until
    // the phase completes), so a budget of one poll gives up on any phase
    // still pending.
    if (mbar_test_wait(bar, parity)) return true;
    for (unsigned it = 1; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 1023u) == 1023u && *abort_flag) return false;
    }
    return false;
}

// A CTA that gave up waits (bounded) for the last fill it issued on each of
// its NS stages to land before it exits: a bulk copy must not write into the
// shared memory of an exited CTA.  `nfills` counts the operations that
// completed or will complete a phase of a full barrier (a tile's copies, or
// the arrive of "no tile"); fill f went to stage f % NS, and all but the last
// fill of a stage had completed before the producer could issue the next.
template <int NS>
__device__ __forceinline__ void drain_fills(uint64_t* full, unsigned nfills)
{
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        const unsigned fk = (nfills + (unsigned)(NS - 1 - k)) / NS;     // fills of stage k
        if (fk == 0) continue;
        const unsigned par = (fk - 1u) & 1u;
        for (unsigned it = 0; it < DRAIN_LIMIT && !mbar_try_wait(&full[k], par); ++it) __nanosleep(64);
    }
}

// n / d for 0 <= n < 2^24, d >= 1, from a float reciprocal of d: float(n) is
// exact and the estimate is within 2 of the quotient, which two corrections
// each way make exact (no integer division on the producer's path).
__device__ __forceinline__ int div_small(int n, int d, float inv_d)
{
    int q = (int)((float)n * inv_d);
    q -= q * d > n;
    q -= q * d > n;
    q += (q + 1) * d <= n;
    q += (q + 1) * d <= n;
    return q;
}

// ---- register window and packed stencil arithmetic ------------------------
// TMA_PZ consecutive floats (16-byte aligned) to / from registers.
__device__ __forceinline__ void ldv(const float* p, float* o)
{
    const float4 a = *reinterpret_cast<const float4*>(p);
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
}

__device__ __forceinline__ void stv(float* p, const float* o)
{
    *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
}

// The register window of one thread: rows r0-1 .. r0+PZ of columns c-1 .. c+1
// for U, V, W, plus V at c-2 / c+2 (rows r0 .. r0+PZ-1) and W at rows r0-2
// and r0+PZ+1 of column c, from a buffer of field stride FS.
struct Window {
    static constexpr int R = TMA_PZ + 2;
    float u[3][R], v[3][R], w[3][R], v2m[TMA_PZ], v2p[TMA_PZ], wz[2];
    template <int FS>
    __device__ __forceinline__ void load(const float* base, int c, int r0)
    {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
            const float* fu = base + (c - 1 + cc) * BZ + r0;
            const float* fv = fu + FS;
            const float* fw = fu + 2 * FS;
            u[cc][0] = fu[-1]; ldv(fu, &u[cc][1]); u[cc][R - 1] = fu[TMA_PZ];
            v[cc][0] = fv[-1]; ldv(fv, &v[cc][1]); v[cc][R - 1] = fv[TMA_PZ];
            w[cc][0] = fw[-1]; ldv(fw, &w[cc][1]); w[cc][R - 1] = fw[TMA_PZ];
        }
        ldv(base + FS + (c - 2) * BZ + r0, v2m);
        ldv(base + FS + (c + 2) * BZ + r0, v2p);
        wz[0] = base[2 * FS + c * BZ + r0 - 2];
        wz[1] = base[2 * FS + c * BZ + r0 + TMA_PZ + 1];
    }
};

// Packed FP32x2 arithmetic (one instruction for two z-points).  Each lane is
// the IEEE operation of the scalar form, so results do not depend on the
// packing.
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 psub(float2 a, float2 b)
{
    unsigned long long x = *reinterpret_cast<unsigned long long*>(&a);
    unsigned long long y = *reinterpret_cast<unsigned long long*>(&b), z;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(z) : "l"(x), "l"(y));
    return *reinterpret_cast<float2*>(&z);
}
__device__ __forceinline__ float2 pr(float a, float b) { return make_float2(a, b); }

// The stencil sums su, sv, sw (see mnad_update) of the 4 points of a thread,
// as two z-pairs (points 0,1 and 2,3).  Side columns enter through their
// row sums S = F(c-1) + F(c+1) and differences D = F(c-1) - F(c+1), shared
// between rows: e.g. the diagonal sum of point k is S[k] + S[k+2] and the odd
// diagonal of Avu_gen.m is D[k] + D[k+2].  Per point the operations, their
// order and their rounding are those of mnad_update.
__device__ __forceinline__ void mnad_update_pairs(const Coefs2& K, const Window& win, const float* rr, float2* su,
                                                  float2* sv, float2* sw)
{
    const float2* a = K.alpha;
    const float2* b = K.beta;
    const float* U = win.u[1];
    const float* V = win.v[1];
    const float* W = win.w[1];
    // row sums / differences of the side columns: rows 1..4 as pairs, rows 0 and 5 alone
    float2 SUp[2], DUp[2], SVp[2], DVp[2], SWp[2], DWp[2];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int r = 1 + 2 * m;
        SUp[m] = padd(pr(win.u[0][r], win.u[0][r + 1]), pr(win.u[2][r], win.u[2][r + 1]));
        DUp[m] = psub(pr(win.u[0][r], win.u[0][r + 1]), pr(win.u[2][r], win.u[2][r + 1]));
        SVp[m] = padd(pr(win.v[0][r], win.v[0][r + 1]), pr(win.v[2][r], win.v[2][r + 1]));
        DVp[m] = psub(pr(win.v[0][r], win.v[0][r + 1]), pr(win.v[2][r], win.v[2][r + 1]));
        SWp[m] = padd(pr(win.w[0][r], win.w[0][r + 1]), pr(win.w[2][r], win.w[2][r + 1]));
        DWp[m] = psub(pr(win.w[0][r], win.w[0][r + 1]), pr(win.w[2][r], win.w[2][r + 1]));
    }
    float SU[6], DU[6], SV[6], DV[6], SW[6], DW[6];
    SU[0] = win.u[0][0] + win.u[2][0]; DU[0] = win.u[0][0] - win.u[2][0];
    SV[0] = win.v[0][0] + win.v[2][0]; DV[0] = win.v[0][0] - win.v[2][0];
    SW[0] = win.w[0][0] + win.w[2][0]; DW[0] = win.w[0][0] - win.w[2][0];
    SU[5] = win.u[0][5] + win.u[2][5]; DU[5] = win.u[0][5] - win.u[2][5];
    SV[5] = win.v[0][5] + win.v[2][5]; DV[5] = win.v[0][5] - win.v[2][5];
    SW[5] = win.w[0][5] + win.w[2][5]; DW[5] = win.w[0][5] - win.w[2][5];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        SU[1 + 2 * m] = SUp[m].x; SU[2 + 2 * m] = SUp[m].y; DU[1 + 2 * m] = DUp[m].x; DU[2 + 2 * m] = DUp[m].y;
        SV[1 + 2 * m] = SVp[m].x; SV[2 + 2 * m] = SVp[m].y; DV[1 + 2 * m] = DVp[m].x; DV[2 + 2 * m] = DVp[m].y;
        SW[1 + 2 * m] = SWp[m].x; SW[2 + 2 * m] = SWp[m].y; DW[1 + 2 * m] = DWp[m].x; DW[2 + 2 * m] = DWp[m].y;
    }
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int k = 2 * m;              // points k, k+1 (window rows k+1, k+2)
        const float2 r = pr(rr[k], rr[k + 1]);
        const float2 q = pmul(r, r);
        const float2 u0 = pr(U[k + 1], U[k + 2]), v0 = pr(V[k + 1], V[k + 2]), w0 = pr(W[k + 1], W[k + 2]);
        const float2 u2 = padd(u0, u0), v2 = padd(v0, v0), w2 = padd(w0, w0);
        const float2 uzs = pr(U[k] + U[k + 2], U[k + 1] + U[k + 3]);
        const float2 vzs = pr(V[k] + V[k + 2], V[k + 1] + V[k + 3]);
        const float2 wzs = pr(W[k] + W[k + 2], W[k + 1] + W[k + 3]);
        // U combinations (Auu, Avu, Awu)
        const float2 dUz = psub(uzs, u2), dUx = psub(SUp[m], u2);
        const float2 dUd = psub(pr(SU[k] + SU[k + 2], SU[k + 1] + SU[k + 3]), padd(u2, u2));
        const float2 uLx = DUp[m], uLz = pr(U[k] - U[k + 2], U[k + 1] - U[k + 3]);
        const float2 uDx = pr(DU[k] + DU[k + 2], DU[k + 1] + DU[k + 3]);
        const float2 uDz = pr(SU[k] - SU[k + 2], SU[k + 1] - SU[k + 3]);
        // V combinations (Avv, Auv, Awv); vX1 and vDx enter with negative sign
        const float2 dVz = psub(vzs, v2), dVx = psub(SVp[m], v2);
        const float2 dVd = psub(pr(SV[k] + SV[k + 2], SV[k + 1] + SV[k + 3]), padd(v2, v2));
        const float2 nvX1 = DVp[m], nvDx = pr(DV[k] + DV[k + 2], DV[k + 1] + DV[k + 3]);
        const float2 vX2 = psub(pr(win.v2m[k], win.v2m[k + 1]), pr(win.v2p[k], win.v2p[k + 1]));
        const float2 vXZ = pr(DV[k] - DV[k + 2], DV[k + 1] - DV[k + 3]);
        // W combinations (Aww, Auw, Avw)
        const float2 wzm2 = m == 0 ? pr(win.wz[0], W[0]) : pr(W[1], W[2]);
        const float2 wzp2 = m == 0 ? pr(W[3], W[4]) : pr(W[5], win.wz[1]);
        const float2 dWz = psub(wzs, w2), dWx = psub(SWp[m], w2);
        const float2 dWd = psub(pr(SW[k] + SW[k + 2], SW[k + 1] + SW[k + 3]), padd(w2, w2));
        const float2 wZ1 = pr(W[k + 2] - W[k], W[k + 3] - W[k + 1]);
        const float2 wDz = pr(SW[k + 2] - SW[k], SW[k + 3] - SW[k + 1]);
        const float2 wZ2 = psub(wzm2, wzp2), wXZ = pr(DW[k] - DW[k + 2], DW[k + 1] - DW[k + 3]);
        // nU row
        float2 ra = pmul(a[K_UU_Z], dUz);
        ra = pfma(a[K_UU_X], dUx, ra);
        ra = pfma(a[K_UV_X1], nvX1, ra);       // negated pair
        ra = pfma(a[K_UV_X2], vX2, ra);
        ra = pfma(a[K_UW_Z1], wZ1, ra);
        ra = pfma(a[K_UW_Z2], wZ2, ra);
        float2 qa = pmul(b[K_UU_Z], dUz);
        qa = pfma(b[K_UU_X], dUx, qa);
        qa = pfma(b[K_UU_D], dUd, qa);
        qa = pfma(b[K_UV_X1], nvX1, qa);       // negated pair
        qa = pfma(b[K_UV_D], nvDx, qa);        // negated pair
        qa = pfma(b[K_UV_X2], vX2, qa);
        qa = pfma(b[K_UW_Z1], wZ1, qa);
        qa = pfma(b[K_UW_D], wDz, qa);
        qa = pfma(b[K_UW_Z2], wZ2, qa);
        su[m] = pfma(q, qa, pmul(r, ra));
        // nV row
        float2 rb = pmul(a[K_VV_Z], dVz);
        rb = pfma(a[K_VV_X], dVx, rb);
        rb = pfma(a[K_VV_R], v0, rb);
        rb = pfma(a[K_VU_X1], uLx, rb);
        rb = pfma(a[K_VU_D], uDx, rb);
        rb = pfma(a[K_VW], wXZ, rb);
        float2 qb = pmul(b[K_VV_Z], dVz);
        qb = pfma(b[K_VV_X], dVx, qb);
        qb = pfma(b[K_VV_D], dVd, qb);
        qb = pfma(b[K_VV_R], v0, qb);
        qb = pfma(b[K_VU_X1], uLx, qb);
        qb = pfma(b[K_VU_D], uDx, qb);
        qb = pfma(b[K_VW], wXZ, qb);
        sv[m] = pfma(q, qb, pmul(r, rb));
        // nW row
        float2 rc = pmul(a[K_WW_Z], dWz);
        rc = pfma(a[K_WW_X], dWx, rc);
        rc = pfma(a[K_WW_R], w0, rc);
        rc = pfma(a[K_WU_Z1], uLz, rc);
        rc = pfma(a[K_WU_D], uDz, rc);
        rc = pfma(a[K_WV], vXZ, rc);
        float2 qc = pmul(b[K_WW_Z], dWz);
        qc = pfma(b[K_WW_X], dWx, qc);
        qc = pfma(b[K_WW_D], dWd, qc);
        qc = pfma(b[K_WW_R], w0, qc);
        qc = pfma(b[K_WU_Z1], uLz, qc);
        qc = pfma(b[K_WU_D], uDz, qc);
        qc = pfma(b[K_WV], vXZ, qc);
        sw[m] = pfma(q, qc, pmul(r, rc));
    }
}

// ---- receivers ------------------------------------------------------------
// Forward receiver sampling (fwd_PDE_exact_MNAD.m:119-123) of the entries
// rbeg..rend of a tile from a staged buffer of field stride FS whose column 0
// holds grid column i0 - col0 and whose row 0 holds grid row j0 - 4: the
// buffer holds U, V, W after this step's injection and before its update.
template <int FS>
__device__ __forceinline__ void record_tile(const PropDesc& P, const float* base, int col0, int tt, int rbeg, int rend,
                                            int j0, int i0)
{
    for (int e = rbeg + (int)threadIdx.x; e < rend; e += (int)blockDim.x) {
        const int pt = __ldg(P.rec_pt + e);
        const int ic = pt / P.ld, jr = pt - ic * P.ld;              // storage column / row
        const int cx = ic - HX - i0 + col0, rz = jr - HZ - j0 + 4;  // position in the buffer
        const size_t o = (size_t)__ldg(P.rec_id + e) * P.nt + (tt - 1);
        const float u = base[cx * BZ + rz];
        if (!isfinite(u)) atomicOr(P.status, ST_NONFINITE);
        P.data[o] = u;
        if (P.datav) P.datav[o] = base[FS + cx * BZ + rz];
        if (P.dataw) P.dataw[o] = base[2 * FS + cx * BZ + rz];
    }
}

// Adjoint receiver injection r*data(tt+1) of the TMA_PZ points p.. of local
// column c of receiver-bucket tile tl: only the entries of that column are
// scanned, in entry order, so receivers at one point add up in the order of
// the whole list.  The amounts come from the propagation's injection table
// (row tt), so an entry costs two independent loads.
__device__ __forceinline__ void injection(const PropDesc& P, int tt, int tl, int c, int p, float* inj)
{
    const int cb = __ldg(P.col_rec + tl * TMA_TX + c), ce = __ldg(P.col_rec + tl * TMA_TX + c + 1);
    const float* row = P.inj + (size_t)tt * P.nr;
    for (int e = cb; e < ce; ++e) {
        const int k = __ldg(P.rec_pt + e) - p;
        const float x = __ldg(row + e);
        if (k < 0 || k >= TMA_PZ) continue;
#pragma unroll
        for (int q = 0; q < TMA_PZ; ++q)
            if (q == k) inj[q] += x;
    }
}

// ---- CPML ---------------------------------------------------------------
// C_cof.m:6-16 at a z-pair of points: (c1, c2, c3) of a side from the
// velocities and the distance terms X (X = 0 outside the strip gives exactly
// 1, 0, 0), in packed FP32x2.  An approximate reciprocal is used for these
// damping coefficients only.
struct CpmlC {
    float2 c1, c2, c3;
};
__device__ __forceinline__ CpmlC cpml_c2(float K, float2 vel, float2 X, float dt)
{
    const float2 s0 = pmul(pr(K, K), vel);
    const float2 sig = pmul(s0, pmul(X, X));
    const float2 a = pmul(sig, pr(0.5f * dt, 0.5f * dt));
    const float2 den = padd(pr(1.0f, 1.0f), a);
    const float2 inv = pr(__fdividef(1.0f, den.x), __fdividef(1.0f, den.y));
    CpmlC c;
    c.c1 = pmul(psub(pr(1.0f, 1.0f), a), inv);
    c.c2 = pmul(pmul(pmul(pmul(pr(2.0f, 2.0f), s0), X), pr(dt, dt)), inv);
    c.c3 = pmul(pmul(sig, pr(dt, dt)), inv);
    return c;
}

// One side of Ux123_gen.m / Uz123_gen.m for one field at a z-pair of points
// (cpml_mem of the per-point kernels, in packed FP32x2): gr = (behind -
// ahead) on the low side, (ahead - behind) on the high side; lap = behind -
// 2 F + ahead.  Updates m1..m3 in place, returns the new m1.
__device__ __forceinline__ float2 cpml_mem2(const CpmlC& c, float2 ih, float2 ih2, float2 gr, float2 lap, float2& m1,
                                            float2& m2, float2& m3)
{
    const float2 g2 = pmul(pmul(c.c2, ih), gr);
    const float2 hg = pmul(pr(0.5f, 0.5f), g2);
    m3 = pfma(c.c1, m3, hg);
    m2 = padd(pfma(c.c1, m2, g2), pmul(c.c3, pfma(lap, ih2, pr(-m3.x, -m3.y))));
    m1 = padd(pfma(c.c1, m1, hg), pmul(c.c3, pfma(pmul(pr(2.0f, 2.0f), lap), ih2, pr(-m2.x, -m2.y))));
    return m1;
}

// Memory-variable storage of one bank: x strips [side 2][var 9][d][ld],
// z strips [side 2][var 9][nx][dpz].
struct MemBank {
    float* mx;
    float* mz;
};

// L2 prefetch of the memory variables that cpml_vec will read for the
// TMA_PZ points j.. of column i: issued when a general tile starts, so that
// their DRAM latency overlaps the stencil arithmetic.
__device__ __forceinline__ void prefetch_strip_state(const PropDesc& P, MemBank m, int j, int i)
{
    constexpr int Q = TMA_PZ;
    const int d = P.d, nz = P.nz, nx = P.nx, ld = P.ld;
    if (i < d || i >= nx - d) {
        const int side = i < d ? 0 : 1;
        const int kx = side ? i - (nx - d) : i;
        const float* b = m.mx + ((side * 9) * d + kx) * ld + j;
#pragma unroll
        for (int v = 0; v < 9; ++v) asm volatile("prefetch.global.L2 [%0];" ::"l"(b + v * (d * ld)));
    }
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        if (side == 0 ? !(j < d) : !(j + Q - 1 >= nz - d)) continue;
        const int k0 = side ? j - P.zb0 : j;
        const float* b = m.mz + ((side * 9) * nx + i) * P.dpz + k0;
#pragma unroll
        for (int v = 0; v < 9; ++v) asm volatile("prefetch.global.L2 [%0];" ::"l"(b + v * (nx * P.dpz)));
    }
}

// Ux123_gen.m / Uz123_gen.m for the TMA_PZ points j.. of column i (one
// thread), vectorized over the points: the memory variables of a field and
// side are TMA_PZ consecutive, aligned floats.  The fields come from column c,
// rows r0.., of a staged buffer of field stride FS.  Memory variables are read
// from bank `rd` and, when `store`, written to bank `wr` (the same bank for a
// kernel that advances one step per pass).  Adds F1_x + F1_z of U, V, W into
// cu, cv, cw (as the z-pairs of points 0,1 and 2,3; packed FP32x2 throughout).
// U is taken before this step's source injection (fwd_PDE_exact_MNAD.m:95-111):
// the staged U already holds it.
template <int FS>
__device__ __forceinline__ void cpml_vec(const PropDesc& P, const float* fbase, int c, int r0, int tt, int j, int i,
                                         int p, bool has_src, const float* r, MemBank rd, MemBank wr, bool store,
                                         float2* cu, float2* cv, float2* cw)
{
    constexpr int Q = TMA_PZ;
    const int d = P.d, nz = P.nz, nx = P.nx, ld = P.ld;
    if (d <= 0) return;                 // no CPML strips (and no memory-variable storage)
    float2 vel[2];
#pragma unroll
    for (int m = 0; m < 2; ++m)
        vel[m] = pmul(pmul(pr(r[2 * m], r[2 * m + 1]), pr(rsqrtf(r[2 * m]), rsqrtf(r[2 * m + 1]))),
                      pr(P.inv_dt, P.inv_dt));
    const float srcamp = (has_src && P.mode == MODE_FWD && P.src >= 0) ? P.src_amp[tt - 1] : 0.0f;
    const int src = P.src;
    // One field's term of one direction: F0 at the points, Fa / Fd ahead /
    // behind along the direction (staged, pre-injection values); mv holds
    // m1, m2, m3 of the 4 points and is updated in place.
    auto field = [&](int f, int side, const CpmlC* cc, float2 ih, float2 ih2, const float* F0, const float* Fa,
                     const float* Fd, float* mv) {
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const float2 f0 = pr(F0[2 * m], F0[2 * m + 1]), fa = pr(Fa[2 * m], Fa[2 * m + 1]),
                         fd = pr(Fd[2 * m], Fd[2 * m + 1]);
            const float2 gr = side ? psub(fa, fd) : psub(fd, fa);
            const float2 lap = psub(padd(fd, fa), pmul(pr(2.0f, 2.0f), f0));
            float2 m1 = pr(mv[2 * m], mv[2 * m + 1]);
            float2 m2 = pr(mv[Q + 2 * m], mv[Q + 2 * m + 1]);
            float2 m3 = pr(mv[2 * Q + 2 * m], mv[2 * Q + 2 * m + 1]);
            const float2 o = cpml_mem2(cc[m], ih, ih2, gr, lap, m1, m2, m3);
            if (f == 0) cu[m] = padd(cu[m], o); else if (f == 1) cv[m] = padd(cv[m], o); else cw[m] = padd(cw[m], o);
            mv[2 * m] = m1.x; mv[2 * m + 1] = m1.y;
            mv[Q + 2 * m] = m2.x; mv[Q + 2 * m + 1] = m2.y;
            mv[2 * Q + 2 * m] = m3.x; mv[2 * Q + 2 * m + 1] = m3.y;
        }
    };
    // x direction: the whole column lies in the strip
    if (i < d || i >= nx - d) {
        const int side = i < d ? 0 : 1;
        const int kx = side ? i - (nx - d) : i;
        const float X = side ? float(kx + 1) * P.dx : float(d - i) * P.dx;
        const float inv_h = 1.0f / P.dx;
        const float2 ih = pr(inv_h, inv_h), ih2 = pmul(ih, ih);
        CpmlC cc[2];
#pragma unroll
        for (int m = 0; m < 2; ++m) cc[m] = cpml_c2(P.kx, vel[m], pr(X, X), P.dt);
        const int vs = d * ld;
        const int off = ((side * 9) * d + kx) * ld + j;
        const float* rbase = rd.mx + off;
        float* wbase = wr.mx + off;
        // the next field's memory variables are loaded before this field's
        // stores (which the compiler must assume could alias them)
        float nm[3 * Q];
#pragma unroll
        for (int v = 0; v < 3; ++v) ldv(rbase + v * vs, &nm[v * Q]);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            float F0v[Q], Fav[Q], Fdv[Q];
            const float* col = fbase + f * FS + c * BZ + r0;
            ldv(col, F0v);
            ldv(col + BZ, Fav);
            ldv(col - BZ, Fdv);
            float mv[3 * Q];
#pragma unroll
            for (int k = 0; k < 3 * Q; ++k) mv[k] = nm[k];
            if (f < 2) {
#pragma unroll
                for (int v = 0; v < 3; ++v) ldv(rbase + (f * 3 + 3 + v) * vs, &nm[v * Q]);
            }
            if (f == 0 && srcamp != 0.0f) {
#pragma unroll
                for (int k = 0; k < Q; ++k) {
                    if (src == p + k) F0v[k] -= srcamp;
                    if (src == p + k + ld) Fav[k] -= srcamp;
                    if (src == p + k - ld) Fdv[k] -= srcamp;
                }
            }
            field(f, side, cc, ih, ih2, F0v, Fav, Fdv, mv);
            if (store) {
                float* mw = wbase + (f * 3) * vs;
                stv(mw, &mv[0]);
                stv(mw + vs, &mv[Q]);
                stv(mw + 2 * vs, &mv[2 * Q]);
            }
        }
    }
    // z direction: the top and/or bottom strip may cover part of the group
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        // the group j..j+Q-1 (j < nz) must overlap the strip rows [0, d) or [nz-d, nz)
        if (side == 0 ? !(j < d) : !(j + Q - 1 >= nz - d)) continue;
        const int k0 = side ? j - P.zb0 : j;
        const float inv_h = 1.0f / P.dz;
        const float2 ih = pr(inv_h, inv_h), ih2 = pmul(ih, ih);
        float X[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const int jk = j + k;
            X[k] = 0.0f;                                     // outside: c = (1, 0, 0)
            if (side == 0 && jk < d) X[k] = float(d - jk) * P.dz;
            if (side == 1 && jk >= nz - d && jk < nz) X[k] = float(jk - (nz - d) + 1) * P.dz;
        }
        CpmlC cc[2];
#pragma unroll
        for (int m = 0; m < 2; ++m) cc[m] = cpml_c2(P.kz, vel[m], pr(X[2 * m], X[2 * m + 1]), P.dt);
        const int vs = nx * P.dpz;
        const int off = ((side * 9) * nx + i) * P.dpz + k0;
        const float* rbase = rd.mz + off;
        float* wbase = wr.mz + off;
        float nm[3 * Q];
#pragma unroll
        for (int v = 0; v < 3; ++v) ldv(rbase + v * vs, &nm[v * Q]);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const float* col = fbase + f * FS + c * BZ + r0;
            float Fc[Q + 2];
            Fc[0] = col[-1];
            ldv(col, &Fc[1]);
            Fc[Q + 1] = col[Q];
            float mv[3 * Q];
#pragma unroll
            for (int k = 0; k < 3 * Q; ++k) mv[k] = nm[k];
            if (f < 2) {
#pragma unroll
                for (int v = 0; v < 3; ++v) ldv(rbase + (f * 3 + 3 + v) * vs, &nm[v * Q]);
            }
            float F0v[Q], Fav[Q], Fdv[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) { F0v[k] = Fc[k + 1]; Fav[k] = Fc[k + 2]; Fdv[k] = Fc[k]; }
            if (f == 0 && srcamp != 0.0f) {
#pragma unroll
                for (int k = 0; k < Q; ++k) {
                    if (src == p + k) F0v[k] -= srcamp;
                    if (src == p + k + 1) Fav[k] -= srcamp;
                    if (src == p + k - 1) Fdv[k] -= srcamp;
                }
            }
            field(f, side, cc, ih, ih2, F0v, Fav, Fdv, mv);
            if (store) {
                float* mw = wbase + (f * 3) * vs;
                stv(mw, &mv[0]);
                stv(mw + vs, &mv[Q]);
                stv(mw + 2 * vs, &mv[2 * Q]);
            }
        }
    }
}

}  // namespace tile
}  // namespace mnad
