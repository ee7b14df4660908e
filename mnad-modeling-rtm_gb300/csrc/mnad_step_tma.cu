// step_tma: persistent, TMA-pipelined MNAD time step.
//
// A grid of at most TMA_CTAS_PER_SM CTAs per SM works through the flat tile
// list of a launch group (one geometry, so tile t maps arithmetically to its
// propagation and origin).  Tiles are claimed dynamically from a per-launch
// counter, since strip tiles cost more than interior ones.
//
// Each CTA keeps TMA_STAGES tiles in flight.  For a tile, thread 0 (the
// producer) fills one shared-memory stage with a single mbarrier
// transaction: 2-D bulk tensor copies of U, V, W of the current time level as
// TMA_TZ+8 x TMA_TX+4 boxes (tile plus a 4-row / 2-column halo) and of pU, pV,
// pW, r as TMA_TZ x TMA_TX boxes, plus 1-D bulk copies of the propagation's
// descriptor and the tile's metadata.  Consumers (all TMA_THREADS threads,
// thread 0 included) wait on that stage's "full" barrier, compute the tile
// (each thread TMA_PZ consecutive z points of one column, a register window
// along z; a warp covers 32 x TMA_PZ rows of one column) and write nU, nV, nW
// with vector stores over pU, pV, pW; each warp then
// arrives on the stage's "empty" barrier.  Only the producer waits for
// "empty" before refilling the stage, so no global-memory latency and no
// CTA-wide barrier sits on the consumers' path; the producer's own tile
// claim is an atomic issued one tile ahead.
//
// Interior points take a lean path; CPML strip points add the memory-
// variable updates of Ux123_gen.m / Uz123_gen.m.
//
// No copy starts at a negative coordinate: the padded storage has a zero
// halo of HZ = 4 rows and HX = 2 columns, so the halo box of the tile at
// point (j0, i0) starts at storage (j0, i0) and the point box at
// (j0 + 4, i0 + 2); j0 is a multiple of TMA_TZ, so the innermost coordinate
// times 4 bytes is a multiple of 16.  Boxes past the end of the array are
// zero-filled, which is the reference's omitted out-of-grid neighbour.  Every
// wait is bounded (StepArgs::spin_limit polls); a wait that runs out sets
// ST_TIMEOUT in the launch's status word, and the CTA leaves only after the
// last copy it issued on each stage has landed (itself a bounded wait).
#include <cuda.h>

#include <cstddef>

#include "mnad_kernels.h"
#include "mnad_point.cuh"

namespace mnad {

namespace {

constexpr int BZ = TMA_TZ + 8;     // halo box rows (z)
constexpr int BX = TMA_TX + 4;     // halo box columns (x)

struct __align__(128) Stage {
    float halo[3][BX][BZ];         // U, V, W with halo
    float pts[4][TMA_TX][TMA_TZ];  // pU, pV, pW, r
    PropDesc desc;                 // the tile's propagation
    int4 info;                     // receiver bucket begin/end, flags, j0 | i0 << 16
};
constexpr unsigned FIELD_BYTES = sizeof(float) * (3 * BX * BZ + 4 * TMA_TX * TMA_TZ);
constexpr unsigned STAGE_BYTES = FIELD_BYTES + sizeof(PropDesc) + sizeof(int4);
static_assert(offsetof(Stage, desc) == FIELD_BYTES, "descriptor follows the field boxes");
static_assert(sizeof(PropDesc) % 16 == 0, "bulk copies move multiples of 16 bytes");
static_assert(TMA_PZ == 2 || TMA_PZ == 4, "vector accesses cover 2 or 4 consecutive z points");
static_assert(TMA_TZY == 16 || TMA_TZY == 32, "a warp spans whole tile columns");
static_assert((BZ * 4) % 16 == 0 && (TMA_TZ * 4) % 16 == 0, "box inner extents must be multiples of 16 bytes");

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

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_addr(dst)), "l"(map), "r"(c0), "r"(c1), "r"(smem_addr(bar))
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
// has aborted.
__device__ __forceinline__ bool wait_bounded(uint64_t* bar, unsigned parity, const volatile int* abort_flag,
                                             unsigned limit)
{
    for (unsigned it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 1023u) == 1023u && *abort_flag) return false;
    }
    return false;
}

// Thread 0: fill `stage` with tile t of the launch (one transaction).
__device__ __forceinline__ void issue_tile(const StepArgs& A, int t, Stage& st, uint64_t* bar, int cur)
{
    const int pi = t / A.tiles_per_prop;
    const int tl = t - pi * A.tiles_per_prop;
    const int j0 = (tl % A.ntz) * TMA_TZ, i0 = (tl / A.ntz) * TMA_TX;
    const CUtensorMap* maps = static_cast<const CUtensorMap*>(A.tmaps) + (size_t)pi * TMAPS_PER_PROP;
    mbar_expect_tx(bar, STAGE_BYTES);
    bulk_load(&st.desc, A.props + pi, sizeof(PropDesc), bar);
    bulk_load(&st.info, A.tile_info + t, sizeof(int4), bar);
#pragma unroll
    for (int f = 0; f < 3; ++f) tma_load_2d(&st.halo[f][0][0], maps + TMAP_HALO + cur * 3 + f, bar, j0, i0);
#pragma unroll
    for (int f = 0; f < 3; ++f)
        tma_load_2d(&st.pts[f][0][0], maps + TMAP_POINT + (cur ^ 1) * 3 + f, bar, j0 + HZ, i0 + HX);
    tma_load_2d(&st.pts[3][0][0], maps + TMAP_R, bar, j0 + HZ, i0 + HX);
}

// TMA_PZ consecutive floats (8- or 16-byte aligned) to / from registers.
__device__ __forceinline__ void ldv(const float* p, float* o)
{
    if constexpr (TMA_PZ == 4) {
        const float4 a = *reinterpret_cast<const float4*>(p);
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    } else {
        const float2 a = *reinterpret_cast<const float2*>(p);
        o[0] = a.x; o[1] = a.y;
    }
}

__device__ __forceinline__ void stv(float* p, const float* o)
{
    if constexpr (TMA_PZ == 4) *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
    else *reinterpret_cast<float2*>(p) = make_float2(o[0], o[1]);
}

// The register window of one thread: rows r0-1 .. r0+PZ of columns c-1 .. c+1
// for U, V, W, plus V at c-2 / c+2 (rows r0 .. r0+PZ-1) and W at rows r0-2
// and r0+PZ+1 of column c.
struct Window {
    static constexpr int R = TMA_PZ + 2;
    float u[3][R], v[3][R], w[3][R], v2m[TMA_PZ], v2p[TMA_PZ], wz[2];
    __device__ __forceinline__ void load(const Stage& st, int c, int r0)
    {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
            const float* fu = &st.halo[0][c - 1 + cc][r0];
            const float* fv = &st.halo[1][c - 1 + cc][r0];
            const float* fw = &st.halo[2][c - 1 + cc][r0];
            u[cc][0] = fu[-1]; ldv(fu, &u[cc][1]); u[cc][R - 1] = fu[TMA_PZ];
            v[cc][0] = fv[-1]; ldv(fv, &v[cc][1]); v[cc][R - 1] = fv[TMA_PZ];
            w[cc][0] = fw[-1]; ldv(fw, &w[cc][1]); w[cc][R - 1] = fw[TMA_PZ];
        }
        ldv(&st.halo[1][c - 2][r0], v2m);
        ldv(&st.halo[1][c + 2][r0], v2p);
        wz[0] = st.halo[2][c][r0 - 2];
        wz[1] = st.halo[2][c][r0 + TMA_PZ + 1];
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
    static_assert(TMA_PZ == 4, "two z-pairs per thread");
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

// Forward receiver sampling (fwd_PDE_exact_MNAD.m:119-123) of the entries
// rbeg..rend of a tile, read from the stage: its halo boxes hold the current
// U, V, W of every point of the tile.
__device__ __forceinline__ void record_tile(const PropDesc& P, const Stage& st, int tt, int rbeg, int rend, int j0,
                                            int i0)
{
    for (int e = rbeg + (int)threadIdx.x; e < rend; e += TMA_THREADS) {
        const int pt = __ldg(P.rec_pt + e);
        const int ic = pt / P.ld, jr = pt - ic * P.ld;          // storage column / row
        const int cx = ic - HX - i0 + 2, rz = jr - HZ - j0 + 4; // position in the halo box
        const size_t o = (size_t)__ldg(P.rec_id + e) * P.nt + (tt - 1);
        const float u = st.halo[0][cx][rz];
        if (!isfinite(u)) atomicOr(P.status, ST_NONFINITE);
        P.data[o] = u;
        if (P.datav) P.datav[o] = st.halo[1][cx][rz];
        if (P.dataw) P.dataw[o] = st.halo[2][cx][rz];
    }
}

// Adjoint receiver injection r*data(tt+1) of the TMA_PZ points p.. of local
// column c of tile tl: only the entries of that column are scanned, in entry
// order, so receivers at one point add up in the order of the whole list.
__device__ __forceinline__ void injection(const PropDesc& P, int tt, int tl, int c, int p, float* inj)
{
    const int cb = __ldg(P.col_rec + tl * TMA_TX + c), ce = __ldg(P.col_rec + tl * TMA_TX + c + 1);
    for (int e = cb; e < ce; ++e) {
        const int k = __ldg(P.rec_pt + e) - p;
        if (k < 0 || k >= TMA_PZ) continue;
        const float x = (float)(__ldg(P.rec_r + e) * __ldg(P.data + (size_t)__ldg(P.rec_id + e) * P.nt + tt));
#pragma unroll
        for (int q = 0; q < TMA_PZ; ++q)
            if (q == k) inj[q] += x;
    }
}

}  // namespace

// C_cof.m:6-16 at one point: (c1, c2, c3) of a side from the distance term X
// (X = 0 outside the strip gives exactly 1, 0, 0).  Approximate reciprocal and
// square root are used for these damping coefficients only.
__device__ __forceinline__ void cpml_c(float K, float vel, float X, float dt, float& c1, float& c2, float& c3)
{
    const float s0 = K * vel;
    const float sig = s0 * (X * X);
    const float a = sig * (0.5f * dt);
    const float inv = __fdividef(1.0f, 1.0f + a);
    c1 = (1.0f - a) * inv;
    c2 = (2.0f * s0 * X) * dt * inv;
    c3 = (sig * dt) * inv;
}

// L2 prefetch of the memory variables that cpml_vec will read and write for
// the TMA_PZ points j.. of column i: issued when a general tile starts, so
// that their DRAM latency overlaps the stencil arithmetic.
__device__ __forceinline__ void prefetch_strip_state(const PropDesc& P, int j, int i)
{
    constexpr int Q = TMA_PZ;
    const int d = P.d, nz = P.nz, nx = P.nx, ld = P.ld;
    if (i < d || i >= nx - d) {
        const int side = i < d ? 0 : 1;
        const int kx = side ? i - (nx - d) : i;
        const float* m = P.mx + ((side * 9) * d + kx) * ld + j;
#pragma unroll
        for (int v = 0; v < 9; ++v) asm volatile("prefetch.global.L2 [%0];" ::"l"(m + v * (d * ld)));
    }
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        if (side == 0 ? !(j < d) : !(j + Q - 1 >= nz - d)) continue;
        const int k0 = side ? j - P.zb0 : j;
        const float* m = P.mz + ((side * 9) * nx + i) * P.dpz + k0;
#pragma unroll
        for (int v = 0; v < 9; ++v) asm volatile("prefetch.global.L2 [%0];" ::"l"(m + v * (nx * P.dpz)));
    }
}

// Ux123_gen.m / Uz123_gen.m for the TMA_PZ points j.. of column i (one
// thread), vectorized over the points: the memory variables of a field and
// side are TMA_PZ consecutive, aligned floats.  Adds F1_x + F1_z of
// U, V, W into cu, cv, cw.  U is taken before this step's source injection
// (fwd_PDE_exact_MNAD.m:95-111): the stored U already holds it.
__device__ __forceinline__ void cpml_vec(const PropDesc& P, const Stage& st, int c, int r0, int tt, int j, int i,
                                         int p, bool has_src, const float* r, float* cu, float* cv, float* cw)
{
    constexpr int Q = TMA_PZ;
    const int d = P.d, nz = P.nz, nx = P.nx, ld = P.ld;
    float vel[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) vel[k] = r[k] * rsqrtf(r[k]) * P.inv_dt;
    const float srcamp = (has_src && P.mode == MODE_FWD && P.src >= 0) ? P.src_amp[tt - 1] : 0.0f;
    const int src = P.src;
    if (d <= 0) return;                 // no CPML strips (and no memory-variable storage)
    // x direction: the whole column lies in the strip
    if (i < d || i >= nx - d) {
        const int side = i < d ? 0 : 1;
        const int kx = side ? i - (nx - d) : i;
        const float X = side ? float(kx + 1) * P.dx : float(d - i) * P.dx;
        const float inv_h = 1.0f / P.dx;
        float c1[Q], c2[Q], c3[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) cpml_c(P.kx, vel[k], X, P.dt, c1[k], c2[k], c3[k]);
        const int vs = d * ld;
        float* base = P.mx + ((side * 9) * d + kx) * ld + j;
        // the next field's memory variables are loaded before this field's
        // stores (which the compiler must assume could alias them)
        float nm[3][Q];
#pragma unroll
        for (int v = 0; v < 3; ++v) ldv(base + v * vs, nm[v]);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            float F0v[Q], Fav[Q], Fdv[Q];
            ldv(&st.halo[f][c][r0], F0v);
            ldv(&st.halo[f][c + 1][r0], Fav);
            ldv(&st.halo[f][c - 1][r0], Fdv);
            float* m = base + (f * 3) * vs;
            float m1[Q], m2[Q], m3[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) { m1[k] = nm[0][k]; m2[k] = nm[1][k]; m3[k] = nm[2][k]; }
            if (f < 2) {
#pragma unroll
                for (int v = 0; v < 3; ++v) ldv(m + (3 + v) * vs, nm[v]);
            }
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                float F0 = F0v[k], Fa = Fav[k], Fd = Fdv[k];
                if (f == 0 && srcamp != 0.0f) {
                    if (src == p + k) F0 -= srcamp;
                    if (src == p + k + ld) Fa -= srcamp;
                    if (src == p + k - ld) Fd -= srcamp;
                }
                const float gr = side ? Fa - Fd : Fd - Fa;
                const float lap = (Fd + Fa) - 2.0f * F0;
                const float o = cpml_mem(c1[k], c2[k], c3[k], inv_h, gr, lap, m1[k], m2[k], m3[k]);
                if (f == 0) cu[k] += o; else if (f == 1) cv[k] += o; else cw[k] += o;
            }
            stv(m, m1);
            stv(m + vs, m2);
            stv(m + 2 * vs, m3);
        }
    }
    // z direction: the top and/or bottom strip may cover part of the group
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        // the group j..j+Q-1 (j < nz) must overlap the strip rows [0, d) or [nz-d, nz)
        if (side == 0 ? !(j < d) : !(j + Q - 1 >= nz - d)) continue;
        const int k0 = side ? j - P.zb0 : j;
        const float inv_h = 1.0f / P.dz;
        float c1[Q], c2[Q], c3[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const int jk = j + k;
            float X = 0.0f;                                  // outside: c = (1, 0, 0)
            if (side == 0 && jk < d) X = float(d - jk) * P.dz;
            if (side == 1 && jk >= nz - d && jk < nz) X = float(jk - (nz - d) + 1) * P.dz;
            cpml_c(P.kz, vel[k], X, P.dt, c1[k], c2[k], c3[k]);
        }
        const int vs = nx * P.dpz;
        float* base = P.mz + ((side * 9) * nx + i) * P.dpz + k0;
        float nm[3][Q];
#pragma unroll
        for (int v = 0; v < 3; ++v) ldv(base + v * vs, nm[v]);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const float* col = &st.halo[f][c][r0];
            float Fc[Q + 2];
            Fc[0] = col[-1];
            ldv(col, &Fc[1]);
            Fc[Q + 1] = col[Q];
            float* m = base + (f * 3) * vs;
            float m1[Q], m2[Q], m3[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) { m1[k] = nm[0][k]; m2[k] = nm[1][k]; m3[k] = nm[2][k]; }
            if (f < 2) {
#pragma unroll
                for (int v = 0; v < 3; ++v) ldv(m + (3 + v) * vs, nm[v]);
            }
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                float F0 = Fc[k + 1], Fa = Fc[k + 2], Fd = Fc[k];
                if (f == 0 && srcamp != 0.0f) {
                    if (src == p + k) F0 -= srcamp;
                    if (src == p + k + 1) Fa -= srcamp;
                    if (src == p + k - 1) Fd -= srcamp;
                }
                const float gr = side ? Fa - Fd : Fd - Fa;
                const float lap = (Fd + Fa) - 2.0f * F0;
                const float o = cpml_mem(c1[k], c2[k], c3[k], inv_h, gr, lap, m1[k], m2[k], m3[k]);
                if (f == 0) cu[k] += o; else if (f == 1) cv[k] += o; else cw[k] += o;
            }
            stv(m, m1);
            stv(m + vs, m2);
            stv(m + 2 * vs, m3);
        }
    }
}

// Shared-memory layout: TMA_STAGES stages, their full and empty barriers,
// the tile held by each stage, the abort flag.
constexpr size_t OFF_FULL = TMA_STAGES * sizeof(Stage);
constexpr size_t OFF_EMPTY = OFF_FULL + TMA_STAGES * sizeof(uint64_t);
constexpr size_t OFF_TILE = OFF_EMPTY + TMA_STAGES * sizeof(uint64_t);
constexpr size_t OFF_FLAG = OFF_TILE + TMA_STAGES * sizeof(int);
constexpr int NWARPS = TMA_THREADS / 32;

__global__ void __launch_bounds__(TMA_THREADS, TMA_CTAS_PER_SM) step_tma(const __grid_constant__ StepArgs A)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Stage* stages = reinterpret_cast<Stage*>(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + OFF_FULL);
    uint64_t* empty = reinterpret_cast<uint64_t*>(smem_raw + OFF_EMPTY);
    volatile int* stage_tile = reinterpret_cast<volatile int*>(smem_raw + OFF_TILE);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem_raw + OFF_FLAG);
    const int tid = threadIdx.x, lane = tid & 31;
    if (smem_addr(smem_raw) & 127u) {       // TMA destinations need aligned stages
        if (tid == 0 && A.ntiles > 0) atomicOr(A.status, ST_TIMEOUT);
        return;
    }
    const int cur = A.s & 1;
    const unsigned limit = A.spin_limit ? A.spin_limit : SPIN_LIMIT_DEFAULT;
    int next_claim = -1;                    // producer: tile claimed one refill ahead
    // producer: operations that complete a phase of each stage's full barrier
    // (a tile's copies, or the arrive of "no tile"); the last of them is the
    // only one that can still be in flight
    unsigned fills[TMA_STAGES];
#pragma unroll
    for (int k = 0; k < TMA_STAGES; ++k) fills[k] = 0;
    if (tid == 0) {
        for (int k = 0; k < TMA_STAGES; ++k) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], NWARPS);
        }
        fence_mbar_init();
        *abort_flag = 0;
        for (int k = 0; k < TMA_STAGES; ++k) {
            const int t = atomicAdd(A.tile_counter, 1);
            stage_tile[k] = t < A.ntiles ? t : -1;
        }
        next_claim = atomicAdd(A.tile_counter, 1);
    }
    __syncthreads();
    if (tid == 0)
#pragma unroll
        for (int k = 0; k < TMA_STAGES; ++k) {
            if (stage_tile[k] >= 0) issue_tile(A, stage_tile[k], stages[k], &full[k], cur);
            else mbar_arrive(&full[k]);     // releases the consumers: no tile
            fills[k] = 1;
        }
    const int tzt = tid % TMA_TZY, txt = tid / TMA_TZY;
    const int c = txt + 2, r0 = tzt * TMA_PZ + 4;
    bool producing = true;

    for (int n = 0;; ++n) {
        const int sidx = n % TMA_STAGES;
        const unsigned parity = (unsigned)(n / TMA_STAGES) & 1u;
        // the warp leaves together if any of its lanes' waits ran out (no
        // lane may be left behind at a warp-wide synchronisation)
        if (!__all_sync(0xffffffffu, wait_bounded(&full[sidx], parity, abort_flag, limit))) {
            if (lane == 0 && atomicExch((int*)abort_flag, 1) == 0) atomicOr(A.status, ST_TIMEOUT);
            break;
        }
        const int t = stage_tile[sidx];      // written before the producer's arrive
        if (t < 0) break;
        const Stage& st = stages[sidx];
        const PropDesc& P = st.desc;
        const int4 info = st.info;
        // Per-tile scalars in registers.
        const int tt = step_tt(P, A.s);
        const int j0 = info.w & 0xffff, i0 = info.w >> 16;
        const int tl = j0 / TMA_TZ + (i0 / TMA_TX) * P.ntz;
        const int nz = P.nz, nx = P.nx, d = P.d, ld = P.ld, nt = P.nt, mode = P.mode;
        if (tt != 0 && (info.z & TILE_RECEIVERS) && mode == MODE_FWD) record_tile(P, st, tt, info.x, info.y, j0, i0);
        const int j = j0 + tzt * TMA_PZ;
        const int i = i0 + txt;
        // tt / T and tt % T without an integer division: (tt + 0.5) / T is
        // never within 0.5/T of an integer, far beyond float rounding.
        const int tq = (int)(((float)tt + 0.5f) * P.invT);
        const bool snap_step = P.T > 0 && tt - tq * P.T == 0;
        // A plain tile (image region only, no source, no receivers, no
        // snapshot or imaging at this step) is stencil arithmetic and stores.
        // At snapshot / imaging steps (from tt = 3 on) a plain tile also stores its
        // snapshot and illumination (forward) or adds its image term (adjoint).
        const bool plain = !(info.z & (TILE_STRIP | TILE_RECEIVERS | TILE_SOURCE)) && (!snap_step || tt > 2);
        if (tt != 0 && plain) {
            constexpr int Q = TMA_PZ;
            float rr[Q];
            ldv(&st.pts[3][txt][tzt * Q], rr);
            const int p = (i + HX) * ld + (j + HZ);
            float2 su[2], sv[2], sw[2];
            {
                Window win;
                win.load(st, c, r0);
                mnad_update_pairs(A.coef2, win, rr, su, sv, sw);
            }
            const float4 pu = *reinterpret_cast<const float4*>(&st.pts[0][txt][tzt * Q]);
            const float4 pv = *reinterpret_cast<const float4*>(&st.pts[1][txt][tzt * Q]);
            const float4 pw = *reinterpret_cast<const float4*>(&st.pts[2][txt][tzt * Q]);
            const float4 uc = *reinterpret_cast<const float4*>(&st.halo[0][c][r0]);
            const float4 vc = *reinterpret_cast<const float4*>(&st.halo[1][c][r0]);
            const float4 wc = *reinterpret_cast<const float4*>(&st.halo[2][c][r0]);
            // nF = F + ((F - pF) + sF)
            const float2 u01 = pr(uc.x, uc.y), u23 = pr(uc.z, uc.w);
            const float2 v01 = pr(vc.x, vc.y), v23 = pr(vc.z, vc.w);
            const float2 w01 = pr(wc.x, wc.y), w23 = pr(wc.z, wc.w);
            const float2 nu01 = padd(u01, padd(psub(u01, pr(pu.x, pu.y)), su[0]));
            const float2 nu23 = padd(u23, padd(psub(u23, pr(pu.z, pu.w)), su[1]));
            const float2 nv01 = padd(v01, padd(psub(v01, pr(pv.x, pv.y)), sv[0]));
            const float2 nv23 = padd(v23, padd(psub(v23, pr(pv.z, pv.w)), sv[1]));
            const float2 nw01 = padd(w01, padd(psub(w01, pr(pw.x, pw.y)), sw[0]));
            const float2 nw23 = padd(w23, padd(psub(w23, pr(pw.z, pw.w)), sw[1]));
            *reinterpret_cast<float4*>(P.fld[cur ^ 1][0] + p) = make_float4(nu01.x, nu01.y, nu23.x, nu23.y);
            *reinterpret_cast<float4*>(P.fld[cur ^ 1][1] + p) = make_float4(nv01.x, nv01.y, nv23.x, nv23.y);
            *reinterpret_cast<float4*>(P.fld[cur ^ 1][2] + p) = make_float4(nw01.x, nw01.y, nw23.x, nw23.y);
            if (snap_step) {
                const int niz = nz - 2 * d;
                const size_t nint = (size_t)niz * (nx - 2 * d);
                const size_t q0 = (size_t)(j - d) + (size_t)(i - d) * niz;
                if (mode == MODE_FWD) {
                    // fwd_PDE_exact_MNAD.m:128-141 for tt > 2: d2u = nU - 2U + pU = su
                    const float d2u[Q] = {su[0].x * P.inv_dt2, su[0].y * P.inv_dt2, su[1].x * P.inv_dt2,
                                          su[1].y * P.inv_dt2};
                    const int slot = P.snap_stage ? 0 : tq - 1 - P.snap_col0;
                    if ((P.snap_flags & SNAP_WRITE) && slot >= 0 && slot < P.snap_cols) {
                        const size_t o = (size_t)slot * nint + q0;
#pragma unroll
                        for (int k = 0; k < Q; ++k) {
                            if (P.codec == CODEC_BF16)
                                static_cast<__nv_bfloat16*>(P.snap)[o + k] = __float2bfloat16_rn(d2u[k]);
                            else static_cast<float*>(P.snap)[o + k] = d2u[k];
                        }
                    }
                    if (P.snap_flags & SNAP_ILLUM) {
#pragma unroll
                        for (int k = 0; k < Q; ++k)
                            P.illum[q0 + k] = fma((double)d2u[k], (double)d2u[k], P.illum[q0 + k]);
                    }
                } else {
                    // Born_adj_MNAD.m:127-134
                    int col = (P.pairing == PAIR_REFERENCE ? P.ncols : P.nsnap) - (P.img_steps - tq);
                    if (col >= 1 && col <= P.nsnap && col - 1 >= P.snap_col0 && col - 1 - P.snap_col0 < P.snap_cols) {
                        const float sc = P.codec == CODEC_F16 ? P.snap_scale[col - 1] : 1.0f;
                        const size_t o = (size_t)(col - 1 - P.snap_col0) * nint + q0;
                        const float ou[Q] = {nu01.x, nu01.y, nu23.x, nu23.y};
#pragma unroll
                        for (int k = 0; k < Q; ++k) {
                            const float us = snap_decode(P.snap, P.codec, o + k, sc);
                            P.image[q0 + k] = fma((double)us, (double)ou[k], P.image[q0 + k]);
                        }
                    }
                }
            }
        } else if (tt != 0 && j < nz && i < nx) {
            constexpr int Q = TMA_PZ;
            float rr[Q];
            ldv(&st.pts[3][txt][tzt * Q], rr);
            const int p = (i + HX) * ld + (j + HZ);
            const int rbeg = info.x, rend = info.y;
            const bool adj_inj = mode == MODE_ADJ && tt < nt && rbeg < rend;
            const bool has_src = (info.z & TILE_SOURCE) != 0;
            const int niz = nz - 2 * d;
            const size_t nint = (size_t)niz * (nx - 2 * d);
            const long long q0 = (long long)(j - d) + (long long)(i - d) * niz;
            // imaging column of this step (Born_adj_MNAD.m:128), 0 when none
            int col = 0;
            if (mode == MODE_ADJ && snap_step) {
                col = (P.pairing == PAIR_REFERENCE ? P.ncols : P.nsnap) - (P.img_steps - tq);
                if (col < 1 || col > P.nsnap || col - 1 < P.snap_col0 || col - 1 - P.snap_col0 >= P.snap_cols) col = 0;
            }
            const int src = P.src;
            const float src_next = (has_src && mode == MODE_FWD && src >= p && src < p + Q && tt < nt)
                                       ? P.src_amp[tt] : 0.0f;
            // lean: every point of the group inside the image region (no CPML, no edge)
            const bool lean = i >= d && i < nx - d && j >= d && j + Q - 1 < nz - d;
            float2 s2u[2], s2v[2], s2w[2];
            if (!lean && d > 0) prefetch_strip_state(P, j, i);
            {
                Window win;            // dies here: later phases re-read the stage
                win.load(st, c, r0);
                mnad_update_pairs(A.coef2, win, rr, s2u, s2v, s2w);
            }
            if (!lean) {
                float cu[Q], cv[Q], cw[Q];
#pragma unroll
                for (int k = 0; k < Q; ++k) cu[k] = cv[k] = cw[k] = 0.0f;
                cpml_vec(P, st, c, r0, tt, j, i, p, has_src, rr, cu, cv, cw);
                // sF -= r * (F1_x + F1_z), per point fmaf(-r, c, s)
#pragma unroll
                for (int m = 0; m < 2; ++m) {
                    const float2 nr = pr(-rr[2 * m], -rr[2 * m + 1]);
                    s2u[m] = pfma(nr, pr(cu[2 * m], cu[2 * m + 1]), s2u[m]);
                    s2v[m] = pfma(nr, pr(cv[2 * m], cv[2 * m + 1]), s2v[m]);
                    s2w[m] = pfma(nr, pr(cw[2 * m], cw[2 * m + 1]), s2w[m]);
                }
            }
            const float4 pu4 = *reinterpret_cast<const float4*>(&st.pts[0][txt][tzt * Q]);
            const float4 pv4 = *reinterpret_cast<const float4*>(&st.pts[1][txt][tzt * Q]);
            const float4 pw4 = *reinterpret_cast<const float4*>(&st.pts[2][txt][tzt * Q]);
            const float4 uc4 = *reinterpret_cast<const float4*>(&st.halo[0][c][r0]);
            const float4 vc4 = *reinterpret_cast<const float4*>(&st.halo[1][c][r0]);
            const float4 wc4 = *reinterpret_cast<const float4*>(&st.halo[2][c][r0]);
            // nF = F + ((F - pF) + sF)
            const float2 nu01 = padd(pr(uc4.x, uc4.y), padd(psub(pr(uc4.x, uc4.y), pr(pu4.x, pu4.y)), s2u[0]));
            const float2 nu23 = padd(pr(uc4.z, uc4.w), padd(psub(pr(uc4.z, uc4.w), pr(pu4.z, pu4.w)), s2u[1]));
            const float2 nv01 = padd(pr(vc4.x, vc4.y), padd(psub(pr(vc4.x, vc4.y), pr(pv4.x, pv4.y)), s2v[0]));
            const float2 nv23 = padd(pr(vc4.z, vc4.w), padd(psub(pr(vc4.z, vc4.w), pr(pv4.z, pv4.w)), s2v[1]));
            const float2 nw01 = padd(pr(wc4.x, wc4.y), padd(psub(pr(wc4.x, wc4.y), pr(pw4.x, pw4.y)), s2w[0]));
            const float2 nw23 = padd(pr(wc4.z, wc4.w), padd(psub(pr(wc4.z, wc4.w), pr(pw4.z, pw4.w)), s2w[1]));
            float ou[Q] = {nu01.x, nu01.y, nu23.x, nu23.y};
            float ov[Q] = {nv01.x, nv01.y, nv23.x, nv23.y};
            float ow[Q] = {nw01.x, nw01.y, nw23.x, nw23.y};
            const float su[Q] = {s2u[0].x, s2u[0].y, s2u[1].x, s2u[1].y};
            const float pu[Q] = {pu4.x, pu4.y, pu4.z, pu4.w};
            const float uc[Q] = {uc4.x, uc4.y, uc4.z, uc4.w};
            if (mode == MODE_FWD) {
                if (snap_step) {
#pragma unroll
                    for (int k = 0; k < Q; ++k) {
                        const int jk = j + k;
                        if (!(jk >= d && jk < nz - d && i >= d && i < nx - d)) continue;
                        // fwd_PDE_exact_MNAD.m:128-141; nU - 2U + pU = su
                        float d2u = su[k];
                        if (tt == 1) d2u = fmaf(2.0f, uc[k], su[k] - pu[k]);
                        else if (tt == 2) d2u = su[k] - pu[k];
                        d2u *= P.inv_dt2;
                        const size_t q = (size_t)(q0 + k);
                        const int slot = P.snap_stage ? 0 : tq - 1 - P.snap_col0;
                        if ((P.snap_flags & SNAP_WRITE) && slot >= 0 && slot < P.snap_cols) {
                            const size_t o = (size_t)slot * nint + q;
                            if (P.codec == CODEC_BF16)
                                static_cast<__nv_bfloat16*>(P.snap)[o] = __float2bfloat16_rn(d2u);
                            else static_cast<float*>(P.snap)[o] = d2u;
                        }
                        if (P.snap_flags & SNAP_ILLUM) P.illum[q] = fma((double)d2u, (double)d2u, P.illum[q]);
                    }
                }
                if (src_next != 0.0f) {
#pragma unroll
                    for (int k = 0; k < Q; ++k)
                        if (p + k == src) ou[k] += src_next;
                }
            } else {
                if (adj_inj) {
                    float inj[Q];
#pragma unroll
                    for (int k = 0; k < Q; ++k) inj[k] = 0.0f;
                    injection(P, tt, tl, txt, p, inj);
#pragma unroll
                    for (int k = 0; k < Q; ++k) ou[k] -= inj[k];
                }
                if (col) {
#pragma unroll
                    for (int k = 0; k < Q; ++k) {
                        const int jk = j + k;
                        if (!(jk >= d && jk < nz - d && i >= d && i < nx - d)) continue;
                        const size_t q = (size_t)(q0 + k);
                        const float sc = P.codec == CODEC_F16 ? P.snap_scale[col - 1] : 1.0f;
                        const float us = snap_decode(P.snap, P.codec, (size_t)(col - 1 - P.snap_col0) * nint + q, sc);
                        P.image[q] = fma((double)us, (double)ou[k], P.image[q]);
                    }
                }
            }
            if (j + Q > nz) {
#pragma unroll
                for (int k = 0; k < Q; ++k)
                    if (j + k >= nz) ou[k] = ov[k] = ow[k] = 0.0f;   // rows past nz are the zero halo
            }
            stv(P.fld[cur ^ 1][0] + p, ou);
            stv(P.fld[cur ^ 1][1] + p, ov);
            stv(P.fld[cur ^ 1][2] + p, ow);
        }
        // This warp is done with the stage.
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[sidx]);
        bool gave_up = false;
        if (tid == 0 && producing) {
            // Refill the stage with the tile claimed earlier once every warp
            // has released it; claim the one after that.
            gave_up = !wait_bounded(&empty[sidx], parity, abort_flag, limit);
            if (gave_up) {
                if (atomicExch((int*)abort_flag, 1) == 0) atomicOr(A.status, ST_TIMEOUT);
                producing = false;
            }
        }
        if (tid == 0 && producing) {
            const int t2 = next_claim < A.ntiles ? next_claim : -1;
            stage_tile[sidx] = t2;
            if (t2 >= 0) {
                issue_tile(A, t2, stages[sidx], &full[sidx], cur);
                next_claim = atomicAdd(A.tile_counter, 1);
            } else {
                mbar_arrive(&full[sidx]);   // releases the consumers: no tile
                producing = false;
            }
#pragma unroll
            for (int k = 0; k < TMA_STAGES; ++k) fills[k] += k == sidx;
        }
        // warp 0 reconverges after the producer's work, and leaves together
        // with it if its wait ran out
        if (__shfl_sync(0xffffffffu, (int)gave_up, 0)) break;
    }
    if (tid == 0 && *abort_flag) {
        // A wait ran out.  Before the CTA exits, the last fill issued on each
        // stage (phase fills[k] - 1 of its full barrier; every earlier phase
        // completed before the producer could issue the next) must have
        // landed: a bulk copy must not write into the shared memory of an
        // exited CTA.  Bounded too, by DRAIN_LIMIT polls.
#pragma unroll
        for (int k = 0; k < TMA_STAGES; ++k) {
            if (fills[k] == 0) continue;
            const unsigned par = (fills[k] - 1u) & 1u;
            for (unsigned it = 0; it < DRAIN_LIMIT && !mbar_try_wait(&full[k], par); ++it) __nanosleep(64);
        }
    }
}

size_t step_tma_smem_bytes() { return OFF_FLAG + 16; }

}  // namespace mnad
