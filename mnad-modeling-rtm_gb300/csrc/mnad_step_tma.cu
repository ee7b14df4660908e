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
// wait is bounded; a wait that runs out sets ST_TIMEOUT and the CTA leaves
// after giving its own copies in flight a bounded time to land.
#include <cuda.h>

#include <cstddef>

#include "mnad_kernels.h"
#include "mnad_point.cuh"

namespace mnad {

namespace {

constexpr int BZ = TMA_TZ + 8;     // halo box rows (z)
constexpr int BX = TMA_TX + 4;     // halo box columns (x)
constexpr unsigned SPIN_LIMIT = 1u << 22;   // bounded mbarrier wait

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

// Bounded wait; gives up early once another thread has aborted.
__device__ __forceinline__ bool wait_bounded(uint64_t* bar, unsigned parity, const volatile int* abort_flag)
{
    for (unsigned it = 0; it < SPIN_LIMIT; ++it) {
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
    __device__ __forceinline__ void hood(int k, Hood& h) const
    {
        h.u00 = u[1][k + 1]; h.uzm = u[1][k]; h.uzp = u[1][k + 2]; h.uxm = u[0][k + 1]; h.uxp = u[2][k + 1];
        h.umm = u[0][k]; h.upm = u[0][k + 2]; h.ump = u[2][k]; h.upp = u[2][k + 2];
        h.v00 = v[1][k + 1]; h.vzm = v[1][k]; h.vzp = v[1][k + 2]; h.vxm = v[0][k + 1]; h.vxp = v[2][k + 1];
        h.vmm = v[0][k]; h.vpm = v[0][k + 2]; h.vmp = v[2][k]; h.vpp = v[2][k + 2];
        h.vxm2 = v2m[k]; h.vxp2 = v2p[k];
        h.w00 = w[1][k + 1]; h.wzm = w[1][k]; h.wzp = w[1][k + 2]; h.wxm = w[0][k + 1]; h.wxp = w[2][k + 1];
        h.wmm = w[0][k]; h.wpm = w[0][k + 2]; h.wmp = w[2][k]; h.wpp = w[2][k + 2];
        h.wzm2 = k == 0 ? wz[0] : w[1][k - 1];
        h.wzp2 = k == TMA_PZ - 1 ? wz[1] : w[1][k + 3];
    }
};

// The stencil sums su, sv, sw (see mnad_update) of the TMA_PZ points of a
// thread, with the combinations of the side columns shared between rows:
// per row r, S = F(c-1) + F(c+1) and D = F(c-1) - F(c+1), so that e.g. the
// diagonal sum of point k is S[k] + S[k+2] and the odd diagonal of
// Avu_gen.m is D[k] + D[k+2].
__device__ __forceinline__ void mnad_update_window(const Coefs& K, const Window& win, const float* rr, float* su,
                                                   float* sv, float* sw)
{
    constexpr int R = Window::R;
    const float* a = K.alpha;
    const float* b = K.beta;
    float SU[R], DU[R], SV[R], DV[R], SW[R], DW[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        SU[r] = win.u[0][r] + win.u[2][r]; DU[r] = win.u[0][r] - win.u[2][r];
        SV[r] = win.v[0][r] + win.v[2][r]; DV[r] = win.v[0][r] - win.v[2][r];
        SW[r] = win.w[0][r] + win.w[2][r]; DW[r] = win.w[0][r] - win.w[2][r];
    }
#pragma unroll
    for (int k = 0; k < TMA_PZ; ++k) {
        const float r = rr[k], q = r * r;
        const float u0 = win.u[1][k + 1], v0 = win.v[1][k + 1], w0 = win.w[1][k + 1];
        const float u2 = u0 + u0, v2 = v0 + v0, w2 = w0 + w0;
        const float uzs = win.u[1][k] + win.u[1][k + 2], vzs = win.v[1][k] + win.v[1][k + 2];
        const float wzs = win.w[1][k] + win.w[1][k + 2];
        // U combinations (Auu, Avu, Awu)
        const float dUz = uzs - u2, dUx = SU[k + 1] - u2, dUd = (SU[k] + SU[k + 2]) - (u2 + u2);
        const float uLx = DU[k + 1], uLz = win.u[1][k] - win.u[1][k + 2];
        const float uDx = DU[k] + DU[k + 2], uDz = SU[k] - SU[k + 2];
        // V combinations (Avv, Auv, Awv); vX1 and vDx enter with negative sign
        const float dVz = vzs - v2, dVx = SV[k + 1] - v2, dVd = (SV[k] + SV[k + 2]) - (v2 + v2);
        const float nvX1 = DV[k + 1], nvDx = DV[k] + DV[k + 2];
        const float vX2 = win.v2m[k] - win.v2p[k], vXZ = DV[k] - DV[k + 2];
        // W combinations (Aww, Auw, Avw)
        const float wzm2 = k == 0 ? win.wz[0] : win.w[1][k - 1];
        const float wzp2 = k == TMA_PZ - 1 ? win.wz[1] : win.w[1][k + 3];
        const float dWz = wzs - w2, dWx = SW[k + 1] - w2, dWd = (SW[k] + SW[k + 2]) - (w2 + w2);
        const float wZ1 = win.w[1][k + 2] - win.w[1][k], wDz = SW[k + 2] - SW[k];
        const float wZ2 = wzm2 - wzp2, wXZ = DW[k] - DW[k + 2];
        // nU row
        float ra = a[K_UU_Z] * dUz;
        ra = fmaf(a[K_UU_X], dUx, ra);
        ra = fmaf(-a[K_UV_X1], nvX1, ra);
        ra = fmaf(a[K_UV_X2], vX2, ra);
        ra = fmaf(a[K_UW_Z1], wZ1, ra);
        ra = fmaf(a[K_UW_Z2], wZ2, ra);
        float qa = b[K_UU_Z] * dUz;
        qa = fmaf(b[K_UU_X], dUx, qa);
        qa = fmaf(b[K_UU_D], dUd, qa);
        qa = fmaf(-b[K_UV_X1], nvX1, qa);
        qa = fmaf(-b[K_UV_D], nvDx, qa);
        qa = fmaf(b[K_UV_X2], vX2, qa);
        qa = fmaf(b[K_UW_Z1], wZ1, qa);
        qa = fmaf(b[K_UW_D], wDz, qa);
        qa = fmaf(b[K_UW_Z2], wZ2, qa);
        su[k] = fmaf(q, qa, r * ra);
        // nV row
        float rb = a[K_VV_Z] * dVz;
        rb = fmaf(a[K_VV_X], dVx, rb);
        rb = fmaf(a[K_VV_R], v0, rb);
        rb = fmaf(a[K_VU_X1], uLx, rb);
        rb = fmaf(a[K_VU_D], uDx, rb);
        rb = fmaf(a[K_VW], wXZ, rb);
        float qb = b[K_VV_Z] * dVz;
        qb = fmaf(b[K_VV_X], dVx, qb);
        qb = fmaf(b[K_VV_D], dVd, qb);
        qb = fmaf(b[K_VV_R], v0, qb);
        qb = fmaf(b[K_VU_X1], uLx, qb);
        qb = fmaf(b[K_VU_D], uDx, qb);
        qb = fmaf(b[K_VW], wXZ, qb);
        sv[k] = fmaf(q, qb, r * rb);
        // nW row
        float rc = a[K_WW_Z] * dWz;
        rc = fmaf(a[K_WW_X], dWx, rc);
        rc = fmaf(a[K_WW_R], w0, rc);
        rc = fmaf(a[K_WU_Z1], uLz, rc);
        rc = fmaf(a[K_WU_D], uDz, rc);
        rc = fmaf(a[K_WV], vXZ, rc);
        float qc = b[K_WW_Z] * dWz;
        qc = fmaf(b[K_WW_X], dWx, qc);
        qc = fmaf(b[K_WW_D], dWd, qc);
        qc = fmaf(b[K_WW_R], w0, qc);
        qc = fmaf(b[K_WU_Z1], uLz, qc);
        qc = fmaf(b[K_WU_D], uDz, qc);
        qc = fmaf(b[K_WV], vXZ, qc);
        sw[k] = fmaf(q, qc, r * rc);
    }
}

// Receiver injection of the adjoint at storage offset p (entries rbeg..rend).
__device__ __forceinline__ float injection(const PropDesc& P, int tt, int rbeg, int rend, int p)
{
    float inj = 0.0f;
    for (int e = rbeg; e < rend; ++e)
        if (__ldg(P.rec_pt + e) == p)
            inj += (float)(__ldg(P.rec_r + e) * __ldg(P.data + (size_t)__ldg(P.rec_id + e) * P.nt + tt));
    return inj;
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

// Ux123_gen.m / Uz123_gen.m for the TMA_PZ points j.. of column i (one
// thread), vectorized over the points: the memory variables of a field and
// side are TMA_PZ consecutive, aligned floats.  Adds F1_x + F1_z of
// U, V, W into cu, cv, cw.  U is taken before this step's source injection
// (fwd_PDE_exact_MNAD.m:95-111): the stored U already holds it.
__device__ __forceinline__ void cpml_vec(const PropDesc& P, const Stage& st, int c, int r0, int tt, int j, int i,
                                         int p, const float* r, float* cu, float* cv, float* cw)
{
    constexpr int Q = TMA_PZ;
    const int d = P.d, nz = P.nz, nx = P.nx, ld = P.ld;
    float vel[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) vel[k] = r[k] * rsqrtf(r[k]) * P.inv_dt;
    const float srcamp = (P.mode == MODE_FWD && P.src >= 0) ? P.src_amp[tt - 1] : 0.0f;
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
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            float F0v[Q], Fav[Q], Fdv[Q];
            ldv(&st.halo[f][c][r0], F0v);
            ldv(&st.halo[f][c + 1][r0], Fav);
            ldv(&st.halo[f][c - 1][r0], Fdv);
            float* m = base + (f * 3) * vs;
            float m1[Q], m2[Q], m3[Q];
            ldv(m, m1);
            ldv(m + vs, m2);
            ldv(m + 2 * vs, m3);
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
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const float* col = &st.halo[f][c][r0];
            float Fc[Q + 2];
            Fc[0] = col[-1];
            ldv(col, &Fc[1]);
            Fc[Q + 1] = col[Q];
            float* m = base + (f * 3) * vs;
            float m1[Q], m2[Q], m3[Q];
            ldv(m, m1);
            ldv(m + vs, m2);
            ldv(m + 2 * vs, m3);
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
        if (tid == 0 && A.ntiles > 0) atomicOr(A.props[0].status, ST_TIMEOUT);
        return;
    }
    const int cur = A.s & 1;
    int next_claim = -1;                    // producer: tile claimed one refill ahead
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
        for (int k = 0; k < TMA_STAGES; ++k) {
            if (stage_tile[k] >= 0) issue_tile(A, stage_tile[k], stages[k], &full[k], cur);
            else mbar_arrive(&full[k]);     // releases the consumers: no tile
        }
    const int tzt = tid % TMA_TZY, txt = tid / TMA_TZY;
    const int c = txt + 2, r0 = tzt * TMA_PZ + 4;
    const Coefs& K = A.coef;
    bool producing = true;

    for (int n = 0;; ++n) {
        const int sidx = n % TMA_STAGES;
        const unsigned parity = (unsigned)(n / TMA_STAGES) & 1u;
        if (!wait_bounded(&full[sidx], parity, abort_flag)) {
            if (atomicExch((int*)abort_flag, 1) == 0) atomicOr(A.props[0].status, ST_TIMEOUT);
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
        if (tt != 0 && (info.z & TILE_RECEIVERS) && mode == MODE_FWD)
            record_receivers(P, tt, tl, P.fld[cur][0], P.fld[cur][1], P.fld[cur][2]);
        const int j = j0 + tzt * TMA_PZ;
        const int i = i0 + txt;
        if (tt != 0 && j < nz && i < nx) {
            constexpr int Q = TMA_PZ;
            float rr[Q];
            ldv(&st.pts[3][txt][tzt * Q], rr);
            const int p = (i + HX) * ld + (j + HZ);
            const int rbeg = info.x, rend = info.y;
            const bool adj_inj = mode == MODE_ADJ && tt < nt && rbeg < rend;
            // tt / T and tt % T without an integer division: (tt + 0.5) / T is
            // never within 0.5/T of an integer, far beyond float rounding.
            const int tq = (int)(((float)tt + 0.5f) * P.invT);
            const bool snap_step = P.T > 0 && tt - tq * P.T == 0;
            const int niz = nz - 2 * d;
            const size_t nint = (size_t)niz * (nx - 2 * d);
            const long long q0 = (long long)(j - d) + (long long)(i - d) * niz;
            // imaging column of this step (Born_adj_MNAD.m:128), 0 when none
            int col = 0;
            if (mode == MODE_ADJ && snap_step) {
                col = (P.pairing == PAIR_REFERENCE ? P.ncols : P.nsnap) - (P.img_steps - tq);
                if (col < 1 || col > P.nsnap) col = 0;
            }
            const int src = P.src;
            const float src_next = (mode == MODE_FWD && src >= p && src < p + Q && tt < nt) ? P.src_amp[tt] : 0.0f;
            // lean: every point of the group inside the image region (no CPML, no edge)
            const bool lean = i >= d && i < nx - d && j >= d && j + Q - 1 < nz - d;
            float su[Q], sv[Q], sw[Q];
            {
                Window win;            // dies here: later phases re-read the stage
                win.load(st, c, r0);
                mnad_update_window(K, win, rr, su, sv, sw);
            }
            if (!lean) {
                float cu[Q], cv[Q], cw[Q];
#pragma unroll
                for (int k = 0; k < Q; ++k) cu[k] = cv[k] = cw[k] = 0.0f;
                cpml_vec(P, st, c, r0, tt, j, i, p, rr, cu, cv, cw);
#pragma unroll
                for (int k = 0; k < Q; ++k) {
                    su[k] = fmaf(-rr[k], cu[k], su[k]);
                    sv[k] = fmaf(-rr[k], cv[k], sv[k]);
                    sw[k] = fmaf(-rr[k], cw[k], sw[k]);
                }
            }
            float pu[Q], pv[Q], pw[Q], uc[Q], vc[Q], wc[Q];
            ldv(&st.pts[0][txt][tzt * Q], pu);
            ldv(&st.pts[1][txt][tzt * Q], pv);
            ldv(&st.pts[2][txt][tzt * Q], pw);
            ldv(&st.halo[0][c][r0], uc);
            ldv(&st.halo[1][c][r0], vc);
            ldv(&st.halo[2][c][r0], wc);
            float ou[Q], ov[Q], ow[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                const int jk = j + k;
                const bool inner = lean || (jk >= d && jk < nz - d && i >= d && i < nx - d);
                const float u0 = uc[k], v0 = vc[k], w0 = wc[k];
                float xu = u0 + ((u0 - pu[k]) + su[k]);
                float xv = v0 + ((v0 - pv[k]) + sv[k]);
                float xw = w0 + ((w0 - pw[k]) + sw[k]);
                if (mode == MODE_FWD) {
                    if (snap_step && inner) {
                        // fwd_PDE_exact_MNAD.m:128-141; nU - 2U + pU = su
                        float d2u = su[k];
                        if (tt == 1) d2u = fmaf(2.0f, u0, su[k] - pu[k]);
                        else if (tt == 2) d2u = su[k] - pu[k];
                        d2u *= P.inv_dt2;
                        const size_t q = (size_t)(q0 + k);
                        const size_t o = (P.snap_stage ? (size_t)0 : (size_t)(tq - 1)) * nint + q;
                        if (P.codec == CODEC_BF16) static_cast<__nv_bfloat16*>(P.snap)[o] = __float2bfloat16_rn(d2u);
                        else static_cast<float*>(P.snap)[o] = d2u;
                        P.illum[q] = fma((double)d2u, (double)d2u, P.illum[q]);
                    }
                    if (p + k == src) xu += src_next;
                } else {
                    if (adj_inj) xu -= injection(P, tt, rbeg, rend, p + k);
                    if (col && inner) {
                        const size_t q = (size_t)(q0 + k);
                        const float sc = P.codec == CODEC_F16 ? P.snap_scale[col - 1] : 1.0f;
                        const float us = snap_decode(P.snap, P.codec, (size_t)(col - 1) * nint + q, sc);
                        P.image[q] = fma((double)us, (double)xu, P.image[q]);
                    }
                }
                if (jk >= nz) xu = xv = xw = 0.0f;   // rows past nz are the zero halo
                ou[k] = xu;
                ov[k] = xv;
                ow[k] = xw;
            }
            stv(P.fld[cur ^ 1][0] + p, ou);
            stv(P.fld[cur ^ 1][1] + p, ov);
            stv(P.fld[cur ^ 1][2] + p, ow);
        }
        // This warp is done with the stage.
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[sidx]);
        if (tid == 0 && producing) {
            // Refill the stage with the tile claimed earlier once every warp
            // has released it; claim the one after that.
            if (!wait_bounded(&empty[sidx], parity, abort_flag)) {
                if (atomicExch((int*)abort_flag, 1) == 0) atomicOr(A.props[0].status, ST_TIMEOUT);
                break;
            }
            const int t2 = next_claim < A.ntiles ? next_claim : -1;
            stage_tile[sidx] = t2;
            if (t2 >= 0) {
                issue_tile(A, t2, stages[sidx], &full[sidx], cur);
                next_claim = atomicAdd(A.tile_counter, 1);
            } else {
                mbar_arrive(&full[sidx]);   // releases the consumers: no tile
                producing = false;
            }
        }
        __syncwarp();   // warp 0 reconverges after the producer's work
    }
    if (tid == 0 && *abort_flag) {
        // let this CTA's copies still in flight land (bounded) before leaving
        for (int k = 0; k < TMA_STAGES; ++k)
            for (unsigned it = 0; it < SPIN_LIMIT; ++it)
                if (mbar_try_wait(&full[k], 0) || mbar_try_wait(&full[k], 1)) break;
    }
}

size_t step_tma_smem_bytes() { return OFF_FLAG + 16; }

}  // namespace mnad
