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
// descriptor and the tile's metadata.  Consumers (all 256 threads, thread 0
// included) wait on that stage's "full" barrier, compute the tile (each
// TMA_PZ consecutive z points of one column, a register window along z) and
// write nU, nV, nW with 128-bit stores over pU, pV, pW; each warp then
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
    int4 info;                     // receiver bucket begin/end, flags, local tile index
};
constexpr unsigned FIELD_BYTES = sizeof(float) * (3 * BX * BZ + 4 * TMA_TX * TMA_TZ);
constexpr unsigned STAGE_BYTES = FIELD_BYTES + sizeof(PropDesc) + sizeof(int4);
static_assert(offsetof(Stage, desc) == FIELD_BYTES, "descriptor follows the field boxes");
static_assert(sizeof(PropDesc) % 16 == 0, "bulk copies move multiples of 16 bytes");
static_assert(TMA_PZ == 4, "the register window below is written for 4 points per thread");
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

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }

// The register window of one thread: rows r0-1 .. r0+4 of columns c-1 .. c+1
// for U, V, W, plus V at c-2 / c+2 (rows r0 .. r0+3) and W at rows r0-2, r0+5.
struct Window {
    float u[3][6], v[3][6], w[3][6], v2m[4], v2p[4], wz[2];
    __device__ __forceinline__ void load(const Stage& st, int c, int r0)
    {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
            const float* fu = &st.halo[0][c - 1 + cc][r0];
            const float* fv = &st.halo[1][c - 1 + cc][r0];
            const float* fw = &st.halo[2][c - 1 + cc][r0];
            const float4 a = ld4(fu), b = ld4(fv), e = ld4(fw);
            u[cc][0] = fu[-1]; u[cc][1] = a.x; u[cc][2] = a.y; u[cc][3] = a.z; u[cc][4] = a.w; u[cc][5] = fu[4];
            v[cc][0] = fv[-1]; v[cc][1] = b.x; v[cc][2] = b.y; v[cc][3] = b.z; v[cc][4] = b.w; v[cc][5] = fv[4];
            w[cc][0] = fw[-1]; w[cc][1] = e.x; w[cc][2] = e.y; w[cc][3] = e.z; w[cc][4] = e.w; w[cc][5] = fw[4];
        }
        const float4 a = ld4(&st.halo[1][c - 2][r0]), b = ld4(&st.halo[1][c + 2][r0]);
        v2m[0] = a.x; v2m[1] = a.y; v2m[2] = a.z; v2m[3] = a.w;
        v2p[0] = b.x; v2p[1] = b.y; v2p[2] = b.z; v2p[3] = b.w;
        wz[0] = st.halo[2][c][r0 - 2];
        wz[1] = st.halo[2][c][r0 + 5];
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
        h.wzp2 = k == 3 ? wz[1] : w[1][k + 3];
    }
};

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

__device__ __forceinline__ float4 ld4g(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4g(float* p, float a, float b, float c, float d)
{
    *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}

// Ux123_gen.m / Uz123_gen.m for the four points j..j+3 of column i (one
// thread), vectorized over the points: the memory variables of a field and
// side are four consecutive, 16-byte aligned floats.  Adds F1_x + F1_z of
// U, V, W into cu, cv, cw.  U is taken before this step's source injection
// (fwd_PDE_exact_MNAD.m:95-111): the stored U already holds it.
__device__ __forceinline__ void cpml_vec(const PropDesc& P, const Window& win, int tt, int j, int i, int p,
                                         const float r[4], float cu[4], float cv[4], float cw[4])
{
    const int d = P.d, nz = P.nz, nx = P.nx, ld = P.ld;
    float vel[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) vel[k] = r[k] * rsqrtf(r[k]) * P.inv_dt;
    const float srcamp = (P.mode == MODE_FWD && P.src >= 0) ? P.src_amp[tt - 1] : 0.0f;
    const int src = P.src;
    if (d <= 0) return;                 // no CPML strips (and no memory-variable storage)
    // x direction: the whole column lies in the strip
    if (i < d || i >= nx - d) {
        const int side = i < d ? 0 : 1;
        const int kx = side ? i - (nx - d) : i;
        const float X = side ? float(kx + 1) * P.dx : float(d - i) * P.dx;
        const float inv_h = 1.0f / P.dx;
        float c1[4], c2[4], c3[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) cpml_c(P.kx, vel[k], X, P.dt, c1[k], c2[k], c3[k]);
        const int vs = d * ld;
        float* base = P.mx + ((side * 9) * d + kx) * ld + j;
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const float(*F)[6] = f == 0 ? win.u : (f == 1 ? win.v : win.w);
            float* m = base + (f * 3) * vs;
            const float4 a1 = ld4g(m), a2 = ld4g(m + vs), a3 = ld4g(m + 2 * vs);
            float m1[4] = {a1.x, a1.y, a1.z, a1.w}, m2[4] = {a2.x, a2.y, a2.z, a2.w}, m3[4] = {a3.x, a3.y, a3.z, a3.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float F0 = F[1][k + 1], Fa = F[2][k + 1], Fd = F[0][k + 1];
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
            st4g(m, m1[0], m1[1], m1[2], m1[3]);
            st4g(m + vs, m2[0], m2[1], m2[2], m2[3]);
            st4g(m + 2 * vs, m3[0], m3[1], m3[2], m3[3]);
        }
    }
    // z direction: the top and/or bottom strip may cover part of the group
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        // the group j..j+3 (j < nz) must overlap the strip rows [0, d) or [nz-d, nz)
        if (side == 0 ? !(j < d) : !(j + 3 >= nz - d)) continue;
        const int k0 = side ? j - P.zb0 : j;
        const float inv_h = 1.0f / P.dz;
        float c1[4], c2[4], c3[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
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
            const float(*F)[6] = f == 0 ? win.u : (f == 1 ? win.v : win.w);
            float* m = base + (f * 3) * vs;
            const float4 a1 = ld4g(m), a2 = ld4g(m + vs), a3 = ld4g(m + 2 * vs);
            float m1[4] = {a1.x, a1.y, a1.z, a1.w}, m2[4] = {a2.x, a2.y, a2.z, a2.w}, m3[4] = {a3.x, a3.y, a3.z, a3.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float F0 = F[1][k + 1], Fa = F[1][k + 2], Fd = F[1][k];
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
            st4g(m, m1[0], m1[1], m1[2], m1[3]);
            st4g(m + vs, m2[0], m2[1], m2[2], m2[3]);
            st4g(m + 2 * vs, m3[0], m3[1], m3[2], m3[3]);
        }
    }
}

// Shared-memory layout: TMA_STAGES stages, their full and empty barriers,
// the tile held by each stage, the abort flag.
constexpr size_t OFF_FULL = TMA_STAGES * sizeof(Stage);
constexpr size_t OFF_EMPTY = OFF_FULL + TMA_STAGES * sizeof(uint64_t);
constexpr size_t OFF_TILE = OFF_EMPTY + TMA_STAGES * sizeof(uint64_t);
constexpr size_t OFF_FLAG = OFF_TILE + TMA_STAGES * sizeof(int);
constexpr int NWARPS = TMA_TZY * TMA_TX / 32;

__global__ void __launch_bounds__(TMA_TZY * TMA_TX, TMA_CTAS_PER_SM) step_tma(const __grid_constant__ StepArgs A)
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
        const int tl = info.w;
        const int j0 = (tl % P.ntz) * TMA_TZ, i0 = (tl / P.ntz) * TMA_TX;
        const int nz = P.nz, nx = P.nx, d = P.d, ld = P.ld, nt = P.nt, mode = P.mode;
        if (tt != 0 && (info.z & TILE_RECEIVERS) && mode == MODE_FWD)
            record_receivers(P, tt, tl, P.fld[cur][0], P.fld[cur][1], P.fld[cur][2]);
        const int j = j0 + tzt * TMA_PZ;
        const int i = i0 + txt;
        if (tt != 0 && j < nz && i < nx) {
            Window win;
            win.load(st, c, r0);
            const float4 pu4 = ld4(&st.pts[0][txt][tzt * TMA_PZ]);
            const float4 pv4 = ld4(&st.pts[1][txt][tzt * TMA_PZ]);
            const float4 pw4 = ld4(&st.pts[2][txt][tzt * TMA_PZ]);
            const float4 r4 = ld4(&st.pts[3][txt][tzt * TMA_PZ]);
            const float pu[4] = {pu4.x, pu4.y, pu4.z, pu4.w}, pv[4] = {pv4.x, pv4.y, pv4.z, pv4.w};
            const float pw[4] = {pw4.x, pw4.y, pw4.z, pw4.w}, rr[4] = {r4.x, r4.y, r4.z, r4.w};
            const int p = (i + HX) * ld + (j + HZ);
            const int rbeg = info.x, rend = info.y;
            const bool adj_inj = mode == MODE_ADJ && tt < nt && rbeg < rend;
            const bool snap_step = P.T > 0 && tt % P.T == 0;
            const int niz = nz - 2 * d;
            const size_t nint = (size_t)niz * (nx - 2 * d);
            const long long q0 = (long long)(j - d) + (long long)(i - d) * niz;
            // imaging column of this step (Born_adj_MNAD.m:128), 0 when none
            int col = 0;
            if (mode == MODE_ADJ && snap_step) {
                col = (P.pairing == PAIR_REFERENCE ? P.ncols : P.nsnap) - (P.img_steps - tt / P.T);
                if (col < 1 || col > P.nsnap) col = 0;
            }
            const int src = P.src;
            const float src_next = (mode == MODE_FWD && src >= p && src < p + 4 && tt < nt) ? P.src_amp[tt] : 0.0f;
            // lean: all four points inside the image region (no CPML, no edge)
            const bool lean = i >= d && i < nx - d && j >= d && j + 3 < nz - d;
            float su[4], sv[4], sw[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                Hood h;
                win.hood(k, h);
                mnad_update(K, rr[k], h, su[k], sv[k], sw[k]);
            }
            if (!lean) {
                float cu[4] = {0.f, 0.f, 0.f, 0.f}, cv[4] = {0.f, 0.f, 0.f, 0.f}, cw[4] = {0.f, 0.f, 0.f, 0.f};
                cpml_vec(P, win, tt, j, i, p, rr, cu, cv, cw);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    su[k] = fmaf(-rr[k], cu[k], su[k]);
                    sv[k] = fmaf(-rr[k], cv[k], sv[k]);
                    sw[k] = fmaf(-rr[k], cw[k], sw[k]);
                }
            }
            float ou[4], ov[4], ow[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int jk = j + k;
                const bool inner = lean || (jk >= d && jk < nz - d && i >= d && i < nx - d);
                const float u0 = win.u[1][k + 1], v0 = win.v[1][k + 1], w0 = win.w[1][k + 1];
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
                        const size_t o = (size_t)(tt / P.T - 1) * nint + q;
                        if (P.codec == CODEC_BF16) static_cast<__nv_bfloat16*>(P.snap)[o] = __float2bfloat16_rn(d2u);
                        else static_cast<float*>(P.snap)[o] = d2u;
                        P.illum[q] = fma((double)d2u, (double)d2u, P.illum[q]);
                    }
                    if (p + k == src) xu += src_next;
                } else {
                    if (adj_inj) xu -= injection(P, tt, rbeg, rend, p + k);
                    if (col && inner) {
                        const size_t q = (size_t)(q0 + k);
                        const float us = snap_decode(P.snap, P.codec, (size_t)(col - 1) * nint + q, 1.0f);
                        P.image[q] = fma((double)us, (double)xu, P.image[q]);
                    }
                }
                if (jk >= nz) xu = xv = xw = 0.0f;   // rows past nz are the zero halo
                ou[k] = xu;
                ov[k] = xv;
                ow[k] = xw;
            }
            float* nU = P.fld[cur ^ 1][0];
            float* nV = P.fld[cur ^ 1][1];
            float* nW = P.fld[cur ^ 1][2];
            *reinterpret_cast<float4*>(nU + p) = make_float4(ou[0], ou[1], ou[2], ou[3]);
            *reinterpret_cast<float4*>(nV + p) = make_float4(ov[0], ov[1], ov[2], ov[3]);
            *reinterpret_cast<float4*>(nW + p) = make_float4(ow[0], ow[1], ow[2], ow[3]);
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
