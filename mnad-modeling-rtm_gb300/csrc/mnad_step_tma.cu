// step_tma: persistent, TMA-pipelined MNAD time step.
//
// A grid of at most TMA_CTAS_PER_SM CTAs per SM walks the flat tile list of a
// launch group (tile t goes to CTA t mod gridDim).  Each CTA keeps
// TMA_STAGES tiles in flight: for every tile, thread 0 issues seven 2-D bulk
// tensor copies into one shared-memory stage, completing on that stage's
// mbarrier -- U, V, W of the current time level as TMA_TZ+8 x TMA_TX+4 boxes
// (tile plus a 4-row / 2-column halo) and pU, pV, pW, r as TMA_TZ x TMA_TX
// boxes.  While the copies of later tiles are in flight, the 256 threads
// compute the current tile (each TMA_PZ consecutive z points of one column,
// a register window along z), then write nU, nV, nW with 128-bit stores over
// pU, pV, pW.  After a CTA barrier the freed stage is refilled with the tile
// TMA_STAGES ahead.
//
// Tiles wholly inside the interior (no CPML strip) take a lean path; the
// others run the general per-point code with the CPML memory variables.
//
// No copy starts at a negative coordinate: the padded storage has a zero
// halo of HZ = 4 rows and HX = 2 columns, so the halo box of the tile at
// point (j0, i0) starts at storage (j0, i0) and the point box at
// (j0 + 4, i0 + 2); j0 is a multiple of TMA_TZ, so the innermost coordinate
// times 4 bytes is a multiple of 16.  Boxes past the end of the array are
// zero-filled, which is the reference's omitted out-of-grid neighbour.
#include <cuda.h>

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
};
constexpr unsigned STAGE_BYTES = sizeof(float) * (3 * BX * BZ + 4 * TMA_TX * TMA_TZ);
static_assert(sizeof(Stage) == STAGE_BYTES, "stage layout must equal the bytes the copies deliver");
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

__device__ __forceinline__ bool wait_bounded(uint64_t* bar, unsigned parity)
{
    for (unsigned it = 0; it < SPIN_LIMIT; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Thread 0: fill `stage` with tile t of the launch.
__device__ __forceinline__ void issue_tile(const StepArgs& A, int t, Stage& st, uint64_t* bar, int cur)
{
    const int4 info = __ldg(A.tile_info + t);
    const CUtensorMap* maps = static_cast<const CUtensorMap*>(A.tmaps) + (size_t)info.x * TMAPS_PER_PROP;
    mbar_expect_tx(bar, STAGE_BYTES);
#pragma unroll
    for (int f = 0; f < 3; ++f) tma_load_2d(&st.halo[f][0][0], maps + TMAP_HALO + cur * 3 + f, bar, info.y, info.z);
#pragma unroll
    for (int f = 0; f < 3; ++f)
        tma_load_2d(&st.pts[f][0][0], maps + TMAP_POINT + (cur ^ 1) * 3 + f, bar, info.y + HZ, info.z + HX);
    tma_load_2d(&st.pts[3][0][0], maps + TMAP_R, bar, info.y + HZ, info.z + HX);
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

__global__ void __launch_bounds__(TMA_TZY * TMA_TX, TMA_CTAS_PER_SM) step_tma(const __grid_constant__ StepArgs A)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Stage* stages = reinterpret_cast<Stage*>(smem_raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + TMA_STAGES * sizeof(Stage));
    int& abort_flag = *reinterpret_cast<int*>(bars + TMA_STAGES);
    const int tid = threadIdx.x;
    if (smem_addr(smem_raw) & 127u) {       // TMA destinations need aligned stages
        if (tid == 0 && A.ntiles > 0) atomicOr(A.props[0].status, ST_TIMEOUT);
        return;
    }
    const int G = gridDim.x;
    const int cur = A.s & 1;
    if (tid == 0) {
        for (int k = 0; k < TMA_STAGES; ++k) mbar_init(&bars[k], 1);
        fence_mbar_init();
        abort_flag = 0;
    }
    __syncthreads();
    if (tid == 0)
        for (int k = 0; k < TMA_STAGES; ++k) {
            const int t = blockIdx.x + k * G;
            if (t < A.ntiles) issue_tile(A, t, stages[k], &bars[k], cur);
        }
    const int tzt = tid % TMA_TZY, txt = tid / TMA_TZY;
    const int c = txt + 2, r0 = tzt * TMA_PZ + 4;
    const Coefs& K = A.coef;

    for (int n = 0;; ++n) {
        const int t = blockIdx.x + n * G;
        if (t >= A.ntiles) break;
        const int sidx = n % TMA_STAGES;
        const unsigned parity = (unsigned)(n / TMA_STAGES) & 1u;
        const int4 info = __ldg(A.tile_info + t);
        const PropDesc& P = A.props[info.x];
        const int tt = step_tt(P, A.s);
        const int j0 = info.y, i0 = info.z;
        const int tl = (j0 / TMA_TZ) + (i0 / TMA_TX) * P.ntz;
        if (tt != 0 && (info.w & TILE_RECEIVERS) && P.mode == MODE_FWD)
            record_receivers(P, tt, tl, P.fld[cur][0], P.fld[cur][1], P.fld[cur][2]);

        if (!wait_bounded(&bars[sidx], parity)) atomicExch(&abort_flag, 1);
        __syncthreads();
        if (abort_flag) {
            if (tid == 0) {
                atomicOr(P.status, ST_TIMEOUT);
                // let every copy still in flight land (bounded) before leaving
                for (int k = 0; k < TMA_STAGES; ++k)
                    if (blockIdx.x + (n + k) * G < A.ntiles)
                        wait_bounded(&bars[(n + k) % TMA_STAGES], (unsigned)((n + k) / TMA_STAGES) & 1u);
            }
            return;
        }
        const Stage& st = stages[sidx];
        const int j = j0 + tzt * TMA_PZ;
        const int i = i0 + txt;
        if (tt != 0 && j < P.nz && i < P.nx) {
            Window win;
            win.load(st, c, r0);
            const float4 pu4 = ld4(&st.pts[0][txt][tzt * TMA_PZ]);
            const float4 pv4 = ld4(&st.pts[1][txt][tzt * TMA_PZ]);
            const float4 pw4 = ld4(&st.pts[2][txt][tzt * TMA_PZ]);
            const float4 r4 = ld4(&st.pts[3][txt][tzt * TMA_PZ]);
            const float pu[4] = {pu4.x, pu4.y, pu4.z, pu4.w}, pv[4] = {pv4.x, pv4.y, pv4.z, pv4.w};
            const float pw[4] = {pw4.x, pw4.y, pw4.z, pw4.w}, rr[4] = {r4.x, r4.y, r4.z, r4.w};
            const int p = (i + HX) * P.ld + (j + HZ);
            const int rbeg = (info.w & TILE_RECEIVERS) ? __ldg(P.tile_rec + tl) : 0;
            const int rend = (info.w & TILE_RECEIVERS) ? __ldg(P.tile_rec + tl + 1) : 0;
            const bool adj_inj = P.mode == MODE_ADJ && tt < P.nt && rbeg < rend;
            float ou[4], ov[4], ow[4];
            if (info.w & TILE_STRIP) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    Hood h;
                    win.hood(k, h);
                    float su, sv, sw;
                    mnad_update(K, rr[k], h, su, sv, sw);
                    const float inj = adj_inj ? injection(P, tt, rbeg, rend, p + k) : 0.0f;
                    if (j + k < P.nz)
                        finish_point(P, tt, j + k, i, (size_t)(p + k), rr[k], h, su, sv, sw, pu[k], pv[k], pw[k], inj,
                                     ou[k], ov[k], ow[k]);
                    else
                        ou[k] = ov[k] = ow[k] = 0.0f;   // rows past nz are the zero halo
                }
            } else {
                // Interior tile: no CPML; every point is inside the image region.
                const bool snap_step = P.T > 0 && tt % P.T == 0;
                const int d = P.d, niz = P.nz - 2 * d;
                const size_t q0 = (size_t)(j - d) + (size_t)(i - d) * niz;
                const size_t nint = (size_t)niz * (P.nx - 2 * d);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    Hood h;
                    win.hood(k, h);
                    float su, sv, sw;
                    mnad_update(K, rr[k], h, su, sv, sw);
                    float xu = h.u00 + ((h.u00 - pu[k]) + su);
                    ov[k] = h.v00 + ((h.v00 - pv[k]) + sv);
                    ow[k] = h.w00 + ((h.w00 - pw[k]) + sw);
                    if (P.mode == MODE_FWD) {
                        if (snap_step) {
                            // fwd_PDE_exact_MNAD.m:128-141; nU - 2U + pU = su
                            float d2u = su;
                            if (tt == 1) d2u = fmaf(2.0f, h.u00, su - pu[k]);
                            else if (tt == 2) d2u = su - pu[k];
                            d2u *= P.inv_dt2;
                            const size_t q = q0 + k;
                            const size_t o = (size_t)(tt / P.T - 1) * nint + q;
                            if (P.codec == CODEC_BF16) static_cast<__nv_bfloat16*>(P.snap)[o] = __float2bfloat16_rn(d2u);
                            else static_cast<float*>(P.snap)[o] = d2u;
                            P.illum[q] = fma((double)d2u, (double)d2u, P.illum[q]);
                        }
                        if (p + k == P.src && tt < P.nt) xu += P.src_amp[tt];
                    } else {
                        if (adj_inj) xu -= injection(P, tt, rbeg, rend, p + k);
                        if (snap_step) {
                            // Born_adj_MNAD.m:127-134
                            const int ttt = P.img_steps - tt / P.T;
                            const int col = (P.pairing == PAIR_REFERENCE ? P.ncols : P.nsnap) - ttt;
                            if (col >= 1 && col <= P.nsnap) {
                                const size_t q = q0 + k;
                                const float us = snap_decode(P.snap, P.codec, (size_t)(col - 1) * nint + q, 1.0f);
                                P.image[q] = fma((double)us, (double)xu, P.image[q]);
                            }
                        }
                    }
                    ou[k] = xu;
                }
            }
            float* nU = P.fld[cur ^ 1][0];
            float* nV = P.fld[cur ^ 1][1];
            float* nW = P.fld[cur ^ 1][2];
            *reinterpret_cast<float4*>(nU + p) = make_float4(ou[0], ou[1], ou[2], ou[3]);
            *reinterpret_cast<float4*>(nV + p) = make_float4(ov[0], ov[1], ov[2], ov[3]);
            *reinterpret_cast<float4*>(nW + p) = make_float4(ow[0], ow[1], ow[2], ow[3]);
        }
        __syncthreads();   // the stage is free again
        if (tid == 0) {
            const int t2 = t + TMA_STAGES * G;
            if (t2 < A.ntiles) issue_tile(A, t2, stages[sidx], &bars[sidx], cur);
        }
    }
}

size_t step_tma_smem_bytes() { return TMA_STAGES * sizeof(Stage) + TMA_STAGES * sizeof(uint64_t) + 16; }

}  // namespace mnad
