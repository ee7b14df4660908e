// step_tma2: persistent, TMA-pipelined MNAD kernel that advances every
// propagation of a launch group by two time steps per pass (temporal
// blocking of depth 2).
//
// A pass at even global step s runs steps s and s+1.  For a 64 x 16 tile
// (TMA_TZ x TMA_TX, the receiver-bucket tiling) one mbarrier transaction
// stages
//   * level n   (U, V, W after s steps) on the tile plus a 4-point halo:
//     72 x 24 boxes, columns i0-4 .. i0+19, rows j0-4 .. j0+67;
//   * level n-1 and r on the ring region R1 = the tile plus 2 points:
//     72 x 20 boxes, columns i0-2 .. i0+17, same rows;
//   * the propagation descriptor and the tile's metadata.
// Sub-step 1 (step s) computes level n+1 on all of R1 into shared memory,
// over the level n-1 values it replaces: 18 four-point row groups x 20
// columns, two rounds of the 256 threads.  Rows j0-4, j0-3, j0+66, j0+67 come
// out wrong (their stencil reaches beyond the staged rows) but sub-step 2
// never reads them; points outside the grid are set to zero, the reference's
// omitted neighbours.  After a CTA barrier, sub-step 2 (step s+1) computes
// level n+2 on the tile from level n+1 in shared memory and level n as its
// previous level; each thread then stores both new levels of its 4 points.
//
// Levels are kept in four buffers (level L in buffer L & 3), so no pass
// writes a buffer that a neighbouring tile of the same pass still reads.  The
// CPML memory variables likewise alternate between two banks: a pass reads
// bank (s/2) & 1 on R1 and writes the other bank on its own tile only (sub-
// step 1 writes it, sub-step 2 updates it in place).
//
// Every per-step event of fwd_PDE_exact_MNAD.m:92-157 and
// Born_adj_MNAD.m:85-136 happens at its own sub-step: CPML on the pre-
// injection U, the update, the source injection of the next step, the
// receivers of each step (from the staged level n and from level n+1 in
// shared memory), d2u snapshots with illumination, the adjoint's residual
// injection after the update (on all of R1 in sub-step 1, since sub-step 2
// reads it there) and the imaging condition.  Per point the arithmetic is
// that of step_tma, so results are bitwise those of two single steps.
//
// Propagations must start at global step 0 and run without step windows;
// a propagation whose last step is s runs sub-step 1 only.  Waits are
// bounded as in step_tma: a CTA whose wait runs out sets ST_TIMEOUT and
// leaves, with the whole CTA, after its own copies in flight have landed.
#include <cuda.h>

#include <cstddef>

#include "mnad_tile.cuh"

namespace mnad {

namespace {

using namespace tile;

constexpr int CX = TMA_TX + 8;       // columns of the level-n buffer
constexpr int RX = TMA_TX + 4;       // columns of the ring region R1
constexpr int FSC = CX * BZ;         // field strides (floats)
constexpr int FSR = RX * BZ;
constexpr int QROWS = BZ / TMA_PZ;   // four-point row groups of R1 (18)
constexpr int NQ1 = QROWS * RX;      // sub-step-1 quads (360)
constexpr int NSTAGE = 2;

struct __align__(128) Stage2 {
    float cur[3][CX][BZ];            // level n of U, V, W
    float ring[3][RX][BZ];           // level n-1 on R1, overwritten by level n+1
    float r[RX][BZ];                 // v^2 dt^2 on R1
    PropDesc desc;
    int4 info;                       // receiver bucket begin/end, TILE_* flags (of R1), j0 | i0 << 16
};
constexpr unsigned FIELD_BYTES2 = sizeof(float) * (3 * CX * BZ + 3 * RX * BZ + RX * BZ);
constexpr unsigned STAGE_BYTES2 = FIELD_BYTES2 + sizeof(PropDesc) + sizeof(int4);
static_assert(offsetof(Stage2, desc) == FIELD_BYTES2, "descriptor follows the field boxes");
static_assert(sizeof(PropDesc) % 16 == 0, "bulk copies move multiples of 16 bytes");

// Thread 0: fill `st` with tile t (one transaction).  Storage coordinates:
// row j0 holds grid row j0 - 4 (HZ = 4), column i0 + HX - 4 = i0 - 2 holds
// grid column i0 - 4 (negative for the first tile column: the copy fills
// zeros there; the innermost coordinate j0 is a multiple of 4 floats).
__device__ __forceinline__ void issue_tile2(const StepArgs& A, int t, Stage2& st, uint64_t* bar, int lc, int lp)
{
    const int pi = t / A.tiles_per_prop;
    const int tl = t - pi * A.tiles_per_prop;
    const int j0 = (tl % A.ntz) * TMA_TZ, i0 = (tl / A.ntz) * TMA_TX;
    const CUtensorMap* maps = static_cast<const CUtensorMap*>(A.tmaps) + (size_t)pi * TMAPS_PER_PROP2;
    mbar_expect_tx(bar, STAGE_BYTES2);
    bulk_load(&st.desc, A.props + pi, sizeof(PropDesc), bar);
    bulk_load(&st.info, A.tile_info + t, sizeof(int4), bar);
    tma_load_3d(&st.cur[0][0][0], maps + TMAP2_CUR + lc, bar, j0, i0 + HX - 4, 0);
    tma_load_3d(&st.ring[0][0][0], maps + TMAP2_RING + lp, bar, j0, i0 + HX - 2, 0);
    tma_load_2d(&st.r[0][0], maps + TMAP2_R, bar, j0, i0 + HX - 2);
}

// One sub-step for the TMA_PZ points j.. of grid column i (all inside the
// grid, rows past nz excepted): the stencil from the window buffer (field
// stride WFS, column wc), the previous level from buffer P (stride PFS,
// column pc), r from column rc of the r buffer, all at rows r0...  `general`
// adds CPML, source and receiver injection; `owned` marks points of the
// pass's own tile (memory variables stored, snapshots and imaging).
// Returns the new U, V, W (zero in rows past nz).
template <int WFS, int PFS>
__device__ __forceinline__ void quad_step(const StepArgs& A, const PropDesc& P, int tt, const float* wbase, int wc,
                                          const float* pbase, int pc, const float* rb, int rc, int r0, int j, int i,
                                          bool general, bool src_tile, bool rec_tile, bool owned, int rd_bank,
                                          int wr_bank, float* ou, float* ov, float* ow)
{
    constexpr int Q = TMA_PZ;
    const int nz = P.nz, nx = P.nx, d = P.d, ld = P.ld, nt = P.nt, mode = P.mode;
    const int p = (i + HX) * ld + (j + HZ);
    float rr[Q];
    ldv(rb + rc * BZ + r0, rr);
    const bool lean = !general || (i >= d && i < nx - d && j >= d && j + Q - 1 < nz - d);
    const MemBank rd = rd_bank ? MemBank{P.mx2, P.mz2} : MemBank{P.mx, P.mz};
    const MemBank wr = wr_bank ? MemBank{P.mx2, P.mz2} : MemBank{P.mx, P.mz};
    if (!lean && d > 0) prefetch_strip_state(P, rd, j, i);
    float2 su[2], sv[2], sw[2];
    {
        Window win;
        win.load<WFS>(wbase, wc, r0);
        mnad_update_pairs(A.coef2, win, rr, su, sv, sw);
    }
    if (!lean) {
        float2 cu[2], cv[2], cw[2];
#pragma unroll
        for (int m = 0; m < 2; ++m) cu[m] = cv[m] = cw[m] = pr(0.0f, 0.0f);
        cpml_vec<WFS>(P, wbase, wc, r0, tt, j, i, p, src_tile, rr, rd, wr, owned, cu, cv, cw);
        // sF -= r * (F1_x + F1_z), per point fmaf(-r, c, s)
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const float2 nr = pr(-rr[2 * m], -rr[2 * m + 1]);
            su[m] = pfma(nr, cu[m], su[m]);
            sv[m] = pfma(nr, cv[m], sv[m]);
            sw[m] = pfma(nr, cw[m], sw[m]);
        }
    }
    const float4 pu4 = *reinterpret_cast<const float4*>(pbase + pc * BZ + r0);
    const float4 pv4 = *reinterpret_cast<const float4*>(pbase + PFS + pc * BZ + r0);
    const float4 pw4 = *reinterpret_cast<const float4*>(pbase + 2 * PFS + pc * BZ + r0);
    const float4 uc4 = *reinterpret_cast<const float4*>(wbase + wc * BZ + r0);
    const float4 vc4 = *reinterpret_cast<const float4*>(wbase + WFS + wc * BZ + r0);
    const float4 wc4 = *reinterpret_cast<const float4*>(wbase + 2 * WFS + wc * BZ + r0);
    // nF = F + ((F - pF) + sF)
    const float2 nu01 = padd(pr(uc4.x, uc4.y), padd(psub(pr(uc4.x, uc4.y), pr(pu4.x, pu4.y)), su[0]));
    const float2 nu23 = padd(pr(uc4.z, uc4.w), padd(psub(pr(uc4.z, uc4.w), pr(pu4.z, pu4.w)), su[1]));
    const float2 nv01 = padd(pr(vc4.x, vc4.y), padd(psub(pr(vc4.x, vc4.y), pr(pv4.x, pv4.y)), sv[0]));
    const float2 nv23 = padd(pr(vc4.z, vc4.w), padd(psub(pr(vc4.z, vc4.w), pr(pv4.z, pv4.w)), sv[1]));
    const float2 nw01 = padd(pr(wc4.x, wc4.y), padd(psub(pr(wc4.x, wc4.y), pr(pw4.x, pw4.y)), sw[0]));
    const float2 nw23 = padd(pr(wc4.z, wc4.w), padd(psub(pr(wc4.z, wc4.w), pr(pw4.z, pw4.w)), sw[1]));
    ou[0] = nu01.x; ou[1] = nu01.y; ou[2] = nu23.x; ou[3] = nu23.y;
    ov[0] = nv01.x; ov[1] = nv01.y; ov[2] = nv23.x; ov[3] = nv23.y;
    ow[0] = nw01.x; ow[1] = nw01.y; ow[2] = nw23.x; ow[3] = nw23.y;
    // tt / T and tt % T without an integer division: (tt + 0.5) / T is
    // never within 0.5/T of an integer, far beyond float rounding.
    const int tq = (int)(((float)tt + 0.5f) * P.invT);
    const bool snap_step = owned && P.T > 0 && tt - tq * P.T == 0;
    const int niz = nz - 2 * d;
    const size_t nint = (size_t)niz * (nx - 2 * d);
    const long long q0 = (long long)(j - d) + (long long)(i - d) * niz;
    if (mode == MODE_FWD) {
        if (snap_step) {
            const float sus[Q] = {su[0].x, su[0].y, su[1].x, su[1].y};
            const float pus[Q] = {pu4.x, pu4.y, pu4.z, pu4.w};
            const float ucs[Q] = {uc4.x, uc4.y, uc4.z, uc4.w};
            const int slot = P.snap_stage ? 0 : tq - 1 - P.snap_col0;
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                const int jk = j + k;
                if (!(jk >= d && jk < nz - d && i >= d && i < nx - d)) continue;
                // fwd_PDE_exact_MNAD.m:128-141; nU - 2U + pU = su
                float d2u = sus[k];
                if (tt == 1) d2u = fmaf(2.0f, ucs[k], sus[k] - pus[k]);
                else if (tt == 2) d2u = sus[k] - pus[k];
                d2u *= P.inv_dt2;
                const size_t q = (size_t)(q0 + k);
                if ((P.snap_flags & SNAP_WRITE) && slot >= 0 && slot < P.snap_cols) {
                    const size_t o = (size_t)slot * nint + q;
                    if (P.codec == CODEC_BF16) static_cast<__nv_bfloat16*>(P.snap)[o] = __float2bfloat16_rn(d2u);
                    else static_cast<float*>(P.snap)[o] = d2u;
                }
                if (P.snap_flags & SNAP_ILLUM) accumulate_product(&P.illum[q], d2u, d2u);
            }
        }
        // the next step's injection (fwd_PDE_exact_MNAD.m:111): stored U holds it
        const int src = P.src;
        if (src_tile && src >= p && src < p + Q && tt < nt) {
            const float a = P.src_amp[tt];
#pragma unroll
            for (int k = 0; k < Q; ++k)
                if (p + k == src) ou[k] += a;
        }
    } else {
        // Born_adj_MNAD.m:109-111: the residual of step tt+1 enters U after the update
        if (rec_tile && tt < nt) {
            float inj[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) inj[k] = 0.0f;
            injection(P, tt, (j / TMA_TZ) + (i / TMA_TX) * P.ntz, i % TMA_TX, p, inj);
#pragma unroll
            for (int k = 0; k < Q; ++k) ou[k] -= inj[k];
        }
        if (snap_step) {
            // Born_adj_MNAD.m:127-134: column ncols - ttt + 1 of UU
            const int col = (P.pairing == PAIR_REFERENCE ? P.ncols : P.nsnap) - (P.img_steps - tq);
            if (col >= 1 && col <= P.nsnap && col - 1 >= P.snap_col0 && col - 1 - P.snap_col0 < P.snap_cols) {
                const float sc = P.codec == CODEC_F16 ? P.snap_scale[col - 1] : 1.0f;
                const size_t o = (size_t)(col - 1 - P.snap_col0) * nint;
#pragma unroll
                for (int k = 0; k < Q; ++k) {
                    const int jk = j + k;
                    if (!(jk >= d && jk < nz - d && i >= d && i < nx - d)) continue;
                    const size_t q = (size_t)(q0 + k);
                    const float us = snap_decode(P.snap, P.codec, o + q, sc);
                    accumulate_product(&P.image[q], us, ou[k]);
                }
            }
        }
    }
    if (j + Q > nz) {
#pragma unroll
        for (int k = 0; k < Q; ++k)
            if (j + k >= nz) ou[k] = ov[k] = ow[k] = 0.0f;   // rows past nz are the zero halo
    }
}

constexpr size_t OFF_FULL2 = NSTAGE * sizeof(Stage2);
constexpr size_t OFF_EMPTY2 = OFF_FULL2 + NSTAGE * sizeof(uint64_t);
constexpr size_t OFF_TILE2 = OFF_EMPTY2 + NSTAGE * sizeof(uint64_t);
constexpr size_t OFF_FLAG2 = OFF_TILE2 + NSTAGE * sizeof(int);
constexpr int NWARPS2 = TMA_THREADS / 32;

}  // namespace

__global__ void __launch_bounds__(TMA_THREADS, TMA_CTAS_PER_SM) step_tma2(const __grid_constant__ StepArgs A)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Stage2* stages = reinterpret_cast<Stage2*>(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + OFF_FULL2);
    uint64_t* empty = reinterpret_cast<uint64_t*>(smem_raw + OFF_EMPTY2);
    volatile int* stage_tile = reinterpret_cast<volatile int*>(smem_raw + OFF_TILE2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem_raw + OFF_FLAG2);
    const int tid = threadIdx.x, lane = tid & 31;
    if (smem_addr(smem_raw) & 127u) {       // TMA destinations need aligned stages
        if (tid == 0 && A.ntiles > 0) atomicOr(A.status, ST_TIMEOUT);
        return;
    }
    const int s = A.s;                      // even: this pass runs steps s and s + 1
    const int lc = s & 3, lp = (s + 3) & 3, l1 = (s + 1) & 3, l2 = (s + 2) & 3;
    const int bank = (s >> 1) & 1;
    int next_claim = -1;
    unsigned nfills = 0;                    // producer: fills issued; fill f goes to stage f % NSTAGE
    bool gave_up = false;                   // producer: its wait for a free stage ran out
    if (tid == 0) {
        for (int k = 0; k < NSTAGE; ++k) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], NWARPS2);
        }
        fence_mbar_init();
        *abort_flag = 0;
        for (int k = 0; k < NSTAGE; ++k) {
            const int t = atomicAdd(A.tile_counter, 1);
            stage_tile[k] = t < A.ntiles ? t : -1;
        }
        next_claim = atomicAdd(A.tile_counter, 1);
    }
    __syncthreads();
    if (tid == 0)
#pragma unroll
        for (int k = 0; k < NSTAGE; ++k) {
            if (stage_tile[k] >= 0) issue_tile2(A, stage_tile[k], stages[k], &full[k], lc, lp);
            else mbar_arrive(&full[k]);
            ++nfills;
        }
    const int tzt = tid % TMA_TZY, txt = tid / TMA_TZY;

    for (int n = 0;; ++n) {
        const int sidx = n & 1;
        const unsigned parity = (unsigned)(n >> 1) & 1u;
        // the CTA goes on only if every thread's wait succeeded (the pass has
        // CTA-wide barriers, so nobody may be left behind)
        const bool ok = gave_up ? false : wait_bounded(&full[sidx], parity, abort_flag, A.spin_limit);
        if (!__syncthreads_and(ok)) {
            if (tid == 0 && atomicExch((int*)abort_flag, 1) == 0) atomicOr(A.status, ST_TIMEOUT);
            break;
        }
        const int t = stage_tile[sidx];
        if (t < 0) break;
        Stage2& st = stages[sidx];
        const PropDesc& P = st.desc;
        const int4 info = st.info;
        const int tt1 = step_tt(P, s), tt2 = step_tt(P, s + 1);
        const int j0 = info.w & 0xffff, i0 = info.w >> 16;
        const int nz = P.nz, nx = P.nx, ld = P.ld;
        const bool general = (info.z & (TILE_STRIP | TILE_RECEIVERS | TILE_SOURCE)) != 0;
        const bool src_tile = (info.z & TILE_SOURCE) != 0, rec_tile = (info.z & TILE_RECEIVERS) != 0;
        const bool fwd = P.mode == MODE_FWD;
        if (tt1 != 0) {
            if (rec_tile && fwd) record_tile<FSC>(P, &st.cur[0][0][0], 4, tt1, info.x, info.y, j0, i0);
            // sub-step 1: level n+1 on R1
#pragma unroll 1
            for (int q = tid; q < NQ1; q += TMA_THREADS) {
                const int c1 = q / QROWS, qr = q - c1 * QROWS;
                const int r0 = qr * TMA_PZ, j = j0 - 4 + r0, i = i0 - 2 + c1;
                float ou[TMA_PZ], ov[TMA_PZ], ow[TMA_PZ];
                if (i < 0 || i >= nx || j < 0 || j >= nz) {
#pragma unroll
                    for (int k = 0; k < TMA_PZ; ++k) ou[k] = ov[k] = ow[k] = 0.0f;   // outside the grid
                } else {
                    const bool owned = c1 >= 2 && c1 < 2 + TMA_TX && qr >= 1 && qr <= TMA_TZY;
                    quad_step<FSC, FSR>(A, P, tt1, &st.cur[0][0][0], c1 + 2, &st.ring[0][0][0], c1, &st.r[0][0], c1,
                                        r0, j, i, general, src_tile, rec_tile, owned, bank, bank ^ 1, ou, ov, ow);
                }
                stv(&st.ring[0][c1][r0], ou);
                stv(&st.ring[1][c1][r0], ov);
                stv(&st.ring[2][c1][r0], ow);
            }
        }
        __syncthreads();      // level n+1 complete on R1 (and the memory variables of the tile in the other bank)
        if (tt1 != 0) {
            const int r0 = 4 + tzt * TMA_PZ, j = j0 + tzt * TMA_PZ, i = i0 + txt;
            if (j < nz && i < nx) {
                const int p = (i + HX) * ld + (j + HZ);
                // level n+1 of the tile point group
#pragma unroll
                for (int f = 0; f < 3; ++f)
                    *reinterpret_cast<float4*>(P.fld[l1][f] + p) =
                        *reinterpret_cast<const float4*>(&st.ring[f][txt + 2][r0]);
                if (tt2 != 0) {
                    // sub-step 2: level n+2 on the tile
                    float ou[TMA_PZ], ov[TMA_PZ], ow[TMA_PZ];
                    quad_step<FSR, FSC>(A, P, tt2, &st.ring[0][0][0], txt + 2, &st.cur[0][0][0], txt + 4, &st.r[0][0],
                                        txt + 2, r0, j, i, general, src_tile, rec_tile, true, bank ^ 1, bank ^ 1, ou, ov, ow);
                    stv(P.fld[l2][0] + p, ou);
                    stv(P.fld[l2][1] + p, ov);
                    stv(P.fld[l2][2] + p, ow);
                }
            }
            if (tt2 != 0 && rec_tile && fwd) record_tile<FSR>(P, &st.ring[0][0][0], 2, tt2, info.x, info.y, j0, i0);
        }
        // This warp is done with the stage.  Its writes of level n+1 into the
        // stage (generic proxy) are ordered before the bulk copies that will
        // refill it (async proxy).
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[sidx]);
        if (tid == 0 && !gave_up) {
            // refill the stage once every warp has released it
            if (!wait_bounded(&empty[sidx], parity, abort_flag, A.spin_limit)) {
                gave_up = true;     // the next full-barrier check takes the whole CTA out
            } else {
                const int t2 = next_claim < A.ntiles ? next_claim : -1;
                stage_tile[sidx] = t2;
                if (t2 >= 0) {
                    issue_tile2(A, t2, stages[sidx], &full[sidx], lc, lp);
                    next_claim = atomicAdd(A.tile_counter, 1);
                } else {
                    mbar_arrive(&full[sidx]);
                }
                ++nfills;
            }
        }
    }
    // a wait ran out: the copies this CTA issued must land before it exits
    if (tid == 0 && *abort_flag) drain_fills<NSTAGE>(full, nfills);
}

size_t step_tma2_smem_bytes() { return OFF_FLAG2 + 16; }

}  // namespace mnad
