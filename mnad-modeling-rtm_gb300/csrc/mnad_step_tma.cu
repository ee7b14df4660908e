// step_tma: persistent, TMA-pipelined MNAD time step.
//
// A grid of at most TMA_CTAS_PER_SM CTAs per SM works through the flat tile
// list of a launch group (one geometry, so tile t maps arithmetically to its
// propagation and origin).  Tiles are claimed dynamically from a per-launch
// counter, since strip tiles cost more than interior ones.
//
// Each CTA keeps TMA_STAGES tiles in flight.  A stage is filled with a single
// mbarrier transaction: one 3-D bulk tensor copy of U, V, W of the current
// time level as a TMA_TZ+8 x TMA_TX+4 x 3 box (tile plus a 4-row / 2-column
// halo), one of pU, pV, pW as a TMA_TZ x TMA_TX x 3 box, a 2-D copy of r,
// and 1-D bulk copies of the propagation's descriptor and the tile's
// metadata.  Consumers (all TMA_THREADS threads) wait on that stage's "full"
// barrier, compute the tile (each thread TMA_PZ consecutive z points of one
// column, a register window along z; a warp covers two columns of TMA_TZ
// rows) and write nU, nV, nW with vector stores over pU, pV, pW.  Each warp
// then counts itself in the stage's release count; the warp that completes
// the count refills the stage with the tile thread 0 claimed for it one
// iteration earlier.  So no global-memory latency and no CTA-wide barrier
// sits on the consumers' path, and the producer work of a tile falls on the
// warp that finished it last.

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

#include "mnad_tile.cuh"

namespace mnad {

namespace {

using namespace tile;

// One stage of a tile TMA_TZ x TX points wide (TX = TMA_TX, or a narrower
// tile that nests in the receiver-bucket tiles).
template <int TX>
struct __align__(128) Stage {
    static constexpr int BX = TX + 4;                 // halo box columns (x)
    static constexpr int FS = BX * BZ;                // field stride of the halo buffer (floats)
    float halo[3][BX][BZ];         // U, V, W with halo
    float pts[4][TX][TMA_TZ];      // pU, pV, pW, r
    PropDesc desc;                 // the tile's propagation
    int4 info;                     // receiver entries begin/end, flags, j0 | i0 << 16
    static constexpr unsigned FIELD_BYTES = sizeof(float) * (3 * BX * BZ + 4 * TX * TMA_TZ);
    static constexpr unsigned BYTES = FIELD_BYTES + sizeof(PropDesc) + sizeof(int4);
};
static_assert(offsetof(Stage<TMA_TX>, desc) == Stage<TMA_TX>::FIELD_BYTES, "descriptor follows the field boxes");
static_assert(offsetof(Stage<TMA_TX_NARROW>, desc) == Stage<TMA_TX_NARROW>::FIELD_BYTES,
              "descriptor follows the field boxes");
static_assert(sizeof(PropDesc) % 16 == 0, "bulk copies move multiples of 16 bytes");

// Thread 0: fill `stage` with tile t of the launch (one transaction).
template <int TX>
__device__ __forceinline__ void issue_tile(const StepArgs& A, int t, Stage<TX>& st, uint64_t* bar, int cur)
{
    const int pi = div_small(t, A.tiles_per_prop, A.inv_tiles_per_prop);
    const int tl = t - pi * A.tiles_per_prop;
    const int tx = div_small(tl, A.ntz, A.inv_ntz);
    const int j0 = (tl - tx * A.ntz) * TMA_TZ, i0 = tx * TX;
    const CUtensorMap* maps = static_cast<const CUtensorMap*>(A.tmaps) + (size_t)pi * TMAPS_PER_PROP;
    mbar_expect_tx(bar, Stage<TX>::BYTES);
    bulk_load(&st.desc, A.props + pi, sizeof(PropDesc), bar);
    bulk_load(&st.info, A.tile_info + t, sizeof(int4), bar);
    // U, V, W of a level in one 3-D box each: [f][x][z] is the stage's layout
    tma_load_3d(&st.halo[0][0][0], maps + TMAP_HALO + cur, bar, j0, i0, 0);
    tma_load_3d(&st.pts[0][0][0], maps + TMAP_POINT + (cur ^ 1), bar, j0 + HZ, i0 + HX, 0);
    tma_load_2d(&st.pts[3][0][0], maps + TMAP_R, bar, j0 + HZ, i0 + HX);
}

// Shared-memory layout: NST stages and their full barriers; per stage the
// count of warps that released it, the tile claimed for its next fill and
// the tile it holds; the abort flag; the count of fills issued.
template <int TX, int NST>
struct Layout {
    static constexpr size_t FULL = NST * sizeof(Stage<TX>);
    static constexpr size_t REL = FULL + NST * sizeof(uint64_t);
    static constexpr size_t NEXT = REL + NST * sizeof(int);
    static constexpr size_t TILE = NEXT + NST * sizeof(int);
    static constexpr size_t FLAG = TILE + NST * sizeof(int);
    static constexpr size_t NFILL = FLAG + sizeof(int);
    static constexpr size_t BYTES = NFILL + 16;
};

}  // namespace

// The kernel body for tiles TMA_TZ x TX with NST stages (TMA_TZY x TX threads).
template <int TX, int NST>
__device__ __forceinline__ void step_tma_body(const StepArgs& A)
{
    using St = Stage<TX>;
    using L = Layout<TX, NST>;
    constexpr int FS = St::FS;
    constexpr int NWARPS = TMA_TZY * TX / 32;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    St* stages = reinterpret_cast<St*>(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + L::FULL);
    int* released = reinterpret_cast<int*>(smem_raw + L::REL);
    volatile int* next_tile = reinterpret_cast<volatile int*>(smem_raw + L::NEXT);
    volatile int* stage_tile = reinterpret_cast<volatile int*>(smem_raw + L::TILE);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem_raw + L::FLAG);
    unsigned* nfills = reinterpret_cast<unsigned*>(smem_raw + L::NFILL);
    const int tid = threadIdx.x, lane = tid & 31;
    if (smem_addr(smem_raw) & 127u) {       // TMA destinations need aligned stages
        if (tid == 0 && A.ntiles > 0) atomicOr(A.status, ST_TIMEOUT);
        return;
    }
    const int cur = A.s & 1;
    // Thread 0 claims tiles from the launch's counter, one per iteration and
    // one iteration ahead (the atomic's latency stays off its path); the claim
    // goes to next_tile[stage] for the stage's next fill.  The last warp to
    // release a stage refills it, so the producer work of a tile falls on
    // whichever warp finished it last rather than always on warp 0.
    int next_claim = -1;
    // The first NST tiles of CTA b are b, b + grid, ... (no claim to wait
    // for before the first copies); later tiles are claimed from the counter,
    // which numbers the tiles after those.
    const int first = NST * (int)gridDim.x;
    if (tid == 0) {
        for (int k = 0; k < NST; ++k) {
            mbar_init(&full[k], 1);
            released[k] = 0;
        }
        fence_mbar_init();
        *abort_flag = 0;
#pragma unroll
        for (int k = 0; k < NST; ++k) {
            const int t = (int)blockIdx.x + k * (int)gridDim.x;
            stage_tile[k] = t < A.ntiles ? t : -1;
            if (t < A.ntiles) issue_tile<TX>(A, t, stages[k], &full[k], cur);
            else mbar_arrive(&full[k]);     // releases the consumers: no tile
        }
        // operations that complete a phase of a full barrier (a tile's
        // copies, or the arrive of "no tile"); fill f goes to stage f % NST
        *nfills = NST;
        next_claim = first + atomicAdd(A.tile_counter, 1);
    }
    __syncthreads();
    const int tzt = tid % TMA_TZY, txt = tid / TMA_TZY;
    const int c = txt + 2, r0 = tzt * TMA_PZ + 4;

    for (int n = 0;; ++n) {
        const int sidx = n % NST;
        const unsigned parity = (unsigned)(n / NST) & 1u;
        // the warp leaves together if any of its lanes' waits ran out (no
        // lane may be left behind at a warp-wide synchronisation)
        if (!__all_sync(0xffffffffu, wait_bounded(&full[sidx], parity, abort_flag, A.spin_limit))) {
            if (lane == 0 && atomicExch((int*)abort_flag, 1) == 0) atomicOr(A.status, ST_TIMEOUT);
            break;
        }
        const int t = stage_tile[sidx];      // written before the refill's arrive
        if (t < 0) break;
        if (tid == 0) {                      // the claim for this stage's next fill
            next_tile[sidx] = next_claim;
            next_claim = first + atomicAdd(A.tile_counter, 1);
        }
        const St& st = stages[sidx];
        const PropDesc& P = st.desc;
        const int4 info = st.info;
        // Per-tile scalars in registers.
        const int tt = step_tt(P, A.s);
        const int j0 = info.w & 0xffff, i0 = info.w >> 16;
        const int tl = j0 / TMA_TZ + (i0 / TMA_TX) * P.ntz;     // receiver-bucket tile
        const int cb0 = i0 % TMA_TX;                            // its column holding the tile's first
        const int nz = P.nz, nx = P.nx, d = P.d, ld = P.ld, nt = P.nt, mode = P.mode;
        if (tt != 0 && (info.z & TILE_RECEIVERS) && mode == MODE_FWD)
            record_tile<FS>(P, &st.halo[0][0][0], 2, tt, info.x, info.y, j0, i0);
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
                win.load<FS>(&st.halo[0][0][0], c, r0);
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
                        for (int k = 0; k < Q; ++k) accumulate_product(&P.illum[q0 + k], d2u[k], d2u[k]);
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
                            accumulate_product(&P.image[q0 + k], us, ou[k]);
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
            const MemBank bank{P.mx, P.mz};
            if (!lean && d > 0) prefetch_strip_state(P, bank, j, i);
            {
                Window win;            // dies here: later phases re-read the stage
                win.load<FS>(&st.halo[0][0][0], c, r0);
                mnad_update_pairs(A.coef2, win, rr, s2u, s2v, s2w);
            }
            if (!lean) {
                float2 cu[2], cv[2], cw[2];
#pragma unroll
                for (int m = 0; m < 2; ++m) cu[m] = cv[m] = cw[m] = pr(0.0f, 0.0f);
                cpml_vec<FS>(P, &st.halo[0][0][0], c, r0, tt, j, i, p, has_src, rr, bank, bank, true, cu, cv, cw);
                // sF -= r * (F1_x + F1_z), per point fmaf(-r, c, s)
#pragma unroll
                for (int m = 0; m < 2; ++m) {
                    const float2 nr = pr(-rr[2 * m], -rr[2 * m + 1]);
                    s2u[m] = pfma(nr, cu[m], s2u[m]);
                    s2v[m] = pfma(nr, cv[m], s2v[m]);
                    s2w[m] = pfma(nr, cw[m], s2w[m]);
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
                        if (P.snap_flags & SNAP_ILLUM) accumulate_product(&P.illum[q], d2u, d2u);
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
                    injection(P, tt, tl, cb0 + txt, p, inj);
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
                        accumulate_product(&P.image[q], us, ou[k]);
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
        // This warp is done with the stage: its reads are ordered before the
        // release (warp barrier, then a CTA-scope fence before the count).
        __syncwarp();
        int last = 0;
        if (lane == 0) {
            __threadfence_block();
            last = atomicAdd(&released[sidx], 1) == NWARPS - 1;
        }
        if (__shfl_sync(0xffffffffu, last, 0) && lane == 0) {
            // Every warp has released the stage: refill it with the tile
            // thread 0 claimed for it in this iteration.
            released[sidx] = 0;
            __threadfence_block();
            fence_proxy_async_smem();       // the reads above come before the copies' writes
            const int t2 = next_tile[sidx];
            if (t2 < A.ntiles) {
                stage_tile[sidx] = t2;
                issue_tile<TX>(A, t2, stages[sidx], &full[sidx], cur);
            } else {
                stage_tile[sidx] = -1;
                mbar_arrive(&full[sidx]);   // releases the consumers: no tile
            }
            atomicAdd(nfills, 1u);
        }
        __syncwarp();
    }
    // A wait ran out: the copies this CTA issued must land before it exits.
    // Every warp leaves the loop (each wait is bounded), so after the barrier
    // no refill is in progress and the fills form a prefix of the sequence.
    __syncthreads();
    if (tid == 0 && *abort_flag) drain_fills<NST>(full, *nfills);
}

// 64 x 16 tiles, 3 stages, 256 threads, 2 CTAs per SM (128 registers).
__global__ void __launch_bounds__(TMA_THREADS, TMA_CTAS_PER_SM) step_tma(const __grid_constant__ StepArgs A)
{
    step_tma_body<TMA_TX, TMA_STAGES>(A);
}
size_t step_tma_smem_bytes() { return Layout<TMA_TX, TMA_STAGES>::BYTES; }

// 64 x 8 tiles (half a receiver-bucket tile), 2 stages, 128 threads, 4 CTAs
// per SM (128 registers; 4 CTAs of 2 stages fit the SM's shared memory).
__global__ void __launch_bounds__(TMA_TZY * TMA_TX_NARROW, TMA_CTAS_PER_SM_NARROW)
    step_tma_narrow(const __grid_constant__ StepArgs A)
{
    step_tma_body<TMA_TX_NARROW, TMA_STAGES_NARROW>(A);
}
size_t step_tma_narrow_smem_bytes() { return Layout<TMA_TX_NARROW, TMA_STAGES_NARROW>::BYTES; }

}  // namespace mnad
