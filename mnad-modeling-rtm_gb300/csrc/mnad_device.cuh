// Device-side definitions shared by the MNAD step kernels.
//
// A "propagation" is one shot advancing one wavefield triple (U, V, W) in
// time, forward (fwd_PDE_exact_MNAD.m) or reverse (Born_adj_MNAD.m).  Many
// propagations (shots, possibly on different grids) advance together in one
// launch per time step; each launch covers a flat list of tiles and every
// tile knows its propagation through `tile_prop`.
//
// Storage of every per-point field (U, V, W, both time levels, and r=v^2dt^2)
// is column-major with z fastest, exactly like the MATLAB arrays, with a
// zero halo: element (j, i) lives at base[(i + HX) * ld + (j + HZ)].  The halo
// is never written, so it reproduces the reference's omission of out-of-grid
// neighbours (the index ranges in SRC/MNAD/A??_gen.m) without bounds checks,
// and every 2-D tile including its halo is in-bounds for TMA.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace mnad {

constexpr int HZ = 4;   // zero rows before row 0 (keeps column starts 16-byte aligned)
constexpr int HZB = 4;  // at least this many zero rows after row nz-1
constexpr int HX = 2;   // zero columns on each side (V needs x +- 2)

enum Mode { MODE_FWD = 0, MODE_ADJ = 1 };
enum Codec { CODEC_F32 = 0, CODEC_BF16 = 1, CODEC_F16 = 2 };
enum SnapFlags { SNAP_WRITE = 1, SNAP_ILLUM = 2 };
enum Pairing { PAIR_REFERENCE = 0, PAIR_ALIGNED = 1 };

// Status bits written by kernels (never traps).  ST_NONFINITE goes to the
// propagation's own word (PropDesc::status), ST_TIMEOUT to the launch's
// (StepArgs::status); the host reads both after a run and turns them into
// MNAD_E_NUMERIC / MNAD_E_TIMEOUT.
enum StatusBits : unsigned {
    ST_NONFINITE = 1u,     // a recorded receiver value was not finite
    ST_F16_RANGE = 2u,     // an FP16 snapshot value saturated
    ST_TIMEOUT = 4u,       // a bounded wait for a tile copy ran out
};

// Default bound of a barrier wait (polls), and the bound of the wait with
// which a CTA that gave up lets its own copies in flight land before it exits.
constexpr unsigned SPIN_LIMIT_DEFAULT = 1u << 22;
constexpr unsigned DRAIN_LIMIT = 1u << 24;

// The distinct stencil coefficients of one destination point.  Each is
// alpha*r + beta*r^2 with r = v^2 dt^2 at the destination (the reference's
// v(j,i).^2*dt^2 and v(j,i).^4*dt^4 terms).  The self-coupling blocks (Auu,
// Avv, Aww) are applied in difference form, sum_k c_k (F_k - F_0), which is
// exact for constant fields whatever the rounding of c_k; their centre
// entries therefore reduce to
//   Auu: 2 - sum_k c_k                        (the row sums to exactly 2)
//   Avv: 2 - sum_k c_k + (-15 r/dx^2 + 15 r^2/dx^4)   -> K_VV_R
//   Aww: 2 - sum_k c_k + (-15 r/dz^2 + 15 r^2/dz^4)   -> K_WW_R
// (sums of Auu_gen.m:30-86, Avv_gen.m:29-85, Aww_gen.m:31-87).  The
// sign pattern of the odd couplings is applied in mnad_update().
enum Coef {
    K_UU_Z, K_UU_X, K_UU_D,                  // Auu_gen.m
    K_UV_X1, K_UV_D, K_UV_X2,                // Auv_gen.m
    K_UW_Z1, K_UW_D, K_UW_Z2,                // Auw_gen.m
    K_VU_X1, K_VU_D,                         // Avu_gen.m
    K_VV_Z, K_VV_X, K_VV_D, K_VV_R,          // Avv_gen.m
    K_VW,                                    // Avw_gen.m
    K_WU_Z1, K_WU_D,                         // Awu_gen.m
    K_WV,                                    // Awv_gen.m
    K_WW_Z, K_WW_X, K_WW_D, K_WW_R,          // Aww_gen.m
    NCOEF
};

// 16-byte aligned (and sized) so a CTA can fetch it with one bulk copy.
struct __align__(16) PropDesc {
    int mode;          // MODE_FWD / MODE_ADJ
    int nt;            // steps of this propagation
    int nz, nx;        // padded grid (as passed to the reference)
    int ld;            // z pitch of per-point storage (floats)
    int d;             // CPML thickness (d_pml)
    int dpz;           // pitch of one z-strip column (floats, >= d + 6, multiple of 4)
    int zb0;           // first storage row of the bottom z strip: (nz - d) rounded down to 4
    int tile_base;     // first global tile of this propagation
    int s_off;         // global step at which this propagation started (even)
    int s_begin, s_end;  // global steps [s_begin, s_end) in which it may advance
    int ntz, ntx;      // receiver-bucket (TMA_TZ x TMA_TX) tiles along z / x
    float* fld[4][3];  // [time level][U,V,W], storage origin (halo included); the
                       // one-step kernels keep level s & 1, the two-step kernel
                       // level s & 3 (levels 2, 3 are null without its storage)
    const float* r;    // v^2 dt^2, same storage
    float* mx;         // x-strip memory variables [side 2][var 9][d][ld]
    float* mz;         // z-strip memory variables [side 2][var 9][nx][dpz]; top side slot k
                       // holds row k, bottom side slot k holds row zb0 + k
    float* mx2;        // second bank of both (two-step kernel only, else null)
    float* mz2;
    float kx, kz;      // 3 ln(1/R) / (2 D^3), D = d*dx or d*dz (C_cof.m:6,38)
    float dx, dz, dt, inv_dt;
    // source (forward): storage offset of the point and the amount
    // r_src*w(tt) injected at each step (fwd_PDE_exact_MNAD.m:111)
    int src;                 // -1: none
    const float* src_amp;    // [nt]
    // receivers, bucketed per TMA_TZ x TMA_TX tile (for every step kernel):
    // entries tile_rec[t]..tile_rec[t+1]
    int nr;
    const int* rec_pt;       // storage offset of each entry
    const int* rec_id;       // receiver column rr of each entry
    const double* rec_r;     // r at the receiver (adjoint injection scale)
    const int* tile_rec;     // [ntz*ntx + 1]
    const int* col_rec;      // [ntz*ntx*TMA_TX + 1]: entries of local column c of tile t
                             // are col_rec[t*TMA_TX + c] .. col_rec[t*TMA_TX + c+1]
    double* data;            // [nr][nt] (column-major nt x nr): fwd out / adj in
    double* datav;           // optional fwd outputs
    double* dataw;
    float* inj;              // adjoint: [nt][nr] injection amounts (float)(rec_r[e] * data(tt, rec_id[e]))
                             // in bucket entry order, built when the propagation starts
    // snapshots (forward with indx==1) / imaging (adjoint)
    int T;                   // 0: none
    float invT;              // 1/T (exact quotients of tt/T via (tt + 0.5) * invT)
    int nsnap;               // snapshots filled by the forward: floor(nt/T)
    int ncols;               // columns of the reference's UU matrix
    int codec;
    int pairing;
    int img_steps;           // adjoint: number of imaging steps floor(nt/T)
    void* snap;              // [ncols' = nsnap][nint]
    int snap_stage;          // forward with the FP16 codec: every snapshot is
                             // written in FP32 to one staging slot, then encoded
    const float* snap_scale; // per-snapshot scale (FP16 codec), may be null
    int snap_col0;           // snapshot column (0-based) held in the first slot of `snap`
    int snap_cols;           // slots of `snap`: a forward writes, an adjoint reads only
                             // columns snap_col0 .. snap_col0 + snap_cols - 1
    int snap_flags;          // forward: SNAP_WRITE | SNAP_ILLUM (checkpointed RTM runs them apart)
    double* illum;           // [nint] sum of d2u^2 (forward)
    double* image;           // [nint] sum of US.*UR (adjoint)
    float inv_dt2;
    unsigned* status;
};

// Stencil coefficient polynomials of one grid spacing (dx, dz): passed as
// kernel parameters so the FMAs read them straight from the constant bank.
struct Coefs {
    float alpha[NCOEF], beta[NCOEF];
};

// Arguments of one step launch: the propagations of one (dx, dz) group.
// The same coefficients as (c, c) pairs for packed FP32x2 arithmetic over two
// z-points; the entries that the update applies with a negative sign (K_UV_X1
// of alpha and beta, K_UV_D of beta) are stored negated.
struct Coefs2 {
    float2 alpha[NCOEF], beta[NCOEF];
};

struct StepArgs {
    Coefs coef;
    Coefs2 coef2;          // TMA kernel
    const PropDesc* props;
    const int* tile_prop;
    const void* tmaps;     // CUtensorMap[nprops][TMAPS_PER_PROP] (TMA kernel)
    const int4* tile_info; // per tile: receiver bucket begin/end, flags (TMA kernel)
    int* tile_counter;     // tiles claimed so far in this launch (TMA kernel, zeroed per run)
    int ntiles;
    int ntz;               // tiles along z of every propagation of the group
    int tiles_per_prop;    // ntz * ntx (one geometry per launch group)
    float inv_tiles_per_prop, inv_ntz;   // 1/tiles_per_prop, 1/ntz: division-free tile decode
    int s;                 // global step index
    unsigned* status;      // launch-wide status word (ST_TIMEOUT: the launch did not finish its tiles)
    unsigned spin_limit;   // polls of a bounded barrier wait before it gives up (persistent kernels; set by the host, > 0)
};

// Neighbourhood of one point for the three fields.  Naming: <f><z><x> with
// z/x in {m: -1, 0: 0, p: +1}; the x+-2 (V) and z+-2 (W) reaches are extra.
struct Hood {
    float u00, uzm, uzp, uxm, uxp, umm, upm, ump, upp;
    float v00, vzm, vzp, vxm, vxp, vmm, vpm, vmp, vpp, vxm2, vxp2;
    float w00, wzm, wzp, wxm, wxp, wmm, wpm, wmp, wpp, wzm2, wzp2;
};

// su = nU - 2U + pU (likewise sv, sw) before the CPML term: the nine
// products of fwd_PDE_exact_MNAD.m:114-116 minus the exact 2*F part.  The
// self blocks are taken in difference form, every coefficient is
// alpha_k r + beta_k r^2, and each row is evaluated as
//     r * sum_k alpha_k D_k + r^2 * sum_k beta_k D_k
// over the neighbour combinations D_k (two FMAs per term, constants from the
// kernel parameters).  Signs of the odd couplings follow the J index arrays
// of the generator files (e.g. Auv_gen.m:27-78: +c at i+1, -c at i-1,
// +c at i-2, -c at i+2).
__device__ __forceinline__ void mnad_update(const Coefs& K, float r, const Hood& h,
                                            float& su, float& sv, float& sw)
{
    const float q = r * r;
    const float* a = K.alpha;
    const float* b = K.beta;
    // U combinations
    const float u2 = h.u00 + h.u00;
    const float dUz = (h.uzm + h.uzp) - u2, dUx = (h.uxm + h.uxp) - u2;
    const float uA = h.umm + h.upp, uB = h.upm + h.ump;
    const float dUd = (uA + uB) - (u2 + u2);
    const float uLx = h.uxm - h.uxp;                          // Avu_gen.m:30,37
    const float uLz = h.uzm - h.uzp;                          // Awu_gen.m:29,36
    const float uDx = (h.umm + h.upm) - (h.ump + h.upp);      // Avu_gen.m:44-65
    const float uDz = (h.umm + h.ump) - (h.upm + h.upp);      // Awu_gen.m:44-67
    // V combinations
    const float v2 = h.v00 + h.v00;
    const float dVz = (h.vzm + h.vzp) - v2, dVx = (h.vxm + h.vxp) - v2;
    const float vA = h.vmm + h.vpp, vB = h.vpm + h.vmp;
    const float dVd = (vA + vB) - (v2 + v2);
    const float vX1 = h.vxp - h.vxm;                          // Auv_gen.m:29,36
    const float vDx = (h.vmp + h.vpp) - (h.vmm + h.vpm);      // Auv_gen.m:43-64
    const float vX2 = h.vxm2 - h.vxp2;                        // Auv_gen.m:71,78
    const float vXZ = vA - vB;                                // Awv_gen.m:31-52
    // W combinations
    const float w2 = h.w00 + h.w00;
    const float dWz = (h.wzm + h.wzp) - w2, dWx = (h.wxm + h.wxp) - w2;
    const float wA = h.wmm + h.wpp, wB = h.wpm + h.wmp;
    const float dWd = (wA + wB) - (w2 + w2);
    const float wZ1 = h.wzp - h.wzm;                          // Auw_gen.m:29,36
    const float wDz = (h.wpm + h.wpp) - (h.wmm + h.wmp);      // Auw_gen.m:43-64
    const float wZ2 = h.wzm2 - h.wzp2;                        // Auw_gen.m:71,78
    const float wXZ = wA - wB;                                // Avw_gen.m:29-50
    // nU row
    float ra = a[K_UU_Z] * dUz;
    ra = fmaf(a[K_UU_X], dUx, ra);
    ra = fmaf(a[K_UV_X1], vX1, ra);
    ra = fmaf(a[K_UV_X2], vX2, ra);
    ra = fmaf(a[K_UW_Z1], wZ1, ra);
    ra = fmaf(a[K_UW_Z2], wZ2, ra);
    float qa = b[K_UU_Z] * dUz;
    qa = fmaf(b[K_UU_X], dUx, qa);
    qa = fmaf(b[K_UU_D], dUd, qa);
    qa = fmaf(b[K_UV_X1], vX1, qa);
    qa = fmaf(b[K_UV_D], vDx, qa);
    qa = fmaf(b[K_UV_X2], vX2, qa);
    qa = fmaf(b[K_UW_Z1], wZ1, qa);
    qa = fmaf(b[K_UW_D], wDz, qa);
    qa = fmaf(b[K_UW_Z2], wZ2, qa);
    su = fmaf(q, qa, r * ra);
    // nV row
    float rb = a[K_VV_Z] * dVz;
    rb = fmaf(a[K_VV_X], dVx, rb);
    rb = fmaf(a[K_VV_R], h.v00, rb);
    rb = fmaf(a[K_VU_X1], uLx, rb);
    rb = fmaf(a[K_VU_D], uDx, rb);
    rb = fmaf(a[K_VW], wXZ, rb);
    float qb = b[K_VV_Z] * dVz;
    qb = fmaf(b[K_VV_X], dVx, qb);
    qb = fmaf(b[K_VV_D], dVd, qb);
    qb = fmaf(b[K_VV_R], h.v00, qb);
    qb = fmaf(b[K_VU_X1], uLx, qb);
    qb = fmaf(b[K_VU_D], uDx, qb);
    qb = fmaf(b[K_VW], wXZ, qb);
    sv = fmaf(q, qb, r * rb);
    // nW row
    float rc = a[K_WW_Z] * dWz;
    rc = fmaf(a[K_WW_X], dWx, rc);
    rc = fmaf(a[K_WW_R], h.w00, rc);
    rc = fmaf(a[K_WU_Z1], uLz, rc);
    rc = fmaf(a[K_WU_D], uDz, rc);
    rc = fmaf(a[K_WV], vXZ, rc);
    float qc = b[K_WW_Z] * dWz;
    qc = fmaf(b[K_WW_X], dWx, qc);
    qc = fmaf(b[K_WW_D], dWd, qc);
    qc = fmaf(b[K_WW_R], h.w00, qc);
    qc = fmaf(b[K_WU_Z1], uLz, qc);
    qc = fmaf(b[K_WU_D], uDz, qc);
    qc = fmaf(b[K_WV], vXZ, qc);
    sw = fmaf(q, qc, r * rc);
}

// CPML coefficients of C_cof.m:6-16 at one strip point.  X is the distance
// term of x_b/z_b (D, D-h, ..., h on the low side; h, ..., D on the high side).
__device__ __forceinline__ void cpml_coefs(float K, float v, float X, float dt,
                                           float& c1, float& c2, float& c3)
{
    const float s0 = K * v;
    const float sig = s0 * (X * X);
    const float dsig = 2.0f * s0 * X;
    const float inv_den = 1.0f / fmaf(sig, 0.5f * dt, 1.0f);
    c1 = (1.0f - sig * (0.5f * dt)) * inv_den;
    c2 = (dsig * dt) * inv_den;
    c3 = (sig * dt) * inv_den;
}

// One side of Ux123_gen.m / Uz123_gen.m for one field at one point:
// gr = (behind - ahead) on the low side, (ahead - behind) on the high side;
// lap = behind - 2 F + ahead.  Updates m1..m3 in place, returns the new m1.
__device__ __forceinline__ float cpml_mem(float c1, float c2, float c3, float inv_h,
                                          float gr, float lap, float& m1, float& m2, float& m3)
{
    const float inv_h2 = inv_h * inv_h;
    const float g2 = c2 * inv_h * gr;                 // (c2/h)*gr
    m3 = fmaf(c1, m3, 0.5f * g2);
    m2 = fmaf(c1, m2, g2) + c3 * fmaf(lap, inv_h2, -m3);
    m1 = fmaf(c1, m1, 0.5f * g2) + c3 * fmaf(2.0f * lap, inv_h2, -m2);
    return m1;
}

__device__ __forceinline__ float snap_decode(const void* base, int codec, size_t i, float scale)
{
    if (codec == CODEC_BF16) return __bfloat162float(static_cast<const __nv_bfloat16*>(base)[i]);
    if (codec == CODEC_F16) return __half2float(static_cast<const __half*>(base)[i]) * scale;
    return static_cast<const float*>(base)[i];
}

// The FP64 value of a float, from its IEEE-754 fields with integer
// operations: sign, exponent rebiased from 127 to 1023 (+896), the 23
// mantissa bits shifted to the top of the 52.  Exact for every normal float
// and for zeros; subnormals, infinities and NaNs take the hardware conversion.
__device__ __forceinline__ double widen_f32(float x)
{
    const unsigned u = __float_as_uint(x);
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    if ((u & 0x7fffffffu) == 0u) return __longlong_as_double((long long)sign);
    const unsigned e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)x;
    const unsigned long long bits = sign | ((unsigned long long)(e + 896u) << 52) |
                                    ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)bits);
}

// acc += a * b for the FP64 illumination and image accumulations
// (fwd_PDE_exact_MNAD.m:126-143, Born_adj_MNAD.m:127-134): the product is
// formed in FP32 (one rounding, 2^-24 relative) and added in FP64, so a point
// costs one FP64 operation -- GB300 runs FP64 at a small fraction of its FP32
// rate -- instead of two conversions and an FP64 fused multiply-add.  A zero
// product (the wave has not reached the point) leaves the accumulator, and its
// memory, untouched.
__device__ __forceinline__ void accumulate_product(double* acc, float a, float b)
{
    const float p = __fmul_rn(a, b);
    if (p == 0.0f) return;
    *acc += widen_f32(p);
}

}  // namespace mnad
