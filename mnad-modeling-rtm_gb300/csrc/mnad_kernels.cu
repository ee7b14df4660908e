// MNAD time-step kernels and their small helpers.
//
// step_direct: one fused kernel per time step for a whole batch of
// propagations.  Per point it reads U,V,W (3x3 box, plus x+-2 for V and z+-2
// for W, through the read-only cache), pU,pV,pW and r, and writes nU,nV,nW
// over pU,pV,pW (in-place leapfrog).  In the CPML strips it also updates the
// memory variables of Ux123_gen.m / Uz123_gen.m; the source, the receivers,
// the d2u snapshots + illumination (forward) and the imaging condition
// (adjoint) are fused in as well, so one step is one launch.
#include "mnad_kernels.h"
#include "mnad_point.cuh"

namespace mnad {

__global__ void __launch_bounds__(DIRECT_TZ * DIRECT_TX, 3)
step_direct(const __grid_constant__ StepArgs A)
{
    const Coefs& K = A.coef;
    const PropDesc* __restrict__ props = A.props;
    const int* __restrict__ tile_prop = A.tile_prop;
    const int s = A.s;
    __shared__ __align__(16) PropDesc P;
    const int pi = __ldg(tile_prop + blockIdx.x);
    load_desc(P, props + pi);
    __syncthreads();
    const int tt = step_tt(P, s);
    if (tt == 0) return;
    const int tl = blockIdx.x - P.tile_base;
    const int tz = tl % A.ntz, tx = tl / A.ntz;
    const int j0 = tz * DIRECT_TZ, i0 = tx * DIRECT_TX;
    const int j = j0 + threadIdx.x;
    const int i = i0 + threadIdx.y;
    // receiver buckets are per TMA tile and column; this tile's DIRECT_TX
    // columns are consecutive columns of one TMA tile
    const int cb = (j0 / TMA_TZ + (i0 / TMA_TX) * P.ntz) * TMA_TX + i0 % TMA_TX;
    const int cur = s & 1;
    const float* __restrict__ U = P.fld[cur][0];
    const float* __restrict__ V = P.fld[cur][1];
    const float* __restrict__ W = P.fld[cur][2];
    float* nU = P.fld[cur ^ 1][0];
    float* nV = P.fld[cur ^ 1][1];
    float* nW = P.fld[cur ^ 1][2];
    if (P.mode == MODE_FWD && P.nr > 0) record_receivers(P, tt, cb, j0, U, V, W);
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
    mnad_update(K, r, h, su, sv, sw);
    float xu, xv, xw;
    finish_point(P, tt, j, i, p, r, h, su, sv, sw, pu, pv, pw, adjoint_injection(P, tt, cb + threadIdx.y, p), xu, xv, xw);
    nU[p] = xu;
    nV[p] = xv;
    nW[p] = xw;
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

// Injection table of an adjoint propagation: row tt holds, in receiver-bucket
// entry order, the amount r_e * data(tt+1, id_e) that Born_adj_MNAD.m:109-111
// adds at the receiver after the update of step tt (rounded to float once,
// exactly as the step kernels would).
__global__ void injection_table(const PropDesc* __restrict__ desc)
{
    const PropDesc& P = *desc;
    const size_t nr = (size_t)P.nr, n = (size_t)P.nt * nr;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const size_t tt = k / nr, e = k - tt * nr;
        P.inj[k] = (float)(P.rec_r[e] * P.data[(size_t)P.rec_id[e] * P.nt + tt]);
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

// Largest |x| of one FP32 snapshot (positive floats order like their bits).
__global__ void f16_absmax(const float* __restrict__ x, size_t n, unsigned* __restrict__ maxbits)
{
    float m = 0.0f;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[k]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(maxbits, __float_as_uint(m));
}

// FP16 encoding of one snapshot with a power-of-two scale s chosen from its
// maximum so that max/s < 2^14 (no saturation; the scale multiply is exact).
// Arrays whose maximum is below 2^-100 keep s = 2^-114, so 1/s stays finite.
__global__ void f16_encode(const float* __restrict__ x, size_t n, const unsigned* __restrict__ maxbits,
                           __half* __restrict__ out, float* __restrict__ scale)
{
    const float mx = __uint_as_float(*maxbits);
    int e = 0;
    frexpf(mx, &e);                                   // mx = f * 2^e, 0.5 <= f < 1
    e = max(e, -100);                                 // tiny maxima: keep 2^(14-e) finite
    const float s = mx > 0.0f ? ldexpf(1.0f, e - 14) : 1.0f;
    const float inv = mx > 0.0f ? ldexpf(1.0f, 14 - e) : 1.0f;
    if (blockIdx.x == 0 && threadIdx.x == 0) *scale = s;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        out[k] = __float2half_rn(x[k] * inv);
}

__global__ void f16_decode(const __half* __restrict__ in, size_t n, const float* __restrict__ scale,
                           float* __restrict__ out)
{
    const float s = *scale;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        out[k] = __half2float(in[k]) * s;
}

// Energy of one propagation after a step, in FP64 over the image region:
// 1/2 sum ((Unew - Uold)^2 / r + Vnew^2 + Wnew^2) * dx * dz.
__global__ void energy_reduce(const PropDesc* __restrict__ desc, int lvl_new, double* __restrict__ out)
{
    const PropDesc& P = *desc;
    const int d = P.d, niz = P.nz - 2 * d, nix = P.nx - 2 * d;
    const size_t n = (size_t)niz * nix;
    const float* Un = P.fld[lvl_new][0];
    const float* Uo = P.fld[lvl_new ^ 1][0];
    const float* Vn = P.fld[lvl_new][1];
    const float* Wn = P.fld[lvl_new][2];
    double acc = 0.0;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(k % niz) + d, i = (int)(k / niz) + d;
        const size_t o = (size_t)(i + HX) * P.ld + (j + HZ);
        const double du = (double)Un[o] - (double)Uo[o];
        const double v = Vn[o], w = Wn[o];
        acc += du * du / (double)P.r[o] + v * v + w * w;
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, 0.5 * (double)P.dx * (double)P.dz * acc);
}

// y += a * x in FP64 (the image / illumination stack over shots,
// main_Acoustic_RTM.m:237-244,256-262).
__global__ void axpy_f64(double a, const double* __restrict__ x, size_t n, double* __restrict__ y)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        y[k] = fma(a, x[k], y[k]);
}

// out = num ./ den with IEEE semantics (img_RTM = mean(mhh,3)./illum,
// main_Acoustic_RTM.m:262; a zero illumination gives Inf/NaN as in MATLAB).
__global__ void divide_f64(const double* __restrict__ num, const double* __restrict__ den, size_t n,
                           double* __restrict__ out)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        out[k] = num[k] / den[k];
}

// Scattered data of the RTM workflow: data_sct = data - datas
// (main_Acoustic_RTM.m:225), formed on the device.
__global__ void residual_f64(const double* __restrict__ a, const double* __restrict__ b, size_t n,
                             double* __restrict__ out)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        out[k] = a[k] - b[k];
}

}  // namespace mnad
