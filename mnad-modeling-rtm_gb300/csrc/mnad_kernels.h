// Kernel entry points of the MNAD library (internal; not part of the C ABI).
#pragma once
#include <cstddef>
#include "mnad_device.cuh"

namespace mnad {

// Tile of the direct step kernel: DIRECT_TZ rows (z, one warp) x DIRECT_TX columns.
constexpr int DIRECT_TZ = 32;
constexpr int DIRECT_TX = 8;

// Tile of the TMA step kernel: TMA_TZ x TMA_TX points, TMA_TZY x TMA_TX
// threads, TMA_PZ consecutive z points per thread.
constexpr int TMA_PZ = 4;
constexpr int TMA_TZ = 64;
constexpr int TMA_TX = 16;
constexpr int TMA_TZY = TMA_TZ / TMA_PZ;
constexpr int TMA_THREADS = TMA_TZY * TMA_TX;
// Direct tiles nest in TMA tiles, so both kernels read one receiver bucketing.
static_assert(TMA_TZ % DIRECT_TZ == 0 && TMA_TX % DIRECT_TX == 0, "direct tiles must nest in TMA tiles");
constexpr int TMA_STAGES = 3;         // tiles in flight per CTA
constexpr int TMA_CTAS_PER_SM = 2;
// The narrow variant of the persistent kernel: 64 x 8 tiles (each half of a
// receiver-bucket tile), 128 threads and 2 stages per CTA, 4 CTAs per SM.
constexpr int TMA_TX_NARROW = 8, TMA_STAGES_NARROW = 2, TMA_CTAS_PER_SM_NARROW = 4;
static_assert(TMA_TX % TMA_TX_NARROW == 0, "narrow tiles nest in receiver-bucket tiles");
// Tensor maps of one propagation: per time level one 3-D map over U, V, W
// (the three fields of a level lie at one stride) with the halo box, the same
// with the point box, and the point box of r -- three copies per tile.
constexpr int TMAP_HALO = 0, TMAP_POINT = 2, TMAP_R = 4, TMAPS_PER_PROP = 5;
// Tensor maps of one propagation for the two-step kernel: per time level (four)
// one 3-D map over U, V, W with 72 x 24 boxes (tile + 4-point halo), the same
// with 72 x 20 boxes (tile + 2-point ring), r as a 72 x 20 box.
constexpr int TMAP2_CUR = 0, TMAP2_RING = 4, TMAP2_R = 8, TMAPS_PER_PROP2 = 9;
constexpr int TMA2_BOX_Z = TMA_TZ + 8, TMA2_BOX_X_CUR = TMA_TX + 8, TMA2_BOX_X_RING = TMA_TX + 4;
// tile_info.z flags
constexpr int TILE_STRIP = 1;         // intersects a CPML strip or the grid edge
constexpr int TILE_RECEIVERS = 2;     // has receivers
constexpr int TILE_SOURCE = 4;        // the source point or one of its z/x neighbours

__global__ void step_direct(const __grid_constant__ StepArgs A);
__global__ void step_tma(const __grid_constant__ StepArgs A);
size_t step_tma_smem_bytes();
__global__ void step_tma_narrow(const __grid_constant__ StepArgs A);
size_t step_tma_narrow_smem_bytes();
// Two time steps (A.s even, and A.s + 1) per launch; see mnad_step_tma2.cu.
__global__ void step_tma2(const __grid_constant__ StepArgs A);
size_t step_tma2_smem_bytes();
__global__ void build_r(const double* __restrict__ v, int nz, int nx, double dt, int adjoint,
                        float* __restrict__ r, int ld);
__global__ void seed_sources(const PropDesc* __restrict__ props, int n);
__global__ void injection_table(const PropDesc* __restrict__ desc);
__global__ void snap_export(const void* __restrict__ snap, int codec, const float* __restrict__ scale,
                            size_t nint, int nsnap, int ncols, double* __restrict__ out);
__global__ void snap_import(const double* __restrict__ in, int codec, const float* __restrict__ scale,
                            size_t nint, int nsnap, void* __restrict__ snap);
__global__ void field_export(const float* __restrict__ F, int nz, int nx, int ld, int fix_at, float fix,
                             double* __restrict__ out);
__global__ void scale_f64(const double* __restrict__ in, double s, size_t n, double* __restrict__ out);
__global__ void f16_absmax(const float* __restrict__ x, size_t n, unsigned* __restrict__ maxbits);
__global__ void f16_encode(const float* __restrict__ x, size_t n, const unsigned* __restrict__ maxbits,
                           __half* __restrict__ out, float* __restrict__ scale);
// FP16 -> FP32 of one array stored by f16_encode (value * scale).
__global__ void f16_decode(const __half* __restrict__ in, size_t n, const float* __restrict__ scale,
                           float* __restrict__ out);
__global__ void energy_reduce(const PropDesc* __restrict__ desc, int lvl_new, double* __restrict__ out);
__global__ void axpy_f64(double a, const double* __restrict__ x, size_t n, double* __restrict__ y);
__global__ void divide_f64(const double* __restrict__ num, const double* __restrict__ den, size_t n,
                           double* __restrict__ out);
__global__ void residual_f64(const double* __restrict__ a, const double* __restrict__ b, size_t n,
                             double* __restrict__ out);

}  // namespace mnad
