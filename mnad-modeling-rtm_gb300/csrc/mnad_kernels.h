// Kernel entry points of the MNAD library (internal; not part of the C ABI).
#pragma once
#include <cstddef>
#include "mnad_device.cuh"

namespace mnad {

// Tile of the direct step kernel: DIRECT_TZ rows (z, one warp) x DIRECT_TX columns.
constexpr int DIRECT_TZ = 32;
constexpr int DIRECT_TX = 8;

__global__ void step_direct(const PropDesc* __restrict__ props, const int* __restrict__ tile_prop, int s);
__global__ void build_r(const double* __restrict__ v, int nz, int nx, double dt, int adjoint,
                        float* __restrict__ r, int ld);
__global__ void seed_sources(const PropDesc* __restrict__ props, int n);
__global__ void snap_export(const void* __restrict__ snap, int codec, const float* __restrict__ scale,
                            size_t nint, int nsnap, int ncols, double* __restrict__ out);
__global__ void snap_import(const double* __restrict__ in, int codec, const float* __restrict__ scale,
                            size_t nint, int nsnap, void* __restrict__ snap);
__global__ void field_export(const float* __restrict__ F, int nz, int nx, int ld, int fix_at, float fix,
                             double* __restrict__ out);
__global__ void scale_f64(const double* __restrict__ in, double s, size_t n, double* __restrict__ out);
__global__ void residual_f64(const double* __restrict__ a, const double* __restrict__ b, size_t n,
                             double* __restrict__ out);

}  // namespace mnad
