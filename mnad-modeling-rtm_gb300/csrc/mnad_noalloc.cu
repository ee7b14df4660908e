// mnad_fwd_pde_exact_noalloc: forward modeling of one shot without any
// device-memory allocation.
//
// Some callers cannot let a library call cudaMalloc: a host application whose
// GPU memory is wholly reserved by its own allocator (a framework's caching
// allocator, a server that takes the memory up front), or a process that
// forbids allocation once it is running.  For them this entry point keeps
// every piece of working memory -- wavefield state, CPML memory variables,
// the propagation descriptor, receiver tables, the shot record before it is
// copied out -- in one file-scope device array of NOALLOC_SCRATCH_BYTES.
// Every GPU that loads the library holds that array until the process exits.
//
// The first call on a device looks up the array's device address there
// (cudaGetSymbolAddress with that device current), so that first call should
// come before any stream capture on that device; host code never passes the
// array's host-side name to a kernel.  Each call makes its device current and
// gives the calling thread its previous current device back on return.  All calls share the array and each call
// overwrites what the previous one left: the state is cleared at the start of
// every call, and calls that overlap on the GPU (from several host threads or
// streams) would race, so this library serialises its own callers with a lock.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "mnad_engine.h"
#include "mnad_jobs.h"
#include "mnad_kernels.h"

namespace mnad {
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(64) << 20;   // 64 MiB
constexpr int MAX_DEVICES = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_lock;
void* g_noalloc_addr[MAX_DEVICES] = {};

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

// Makes `device` current for the call and gives the calling thread its own
// current device back on every exit path (the caller -- a MATLAB session, a
// host application with its own CUDA work -- keeps the device it had).
class DeviceScope {
public:
    explicit DeviceScope(int device)
    {
        MNAD_CK(cudaGetDevice(&prev_));
        if (prev_ != device) MNAD_CK(cudaSetDevice(device));
    }
    ~DeviceScope() { cudaSetDevice(prev_); }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
private:
    int prev_ = 0;
};

// Device address of the scratch array on the current device (set-up on the
// first call per device).
unsigned char* scratch_on(int device)
{
    if (device < 0 || device >= MAX_DEVICES) throw Error(MNAD_E_ARG, "device index out of range");
    if (!g_noalloc_addr[device]) {
        void* p = nullptr;
        MNAD_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_addr[device] = p;
    }
    return static_cast<unsigned char*>(g_noalloc_addr[device]);
}

}  // namespace

size_t noalloc_scratch_bytes() { return NOALLOC_SCRATCH_BYTES; }

// Scratch bytes one forward shot needs (0 on invalid geometry).
size_t noalloc_bytes_needed(int nz, int nx, int d, int nt, int nr)
{
    const size_t ld = (size_t)((nz + HZ + HZB + 31) / 32 * 32);
    const size_t S = ld * (nx + 2 * HX);
    const size_t dpz = (size_t)((d + 6 + 3) / 4 * 4);
    const size_t ntiles = (size_t)((nz + DIRECT_TZ - 1) / DIRECT_TZ) * ((nx + DIRECT_TX - 1) / DIRECT_TX);
    const size_t nbt = (size_t)((nz + TMA_TZ - 1) / TMA_TZ) * ((nx + TMA_TX - 1) / TMA_TX);
    size_t b = 0;
    b += align256(sizeof(PropDesc)) + align256(sizeof(unsigned));
    b += align256(ntiles * sizeof(int)) + align256((nbt + 1) * sizeof(int)) + align256((nbt * TMA_TX + 1) * sizeof(int));
    b += align256((size_t)nr * sizeof(int)) * 2 + align256((size_t)nr * sizeof(double));
    b += align256((size_t)nt * sizeof(float));
    b += align256(6 * S * sizeof(float)) + align256(S * sizeof(float));
    if (d > 0) b += align256((size_t)2 * 9 * d * ld * sizeof(float)) + align256((size_t)2 * 9 * nx * dpz * sizeof(float));
    b += align256((size_t)nt * nr * sizeof(double));
    return b;
}

void fwd_noalloc(int device, double dx, int xs, const std::vector<int>& xr, double dz, int zs,
                 const std::vector<int>& zr, const double* v, int nz, int nx, double dt, int nt, const double* w,
                 int d, double* datau)
{
    const int nr = (int)xr.size();
    const size_t need = noalloc_bytes_needed(nz, nx, d, nt, nr);
    if (need > NOALLOC_SCRATCH_BYTES)
        throw Error(MNAD_E_ARG, "shot needs " + std::to_string(need) + " bytes of working memory; the no-allocation "
                                "entry point has " + std::to_string(NOALLOC_SCRATCH_BYTES) +
                                " (use mnad_fwd_pde_exact for larger shots)");
    std::lock_guard<std::mutex> guard(g_noalloc_lock);
    DeviceScope on(device);
    unsigned char* base = scratch_on(device);
    cudaStream_t st = cudaStreamPerThread;

    // Carve the scratch array.
    size_t off = 0;
    auto take = [&](size_t bytes) { unsigned char* p = base + off; off += align256(bytes); return p; };
    const int ld = (nz + HZ + HZB + 31) / 32 * 32;
    const size_t S = (size_t)ld * (nx + 2 * HX);
    const int dpz = (d + 6 + 3) / 4 * 4;
    const int ntz = (nz + DIRECT_TZ - 1) / DIRECT_TZ, ntx = (nx + DIRECT_TX - 1) / DIRECT_TX;
    const int ntiles = ntz * ntx;
    const int bz = (nz + TMA_TZ - 1) / TMA_TZ, bx = (nx + TMA_TX - 1) / TMA_TX, nbt = bz * bx;
    PropDesc* d_desc = reinterpret_cast<PropDesc*>(take(sizeof(PropDesc)));
    unsigned* d_status = reinterpret_cast<unsigned*>(take(sizeof(unsigned)));
    int* d_tile_prop = reinterpret_cast<int*>(take(ntiles * sizeof(int)));
    int* d_tile_rec = reinterpret_cast<int*>(take((nbt + 1) * sizeof(int)));
    int* d_col_rec = reinterpret_cast<int*>(take(((size_t)nbt * TMA_TX + 1) * sizeof(int)));
    int* d_rec_pt = reinterpret_cast<int*>(take((size_t)nr * sizeof(int)));
    int* d_rec_id = reinterpret_cast<int*>(take((size_t)nr * sizeof(int)));
    double* d_rec_r = reinterpret_cast<double*>(take((size_t)nr * sizeof(double)));
    float* d_amp = reinterpret_cast<float*>(take((size_t)nt * sizeof(float)));
    float* d_fields = reinterpret_cast<float*>(take(6 * S * sizeof(float)));
    float* d_r = reinterpret_cast<float*>(take(S * sizeof(float)));
    float* d_mx = nullptr;
    float* d_mz = nullptr;
    if (d > 0) {
        d_mx = reinterpret_cast<float*>(take((size_t)2 * 9 * d * ld * sizeof(float)));
        d_mz = reinterpret_cast<float*>(take((size_t)2 * 9 * nx * dpz * sizeof(float)));
    }
    double* d_data = reinterpret_cast<double*>(take((size_t)nt * nr * sizeof(double)));

    // Host-side tables: receivers bucketed per tile and column, source amplitudes.
    auto at = [&](int j, int i) { return (int)((size_t)(i + HX) * ld + (j + HZ)); };
    std::vector<int> zero(ntiles, 0);
    RecBuckets rb;
    bucket_receivers(nz, nx, ld, zr, xr, v, dt, MODE_FWD, rb);
    std::vector<float> amp(nt);
    const double rs = r_of(v[(size_t)zs + (size_t)xs * nz], dt, MODE_FWD);
    for (int t = 0; t < nt; ++t) amp[t] = (float)(rs * w[t]);

    PropDesc D;
    std::memset(&D, 0, sizeof(D));
    D.s_begin = INT_MIN; D.s_end = INT_MAX;
    D.mode = MODE_FWD; D.nt = nt; D.nz = nz; D.nx = nx; D.ld = ld; D.d = d; D.dpz = dpz; D.zb0 = (nz - d) & ~3;
    D.ntz = bz; D.ntx = bx; D.tile_base = 0;
    for (int t = 0; t < 2; ++t)
        for (int f = 0; f < 3; ++f) D.fld[t][f] = d_fields + (size_t)(t * 3 + f) * S;
    D.r = d_r; D.mx = d_mx; D.mz = d_mz;
    const double R = 1e-4;   // fwd_PDE_exact_MNAD.m:88
    if (d > 0) {
        D.kx = (float)((3 * std::log(1 / R)) / (2 * std::pow(d * dx, 3)));
        D.kz = (float)((3 * std::log(1 / R)) / (2 * std::pow(d * dz, 3)));
    }
    D.dx = (float)dx; D.dz = (float)dz; D.dt = (float)dt; D.inv_dt = (float)(1.0 / dt);
    D.inv_dt2 = (float)(1.0 / (dt * dt));
    D.src = at(zs, xs); D.src_amp = d_amp;
    D.nr = nr; D.rec_pt = d_rec_pt; D.rec_id = d_rec_id; D.rec_r = d_rec_r; D.tile_rec = d_tile_rec;
    D.col_rec = d_col_rec;
    D.data = d_data;
    D.status = d_status;

    // Model -> r (the model is staged in the field area, which is cleared after).
    const size_t N = (size_t)nz * nx;
    MNAD_CK(cudaMemsetAsync(d_r, 0, S * sizeof(float), st));
    MNAD_CK(cudaMemcpyAsync(d_fields, v, N * sizeof(double), cudaMemcpyHostToDevice, st));
    build_r<<<(int)std::min<size_t>((N + 255) / 256, 4096), 256, 0, st>>>(reinterpret_cast<const double*>(d_fields), nz,
                                                                        nx, dt, 0, d_r, ld);
    MNAD_CK(cudaGetLastError());
    // Clear the state left by the previous call.
    MNAD_CK(cudaMemsetAsync(d_fields, 0, 6 * S * sizeof(float), st));
    if (d > 0) {
        MNAD_CK(cudaMemsetAsync(d_mx, 0, (size_t)2 * 9 * d * ld * sizeof(float), st));
        MNAD_CK(cudaMemsetAsync(d_mz, 0, (size_t)2 * 9 * nx * dpz * sizeof(float), st));
    }
    MNAD_CK(cudaMemsetAsync(d_data, 0, (size_t)nt * nr * sizeof(double), st));
    MNAD_CK(cudaMemsetAsync(d_status, 0, sizeof(unsigned), st));
    MNAD_CK(cudaMemcpyAsync(d_desc, &D, sizeof(D), cudaMemcpyHostToDevice, st));
    MNAD_CK(cudaMemcpyAsync(d_tile_prop, zero.data(), ntiles * sizeof(int), cudaMemcpyHostToDevice, st));
    MNAD_CK(cudaMemcpyAsync(d_tile_rec, rb.tile_rec.data(), (nbt + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    MNAD_CK(cudaMemcpyAsync(d_col_rec, rb.col_rec.data(), ((size_t)nbt * TMA_TX + 1) * sizeof(int),
                            cudaMemcpyHostToDevice, st));
    if (nr > 0) {
        MNAD_CK(cudaMemcpyAsync(d_rec_pt, rb.pt.data(), nr * sizeof(int), cudaMemcpyHostToDevice, st));
        MNAD_CK(cudaMemcpyAsync(d_rec_id, rb.id.data(), nr * sizeof(int), cudaMemcpyHostToDevice, st));
        MNAD_CK(cudaMemcpyAsync(d_rec_r, rb.rr.data(), nr * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    MNAD_CK(cudaMemcpyAsync(d_amp, amp.data(), nt * sizeof(float), cudaMemcpyHostToDevice, st));

    seed_sources<<<1, 32, 0, st>>>(d_desc, 1);
    StepArgs a{};
    stencil_polys(dx, dz, a.coef.alpha, a.coef.beta);
    a.props = d_desc;
    a.tile_prop = d_tile_prop;
    a.ntiles = ntiles;
    a.ntz = ntz;
    a.tiles_per_prop = ntiles;
    a.status = d_status;
    for (int s = 0; s < nt; ++s) {
        a.s = s;
        step_direct<<<ntiles, dim3(DIRECT_TZ, DIRECT_TX), 0, st>>>(a);
    }
    MNAD_CK(cudaGetLastError());
    if (nr > 0) MNAD_CK(cudaMemcpyAsync(datau, d_data, (size_t)nt * nr * sizeof(double), cudaMemcpyDeviceToHost, st));
    unsigned bits = 0;
    MNAD_CK(cudaMemcpyAsync(&bits, d_status, sizeof(bits), cudaMemcpyDeviceToHost, st));
    MNAD_CK(cudaStreamSynchronize(st));
    raise_status(bits, "mnad_fwd_pde_exact_noalloc");
}

}  // namespace mnad
