// Host-side engine: device memory, propagation setup, batched time loop.
#include "mnad_engine.h"
#include "mnad_kernels.h"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

namespace mnad {

void check_cuda(cudaError_t e, const char* what, const char* file, int line)
{
    if (e == cudaSuccess) return;
    const int code = (e == cudaErrorMemoryAllocation) ? MNAD_E_OOM : MNAD_E_CUDA;
    throw Error(code, std::string(cudaGetErrorString(e)) + " in " + what + " (" + file + ":" + std::to_string(line) + ")");
}

static size_t round_up(size_t a, size_t b) { return (a + b - 1) / b * b; }

// ---------------------------------------------------------------------------
DevMem::DevMem(Context* c, size_t bytes) : ctx_(c), n_(bytes)
{
    p_ = bytes ? c->alloc(bytes) : nullptr;
}

DevMem& DevMem::operator=(DevMem&& o) noexcept
{
    if (this != &o) {
        reset();
        ctx_ = o.ctx_; p_ = o.p_; n_ = o.n_;
        o.ctx_ = nullptr; o.p_ = nullptr; o.n_ = 0;
    }
    return *this;
}

void DevMem::reset()
{
    if (p_ && ctx_) ctx_->release(p_, n_);
    p_ = nullptr; n_ = 0; ctx_ = nullptr;
}

// ---------------------------------------------------------------------------
Context::Context(int dev, size_t budget_bytes) : device(dev), budget(budget_bytes)
{
    MNAD_CK(cudaSetDevice(dev));
    MNAD_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    MNAD_CK(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
    cudaMemPool_t pool;
    MNAD_CK(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t keep = UINT64_MAX;   // keep freed blocks cached for the next job
    MNAD_CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    MNAD_CK(cudaFuncSetAttribute(step_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)step_tma_smem_bytes()));
    MNAD_CK(cudaFuncSetAttribute(step_tma2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)step_tma2_smem_bytes()));
    MNAD_CK(cudaFuncSetAttribute(step_tma_narrow, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)step_tma_narrow_smem_bytes()));
    MNAD_CK(cudaMalloc(&d_status, sizeof(unsigned)));
    MNAD_CK(cudaMemset(d_status, 0, sizeof(unsigned)));
    opt.snapshot_codec = MNAD_SNAP_F32;
    opt.pairing = MNAD_PAIR_REFERENCE;
    opt.T = 0;
    opt.record_vw = 0;
    opt.use_graphs = 1;
    opt.kernel = MNAD_KERNEL_AUTO;
    opt.energy_every = 0;
    opt.checkpoint_every = 0;
    opt.checkpoint_codec = MNAD_SNAP_F32;
}

Context::~Context()
{
    if (stream) cudaStreamSynchronize(stream);
    wavefields.clear();
    if (d_status) cudaFree(d_status);
    if (stream) cudaStreamSynchronize(stream), cudaStreamDestroy(stream);
}

void* Context::alloc(size_t bytes)
{
    if (budget && in_use + bytes > budget)
        throw Error(MNAD_E_BUDGET, "allocation of " + std::to_string(bytes) + " B exceeds the context budget (" +
                                       std::to_string(in_use) + " of " + std::to_string(budget) + " B in use)");
    void* p = nullptr;
    MNAD_CK(cudaMallocAsync(&p, bytes, stream));
    in_use += bytes;
    peak = std::max(peak, in_use);
    return p;
}

void Context::release(void* p, size_t bytes)
{
    cudaFreeAsync(p, stream);
    in_use -= std::min(in_use, bytes);
}

void Context::sync() { MNAD_CK(cudaStreamSynchronize(stream)); }

unsigned Context::take_status()
{
    unsigned s = 0;
    MNAD_CK(cudaMemcpyAsync(&s, d_status, sizeof(s), cudaMemcpyDeviceToHost, stream));
    MNAD_CK(cudaMemsetAsync(d_status, 0, sizeof(unsigned), stream));
    sync();
    return s;
}

void upload(Context& ctx, void* dst, const void* src, size_t bytes)
{
    if (bytes) MNAD_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx.stream));
    ctx.h2d += bytes;
}

void download(Context& ctx, void* dst, const void* src, size_t bytes)
{
    if (bytes) MNAD_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.d2h += bytes;
}

// ---------------------------------------------------------------------------
TileCfg tile_cfg(int kernel)
{
    return TileCfg{kernel};
}

void bucket_receivers(int nz, int nx, int ld, const std::vector<int>& zr, const std::vector<int>& xr,
                      const double* v, double dt, int mode, RecBuckets& out)
{
    const int ntz = (nz + TMA_TZ - 1) / TMA_TZ, ntx = (nx + TMA_TX - 1) / TMA_TX;
    const int ntiles = ntz * ntx, nb = ntiles * TMA_TX, nr = (int)zr.size();
    std::vector<int> cnt(nb + 1, 0);
    auto bucket = [&](int k) { return ((zr[k] / TMA_TZ) + (xr[k] / TMA_TX) * ntz) * TMA_TX + xr[k] % TMA_TX; };
    for (int k = 0; k < nr; ++k) cnt[1 + bucket(k)]++;
    for (int b = 0; b < nb; ++b) cnt[b + 1] += cnt[b];
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    out.pt.assign(nr, 0);
    out.id.assign(nr, 0);
    out.rr.assign(nr, 0.0);
    for (int k = 0; k < nr; ++k) {
        const int e = fill[bucket(k)]++;
        out.pt[e] = (int)((size_t)(xr[k] + HX) * ld + (zr[k] + HZ));
        out.id[e] = k;
        out.rr[e] = r_of(v[(size_t)zr[k] + (size_t)xr[k] * nz], dt, mode);
    }
    out.tile_rec.assign(ntiles + 1, 0);
    for (int t = 0; t <= ntiles; ++t) out.tile_rec[t] = cnt[(size_t)t * TMA_TX];
    out.col_rec = std::move(cnt);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on libcuda, so the library loads on hosts without a driver).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q{};
        void* p = nullptr;
        MNAD_CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !p) throw Error(MNAD_E_CUDA, "cuTensorMapEncodeTiled is unavailable");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2-D map over one field's padded storage (inner dimension z, ld rows, nx+2HX
// columns) with a box of bz rows x bx columns.
static CUtensorMap field_map(const float* base, int ld, int ncols, int bz, int bx)
{
    CUtensorMap m;
    cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)ncols};
    cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)bz, (cuuint32_t)bx};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides,
                                      box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(MNAD_E_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

// 3-D map over the three fields of one time level (U at base, V and W at
// base + fs and base + 2 fs floats): boxes of bz x bx x 3.
static CUtensorMap fields_map(const float* base, int ld, int ncols, size_t fs, int bz, int bx)
{
    CUtensorMap m;
    cuuint64_t dims[3] = {(cuuint64_t)ld, (cuuint64_t)ncols, 3};
    cuuint64_t strides[2] = {(cuuint64_t)ld * sizeof(float), (cuuint64_t)fs * sizeof(float)};
    cuuint32_t box[3] = {(cuuint32_t)bz, (cuuint32_t)bx, 3};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides,
                                      box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(MNAD_E_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

void model_minmax(const double* v, size_t n, double& vmin, double& vmax)
{
    vmin = INFINITY; vmax = -INFINITY;
    for (size_t k = 0; k < n; ++k) {
        vmin = std::min(vmin, v[k]);
        vmax = std::max(vmax, v[k]);
    }
}

int snapshot_nf(int nt, double vmin, double vmax)
{
    // nf = floor(nt/(2*3*max(v(:))/min(v(:)))), same evaluation order.
    return (int)std::floor((double)nt / (2.0 * 3.0 * vmax / vmin));
}

int snapshot_T(int nt, int nf)
{
    if (nf <= 0)
        throw Error(MNAD_E_ARG, "snapshot plan: nf = floor(nt/(6*vmax/vmin)) is 0, so T = floor(nt/nf/2) is "
                                "undefined; set mnad_options.T");
    return (int)std::floor((double)nt / nf / 2.0);
}

// Stencil coefficient polynomials alpha*r + beta*r^2 (r = v^2 dt^2) of the
// nine generator files (see the Coef enum for the centre entries).
void stencil_polys(double dx, double dz, float* al, float* be)
{
    const double dx2 = dx * dx, dz2 = dz * dz, dx3 = dx2 * dx, dz3 = dz2 * dz;
    const double dx4 = dx2 * dx2, dz4 = dz2 * dz2, dx5 = dx4 * dx, dz5 = dz4 * dz;
    double a[NCOEF] = {}, b[NCOEF] = {};
    // Auu_gen.m:30,37,44,65
    a[K_UU_Z] = (24.0 / 11) / dz2;   b[K_UU_Z] = -(15 / (11 * dz4) + 1 / (dx2 * dz2));
    a[K_UU_X] = (24.0 / 11) / dx2;   b[K_UU_X] = -(15 / (11 * dx4) + 1 / (dx2 * dz2));
    b[K_UU_D] = 1 / (2 * dx2 * dz2);
    // Auv_gen.m:36 (i+1), 57 (diagonals at i+1), 71 (i-2)
    a[K_UV_X1] = (20.0 / 33) / dx;   b[K_UV_X1] = -(47 / (66 * dx3) + 1 / (6 * dx * dz2));
    b[K_UV_D] = 1 / (12 * dx * dz2);
    a[K_UV_X2] = (1.0 / 132) / dx;   b[K_UV_X2] = -(1.0 / 66) / dx3;
    // Auw_gen.m:29 (j+1), 50 (diagonals at j+1), 78 (j-2)
    a[K_UW_Z1] = (20.0 / 33) / dz;   b[K_UW_Z1] = -(47 / (66 * dz3) + 1 / (6 * dz * dx2));
    b[K_UW_D] = 1 / (12 * dz * dx2);
    a[K_UW_Z2] = (1.0 / 132) / dz;   b[K_UW_Z2] = -(1.0 / 66) / dz3;
    // Avu_gen.m:30 (i-1), 44 (diagonals at i-1)
    a[K_VU_X1] = 15 / (2 * dx3) - 1 / (dx * dz2);
    b[K_VU_X1] = -(15 / (2 * dx5) - 1 / (dx * dz4) + 5 / (2 * dx3 * dz2));
    a[K_VU_D] = 1 / (2 * dx * dz2);  b[K_VU_D] = 5 / (4 * dx3 * dz2) - 1 / (2 * dx * dz4);
    // Avv_gen.m:29,36,43,64
    a[K_VV_Z] = 1 / dz2;             b[K_VV_Z] = -2 / (dx2 * dz2);
    a[K_VV_X] = -1.5 / dx2;          b[K_VV_X] = 5 / (2 * dx4) + 1 / (2 * dx2 * dz2);
    // centre -(12/dx^2 + 2/dz^2) r + (10/dx^4 + 4/(dx^2 dz^2)) r^2 minus the
    // off-diagonal sum: the residual of the difference form
    a[K_VV_R] = -15 / dx2;           b[K_VV_R] = 15 / dx4;
    b[K_VV_D] = -1 / (4 * dx2 * dz2);
    // Avw_gen.m:29,50 ((j-1,i-1) and (j+1,i+1))
    a[K_VW] = -1 / (4 * dz * dx);    b[K_VW] = 1 / (4 * dz3 * dx);
    // Awu_gen.m:29 (j-1), 44 (diagonals at j-1)
    a[K_WU_Z1] = 15 / (2 * dz3) - 1 / (dz * dx2);
    b[K_WU_Z1] = -(15 / (2 * dz5) - 1 / (dz * dx4) + 5 / (2 * dz3 * dx2));
    a[K_WU_D] = 1 / (2 * dz * dx2);  b[K_WU_D] = 5 / (4 * dz3 * dx2) - 1 / (2 * dz * dx4);
    // Awv_gen.m:31,52 ((j-1,i-1) and (j+1,i+1))
    a[K_WV] = -1 / (4 * dz * dx);    b[K_WV] = 1 / (4 * dx3 * dz);
    // Aww_gen.m:31,38,45,66
    a[K_WW_Z] = -1.5 / dz2;          b[K_WW_Z] = 5 / (2 * dz4) + 1 / (2 * dx2 * dz2);
    a[K_WW_X] = 1 / dx2;             b[K_WW_X] = -2 / (dz2 * dx2);
    a[K_WW_R] = -15 / dz2;           b[K_WW_R] = 15 / dz4;
    b[K_WW_D] = -1 / (4 * dx2 * dz2);
    for (int k = 0; k < NCOEF; ++k) { al[k] = (float)a[k]; be[k] = (float)b[k]; }
}

double r_of(double v, double dt, int mode)
{
    return mode == MODE_ADJ ? (v * dt) * (v * dt) : (v * v) * (dt * dt);
}

// ---------------------------------------------------------------------------
DevMem make_r(Context& ctx, const double* v, int nz, int nx, double dt, int mode)
{
    const int ld = (int)round_up((size_t)nz + HZ + HZB, 32);
    const size_t S = (size_t)ld * (nx + 2 * HX);
    DevMem r(&ctx, S * sizeof(float));
    MNAD_CK(cudaMemsetAsync(r.get(), 0, r.size(), ctx.stream));
    const size_t N = (size_t)nz * nx;
    DevMem vt(&ctx, N * sizeof(double));
    upload(ctx, vt.get(), v, N * sizeof(double));
    const int blocks = (int)std::min<size_t>((N + 255) / 256, (size_t)ctx.num_sms * 8);
    build_r<<<blocks, 256, 0, ctx.stream>>>(vt.as<double>(), nz, nx, dt, mode == MODE_ADJ, r.as<float>(), ld);
    MNAD_CK(cudaGetLastError());
    return r;
}

void Prop::build(Context& ctx)
{
    const PropSpec& s = spec;
    const int nz = s.nz, nx = s.nx, d = s.d;
    const int ld = (int)round_up((size_t)nz + HZ + HZB, 32);
    S = (size_t)ld * (nx + 2 * HX);
    // z-strip columns hold d rows plus room for the 4-row groups of the TMA
    // kernel that overhang the strip (aligned to 16 bytes at both sides).
    const int dpz = (int)round_up((size_t)d + 6, 4);
    const int zb0 = (nz - d) & ~3;

    const int levels = s.depth2 ? 4 : 2;
    fields = DevMem(&ctx, (size_t)levels * 3 * S * sizeof(float));
    if (!r_ext) r = make_r(ctx, s.v, nz, nx, s.dt, s.mode);
    if (d > 0) {
        mx = DevMem(&ctx, (size_t)2 * 9 * d * ld * sizeof(float));
        mz = DevMem(&ctx, (size_t)2 * 9 * nx * dpz * sizeof(float));
        if (s.depth2) {
            mx2 = DevMem(&ctx, mx.size());
            mz2 = DevMem(&ctx, mz.size());
        }
    }

    PropDesc& D = desc;
    std::memset(&D, 0, sizeof(D));
    D.s_begin = INT_MIN;
    D.s_end = INT_MAX;
    D.mode = s.mode; D.nt = s.nt; D.nz = nz; D.nx = nx; D.ld = ld; D.d = d; D.dpz = dpz; D.zb0 = zb0;
    D.ntz = (nz + TMA_TZ - 1) / TMA_TZ;      // receiver buckets use the TMA tiling for every kernel
    D.ntx = (nx + TMA_TX - 1) / TMA_TX;
    for (int t = 0; t < levels; ++t)
        for (int f = 0; f < 3; ++f) D.fld[t][f] = fields.as<float>() + (size_t)(t * 3 + f) * S;
    D.r = r_ext ? r_ext : r.as<float>();
    D.mx = mx.as<float>();
    D.mz = mz.as<float>();
    D.mx2 = mx2.as<float>();
    D.mz2 = mz2.as<float>();
    const double R = 1e-4;   // fwd_PDE_exact_MNAD.m:88
    if (d > 0) {
        D.kx = (float)((3 * std::log(1 / R)) / (2 * std::pow(d * s.dx, 3)));
        D.kz = (float)((3 * std::log(1 / R)) / (2 * std::pow(d * s.dz, 3)));
    }
    D.dx = (float)s.dx; D.dz = (float)s.dz; D.dt = (float)s.dt; D.inv_dt = (float)(1.0 / s.dt);
    D.inv_dt2 = (float)(1.0 / (s.dt * s.dt));
    stencil_polys(s.dx, s.dz, coefs.alpha, coefs.beta);
    D.status = s.status ? s.status : ctx.d_status;

    auto off = [&](int j, int i) { return (int)((size_t)(i + HX) * ld + (j + HZ)); };
    D.src = -1;
    if (s.mode == MODE_FWD && s.zs >= 0) {
        D.src = off(s.zs, s.xs);
        std::vector<float> amp(s.nt);
        const double rs = r_of(s.v[(size_t)s.zs + (size_t)s.xs * nz], s.dt, MODE_FWD);
        for (int t = 0; t < s.nt; ++t) amp[t] = (float)(rs * s.w[t]);     // fwd_PDE_exact_MNAD.m:111
        src_amp = DevMem(&ctx, s.nt * sizeof(float));
        upload(ctx, src_amp.get(), amp.data(), amp.size() * sizeof(float));
        D.src_amp = src_amp.as<float>();
    }

    // Receivers bucketed by TMA tile and column (bucket_receivers).
    const int nr = (int)s.zr.size();
    RecBuckets rb;
    bucket_receivers(nz, nx, ld, s.zr, s.xr, s.v, s.dt, s.mode, rb);
    const std::vector<int>& pt = rb.pt;
    const std::vector<int>& id = rb.id;
    const std::vector<double>& rr = rb.rr;
    D.nr = nr;
    tile_rec_host = rb.tile_rec;
    tile_rec = DevMem(&ctx, tile_rec_host.size() * sizeof(int));
    upload(ctx, tile_rec.get(), tile_rec_host.data(), tile_rec_host.size() * sizeof(int));
    D.tile_rec = tile_rec.as<int>();
    col_rec_host = rb.col_rec;
    col_rec = DevMem(&ctx, col_rec_host.size() * sizeof(int));
    upload(ctx, col_rec.get(), col_rec_host.data(), col_rec_host.size() * sizeof(int));
    D.col_rec = col_rec.as<int>();
    if (nr > 0) {
        rec_pt = DevMem(&ctx, nr * sizeof(int));
        rec_id = DevMem(&ctx, nr * sizeof(int));
        rec_r = DevMem(&ctx, nr * sizeof(double));
        upload(ctx, rec_pt.get(), pt.data(), nr * sizeof(int));
        upload(ctx, rec_id.get(), id.data(), nr * sizeof(int));
        upload(ctx, rec_r.get(), rr.data(), nr * sizeof(double));
        data = DevMem(&ctx, (size_t)nr * s.nt * sizeof(double));
        if (s.mode == MODE_FWD && s.record_vw) {
            datav = DevMem(&ctx, (size_t)nr * s.nt * sizeof(double));
            dataw = DevMem(&ctx, (size_t)nr * s.nt * sizeof(double));
        }
    }
    D.rec_pt = rec_pt.as<int>(); D.rec_id = rec_id.as<int>(); D.rec_r = rec_r.as<double>();
    D.data = data.as<double>(); D.datav = datav.as<double>(); D.dataw = dataw.as<double>();
    if (s.mode == MODE_ADJ && nr > 0) {
        inj = DevMem(&ctx, (size_t)nr * s.nt * sizeof(float));
        D.inj = inj.as<float>();
    }

    d_desc = DevMem(&ctx, sizeof(PropDesc));
    if (s.mode == MODE_FWD && s.energy_every > 0 && s.nt / s.energy_every > 0)
        energy = DevMem(&ctx, (size_t)(s.nt / s.energy_every) * sizeof(double));
    if (s.T > 0 && s.wf) {
        Wavefield& wf = *s.wf;
        D.T = s.T;
        D.invT = 1.0f / (float)s.T;
        D.nsnap = wf.nsnap;
        D.ncols = wf.ncols;
        D.codec = wf.codec;
        D.pairing = s.pairing;
        D.snap = wf.snap.get();
        D.snap_scale = wf.scale.as<float>();
        D.snap_col0 = 0;
        D.snap_cols = wf.held;
        D.snap_flags = SNAP_WRITE | SNAP_ILLUM;
        if (s.mode == MODE_FWD && wf.codec == MNAD_SNAP_F16) {
            D.snap = wf.stage.get();        // FP32 staging slot, encoded after each snapshot step
            D.codec = CODEC_F32;
            D.snap_stage = 1;
            D.snap_cols = 1;
        }
        if (s.mode == MODE_FWD) {
            D.illum = wf.illum.as<double>();
        } else {
            D.img_steps = s.nt / s.T;
            image = DevMem(&ctx, nint() * sizeof(double));
            D.image = image.as<double>();
        }
    }
}

void Prop::reset(Context& ctx)
{
    cudaStream_t st = ctx.stream;
    MNAD_CK(cudaMemsetAsync(fields.get(), 0, fields.size(), st));
    for (DevMem* m : {&mx, &mz, &mx2, &mz2})
        if (m->get()) MNAD_CK(cudaMemsetAsync(m->get(), 0, m->size(), st));
    if (spec.mode == MODE_FWD) {
        if (data.get()) MNAD_CK(cudaMemsetAsync(data.get(), 0, data.size(), st));
        if (desc.illum) MNAD_CK(cudaMemsetAsync(desc.illum, 0, nint() * sizeof(double), st));
        if (spec.wf && spec.wf->maxbits.get())
            MNAD_CK(cudaMemsetAsync(spec.wf->maxbits.get(), 0, spec.wf->maxbits.size(), st));
    } else {
        if (image.get()) MNAD_CK(cudaMemsetAsync(image.get(), 0, image.size(), st));
        if (inj.get()) {
            const size_t n = inj.size() / sizeof(float);
            const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)ctx.num_sms * 4);
            // d_desc holds this propagation's data and receiver tables (uploaded at build)
            injection_table<<<blocks, 256, 0, st>>>(d_desc.as<PropDesc>());
            MNAD_CK(cudaGetLastError());
        }
    }
    if (energy.get()) MNAD_CK(cudaMemsetAsync(energy.get(), 0, energy.size(), st));
}

void Prop::start(Context& ctx, int s_off)
{
    if (s_off & 1) throw Error(MNAD_E_STATE, "propagations start at even global steps");
    desc.s_off = s_off;
    upload(ctx, d_desc.get(), &desc, sizeof(PropDesc));
    reset(ctx);
    seed_sources<<<1, 32, 0, ctx.stream>>>(d_desc.as<PropDesc>(), 1);
    MNAD_CK(cudaGetLastError());
}

void Prop::setup_checkpoints(Context& ctx, int C, int G, int codec)
{
    Checkpoints& k = ckpt;
    k.C = C;
    k.G = G;
    k.codec = codec;
    if (spec.depth2) throw Error(MNAD_E_STATE, "checkpointed propagations run the one-step kernels only");
    const size_t nf = 6 * S, nmx = mx.size() / sizeof(float), nmz = mz.size() / sizeof(float);
    k.slot = nf + nmx + nmz;
    k.blocks.clear();
    for (int b = 0; b < 6; ++b) k.blocks.emplace_back((size_t)b * S, S);                 // U, V, W x 2 levels
    if (nmx)
        for (int b = 0; b < 18; ++b) k.blocks.emplace_back(nf + (size_t)b * (nmx / 18), nmx / 18);   // [side][var]
    if (nmz)
        for (int b = 0; b < 18; ++b) k.blocks.emplace_back(nf + nmx + (size_t)b * (nmz / 18), nmz / 18);
    if (G <= 1) return;
    const size_t es = codec == MNAD_SNAP_F16 ? 2 : 4;
    k.data = DevMem(&ctx, (size_t)(G - 1) * k.slot * es);
    if (codec == MNAD_SNAP_F16) {
        k.scale = DevMem(&ctx, (size_t)(G - 1) * k.blocks.size() * sizeof(float));
        k.maxbits = DevMem(&ctx, (size_t)(G - 1) * k.blocks.size() * sizeof(unsigned));
    }
}

// The state arrays of a propagation in slot order: the two time levels of
// the one-step kernels, mx, mz (checkpointed propagations never run the
// two-step kernel).
static void state_parts(Prop& p, float* part[3], size_t count[3])
{
    part[0] = p.fields.as<float>(); count[0] = 6 * p.S;
    part[1] = p.mx.as<float>();     count[1] = p.mx.size() / sizeof(float);
    part[2] = p.mz.as<float>();     count[2] = p.mz.size() / sizeof(float);
}

void Prop::save_state(Context& ctx, int g)
{
    Checkpoints& k = ckpt;
    if (g < 1 || g >= k.G) return;
    float* part[3];
    size_t count[3];
    state_parts(*this, part, count);
    cudaStream_t st = ctx.stream;
    if (k.codec == MNAD_SNAP_F32) {
        float* dst = k.data.as<float>() + (size_t)(g - 1) * k.slot;
        for (int a = 0; a < 3; ++a) {
            if (count[a]) MNAD_CK(cudaMemcpyAsync(dst, part[a], count[a] * sizeof(float), cudaMemcpyDeviceToDevice, st));
            dst += count[a];
        }
        return;
    }
    const size_t nb = k.blocks.size();
    unsigned* mb = k.maxbits.as<unsigned>() + (size_t)(g - 1) * nb;
    float* sc = k.scale.as<float>() + (size_t)(g - 1) * nb;
    __half* dst = k.data.as<__half>() + (size_t)(g - 1) * k.slot;
    MNAD_CK(cudaMemsetAsync(mb, 0, nb * sizeof(unsigned), st));
    // slot offsets map onto the three arrays in order
    auto src_of = [&](size_t off) -> const float* {
        for (int a = 0; a < 3; ++a) {
            if (off < count[a]) return part[a] + off;
            off -= count[a];
        }
        return nullptr;
    };
    for (size_t b = 0; b < nb; ++b) {
        const size_t off = k.blocks[b].first, n = k.blocks[b].second;
        const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)ctx.num_sms * 4);
        f16_absmax<<<std::max(blocks, 1), 256, 0, st>>>(src_of(off), n, mb + b);
        f16_encode<<<std::max(blocks, 1), 256, 0, st>>>(src_of(off), n, mb + b, dst + off, sc + b);
    }
    MNAD_CK(cudaGetLastError());
}

void Prop::restore_state(Context& ctx, int g)
{
    Checkpoints& k = ckpt;
    cudaStream_t st = ctx.stream;
    float* part[3];
    size_t count[3];
    state_parts(*this, part, count);
    if (g <= 0) {
        for (int a = 0; a < 3; ++a)
            if (count[a]) MNAD_CK(cudaMemsetAsync(part[a], 0, count[a] * sizeof(float), st));
        seed_sources<<<1, 32, 0, st>>>(d_desc.as<PropDesc>(), 1);
        MNAD_CK(cudaGetLastError());
        return;
    }
    if (g >= k.G) throw Error(MNAD_E_STATE, "no checkpoint " + std::to_string(g));
    if (k.codec == MNAD_SNAP_F32) {
        const float* src = k.data.as<float>() + (size_t)(g - 1) * k.slot;
        for (int a = 0; a < 3; ++a) {
            if (count[a]) MNAD_CK(cudaMemcpyAsync(part[a], src, count[a] * sizeof(float), cudaMemcpyDeviceToDevice, st));
            src += count[a];
        }
        return;
    }
    const size_t nb = k.blocks.size();
    const float* sc = k.scale.as<float>() + (size_t)(g - 1) * nb;
    const __half* src = k.data.as<__half>() + (size_t)(g - 1) * k.slot;
    auto dst_of = [&](size_t off) -> float* {
        for (int a = 0; a < 3; ++a) {
            if (off < count[a]) return part[a] + off;
            off -= count[a];
        }
        return nullptr;
    };
    for (size_t b = 0; b < nb; ++b) {
        const size_t off = k.blocks[b].first, n = k.blocks[b].second;
        const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)ctx.num_sms * 4);
        f16_decode<<<std::max(blocks, 1), 256, 0, st>>>(src + off, n, sc + b, dst_of(off));
    }
    MNAD_CK(cudaGetLastError());
}

double Prop::algorithmic_bytes() const
{
    // Per point-step: read U,V,W,pU,pV,pW,r and write nU,nV,nW (40 B FP32);
    // per CPML strip point and direction: 9 memory variables read + written
    // (72 B); snapshot steps: codec bytes + FP64 illumination r+w (forward)
    // or codec bytes + FP64 image r+w (adjoint).
    const double N = (double)spec.nz * spec.nx;
    const double strip = spec.d > 0 ? 2.0 * spec.d * (spec.nz + spec.nx) : 0.0;
    double b = (N * 40.0 + strip * 72.0) * spec.nt;
    if (spec.T > 0 && spec.wf) {
        const double cb = spec.wf->codec == MNAD_SNAP_F32 ? 4.0 : 2.0;
        b += (double)nint() * (cb + 16.0) * (spec.nt / spec.T);
    }
    return b;
}

// ---------------------------------------------------------------------------
Batch::~Batch()
{
    if (graph_) cudaGraphExecDestroy(graph_);
    if (tick_graph_) cudaGraphExecDestroy(tick_graph_);
}

void Batch::finalize()
{
    groups_.clear();
    nsteps_ = 0;
    ntiles_ = 0;
    std::vector<PropDesc> all;
    for (Prop* p : props_) {
        LaunchGroup* g = nullptr;
        for (auto& x : groups_)
            if (x->dx == p->spec.dx && x->dz == p->spec.dz && x->nz == p->spec.nz && x->nx == p->spec.nx &&
                x->d == p->spec.d)
                g = x.get();
        if (!g) {
            groups_.push_back(std::make_unique<LaunchGroup>());
            g = groups_.back().get();
            g->dx = p->spec.dx;
            g->dz = p->spec.dz;
            g->nz = p->spec.nz;
            g->nx = p->spec.nx;
            g->d = p->spec.d;
            g->coefs = p->coefs;
        }
        g->props.push_back(p);
        nsteps_ = std::max(nsteps_, p->spec.nt);
    }
    for (auto& g : groups_) {
        g->kind = pick_kind(*g);
        const bool tma2 = g->kind == MNAD_KERNEL_TMA2;
        const bool narrow = g->kind == MNAD_KERNEL_TMA_NARROW;
        const bool tma = g->kind == MNAD_KERNEL_TMA || tma2 || narrow;
        const int tx_w = narrow ? TMA_TX_NARROW : TMA_TX;        // tile width of the persistent kernels
        const int ntx_w = (g->nx + tx_w - 1) / tx_w;
        g->ntz = tma ? (g->nz + TMA_TZ - 1) / TMA_TZ : (g->nz + DIRECT_TZ - 1) / DIRECT_TZ;
        g->tiles_per_prop = g->ntz * (tma ? ntx_w : (g->nx + DIRECT_TX - 1) / DIRECT_TX);
        std::vector<PropDesc> descs;
        std::vector<int> tile_prop;
        std::vector<int4> info;
        std::vector<CUtensorMap> maps;
        for (size_t k = 0; k < g->props.size(); ++k) {
            Prop* p = g->props[k];
            PropDesc& D = p->desc;
            D.tile_base = (int)tile_prop.size();
            tile_prop.insert(tile_prop.end(), (size_t)g->tiles_per_prop, (int)k);
            descs.push_back(D);
            all.push_back(D);
            if (!tma) continue;
            const int ncols = D.nx + 2 * HX;
            // the three fields of a level are one array of stride fs
            const int levels = tma2 ? 4 : 2;
            const size_t fs = (size_t)(D.fld[0][1] - D.fld[0][0]);
            for (int t = 0; t < levels; ++t)
                if (D.fld[t][1] - D.fld[t][0] != (ptrdiff_t)fs || D.fld[t][2] - D.fld[t][1] != (ptrdiff_t)fs)
                    throw Error(MNAD_E_CUDA, "the fields of a time level are not evenly spaced");
            if (tma2) {
                for (int t = 0; t < 4; ++t)
                    maps.push_back(fields_map(D.fld[t][0], D.ld, ncols, fs, TMA2_BOX_Z, TMA2_BOX_X_CUR));
                for (int t = 0; t < 4; ++t)
                    maps.push_back(fields_map(D.fld[t][0], D.ld, ncols, fs, TMA2_BOX_Z, TMA2_BOX_X_RING));
                maps.push_back(field_map(D.r, D.ld, ncols, TMA2_BOX_Z, TMA2_BOX_X_RING));
            } else {
                for (int t = 0; t < 2; ++t)
                    maps.push_back(fields_map(D.fld[t][0], D.ld, ncols, fs, TMA_TZ + 8, tx_w + 4));
                for (int t = 0; t < 2; ++t) maps.push_back(fields_map(D.fld[t][0], D.ld, ncols, fs, TMA_TZ, tx_w));
                maps.push_back(field_map(D.r, D.ld, ncols, TMA_TZ, tx_w));
            }
            // The region whose points a tile computes: the tile itself (one
            // step per pass), or the tile and a ring of 2 points, as rows
            // j0-4 .. j0+67 and columns i0-2 .. i0+17 (two steps per pass).
            const int rz0 = tma2 ? -4 : 0, rz1 = tma2 ? TMA_TZ + 4 : TMA_TZ;
            const int rx0 = tma2 ? -2 : 0, rx1 = tma2 ? TMA_TX + 2 : tx_w;
            // tiles whose region holds a receiver (the adjoint injects there)
            std::vector<char> rec_in(tma2 ? (size_t)D.ntz * D.ntx : 0, 0);
            for (size_t e = 0; tma2 && e < p->spec.zr.size(); ++e) {
                const int zr = p->spec.zr[e], xr = p->spec.xr[e];
                for (int tx = std::max(0, (xr - rx1) / TMA_TX); tx < D.ntx && tx * TMA_TX + rx0 <= xr; ++tx)
                    for (int tz = std::max(0, (zr - rz1) / TMA_TZ); tz < D.ntz && tz * TMA_TZ + rz0 <= zr; ++tz)
                        if (xr < tx * TMA_TX + rx1 && zr < tz * TMA_TZ + rz1) rec_in[(size_t)tz + (size_t)tx * D.ntz] = 1;
            }
            for (int tx = 0; tx < ntx_w; ++tx)
                for (int tz = 0; tz < D.ntz; ++tz) {
                    const int j0 = tz * TMA_TZ, i0 = tx * tx_w, d = D.d;
                    const bool interior = j0 + rz0 >= d && j0 + rz1 <= D.nz - d && i0 + rx0 >= d && i0 + rx1 <= D.nx - d;
                    // receiver-bucket tile holding the tile, and the tile's entries
                    // there (its columns i0 % TMA_TX .. + tx_w of the bucket tile)
                    const int tl = tz + (i0 / TMA_TX) * D.ntz;
                    const size_t cb = (size_t)tl * TMA_TX + i0 % TMA_TX;
                    const int rb = p->col_rec_host[cb], re = p->col_rec_host[cb + tx_w];
                    if (j0 >= (1 << 16) || i0 >= (1 << 15)) throw Error(MNAD_E_ARG, "grid too large for the TMA tiling");
                    // the source in the region, or next to it (the CPML term of a neighbour sees it)
                    const int zs = p->spec.zs, xs = p->spec.xs;
                    const bool src = D.src >= 0 && zs >= j0 + rz0 - 1 && zs <= j0 + rz1 && xs >= i0 + rx0 - 1 &&
                                     xs <= i0 + rx1;
                    const bool rec = re > rb || (tma2 && rec_in[tl]);
                    info.push_back(make_int4(rb, re, (interior ? 0 : TILE_STRIP) | (rec ? TILE_RECEIVERS : 0) |
                                                         (src ? TILE_SOURCE : 0),
                                             j0 | (i0 << 16)));
                }
        }
        if (tile_prop.size() >= (size_t(1) << 24))   // the kernels decode tile numbers through float
            throw Error(MNAD_E_ARG, "a launch group holds 2^24 tiles or more; split the batch");
        g->ntiles = (int)tile_prop.size();
        ntiles_ += g->ntiles;
        g->desc = DevMem(&ctx_, descs.size() * sizeof(PropDesc));
        g->tile_prop = DevMem(&ctx_, std::max<size_t>(1, tile_prop.size()) * sizeof(int));
        upload(ctx_, g->desc.get(), descs.data(), descs.size() * sizeof(PropDesc));
        upload(ctx_, g->tile_prop.get(), tile_prop.data(), tile_prop.size() * sizeof(int));
        if (!maps.empty()) {
            g->tmaps = DevMem(&ctx_, maps.size() * sizeof(CUtensorMap));
            upload(ctx_, g->tmaps.get(), maps.data(), maps.size() * sizeof(CUtensorMap));
            g->tile_info = DevMem(&ctx_, info.size() * sizeof(int4));
            upload(ctx_, g->tile_info.get(), info.data(), info.size() * sizeof(int4));
        }
    }
    for (Prop* p : props_) upload(ctx_, p->d_desc.get(), &p->desc, sizeof(PropDesc));
    d_all_desc_ = DevMem(&ctx_, std::max<size_t>(1, all.size()) * sizeof(PropDesc));
    upload(ctx_, d_all_desc_.get(), all.data(), all.size() * sizeof(PropDesc));
}

// The group's step kernel: forced, a tuning trial, a measured choice, or the
// crossover rule.
// The two-step kernel needs its storage on every propagation of the group,
// whole runs from step 0 without step windows, and no per-step host work
// (FP16 snapshot encodes, energy, checkpoints run between single steps).
bool Batch::depth2_allowed(const LaunchGroup& g) const
{
    if (!depth2_ok_ || has_step_hooks()) return false;
    for (const Prop* p : g.props)
        if (!p->spec.depth2) return false;
    return true;
}

int Batch::pick_kind(const LaunchGroup& g) const
{
    const bool d2 = depth2_allowed(g);
    auto valid = [&](int k) { return k == MNAD_KERNEL_TMA2 && !d2 ? MNAD_KERNEL_TMA : k; };
    if (tc_.kind == MNAD_KERNEL_DIRECT || tc_.kind == MNAD_KERNEL_TMA || tc_.kind == MNAD_KERNEL_TMA2 ||
        tc_.kind == MNAD_KERNEL_TMA_NARROW)
        return valid(tc_.kind);
    const double tiles = (double)g.props.size() * ((g.nz + TMA_TZ - 1) / TMA_TZ) * ((g.nx + TMA_TX - 1) / TMA_TX);
    const bool persistent = tiles >= AUTO_TMA_TILES_PER_CTA * ctx_.num_sms * TMA_CTAS_PER_SM;
    if (tc_.kind == MNAD_KERNEL_TUNE) {
        if (trial_kind_ >= 0) return valid(trial_kind_);
        auto it = ctx_.kernel_choice.find(std::make_tuple(g.nz, g.nx, g.d, (int)g.props.size()));
        if (it != ctx_.kernel_choice.end()) return valid(it->second);
        // a group that was not measured itself (the step windows of a
        // checkpointed adjoint leave no room for trial steps): the choice
        // measured on the same grid with the nearest propagation count, if
        // both launches are large enough for the persistent kernels
        int best = -1, gap = INT_MAX;
        for (const auto& kv : ctx_.kernel_choice) {
            const auto& key = kv.first;
            if (std::get<0>(key) != g.nz || std::get<1>(key) != g.nx || std::get<2>(key) != g.d) continue;
            const int dg = std::abs(std::get<3>(key) - (int)g.props.size());
            if (dg < gap && kv.second != MNAD_KERNEL_DIRECT) best = kv.second, gap = dg;
        }
        if (best >= 0 && persistent) return valid(best);
    }
    if (!persistent) return MNAD_KERNEL_DIRECT;
    // Tile width: the narrow tiles win where the CPML strips are a small share
    // of the grid, the 64 x 16 tiles where they are large (measured on GB300:
    // strips 8 % of the 1281 x 4081 grid, narrow +3.8 %; 22 % of 481 x 1281,
    // narrow -2.6 %).
    const double inner = (double)std::max(0, g.nz - 2 * g.d) * std::max(0, g.nx - 2 * g.d);
    const double strip_share = 1.0 - inner / ((double)g.nz * g.nx);
    return strip_share < AUTO_NARROW_STRIP_SHARE ? MNAD_KERNEL_TMA_NARROW : MNAD_KERNEL_TMA;
}

void Batch::tune()
{
    if (tc_.kind != MNAD_KERNEL_TUNE || tuned_) return;
    tuned_ = true;
    const int K = std::min(TUNE_STEPS, nsteps_ - TUNE_WARMUP);
    bool known = true;
    for (const auto& g : groups_)
        known &= ctx_.kernel_choice.count(std::make_tuple(g->nz, g->nx, g->d, (int)g->props.size())) > 0;
    if (known || K < 2 || ntiles_ == 0) return;     // cached, or too short to measure: the rule stands
    const int ng = (int)groups_.size();
    // candidates: one thread per point, the persistent kernel at one and (where
    // the batch allows it) at two steps per pass; the two-step kernel launches
    // at even steps only, so its K steps are timed in K/2 launches
    bool any_d2 = false;
    for (const auto& g : groups_) any_d2 |= depth2_allowed(*g);
    const int kinds[4] = {MNAD_KERNEL_DIRECT, MNAD_KERNEL_TMA, MNAD_KERNEL_TMA_NARROW, MNAD_KERNEL_TMA2};
    const int nk = any_d2 ? 4 : 3;
    std::vector<double> ms[4];
    std::vector<cudaEvent_t> ev((size_t)2 * K * ng, nullptr);
    for (auto& e : ev) MNAD_CK(cudaEventCreate(&e));
    try {
        for (int c = 0; c < nk; ++c) {
            trial_kind_ = kinds[c];
            finalize();
            start();
            const int n = TUNE_WARMUP + K;
            if (has_tma()) {
                const size_t need = reserve_counters(n);
                MNAD_CK(cudaMemsetAsync(d_counters_.get(), 0, need, ctx_.stream));
            }
            for (int s = 0; s < n; ++s)
                for (int gi = 0; gi < ng; ++gi) {
                    const int t = s - TUNE_WARMUP;
                    if (t >= 0) MNAD_CK(cudaEventRecord(ev[(size_t)2 * (t * ng + gi)], ctx_.stream));
                    launch_group(gi, s, s);
                    if (t >= 0) MNAD_CK(cudaEventRecord(ev[(size_t)2 * (t * ng + gi) + 1], ctx_.stream));
                }
            MNAD_CK(cudaGetLastError());
            MNAD_CK(cudaStreamSynchronize(ctx_.stream));
            ms[c].assign(ng, 0.0);
            for (int t = 0; t < K; ++t)
                for (int gi = 0; gi < ng; ++gi) {
                    float x = 0;
                    MNAD_CK(cudaEventElapsedTime(&x, ev[(size_t)2 * (t * ng + gi)], ev[(size_t)2 * (t * ng + gi) + 1]));
                    ms[c][gi] += x;
                }
        }
    } catch (...) {
        for (auto& e : ev) cudaEventDestroy(e);
        trial_kind_ = -1;
        throw;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    for (int gi = 0; gi < ng; ++gi) {
        const LaunchGroup& g = *groups_[gi];
        int best = 0;
        for (int c = 1; c < nk; ++c)
            if (ms[c][gi] < ms[best][gi]) best = c;
        ctx_.kernel_choice[std::make_tuple(g.nz, g.nx, g.d, (int)g.props.size())] = kinds[best];
    }
    trial_kind_ = -1;
    finalize();
}

void Batch::launch_step(int s, int slot)
{
    for (size_t gi = 0; gi < groups_.size(); ++gi) launch_group(gi, s, slot);
}

void Batch::launch_group(size_t gi, int s, int slot)
{
    {
        auto& g = groups_[gi];
        if (g->ntiles == 0) return;
        if (g->kind == MNAD_KERNEL_TMA2 && (s & 1)) return;   // step s ran in the launch at s - 1
        StepArgs a;
        a.coef = g->coefs;
        for (int k = 0; k < NCOEF; ++k) {
            const float sa = k == K_UV_X1 ? -1.0f : 1.0f, sb = (k == K_UV_X1 || k == K_UV_D) ? -1.0f : 1.0f;
            a.coef2.alpha[k] = make_float2(sa * g->coefs.alpha[k], sa * g->coefs.alpha[k]);
            a.coef2.beta[k] = make_float2(sb * g->coefs.beta[k], sb * g->coefs.beta[k]);
        }
        a.props = g->desc.as<PropDesc>();
        a.tile_prop = g->tile_prop.as<int>();
        a.tmaps = g->tmaps.get();
        a.tile_info = g->tile_info.as<int4>();
        a.tile_counter = d_counters_.as<int>() + (d_counters_.get() ? (size_t)slot * groups_.size() + gi : 0);
        a.ntiles = g->ntiles;
        a.ntz = g->ntz;
        a.tiles_per_prop = g->tiles_per_prop;
        a.inv_tiles_per_prop = 1.0f / (float)std::max(1, g->tiles_per_prop);
        a.inv_ntz = 1.0f / (float)std::max(1, g->ntz);
        a.s = s;
        a.status = ctx_.d_status;
        a.spin_limit = ctx_.wait_limit ? ctx_.wait_limit : SPIN_LIMIT_DEFAULT;
        const int grid = std::min(g->ntiles, ctx_.num_sms * TMA_CTAS_PER_SM);
        if (g->kind == MNAD_KERNEL_TMA)
            step_tma<<<grid, TMA_THREADS, step_tma_smem_bytes(), ctx_.stream>>>(a);
        else if (g->kind == MNAD_KERNEL_TMA_NARROW)
            step_tma_narrow<<<std::min(g->ntiles, ctx_.num_sms * TMA_CTAS_PER_SM_NARROW), TMA_TZY * TMA_TX_NARROW,
                              step_tma_narrow_smem_bytes(), ctx_.stream>>>(a);
        else if (g->kind == MNAD_KERNEL_TMA2)
            step_tma2<<<grid, TMA_THREADS, step_tma2_smem_bytes(), ctx_.stream>>>(a);
        else
            step_direct<<<g->ntiles, dim3(DIRECT_TZ, DIRECT_TX), 0, ctx_.stream>>>(a);
    }
}

void Batch::start()
{
    for (Prop* p : props_) p->reset(ctx_);
    if (!props_.empty())
        seed_sources<<<((int)props_.size() + 127) / 128, 128, 0, ctx_.stream>>>(d_all_desc_.as<PropDesc>(),
                                                                            (int)props_.size());
    MNAD_CK(cudaGetLastError());
}

void Batch::encode_snapshots(int s)
{
    for (Prop* p : props_) {
        const PropSpec& sp = p->spec;
        if (sp.mode != MODE_FWD || !sp.wf || sp.wf->codec != MNAD_SNAP_F16 || sp.T <= 0) continue;
        const int tt = s - p->desc.s_off + 1;
        if (tt < 1 || tt > sp.nt || tt % sp.T != 0 || tt / sp.T > sp.wf->nsnap) continue;
        const int k = tt / sp.T - 1;
        Wavefield& wf = *sp.wf;
        const size_t n = wf.nint;
        const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)ctx_.num_sms * 4);
        f16_absmax<<<blocks, 256, 0, ctx_.stream>>>(wf.stage.as<float>(), n, wf.maxbits.as<unsigned>() + k);
        f16_encode<<<blocks, 256, 0, ctx_.stream>>>(wf.stage.as<float>(), n, wf.maxbits.as<unsigned>() + k,
                                                    wf.snap.as<__half>() + (size_t)k * n, wf.scale.as<float>() + k);
    }
}

void Batch::energy_after(int s)
{
    for (Prop* p : props_) {
        const int K = p->spec.energy_every;
        const int sl = s - p->desc.s_off;
        if (!p->energy.get() || sl < 0 || (sl + 1) % K != 0 || sl + 1 > p->spec.nt) continue;
        const size_t n = p->nint();
        const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)ctx_.num_sms * 2);
        // after step s the new fields are time level (s + 1) & 1
        energy_reduce<<<std::max(blocks, 1), 256, 0, ctx_.stream>>>(p->d_desc.as<PropDesc>(), (s + 1) & 1,
                                                                    p->energy.as<double>() + (sl + 1) / K - 1);
    }
}

size_t Batch::reserve_counters(int nsteps)
{
    const size_t need = (size_t)std::max(nsteps, 1) * std::max<size_t>(groups_.size(), 1) * sizeof(int);
    if (d_counters_.size() < need) d_counters_ = DevMem(&ctx_, need);
    return need;
}

void Batch::checkpoint_after(int s)
{
    for (Prop* p : props_) {
        const Checkpoints& k = p->ckpt;
        if (!k.saving || k.C <= 0) continue;
        const int sl = s - p->desc.s_off;
        if (sl < 0 || sl + 1 > p->spec.nt || (sl + 1) % k.C != 0) continue;
        p->save_state(ctx_, (sl + 1) / k.C);
    }
}

void Batch::refresh_descs()
{
    std::vector<PropDesc> all;
    for (auto& g : groups_) {
        std::vector<PropDesc> descs;
        int base = 0;
        for (Prop* p : g->props) {
            PropDesc D = p->desc;
            D.tile_base = base;                 // this batch's tile numbering
            base += g->tiles_per_prop;
            descs.push_back(D);
            all.push_back(D);
        }
        if (!descs.empty()) upload(ctx_, g->desc.get(), descs.data(), descs.size() * sizeof(PropDesc));
    }
    if (!all.empty()) upload(ctx_, d_all_desc_.get(), all.data(), all.size() * sizeof(PropDesc));
}

void Batch::advance(int s0, int s1)
{
    if (ntiles_ == 0) return;
    bool f16 = false, en = false, ck = false;
    for (Prop* p : props_) {
        f16 |= p->spec.mode == MODE_FWD && p->spec.wf && p->spec.wf->codec == MNAD_SNAP_F16;
        en |= p->energy.get() != nullptr;
        ck |= p->ckpt.saving && p->ckpt.C > 0;
    }
    if (has_tma() && s1 > s0) {
        // one tile counter per step and group, zeroed before these launches
        const size_t need = reserve_counters(s1 - s0);
        MNAD_CK(cudaMemsetAsync(d_counters_.get(), 0, need, ctx_.stream));
    }
    for (int s = s0; s < s1; ++s) {
        launch_step(s, s - s0);
        if (f16) encode_snapshots(s);
        if (en) energy_after(s);
        if (ck) checkpoint_after(s);
    }
    MNAD_CK(cudaGetLastError());
}

bool Batch::has_tma() const
{
    for (const auto& g : groups_)
        if ((g->kind == MNAD_KERNEL_TMA || g->kind == MNAD_KERNEL_TMA2 || g->kind == MNAD_KERNEL_TMA_NARROW) &&
            g->ntiles > 0)
            return true;
    return false;
}

int Batch::launches_per_step() const
{
    int n = 0;
    for (const auto& g : groups_) n += g->ntiles > 0;
    return n;
}

int Batch::step_launches() const
{
    int n = 0;
    for (const auto& g : groups_)
        if (g->ntiles > 0) n += g->kind == MNAD_KERNEL_TMA2 ? (nsteps_ + 1) / 2 : nsteps_;
    return n;
}

int Batch::main_kind() const
{
    int kind = -1, most = 0;
    for (const auto& g : groups_)
        if (g->ntiles > most) {
            most = g->ntiles;
            kind = g->kind;
        }
    return kind;
}

int Batch::group_kind_count(int kind) const
{
    int n = 0;
    for (const auto& g : groups_) n += g->ntiles > 0 && g->kind == kind;
    return n;
}

bool Batch::has_step_hooks() const
{
    for (const Prop* p : props_) {
        if (p->spec.mode == MODE_FWD && p->spec.wf && p->spec.wf->codec == MNAD_SNAP_F16) return true;
        if (p->energy.get() || (p->ckpt.saving && p->ckpt.C > 0)) return true;
    }
    return false;
}

void Batch::tick(int K, bool use_graph)
{
    if (ntiles_ == 0 || K <= 0) return;
    if (!use_graph || has_step_hooks()) {
        advance(0, K);
        return;
    }
    if (!tick_graph_ || tick_K_ != K) {
        if (tick_graph_) cudaGraphExecDestroy(tick_graph_);
        tick_graph_ = nullptr;
        if (has_tma()) reserve_counters(K);   // allocate outside the capture
        cudaGraph_t g = nullptr;
        MNAD_CK(cudaStreamBeginCapture(ctx_.stream, cudaStreamCaptureModeThreadLocal));
        advance(0, K);
        cudaError_t e = cudaStreamEndCapture(ctx_.stream, &g);
        MNAD_CK(e);
        e = cudaGraphInstantiate(&tick_graph_, g, 0);
        cudaGraphDestroy(g);
        MNAD_CK(e);
        tick_K_ = K;
    }
    MNAD_CK(cudaGraphLaunch(tick_graph_, ctx_.stream));
}

void Batch::run(bool use_graph)
{
    if (ntiles_ == 0) return;
    if (tc_.kind == MNAD_KERNEL_TUNE && !tuned_) {
        tune();
        if (graph_) {                      // captured with the kernels of the rule
            cudaGraphExecDestroy(graph_);
            graph_ = nullptr;
        }
    }
    auto body = [&]() {
        start();
        advance(0, nsteps_);
    };
    if (!use_graph) {
        body();
        MNAD_CK(cudaGetLastError());
        return;
    }
    if (!graph_) {
        // allocate outside the capture: a graph that allocates memory cannot
        // be relaunched while that memory is held
        if (has_tma()) reserve_counters(nsteps_);
        cudaGraph_t g = nullptr;
        MNAD_CK(cudaStreamBeginCapture(ctx_.stream, cudaStreamCaptureModeThreadLocal));
        body();
        cudaError_t e = cudaStreamEndCapture(ctx_.stream, &g);
        MNAD_CK(e);
        MNAD_CK(cudaGetLastError());
        e = cudaGraphInstantiate(&graph_, g, 0);
        cudaGraphDestroy(g);
        MNAD_CK(e);
    }
    MNAD_CK(cudaGraphLaunch(graph_, ctx_.stream));
}

}  // namespace mnad
