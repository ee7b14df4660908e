// C ABI of libmnad.so (declared in include/mnad.h).
#include "mnad_engine.h"
#include "mnad_jobs.h"
#include "mnad_kernels.h"

#include <algorithm>
#include <climits>
#include <map>
#include <tuple>
#include <cmath>
#include <cstring>
#include <new>

using namespace mnad;

struct mnad_context : Context {
    using Context::Context;
};

static bool use_graph(const Context& c, int nt) { return c.opt.use_graphs != 0 && nt >= 1; }

extern "C" {

MNAD_API int mnad_abi_version(void) { return MNAD_ABI_VERSION; }

MNAD_API const char* mnad_last_error(void) { return last_error().c_str(); }

MNAD_API int mnad_context_create(int device, size_t hbm_budget_bytes, mnad_context** out)
{
    return guard([&] {
        need(out != nullptr, "out is NULL");
        *out = nullptr;
        int n = 0;
        MNAD_CK(cudaGetDeviceCount(&n));
        need(device >= 0 && device < n, "no CUDA device " + std::to_string(device));
        *out = new mnad_context(device, hbm_budget_bytes);
    });
}

MNAD_API int mnad_context_destroy(mnad_context* ctx)
{
    return guard([&] { delete ctx; });
}

MNAD_API int mnad_context_set_options(mnad_context* ctx, const mnad_options* o)
{
    return guard([&] {
        need(ctx && o, "NULL argument");
        need(o->snapshot_codec == MNAD_SNAP_F32 || o->snapshot_codec == MNAD_SNAP_BF16 ||
                 o->snapshot_codec == MNAD_SNAP_F16,
             "snapshot_codec must be MNAD_SNAP_F32, MNAD_SNAP_BF16 or MNAD_SNAP_F16");
        need(o->pairing == MNAD_PAIR_REFERENCE || o->pairing == MNAD_PAIR_ALIGNED, "bad pairing");
        need(o->kernel >= MNAD_KERNEL_AUTO && o->kernel <= MNAD_KERNEL_TMA_NARROW, "bad kernel");
        need(o->energy_every >= 0, "energy_every must be >= 0");
        need(o->checkpoint_every >= 0, "checkpoint_every must be >= 0");
        need(o->checkpoint_codec == MNAD_SNAP_F32 || o->checkpoint_codec == MNAD_SNAP_F16,
             "checkpoint_codec must be MNAD_SNAP_F32 or MNAD_SNAP_F16");
        ctx->opt = *o;
    });
}

MNAD_API int mnad_context_get_options(const mnad_context* ctx, mnad_options* o)
{
    return guard([&] {
        need(ctx && o, "NULL argument");
        *o = ctx->opt;
    });
}

MNAD_API int mnad_context_memory(const mnad_context* ctx, size_t* bytes)
{
    return guard([&] {
        need(ctx && bytes, "NULL argument");
        *bytes = ctx->in_use;
    });
}

MNAD_API int mnad_context_transfers(const mnad_context* ctx, uint64_t* h2d, uint64_t* d2h)
{
    return guard([&] {
        need(ctx != nullptr, "context is NULL");
        if (h2d) *h2d = ctx->h2d;
        if (d2h) *d2h = ctx->d2h;
    });
}

MNAD_API int mnad_context_energy(const mnad_context* ctx, double* out, int max, int* n)
{
    return guard([&] {
        need(ctx != nullptr, "context is NULL");
        const int m = (int)ctx->last_energy.size();
        if (n) *n = m;
        if (out)
            for (int k = 0; k < std::min(m, max); ++k) out[k] = ctx->last_energy[k];
    });
}

MNAD_API int mnad_context_set_wait_limit(mnad_context* ctx, unsigned polls)
{
    return guard([&] {
        need(ctx != nullptr, "context is NULL");
        ctx->wait_limit = polls;
    });
}

MNAD_API int mnad_context_status(mnad_context* ctx, unsigned* flags)
{
    return guard([&] {
        need(ctx && flags, "NULL argument");
        MNAD_CK(cudaSetDevice(ctx->device));
        *flags = ctx->take_status();
    });
}

// ---------------------------------------------------------------------------
MNAD_API int mnad_fwd_pde_exact(mnad_context* ctx, double dx, double xs, const double* xr, int nr,
                                double dz, double zs, const double* zr,
                                const double* v, int nz, int nx, double dt, int nt,
                                const double* w, int d_pml, int ss, int indx,
                                double* datau, double* datav, double* dataw)
{
    return guard([&] {
        need(ctx != nullptr, "context is NULL");
        ModelScans scans;                   // the model is scanned once: checks, then its min / max
        check_grid(nz, nx, d_pml, nt, dx, dz, dt, v, &scans);
        need(w != nullptr, "w is NULL");
        need(nr == 0 || datau != nullptr, "datau is NULL");
        need(indx == 0 || indx == 1, "indx must be 0 or 1");
        Context& c = *ctx;
        MNAD_CK(cudaSetDevice(c.device));
        PropSpec s;
        s.mode = MODE_FWD;
        s.nz = nz; s.nx = nx; s.d = d_pml; s.nt = nt;
        s.dx = dx; s.dz = dz; s.dt = dt; s.v = v; s.w = w;
        s.zs = index1(zs, nz, "zs");
        s.xs = index1(xs, nx, "xs");
        fill_receivers(s, xr, zr, nr);
        s.record_vw = c.opt.record_vw && (datav || dataw);
        s.energy_every = c.opt.energy_every;
        std::unique_ptr<Wavefield> wf;
        if (indx == 1) {
            const auto [vmin, vmax] = scans.scan(v, (size_t)nz * nx);
            const int nf = snapshot_nf(nt, vmin, vmax);                     // :46
            const int T = c.opt.T > 0 ? c.opt.T : snapshot_T(nt, nf);       // :47
            const int k = nt / T;
            wf = new_wavefield(c, nz, nx, d_pml, nt, T, std::max(2 * nf + 1, k), k, c.opt.snapshot_codec);
            s.T = T;
            s.wf = wf.get();
        }
        Prop p;
        p.spec = s;
        p.spec.depth2 = may_use_depth2(c);
        const TileCfg tc = tile_cfg(c.opt.kernel);
        p.build(c);
        Batch b(c, tc, p.spec.depth2);
        b.add(&p);
        b.finalize();
        b.run(use_graph(c, nt));
        const size_t nd = (size_t)nt * nr;
        download(c, datau, p.data.get(), nd * sizeof(double));
        if (s.record_vw && datav) download(c, datav, p.datav.get(), nd * sizeof(double));
        if (s.record_vw && dataw) download(c, dataw, p.dataw.get(), nd * sizeof(double));
        c.last_energy.assign(p.energy.size() / sizeof(double), 0.0);
        if (!c.last_energy.empty()) download(c, c.last_energy.data(), p.energy.get(), p.energy.size());
        check_device_status(c, "mnad_fwd_pde_exact");
        if (wf) c.wavefields[ss] = std::move(wf);
    });
}

MNAD_API int mnad_fwd_fields(mnad_context* ctx, double dx, double xs, const double* xr, int nr,
                             double dz, double zs, const double* zr,
                             const double* v, int nz, int nx, double dt, int nt,
                             const double* w, int d_pml, int nkeep, const int* steps,
                             double* datau, double* fields)
{
    return guard([&] {
        need(ctx != nullptr, "context is NULL");
        check_grid(nz, nx, d_pml, nt, dx, dz, dt, v);
        need(w != nullptr, "w is NULL");
        need(nr == 0 || datau != nullptr, "datau is NULL");
        need(nkeep >= 0 && (nkeep == 0 || (steps && fields)), "steps/fields are NULL");
        for (int k = 0; k < nkeep; ++k)
            need(steps[k] >= 1 && steps[k] <= nt && (k == 0 || steps[k] > steps[k - 1]),
                 "steps must be ascending within 1..nt");
        Context& c = *ctx;
        MNAD_CK(cudaSetDevice(c.device));
        PropSpec s;
        s.mode = MODE_FWD;
        s.nz = nz; s.nx = nx; s.d = d_pml; s.nt = nt;
        s.dx = dx; s.dz = dz; s.dt = dt; s.v = v; s.w = w;
        s.zs = index1(zs, nz, "zs");
        s.xs = index1(xs, nx, "xs");
        fill_receivers(s, xr, zr, nr);
        s.energy_every = c.opt.energy_every;
        Prop p;
        p.spec = s;
        const TileCfg tc = tile_cfg(c.opt.kernel);
        p.build(c);
        Batch b(c, tc);
        b.add(&p);
        b.finalize();
        b.start();
        const size_t N = (size_t)nz * nx;
        const double vs = v[(size_t)s.zs + (size_t)s.xs * nz];
        const double rs = (vs * vs) * (dt * dt);
        DevMem tmp(&c, N * sizeof(double));
        int done = 0;
        for (int k = 0; k < nkeep; ++k) {
            b.advance(done, steps[k]);
            done = steps[k];
            // After step tt the new fields sit in time level tt & 1; the stored
            // U at the source already holds the injection of step tt+1.
            const int lvl = done & 1;
            const float fix = done < nt ? (float)(rs * w[done]) : 0.0f;
            for (int f = 0; f < 3; ++f) {
                field_export<<<(int)std::min<size_t>((N + 255) / 256, 4096), 256, 0, c.stream>>>(
                    p.desc.fld[lvl][f], nz, nx, p.desc.ld, f == 0 ? p.desc.src : -1, f == 0 ? fix : 0.0f,
                    tmp.as<double>());
                MNAD_CK(cudaGetLastError());
                download(c, fields + ((size_t)k * 3 + f) * N, tmp.get(), N * sizeof(double));
            }
        }
        b.advance(done, nt);
        download(c, datau, p.data.get(), (size_t)nt * nr * sizeof(double));
        c.last_energy.assign(p.energy.size() / sizeof(double), 0.0);
        if (!c.last_energy.empty()) download(c, c.last_energy.data(), p.energy.get(), p.energy.size());
        check_device_status(c, "mnad_fwd_fields");
    });
}

MNAD_API int mnad_fwd_pde_exact_noalloc(int device, double dx, double xs, const double* xr, int nr,
                                        double dz, double zs, const double* zr,
                                        const double* v, int nz, int nx, double dt, int nt,
                                        const double* w, int d_pml, double* datau)
{
    return guard([&] {
        check_grid(nz, nx, d_pml, nt, dx, dz, dt, v);
        need(w != nullptr, "w is NULL");
        need(nr == 0 || datau != nullptr, "datau is NULL");
        int n = 0;
        MNAD_CK(cudaGetDeviceCount(&n));
        need(device >= 0 && device < n, "no CUDA device " + std::to_string(device));
        PropSpec s;
        s.nz = nz; s.nx = nx;
        fill_receivers(s, xr, zr, nr);
        fwd_noalloc(device, dx, index1(xs, nx, "xs"), s.xr, dz, index1(zs, nz, "zs"), s.zr, v, nz, nx, dt, nt, w,
                    d_pml, datau);
    });
}

MNAD_API int mnad_born_adj(mnad_context* ctx, double dx, double dz, int nt, double dt,
                           const double* v, int nz, int nx, const double* xr, const double* zr, int nr,
                           const double* data, int d_pml, int ss, double* im)
{
    return guard([&] {
        need(ctx != nullptr, "context is NULL");
        ModelScans scans;                   // the model is scanned once: checks, then its min / max
        check_grid(nz, nx, d_pml, nt, dx, dz, dt, v, &scans);
        need(im != nullptr, "im is NULL");
        need(nr == 0 || data != nullptr, "data is NULL");
        Context& c = *ctx;
        MNAD_CK(cudaSetDevice(c.device));
        auto it = c.wavefields.find(ss);
        if (it == c.wavefields.end())
            throw Error(MNAD_E_NOTFOUND, "no stored source wavefield for shot " + std::to_string(ss) +
                                             " (run the forward with indx=1 or import UU first)");
        Wavefield& wf = *it->second;
        need(wf.nint == (size_t)(nz - 2 * d_pml) * (nx - 2 * d_pml),
             "stored wavefield of shot " + std::to_string(ss) + " has a different interior size");
        const auto [vmin, vmax] = scans.scan(v, (size_t)nz * nx);
        const int T = c.opt.T > 0 ? c.opt.T : snapshot_T(nt, snapshot_nf(nt, vmin, vmax));   // :41-42
        need(nt / T <= wf.ncols, "more imaging steps (floor(nt/T)) than snapshot columns; "
                                 "UU(:,end-ttt+1) would index column < 1");
        PropSpec s;
        s.mode = MODE_ADJ;
        s.nz = nz; s.nx = nx; s.d = d_pml; s.nt = nt;
        s.dx = dx; s.dz = dz; s.dt = dt; s.v = v;
        fill_receivers(s, xr, zr, nr);
        s.T = T;
        s.wf = &wf;
        s.pairing = c.opt.pairing;
        Prop p;
        p.spec = s;
        p.spec.depth2 = may_use_depth2(c);
        const TileCfg tc = tile_cfg(c.opt.kernel);
        p.build(c);
        upload(c, p.data.get(), data, (size_t)nt * nr * sizeof(double));
        Batch b(c, tc, p.spec.depth2);
        b.add(&p);
        b.finalize();
        b.run(use_graph(c, nt));
        const size_t n = p.nint();
        DevMem out(&c, n * sizeof(double));
        scale_f64<<<(int)std::min<size_t>((n + 255) / 256, 4096), 256, 0, c.stream>>>(p.image.as<double>(), (double)T, n,
                                                                                        out.as<double>());
        MNAD_CK(cudaGetLastError());
        download(c, im, out.get(), n * sizeof(double));   // Im = T*Im (:138)
        check_device_status(c, "mnad_born_adj");
    });
}

// ---------------------------------------------------------------------------
MNAD_API int mnad_wavefield_info(mnad_context* ctx, int ss, int64_t* nint, int* ncols, int* nsnap, int* T)
{
    return guard([&] {
        need(ctx != nullptr, "context is NULL");
        auto it = ctx->wavefields.find(ss);
        if (it == ctx->wavefields.end()) throw Error(MNAD_E_NOTFOUND, "no stored wavefield for shot " + std::to_string(ss));
        const Wavefield& wf = *it->second;
        if (nint) *nint = (int64_t)wf.nint;
        if (ncols) *ncols = wf.ncols;
        if (nsnap) *nsnap = wf.nsnap;
        if (T) *T = wf.T;
    });
}

MNAD_API int mnad_wavefield_export(mnad_context* ctx, int ss, double* UU, double* illum)
{
    return guard([&] {
        need(ctx != nullptr, "context is NULL");
        Context& c = *ctx;
        MNAD_CK(cudaSetDevice(c.device));
        auto it = c.wavefields.find(ss);
        if (it == c.wavefields.end()) throw Error(MNAD_E_NOTFOUND, "no stored wavefield for shot " + std::to_string(ss));
        const Wavefield& wf = *it->second;
        if (UU) {
            const size_t n = wf.nint * (size_t)wf.ncols;
            DevMem tmp(&c, std::max<size_t>(1, n * sizeof(double)));
            snap_export<<<(int)std::min<size_t>((n + 255) / 256, 8192), 256, 0, c.stream>>>(
                wf.snap.get(), wf.codec, wf.scale.as<float>(), wf.nint, wf.nsnap, wf.ncols, tmp.as<double>());
            MNAD_CK(cudaGetLastError());
            download(c, UU, tmp.get(), n * sizeof(double));
            c.sync();
        }
        if (illum) {
            const size_t n = wf.nint;
            DevMem tmp(&c, std::max<size_t>(1, n * sizeof(double)));
            scale_f64<<<(int)std::min<size_t>((n + 255) / 256, 4096), 256, 0, c.stream>>>(
                wf.illum.as<double>(), (double)wf.T, n, tmp.as<double>());   // illum = T*illum (:162)
            MNAD_CK(cudaGetLastError());
            download(c, illum, tmp.get(), n * sizeof(double));
            c.sync();
        }
    });
}

MNAD_API int mnad_wavefield_import(mnad_context* ctx, int ss, int nz, int nx, int d_pml, int nt, int T,
                                   int ncols, int nsnap, const double* UU, const double* illum)
{
    return guard([&] {
        need(ctx != nullptr && UU != nullptr, "NULL argument");
        need(nz >= 1 && nx >= 1 && d_pml >= 0 && nz >= 2 * d_pml && nx >= 2 * d_pml, "bad grid");
        need(T >= 1 && nt >= 1, "T and nt must be >= 1");
        need(nsnap >= 0 && nsnap <= ncols, "need 0 <= nsnap <= ncols");
        Context& c = *ctx;
        MNAD_CK(cudaSetDevice(c.device));
        auto wf = new_wavefield(c, nz, nx, d_pml, nt, T, ncols, nsnap, c.opt.snapshot_codec);
        const size_t n = wf->nint * (size_t)nsnap;
        if (wf->codec == MNAD_SNAP_F16 && nsnap > 0) {
            // per-column power-of-two scales, as the forward's encoder picks them
            std::vector<float> sc(nsnap, 1.0f);
            for (int k = 0; k < nsnap; ++k) {
                double mx = 0;
                for (size_t q = 0; q < wf->nint; ++q) mx = std::max(mx, std::fabs(UU[(size_t)k * wf->nint + q]));
                if (mx > 0) {
                    int e = 0;
                    std::frexp((float)mx, &e);
                    sc[k] = std::ldexp(1.0f, e - 14);
                }
            }
            upload(c, wf->scale.get(), sc.data(), sc.size() * sizeof(float));
        }
        if (n) {
            DevMem tmp(&c, n * sizeof(double));
            upload(c, tmp.get(), UU, n * sizeof(double));
            snap_import<<<(int)std::min<size_t>((n + 255) / 256, 8192), 256, 0, c.stream>>>(
                tmp.as<double>(), wf->codec, wf->scale.as<float>(), wf->nint, nsnap, wf->snap.get());
            MNAD_CK(cudaGetLastError());
            c.sync();
        }
        if (illum) {
            DevMem tmp(&c, wf->nint * sizeof(double));
            upload(c, tmp.get(), illum, wf->nint * sizeof(double));
            scale_f64<<<(int)std::min<size_t>((wf->nint + 255) / 256, 4096), 256, 0, c.stream>>>(
                tmp.as<double>(), 1.0 / T, wf->nint, wf->illum.as<double>());
            MNAD_CK(cudaGetLastError());
            c.sync();
        }
        c.wavefields[ss] = std::move(wf);
    });
}

MNAD_API int mnad_wavefield_release(mnad_context* ctx, int ss)
{
    return guard([&] {
        need(ctx != nullptr, "context is NULL");
        auto it = ctx->wavefields.find(ss);
        if (it == ctx->wavefields.end()) throw Error(MNAD_E_NOTFOUND, "no stored wavefield for shot " + std::to_string(ss));
        MNAD_CK(cudaSetDevice(ctx->device));
        ctx->wavefields.erase(it);
        ctx->sync();
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched jobs.
struct mnad_plan {
    mnad_context* ctx = nullptr;
    std::vector<mnad_job> jobs;
    std::vector<std::unique_ptr<Prop>> props;            // owns every propagation
    std::vector<Prop*> fwd_true, fwd_bg, adj;            // per job (nullptr where not used)
    std::vector<std::unique_ptr<Wavefield>> wfs;
    // r of each distinct (host model, grid, dt, mode): shots that pass the same
    // model array share one upload and one device copy
    std::map<std::tuple<const double*, int, int, double, int>, DevMem> rcache;
    std::unique_ptr<Batch> phase1, phase3;
    // checkpointed RTM (options.checkpoint_every > 0): per job the segment
    // length C = m*T, the segment count G and the pairing offset delta
    // (imaging column = tt/T + delta); `recomp` holds the background forwards
    bool ckpt = false;
    std::vector<int> ck_C, ck_m, ck_G, ck_delta;
    std::unique_ptr<Batch> recomp;
    cudaEvent_t ev[4] = {};
    double pts = 0, bytes = 0;
    double bytes_fwd = 0, bytes_adj = 0;        // phase 1 / phase 3 (with the recomputation)
    float run_ms = 0, step_ms = 0, fwd_ms = 0, adj_ms = 0;
    int launches = 0;
    // run once and destroyed (mnad_run_jobs): launch the steps directly --
    // capturing and instantiating a graph of thousands of launches costs more
    // than it saves on a single run, and direct launches overlap the GPU work
    bool once = false;
    ~mnad_plan()
    {
        if (ctx) cudaStreamSynchronize(ctx->stream);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }
};

static Prop* add_prop(mnad_plan& P, const mnad_job& j, int mode, const double* v, Wavefield* wf, int T)
{
    auto p = std::make_unique<Prop>();
    p->spec = job_spec(j, mode, v, wf, T, P.ctx->opt.pairing);
    p->spec.depth2 = !P.ckpt && may_use_depth2(*P.ctx);
    P.props.push_back(std::move(p));
    return P.props.back().get();
}

// Adjoints of a checkpointed plan, segment by segment from the last: restore
// every background forward from its checkpoint, recompute the segment's C
// steps with snapshots into the C/T-column buffer, then run the adjoint steps
// that image with exactly those snapshots.  Each propagation advances only in
// its own window of global steps (s_begin, s_end), with s_off chosen so its
// local step continues where it stands and its time level keeps the parity of
// the global step.  Returns the number of step launches.
static int run_segments(mnad_plan& P)
{
    Context& c = *P.ctx;
    const size_t nj = P.jobs.size();
    P.phase3->start();                              // zero adjoint states and images
    int Gmax = 0;
    for (size_t k = 0; k < nj; ++k)
        if (P.adj[k]) Gmax = std::max(Gmax, P.ck_G[k]);
    auto off = [](Prop* p) { p->desc.s_begin = p->desc.s_end = INT_MIN; };
    for (size_t k = 0; k < nj; ++k)
        if (P.fwd_bg[k]) P.fwd_bg[k]->ckpt.saving = false;   // the recomputation saves nothing
    int R = 0, launches = 0;
    for (int r = 0; r < Gmax; ++r) {
        int L = 0;
        for (size_t k = 0; k < nj; ++k) {
            Prop* b = P.fwd_bg[k];
            if (!b) continue;
            const int g = P.ck_G[k] - 1 - r;
            if (g < 0) { off(b); continue; }
            b->restore_state(c, g);
            const int a0 = g * P.ck_C[k], len = std::min(P.ck_C[k], P.jobs[k].nt - a0);
            b->desc.s_off = R - a0;
            b->desc.s_begin = R;
            b->desc.s_end = R + len;
            b->desc.snap_flags = SNAP_WRITE;
            b->desc.snap_col0 = g * P.ck_m[k];
            L = std::max(L, len);
        }
        P.recomp->refresh_descs();
        P.recomp->advance(R, R + L);
        launches += L;
        R += L + (L & 1);
        L = 0;
        for (size_t k = 0; k < nj; ++k) {
            Prop* a = P.adj[k];
            if (!a) continue;
            const int g = P.ck_G[k] - 1 - r;
            if (g < 0) { off(a); continue; }
            const int nt = P.jobs[k].nt, C = P.ck_C[k], Td = a->spec.T * P.ck_delta[k];
            const int hi = g == P.ck_G[k] - 1 ? nt : (g + 1) * C - Td;
            const int lo = std::max(0, g * C - Td);
            const int sa = nt - hi, len = hi - lo;      // adjoint local steps sa .. sa + len - 1
            const int Rj = R + (sa & 1);
            a->desc.s_off = Rj - sa;
            a->desc.s_begin = Rj;
            a->desc.s_end = Rj + len;
            a->desc.snap_col0 = g * P.ck_m[k];
            L = std::max(L, (sa & 1) + len);
        }
        P.phase3->refresh_descs();
        P.phase3->advance(R, R + L);
        launches += L;
        R += L + (L & 1);
    }
    // back to the whole-run descriptors for the next run
    for (size_t k = 0; k < nj; ++k)
        for (Prop* p : {P.fwd_bg[k], P.adj[k]}) {
            if (!p) continue;
            p->desc.s_off = 0;
            p->desc.s_begin = INT_MIN;
            p->desc.s_end = INT_MAX;
            p->desc.snap_col0 = 0;
            if (p->spec.mode == MODE_FWD) {
                p->desc.snap_flags = SNAP_ILLUM;
                p->ckpt.saving = true;
            }
        }
    P.recomp->refresh_descs();
    P.phase3->refresh_descs();
    MNAD_CK(cudaGetLastError());
    return launches;
}

extern "C" {

MNAD_API int mnad_plan_create(mnad_context* ctx, const mnad_job* jobs, int njobs, mnad_plan** out)
{
    return guard([&] {
        need(ctx && out && (njobs == 0 || jobs), "NULL argument");
        need(njobs >= 0, "njobs must be >= 0");
        *out = nullptr;
        Context& c = *ctx;
        MNAD_CK(cudaSetDevice(c.device));
        auto P = std::make_unique<mnad_plan>();
        P->ctx = ctx;
        P->jobs.assign(jobs, jobs + njobs);
        ModelScans scans;                   // each distinct model is scanned once
        for (int k = 0; k < njobs; ++k) check_job(jobs[k], k, &scans);
        const TileCfg tc = tile_cfg(c.opt.kernel);
        P->ckpt = c.opt.checkpoint_every > 0;
        // whole runs from step 0: the phases may use the two-step kernel
        // (the checkpointed adjoint runs in step windows, so it may not)
        const bool d2 = !P->ckpt && may_use_depth2(c);
        P->phase1 = std::make_unique<Batch>(c, tc, d2);
        P->phase3 = std::make_unique<Batch>(c, tc, d2);
        P->fwd_true.assign(njobs, nullptr);
        P->fwd_bg.assign(njobs, nullptr);
        P->adj.assign(njobs, nullptr);
        P->ck_C.assign(njobs, 0);
        P->ck_m.assign(njobs, 0);
        P->ck_G.assign(njobs, 0);
        P->ck_delta.assign(njobs, 0);
        if (P->ckpt) P->recomp = std::make_unique<Batch>(c, tc);
        for (int k = 0; k < njobs; ++k) {
            const mnad_job& j = jobs[k];
            P->fwd_true[k] = add_prop(*P, j, MODE_FWD, j.v, nullptr, 0);
            if (j.kind == MNAD_JOB_RTM) {
                int T, ncols;
                rtm_snapshot_plan(j, T, ncols, &scans);
                const int k_snap = j.nt / T;
                if (P->ckpt) {
                    // segments of C = m*T steps (C even, so a restored state keeps
                    // its time-level parity); m > delta, so each adjoint chunk
                    // images with the snapshots of one segment only
                    const int delta = c.opt.pairing == MNAD_PAIR_REFERENCE ? ncols - k_snap : 0;
                    int m = std::max((c.opt.checkpoint_every + T - 1) / T, delta + 1);
                    if ((m * T) & 1) ++m;
                    P->ck_C[k] = m * T;
                    P->ck_m[k] = m;
                    P->ck_G[k] = (j.nt + m * T - 1) / (m * T);
                    P->ck_delta[k] = delta;
                    P->wfs.push_back(new_wavefield(c, j.nz, j.nx, j.d_pml, j.nt, T, ncols, k_snap, MNAD_SNAP_F32, m));
                } else {
                    P->wfs.push_back(new_wavefield(c, j.nz, j.nx, j.d_pml, j.nt, T, ncols, k_snap, c.opt.snapshot_codec));
                }
                Wavefield* wf = P->wfs.back().get();
                P->fwd_bg[k] = add_prop(*P, j, MODE_FWD, j.vs, wf, T);
                P->adj[k] = add_prop(*P, j, MODE_ADJ, j.vs, wf, T);
            }
        }
        for (auto& p : P->props) {
            const PropSpec& sp = p->spec;
            const auto key = std::make_tuple(sp.v, sp.nz, sp.nx, sp.dt, sp.mode);
            auto it = P->rcache.find(key);
            if (it == P->rcache.end()) it = P->rcache.emplace(key, make_r(c, sp.v, sp.nz, sp.nx, sp.dt, sp.mode)).first;
            p->r_ext = it->second.as<float>();
            p->build(c);
            (p->spec.mode == MODE_FWD ? P->phase1 : P->phase3)->add(p.get());
            P->pts += p->point_updates();
            P->bytes += p->algorithmic_bytes();
            (p->spec.mode == MODE_FWD ? P->bytes_fwd : P->bytes_adj) += p->algorithmic_bytes();
        }
        if (P->ckpt)
            for (int k = 0; k < njobs; ++k) {
                Prop* b = P->fwd_bg[k];
                if (!b) continue;
                b->desc.snap_flags = SNAP_ILLUM;       // the full forward only accumulates illumination
                b->setup_checkpoints(c, P->ck_C[k], P->ck_G[k], c.opt.checkpoint_codec);
                b->ckpt.saving = true;
                P->recomp->add(b);
                P->pts += b->point_updates();           // the recomputation is work done too
                P->bytes += b->algorithmic_bytes();
                P->bytes_adj += b->algorithmic_bytes();
            }
        if (P->ckpt) P->recomp->finalize();
        P->phase1->finalize();
        P->phase3->finalize();
        for (auto& e : P->ev) MNAD_CK(cudaEventCreate(&e));
        c.sync();
        *out = P.release();
    });
}

MNAD_API int mnad_plan_run(mnad_plan* P)
{
    return guard([&] {
        need(P != nullptr, "plan is NULL");
        Context& c = *P->ctx;
        MNAD_CK(cudaSetDevice(c.device));
        const bool g = c.opt.use_graphs != 0 && !P->once;
        MNAD_CK(cudaEventRecord(P->ev[0], c.stream));
        P->phase1->run(g);
        MNAD_CK(cudaEventRecord(P->ev[1], c.stream));
        for (size_t k = 0; k < P->jobs.size(); ++k) {
            if (!P->adj[k]) continue;
            const size_t n = (size_t)P->jobs[k].nt * P->jobs[k].nr;
            if (n == 0) continue;
            residual_f64<<<(int)std::min<size_t>((n + 255) / 256, 1024), 256, 0, c.stream>>>(
                P->fwd_true[k]->data.as<double>(), P->fwd_bg[k]->data.as<double>(), n, P->adj[k]->data.as<double>());
            MNAD_CK(cudaGetLastError());
        }
        MNAD_CK(cudaEventRecord(P->ev[2], c.stream));
        int seg_launches = 0;
        if (P->ckpt) seg_launches = run_segments(*P);
        else P->phase3->run(g);
        MNAD_CK(cudaEventRecord(P->ev[3], c.stream));
        MNAD_CK(cudaEventSynchronize(P->ev[3]));
        float a = 0, b = 0, t = 0;
        MNAD_CK(cudaEventElapsedTime(&t, P->ev[0], P->ev[3]));
        MNAD_CK(cudaEventElapsedTime(&a, P->ev[0], P->ev[1]));
        MNAD_CK(cudaEventElapsedTime(&b, P->ev[2], P->ev[3]));
        P->run_ms = t;
        P->step_ms = a + b;
        P->fwd_ms = a;
        P->adj_ms = b;
        P->launches = P->phase1->step_launches() + (P->ckpt ? seg_launches : P->phase3->step_launches());
        check_device_status(c, "mnad_plan_run");
    });
}

MNAD_API int mnad_plan_download(mnad_plan* P)
{
    return guard([&] {
        need(P != nullptr, "plan is NULL");
        Context& c = *P->ctx;
        MNAD_CK(cudaSetDevice(c.device));
        std::vector<DevMem> tmp;
        for (size_t k = 0; k < P->jobs.size(); ++k) {
            const mnad_job& j = P->jobs[k];
            const size_t nd = (size_t)j.nt * j.nr;
            if (j.kind == MNAD_JOB_MODEL) {
                if (nd) download(c, j.data_out, P->fwd_true[k]->data.get(), nd * sizeof(double));
                continue;
            }
            Prop* a = P->adj[k];
            if (j.data_out && nd) download(c, j.data_out, a->data.get(), nd * sizeof(double));
            const size_t n = a->nint();
            const int T = a->spec.T;
            tmp.emplace_back(&c, n * sizeof(double));
            scale_f64<<<(int)std::min<size_t>((n + 255) / 256, 4096), 256, 0, c.stream>>>(
                a->image.as<double>(), (double)T, n, tmp.back().as<double>());
            MNAD_CK(cudaGetLastError());
            download(c, j.image_out, tmp.back().get(), n * sizeof(double));
            if (j.illum_out) {
                tmp.emplace_back(&c, n * sizeof(double));
                scale_f64<<<(int)std::min<size_t>((n + 255) / 256, 4096), 256, 0, c.stream>>>(
                    a->spec.wf->illum.as<double>(), (double)T, n, tmp.back().as<double>());
                MNAD_CK(cudaGetLastError());
                download(c, j.illum_out, tmp.back().get(), n * sizeof(double));
            }
        }
        c.sync();
    });
}

MNAD_API int mnad_plan_destroy(mnad_plan* P)
{
    return guard([&] {
        if (P) MNAD_CK(cudaSetDevice(P->ctx->device));
        delete P;
    });
}

MNAD_API int mnad_plan_work(const mnad_plan* P, double* pts, double* bytes)
{
    return guard([&] {
        need(P != nullptr, "plan is NULL");
        if (pts) *pts = P->pts;
        if (bytes) *bytes = P->bytes;
    });
}

MNAD_API int mnad_plan_timing(const mnad_plan* P, double* run_ms, double* step_ms, int* launches)
{
    return guard([&] {
        need(P != nullptr, "plan is NULL");
        if (run_ms) *run_ms = P->run_ms;
        if (step_ms) *step_ms = P->step_ms;
        if (launches) *launches = P->launches;
    });
}

MNAD_API int mnad_plan_phases(const mnad_plan* P, double* forward_ms, double* forward_bytes, double* adjoint_ms,
                              double* adjoint_bytes)
{
    return guard([&] {
        need(P != nullptr, "plan is NULL");
        if (forward_ms) *forward_ms = P->fwd_ms;
        if (forward_bytes) *forward_bytes = P->bytes_fwd;
        if (adjoint_ms) *adjoint_ms = P->adj_ms;
        if (adjoint_bytes) *adjoint_bytes = P->bytes_adj;
    });
}

MNAD_API int mnad_plan_kernels(const mnad_plan* P, int* forward_kernel, int* adjoint_kernel)
{
    return guard([&] {
        need(P != nullptr, "plan is NULL");
        if (forward_kernel) *forward_kernel = P->phase1->main_kind();
        if (adjoint_kernel) *adjoint_kernel = P->phase3->main_kind();
    });
}

MNAD_API int mnad_plan_stack(mnad_plan* P, double* image_sum, double* illum_sum, double* img_rtm)
{
    return guard([&] {
        need(P != nullptr, "plan is NULL");
        Context& c = *P->ctx;
        MNAD_CK(cudaSetDevice(c.device));
        Prop* first = nullptr;
        for (Prop* a : P->adj)
            if (a) {
                if (!first) first = a;
                need(a->nint() == first->nint() && a->spec.nz == first->spec.nz && a->spec.nx == first->spec.nx,
                     "mnad_plan_stack: RTM jobs have different grids");
            }
        need(first != nullptr, "mnad_plan_stack: the plan has no RTM job");
        const size_t n = first->nint();
        const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
        DevMem im(&c, n * sizeof(double)), il(&c, n * sizeof(double)), out(&c, n * sizeof(double));
        MNAD_CK(cudaMemsetAsync(im.get(), 0, im.size(), c.stream));
        MNAD_CK(cudaMemsetAsync(il.get(), 0, il.size(), c.stream));
        for (Prop* a : P->adj) {
            if (!a) continue;
            const double T = (double)a->spec.T;
            axpy_f64<<<blocks, 256, 0, c.stream>>>(T, a->image.as<double>(), n, im.as<double>());
            axpy_f64<<<blocks, 256, 0, c.stream>>>(T, a->spec.wf->illum.as<double>(), n, il.as<double>());
        }
        divide_f64<<<blocks, 256, 0, c.stream>>>(im.as<double>(), il.as<double>(), n, out.as<double>());
        MNAD_CK(cudaGetLastError());
        if (image_sum) download(c, image_sum, im.get(), n * sizeof(double));
        if (illum_sum) download(c, illum_sum, il.get(), n * sizeof(double));
        if (img_rtm) download(c, img_rtm, out.get(), n * sizeof(double));
        c.sync();
    });
}

MNAD_API int mnad_run_jobs(mnad_context* ctx, const mnad_job* jobs, int njobs)
{
    mnad_plan* P = nullptr;
    int rc = mnad_plan_create(ctx, jobs, njobs, &P);
    if (rc != MNAD_OK) return rc;
    P->once = true;
    rc = mnad_plan_run(P);
    if (rc == MNAD_OK) rc = mnad_plan_download(P);
    const std::string keep = last_error();
    const int rc2 = mnad_plan_destroy(P);
    if (rc != MNAD_OK) {
        last_error() = keep;
        return rc;
    }
    return rc2;
}

}  // extern "C"
