// Argument checking, error capture and job set-up shared by the C ABI and the
// serving loop.
#include "mnad_jobs.h"

#include <algorithm>
#include <cmath>
#include <tuple>
#include <vector>

#include "mnad_kernels.h"

namespace mnad {

std::string& last_error()
{
    static thread_local std::string msg;
    return msg;
}

void need(bool ok, const std::string& msg)
{
    if (!ok) throw Error(MNAD_E_ARG, msg);
}

// 1-based grid index passed as a double (MATLAB) -> 0-based int.
int index1(double x, int n, const char* what)
{
    if (!(std::isfinite(x) && x == std::floor(x) && x >= 1 && x <= n))   // the message is built only on failure
        need(false, std::string(what) + " must be an integer grid index in [1, " + std::to_string(n) + "], got " +
                        std::to_string(x));
    return (int)x - 1;
}

std::pair<double, double> ModelScans::scan(const double* v, size_t n)
{
    const auto key = std::make_pair(v, n);
    const auto it = seen.find(key);
    if (it != seen.end()) return it->second;
    double vmin = INFINITY, vmax = -INFINITY;
    for (size_t k = 0; k < n; ++k) {
        if (!(std::isfinite(v[k]) && v[k] > 0))   // the message is built only on failure
            need(false, "velocity must be positive and finite (entry " + std::to_string(k) + ")");
        vmin = std::min(vmin, v[k]);
        vmax = std::max(vmax, v[k]);
    }
    return seen.emplace(key, std::make_pair(vmin, vmax)).first->second;
}

void check_grid(int nz, int nx, int d, int nt, double dx, double dz, double dt, const double* v, ModelScans* scans)
{
    need(v != nullptr, "v is NULL");
    need(nz >= 1 && nx >= 1, "grid must be at least 1 x 1");
    need(d >= 0 && nz >= 2 * d && nx >= 2 * d, "d_pml must satisfy 0 <= 2*d_pml <= min(nz, nx) (C_cof.m builds the strips)");
    need(nt >= 1, "nt must be >= 1");
    need(std::isfinite(dx) && dx > 0 && std::isfinite(dz) && dz > 0 && std::isfinite(dt) && dt > 0,
         "dx, dz, dt must be positive and finite");
    const size_t n = (size_t)nz * nx;
    if (scans) {
        scans->scan(v, n);
        return;
    }
    for (size_t k = 0; k < n; ++k)
        if (!(std::isfinite(v[k]) && v[k] > 0))   // the message is built only on failure
            need(false, "velocity must be positive and finite (entry " + std::to_string(k) + ")");
}

std::unique_ptr<Wavefield> new_wavefield(Context& c, int nz, int nx, int d, int nt, int T, int ncols,
                                                int nsnap, int codec, int held)
{
    auto wf = std::make_unique<Wavefield>();
    wf->nz = nz; wf->nx = nx; wf->d = d; wf->nt = nt; wf->T = T;
    wf->ncols = ncols; wf->nsnap = nsnap; wf->codec = codec;
    wf->held = held < 0 ? nsnap : held;
    wf->nint = (size_t)(nz - 2 * d) * (nx - 2 * d);
    const size_t cb = codec == MNAD_SNAP_F32 ? 4 : 2;
    wf->snap = DevMem(&c, std::max<size_t>(1, wf->nint * (size_t)wf->held * cb));
    wf->illum = DevMem(&c, std::max<size_t>(1, wf->nint * sizeof(double)));
    MNAD_CK(cudaMemsetAsync(wf->illum.get(), 0, wf->illum.size(), c.stream));
    if (codec == MNAD_SNAP_F16) {
        wf->scale = DevMem(&c, std::max(1, nsnap) * sizeof(float));
        std::vector<float> one(std::max(1, nsnap), 1.0f);
        upload(c, wf->scale.get(), one.data(), one.size() * sizeof(float));
        wf->stage = DevMem(&c, std::max<size_t>(1, wf->nint * sizeof(float)));
        wf->maxbits = DevMem(&c, std::max(1, nsnap) * sizeof(unsigned));
        MNAD_CK(cudaMemsetAsync(wf->maxbits.get(), 0, wf->maxbits.size(), c.stream));
    }
    return wf;
}

void fill_receivers(PropSpec& s, const double* xr, const double* zr, int nr)
{
    need(nr >= 0, "nr must be >= 0");
    need(nr == 0 || (xr && zr), "receiver index arrays are NULL");
    s.zr.resize(nr);
    s.xr.resize(nr);
    for (int k = 0; k < nr; ++k) {
        s.zr[k] = index1(zr[k], s.nz, "zr");
        s.xr[k] = index1(xr[k], s.nx, "xr");
    }
}

void check_job(const mnad_job& j, int k, ModelScans* scans)
{
    const std::string pre = "job " + std::to_string(k) + ": ";
    need(j.kind == MNAD_JOB_MODEL || j.kind == MNAD_JOB_RTM, pre + "kind must be MNAD_JOB_MODEL or MNAD_JOB_RTM");
    check_grid(j.nz, j.nx, j.d_pml, j.nt, j.dx, j.dz, j.dt, j.v, scans);
    need(j.w != nullptr, pre + "w is NULL");
    if (j.kind == MNAD_JOB_RTM) {
        check_grid(j.nz, j.nx, j.d_pml, j.nt, j.dx, j.dz, j.dt, j.vs, scans);
        need(j.image_out != nullptr, pre + "image_out is NULL");
    } else {
        need(j.nr == 0 || j.data_out != nullptr, pre + "data_out is NULL");
    }
}


void rtm_snapshot_plan(const mnad_job& j, int& T, int& ncols, ModelScans* scans)
{
    double vmin, vmax;
    if (scans) std::tie(vmin, vmax) = scans->scan(j.vs, (size_t)j.nz * j.nx);
    else model_minmax(j.vs, (size_t)j.nz * j.nx, vmin, vmax);
    const int nf = snapshot_nf(j.nt, vmin, vmax);             // fwd_PDE_exact_MNAD.m:46
    T = j.T > 0 ? j.T : snapshot_T(j.nt, nf);                  // :47
    ncols = std::max(2 * nf + 1, j.nt / T);                    // :53 (grown to k when larger)
}

PropSpec job_spec(const mnad_job& j, int mode, const double* v, Wavefield* wf, int T, int pairing)
{
    PropSpec s;
    s.mode = mode;
    s.nz = j.nz; s.nx = j.nx; s.d = j.d_pml; s.nt = j.nt;
    s.dx = j.dx; s.dz = j.dz; s.dt = j.dt; s.v = v; s.w = j.w;
    if (mode == MODE_FWD) {
        s.zs = index1(j.zs, j.nz, "zs");
        s.xs = index1(j.xs, j.nx, "xs");
    }
    fill_receivers(s, j.xr, j.zr, j.nr);
    s.wf = wf;
    s.T = T;
    s.pairing = pairing;
    return s;
}

void raise_status(unsigned bits, const std::string& what)
{
    if (bits & ST_TIMEOUT)
        throw Error(MNAD_E_TIMEOUT, what + ": a bounded device wait for a tile copy ran out; the outputs are "
                                           "incomplete (the context stays usable)");
    if (bits & ST_NONFINITE)
        throw Error(MNAD_E_NUMERIC, what + ": a recorded wavefield value is not finite (unstable time step "
                                           "v*dt/dx, or non-finite input)");
    if (bits & ST_F16_RANGE) throw Error(MNAD_E_NUMERIC, what + ": an FP16 snapshot value saturated");
}

void check_device_status(Context& c, const std::string& what)
{
    raise_status(c.take_status(), what);
}

bool may_use_depth2(const Context& c)
{
    return c.opt.kernel == MNAD_KERNEL_TMA2 || c.opt.kernel == MNAD_KERNEL_TUNE;
}

}  // namespace mnad
