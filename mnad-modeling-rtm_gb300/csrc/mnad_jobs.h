// Argument checking, error capture and job set-up shared by the C ABI entry
// points (mnad_capi.cu) and the serving loop (mnad_server.cu).  Internal.
#pragma once
#include <map>
#include <memory>
#include <new>
#include <string>
#include <utility>

#include "mnad_engine.h"

namespace mnad {

// Message of the last failed call on this thread (mnad_last_error).
std::string& last_error();

// Runs f, turning exceptions into status codes (the C ABI never throws).
template <class F>
int guard(F&& f)
{
    try {
        f();
        return MNAD_OK;
    } catch (const Error& e) {
        last_error() = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        last_error() = "host allocation failed";
        return MNAD_E_OOM;
    } catch (const std::exception& e) {
        last_error() = e.what();
        return MNAD_E_CUDA;
    }
}

void need(bool ok, const std::string& msg);
// 1-based grid index passed as a double (MATLAB) -> 0-based int.
int index1(double x, int n, const char* what);
// Velocity models scanned during one call.  The jobs of a batch usually
// share their models, so each distinct array is checked (positive, finite)
// and its min / max taken once per call instead of once per job.
struct ModelScans {
    std::map<std::pair<const double*, size_t>, std::pair<double, double>> seen;   // -> (vmin, vmax)
    std::pair<double, double> scan(const double* v, size_t n);
};
void check_grid(int nz, int nx, int d, int nt, double dx, double dz, double dt, const double* v,
                ModelScans* scans = nullptr);
void check_job(const mnad_job& j, int k, ModelScans* scans = nullptr);
void fill_receivers(PropSpec& s, const double* xr, const double* zr, int nr);
// `held` snapshot columns are allocated (< 0: all nsnap).
std::unique_ptr<Wavefield> new_wavefield(Context& c, int nz, int nx, int d, int nt, int T, int ncols, int nsnap,
                                         int codec, int held = -1);
// Snapshot interval of an RTM job (job.T or the reference formula on vs)
// and the UU column count max(2 nf + 1, floor(nt/T)).
void rtm_snapshot_plan(const mnad_job& j, int& T, int& ncols, ModelScans* scans = nullptr);
// Propagation spec of a job: forward (true or background model) or adjoint.
PropSpec job_spec(const mnad_job& j, int mode, const double* v, Wavefield* wf, int T, int pairing);
// Device status bits -> error: ST_TIMEOUT throws MNAD_E_TIMEOUT (a step
// launch gave up on a tile copy, so the outputs are incomplete), ST_NONFINITE
// or ST_F16_RANGE throw MNAD_E_NUMERIC (a recorded value was not finite or a
// snapshot saturated).  `what` names the call.
void raise_status(unsigned bits, const std::string& what);
// Reads and clears the context's status word (synchronising its stream),
// then raise_status().
void check_device_status(Context& c, const std::string& what);
// Whether propagations built under the context's kernel option should carry
// the storage of the two-step kernel (it may then be chosen for them).
bool may_use_depth2(const Context& c);

}  // namespace mnad
