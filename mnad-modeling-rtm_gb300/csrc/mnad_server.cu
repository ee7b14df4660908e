// Serving loop: continuous batching of modeling and RTM shot jobs.
//
// A worker thread owns a private context (its own stream and HBM budget).
// Every tick it advances all running propagations, whatever their grids and
// record lengths, by chunk_steps time steps (one launch per geometry group
// and step).  Between ticks it retires finished propagations, moves RTM jobs
// from their two forward propagations (true and background model, the latter
// keeping the d2u snapshots) to the adjoint, and admits queued jobs in
// arrival order as long as their state fits the budget -- so requests that
// arrive while others run are started at the next tick and share the GPU with
// them.  Each job's result is bitwise the same alone and in a mix: its
// propagations run the same per-point arithmetic whatever else is batched.
//
// Latency is measured per job from submission to the completed copy of its
// outputs into the caller's buffers.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "mnad_jobs.h"
#include "mnad_kernels.h"

using namespace mnad;
using Clock = std::chrono::steady_clock;

namespace {

enum JobState { JS_QUEUED = MNAD_JOB_QUEUED, JS_RUNNING = MNAD_JOB_RUNNING, JS_DONE = MNAD_JOB_DONE, JS_FAILED = MNAD_JOB_FAILED };

struct ServerJob {
    uint64_t ticket = 0;
    mnad_job job{};                          // points into the owned copies below
    std::vector<double> v, vs, w, zr, xr;
    int state = JS_QUEUED;
    int status = MNAD_OK;
    std::string error;
    Clock::time_point t_submit, t_done;
    // running state
    int phase = 0;                           // 1: forward(s), 2: adjoint
    int T = 0;
    DevMem dev_status;                       // device status word of this job's propagations
    std::unique_ptr<Wavefield> wf;
    std::unique_ptr<Prop> fwd_true, fwd_bg, adj;
    double points = 0;                       // grid-point updates of the whole job
};

double percentile(std::vector<double> x, double p)
{
    if (x.empty()) return 0.0;
    std::sort(x.begin(), x.end());
    const double r = p * (x.size() - 1);
    const size_t lo = (size_t)r, hi = std::min(lo + 1, x.size() - 1);
    return x[lo] + (r - lo) * (x[hi] - x[lo]);
}

}  // namespace

struct mnad_server {
    mnad_server_options opt{};
    std::unique_ptr<Context> ctx;
    TileCfg tc{};
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    uint64_t next_ticket = 1;
    std::map<uint64_t, std::unique_ptr<ServerJob>> jobs;
    std::deque<ServerJob*> queue;            // submitted, not admitted (FIFO)
    std::vector<ServerJob*> running;         // owned by the worker thread
    std::unique_ptr<Batch> batch;
    size_t budget = 0, reserve = 0;          // HBM budget; part kept for batch tables
    std::atomic<size_t> mem_in_use{0};       // the context's device bytes, for other threads
    std::atomic<size_t> mem_peak{0};         // the context's largest device bytes so far
    bool dirty = true;
    // Each tick runs global steps 0..K-1; a propagation's local step at tick
    // step s is s - s_off, and s_off drops by K after every tick.
    // statistics (under mu)
    int64_t n_submitted = 0, n_done = 0, n_failed = 0;
    std::vector<double> latencies_ms;
    double points_done = 0, busy_s = 0;
    Clock::time_point t_first_submit{};
    bool any_submit = false;

    void loop();
    bool admit(ServerJob* j);
    void retire(ServerJob* j, int status, const std::string& err);
    void step_phase(ServerJob* j);
};

static void free_running_state(ServerJob* j)
{
    j->fwd_true.reset();
    j->fwd_bg.reset();
    j->adj.reset();
    j->wf.reset();
    j->dev_status.reset();
}

// Reads and clears the job's status word (the stream is synchronised).
static unsigned take_job_status(Context& c, ServerJob* j)
{
    unsigned s = 0;
    MNAD_CK(cudaMemcpyAsync(&s, j->dev_status.get(), sizeof(s), cudaMemcpyDeviceToHost, c.stream));
    MNAD_CK(cudaMemsetAsync(j->dev_status.get(), 0, sizeof(unsigned), c.stream));
    c.sync();
    return s;
}

// Admission: every propagation of the job is built (device state allocated)
// and the forward propagations start at the next tick; the adjoint of an RTM job
// starts when its forwards end.  Allocation stops short of the budget by a
// reserve kept for the batch tables of the ticks.
bool mnad_server::admit(ServerJob* j)
{
    Context& c = *ctx;
    c.budget = budget - reserve;
    try {
        const mnad_job& J = j->job;
        j->dev_status = DevMem(&c, sizeof(unsigned));
        MNAD_CK(cudaMemsetAsync(j->dev_status.get(), 0, sizeof(unsigned), c.stream));
        unsigned* st = j->dev_status.as<unsigned>();
        j->fwd_true = std::make_unique<Prop>();
        j->fwd_true->spec = job_spec(J, MODE_FWD, J.v, nullptr, 0, c.opt.pairing);
        j->fwd_true->spec.status = st;
        j->fwd_true->build(c);
        j->points = (double)J.nz * J.nx * J.nt;
        if (J.kind == MNAD_JOB_RTM) {
            int ncols;
            rtm_snapshot_plan(J, j->T, ncols);
            j->wf = new_wavefield(c, J.nz, J.nx, J.d_pml, J.nt, j->T, ncols, J.nt / j->T, c.opt.snapshot_codec);
            j->fwd_bg = std::make_unique<Prop>();
            j->fwd_bg->spec = job_spec(J, MODE_FWD, J.vs, j->wf.get(), j->T, c.opt.pairing);
            j->fwd_bg->spec.status = st;
            j->fwd_bg->build(c);
            j->adj = std::make_unique<Prop>();
            j->adj->spec = job_spec(J, MODE_ADJ, J.vs, j->wf.get(), j->T, c.opt.pairing);
            j->adj->spec.status = st;
            j->adj->build(c);
            j->points *= 3;
        }
        c.budget = budget;
        j->fwd_true->start(c, 0);
        if (j->fwd_bg) j->fwd_bg->start(c, 0);
        j->phase = 1;
        return true;
    } catch (const Error& e) {
        c.budget = budget;
        free_running_state(j);
        if (e.code == MNAD_E_BUDGET || e.code == MNAD_E_OOM) return false;   // wait for memory
        retire(j, e.code, e.what());
        return true;
    }
}

void mnad_server::retire(ServerJob* j, int status, const std::string& err)
{
    free_running_state(j);
    std::lock_guard<std::mutex> lk(mu);
    j->state = status == MNAD_OK ? JS_DONE : JS_FAILED;
    j->status = status;
    j->error = err;
    j->t_done = Clock::now();
    if (status == MNAD_OK) {
        ++n_done;
        latencies_ms.push_back(std::chrono::duration<double, std::milli>(j->t_done - j->t_submit).count());
        points_done += j->points;
    } else {
        ++n_failed;
    }
    cv_done.notify_all();
}

// Output of n FP64 values times T, the reference's final scaling
// (Born_adj_MNAD.m:138, fwd_PDE_exact_MNAD.m:162), applied on the host after
// the copy (one IEEE multiply per value, as on the device).
static void download_times(Context& c, double* dst, const void* src, size_t n, int T)
{
    download(c, dst, src, n * sizeof(double));
    c.sync();
    for (size_t k = 0; k < n; ++k) dst[k] *= (double)T;
}

// Called when the propagations of the job's current phase are finished.  A
// non-finite value recorded by one of the job's propagations fails this job
// only (its own status word).
void mnad_server::step_phase(ServerJob* j)
{
    Context& c = *ctx;
    const mnad_job& J = j->job;
    const size_t nd = (size_t)J.nt * J.nr;
    const unsigned st = take_job_status(c, j);
    if (st) {
        try {
            raise_status(st, "server job " + std::to_string(j->ticket));
        } catch (const Error& e) {
            retire(j, e.code, e.what());
            return;
        }
    }
    if (j->phase == 1 && J.kind == MNAD_JOB_MODEL) {
        if (nd && J.data_out) download(c, J.data_out, j->fwd_true->data.get(), nd * sizeof(double));
        c.sync();
        retire(j, MNAD_OK, "");
        return;
    }
    if (j->phase == 1) {
        // scattered data (main_Acoustic_RTM.m:225) is the adjoint's record
        if (nd) {
            residual_f64<<<(int)std::min<size_t>((nd + 255) / 256, 1024), 256, 0, c.stream>>>(
                j->fwd_true->data.as<double>(), j->fwd_bg->data.as<double>(), nd, j->adj->data.as<double>());
            MNAD_CK(cudaGetLastError());
            if (J.data_out) download(c, J.data_out, j->adj->data.get(), nd * sizeof(double));
        }
        c.sync();
        j->fwd_true.reset();
        j->fwd_bg.reset();                   // the snapshots stay in j->wf
        j->adj->start(c, 0);
        j->phase = 2;
        return;
    }
    const size_t n = j->adj->nint();
    download_times(c, J.image_out, j->adj->image.get(), n, j->T);
    if (J.illum_out) download_times(c, J.illum_out, j->wf->illum.get(), n, j->T);
    retire(j, MNAD_OK, "");
}

void mnad_server::loop()
{
    MNAD_CK(cudaSetDevice(ctx->device));
    const int K = opt.chunk_steps;
    while (true) {
        // admission in arrival order while the budget (and slot cap) allows
        {
            std::unique_lock<std::mutex> lk(mu);
            if (stop && queue.empty() && running.empty()) break;
            if (queue.empty() && running.empty()) {
                cv_work.wait(lk, [&] { return stop || !queue.empty(); });
                continue;
            }
        }
        while (true) {
            ServerJob* j = nullptr;
            {
                std::lock_guard<std::mutex> lk(mu);
                if (queue.empty()) break;
                if (opt.max_active_jobs > 0 && (int)running.size() >= opt.max_active_jobs) break;
                j = queue.front();
            }
            const bool admitted = admit(j);
            mem_in_use.store(std::max(mem_in_use.load(), ctx->in_use));
            mem_peak.store(ctx->peak);
            if (!admitted) break;            // not enough memory yet: keep FIFO order
            std::lock_guard<std::mutex> lk(mu);
            queue.pop_front();
            if (j->state == JS_QUEUED) {
                j->state = JS_RUNNING;
                running.push_back(j);
                dirty = true;
            }
        }
        if (running.empty()) {
            // the head job does not fit even on an idle GPU: fail it
            std::unique_lock<std::mutex> lk(mu);
            if (!queue.empty()) {
                ServerJob* j = queue.front();
                queue.pop_front();
                lk.unlock();
                retire(j, MNAD_E_BUDGET, "job does not fit the server's HBM budget");
            }
            continue;
        }
        const auto t0 = Clock::now();
        try {
            if (dirty) {
                batch = std::make_unique<Batch>(*ctx, tc);
                for (ServerJob* j : running) {
                    if (j->phase == 2) {
                        batch->add(j->adj.get());
                        continue;
                    }
                    batch->add(j->fwd_true.get());
                    if (j->fwd_bg) batch->add(j->fwd_bg.get());
                }
                batch->finalize();
                dirty = false;
            }
            batch->refresh_descs();
            batch->tick(K, opt.no_graphs == 0);
            for (Prop* p : batch->props()) p->desc.s_off -= K;
            // a launch that gave up (a bounded wait ran out) left tiles of every
            // job of this tick unfinished: those jobs fail, later ones run on
            raise_status(ctx->take_status() & ST_TIMEOUT, "server tick");
            // retire / advance the jobs whose current phase is over
            std::vector<ServerJob*> still;
            for (ServerJob* j : running) {
                const Prop* p = j->phase == 2 ? j->adj.get() : j->fwd_true.get();
                if (-p->desc.s_off >= p->spec.nt) {
                    step_phase(j);
                    dirty = true;
                }
                if (j->state == JS_RUNNING) still.push_back(j);
            }
            running.swap(still);
        } catch (const Error& e) {
            for (ServerJob* j : running) retire(j, e.code, e.what());
            running.clear();
            batch.reset();
            dirty = true;
        }
        mem_in_use.store(ctx->in_use);
        mem_peak.store(ctx->peak);
        std::lock_guard<std::mutex> lk(mu);
        busy_s += std::chrono::duration<double>(Clock::now() - t0).count();
    }
    batch.reset();
}

extern "C" {

MNAD_API int mnad_server_create(int device, const mnad_server_options* o, mnad_server** out)
{
    return guard([&] {
        need(out != nullptr, "out is NULL");
        *out = nullptr;
        int n = 0;
        MNAD_CK(cudaGetDeviceCount(&n));
        need(device >= 0 && device < n, "no CUDA device " + std::to_string(device));
        auto S = std::make_unique<mnad_server>();
        if (o) S->opt = *o;
        if (S->opt.chunk_steps <= 0) S->opt.chunk_steps = 64;
        S->opt.chunk_steps += S->opt.chunk_steps & 1;   // ticks keep the global step even
        need(S->opt.snapshot_codec >= MNAD_SNAP_F32 && S->opt.snapshot_codec <= MNAD_SNAP_F16, "bad snapshot_codec");
        need(S->opt.kernel >= MNAD_KERNEL_AUTO && S->opt.kernel <= MNAD_KERNEL_TMA_NARROW, "bad kernel");
        size_t budget = S->opt.hbm_budget_bytes;
        if (budget == 0) {
            MNAD_CK(cudaSetDevice(device));
            size_t fr = 0, tot = 0;
            MNAD_CK(cudaMemGetInfo(&fr, &tot));
            budget = fr / 10 * 9;
        }
        S->budget = budget;
        S->reserve = std::min<size_t>(budget / 8, size_t(64) << 20);
        S->ctx = std::make_unique<Context>(device, budget);
        S->ctx->opt.snapshot_codec = S->opt.snapshot_codec;
        S->ctx->opt.kernel = S->opt.kernel;
        S->tc = tile_cfg(S->opt.kernel);
        mnad_server* raw = S.get();
        S->worker = std::thread([raw] {
            try {
                raw->loop();
            } catch (const std::exception& e) {
                std::lock_guard<std::mutex> lk(raw->mu);
                for (auto& kv : raw->jobs)
                    if (kv.second->state == JS_QUEUED || kv.second->state == JS_RUNNING) {
                        kv.second->state = JS_FAILED;
                        kv.second->status = MNAD_E_CUDA;
                        kv.second->error = e.what();
                    }
                raw->cv_done.notify_all();
            }
        });
        *out = S.release();
    });
}

MNAD_API int mnad_server_submit(mnad_server* S, const mnad_job* job, uint64_t* ticket)
{
    return guard([&] {
        need(S && job && ticket, "NULL argument");
        check_job(*job, 0);
        auto j = std::make_unique<ServerJob>();
        const size_t N = (size_t)job->nz * job->nx;
        j->job = *job;
        j->v.assign(job->v, job->v + N);
        if (job->kind == MNAD_JOB_RTM) j->vs.assign(job->vs, job->vs + N);
        j->w.assign(job->w, job->w + job->nt);
        if (job->nr > 0) {
            need(job->zr && job->xr, "receiver index arrays are NULL");
            j->zr.assign(job->zr, job->zr + job->nr);
            j->xr.assign(job->xr, job->xr + job->nr);
        }
        j->job.v = j->v.data();
        j->job.vs = j->vs.empty() ? nullptr : j->vs.data();
        j->job.w = j->w.data();
        j->job.zr = j->zr.data();
        j->job.xr = j->xr.data();
        // validate geometry now so a bad job fails at submission
        (void)job_spec(j->job, MODE_FWD, j->job.v, nullptr, 0, MNAD_PAIR_REFERENCE);
        std::lock_guard<std::mutex> lk(S->mu);
        need(!S->stop, "server is shutting down");
        j->ticket = S->next_ticket++;
        j->t_submit = Clock::now();
        if (!S->any_submit) {
            S->any_submit = true;
            S->t_first_submit = j->t_submit;
        }
        ++S->n_submitted;
        *ticket = j->ticket;
        S->queue.push_back(j.get());
        S->jobs[j->ticket] = std::move(j);
        S->cv_work.notify_all();
    });
}

MNAD_API int mnad_server_poll(mnad_server* S, uint64_t ticket, int* state)
{
    return guard([&] {
        need(S && state, "NULL argument");
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->jobs.find(ticket);
        if (it == S->jobs.end()) throw Error(MNAD_E_NOTFOUND, "unknown ticket");
        *state = it->second->state;
    });
}

MNAD_API int mnad_server_wait(mnad_server* S, uint64_t ticket, double timeout_s)
{
    int job_status = MNAD_OK;
    std::string job_error;
    const int rc = guard([&] {
        need(S != nullptr, "server is NULL");
        std::unique_lock<std::mutex> lk(S->mu);
        auto it = S->jobs.find(ticket);
        if (it == S->jobs.end()) throw Error(MNAD_E_NOTFOUND, "unknown ticket");
        ServerJob* j = it->second.get();
        auto done = [&] { return j->state == JS_DONE || j->state == JS_FAILED; };
        if (timeout_s < 0) S->cv_done.wait(lk, done);
        else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
            throw Error(MNAD_E_TIMEOUT, "job " + std::to_string(ticket) + " not finished");
        job_status = j->status;
        job_error = j->error;
    });
    if (rc != MNAD_OK) return rc;
    if (job_status != MNAD_OK) last_error() = job_error;
    return job_status;
}

MNAD_API int mnad_server_get_stats(mnad_server* S, mnad_server_stats* st)
{
    return guard([&] {
        need(S && st, "NULL argument");
        std::lock_guard<std::mutex> lk(S->mu);
        std::memset(st, 0, sizeof(*st));
        st->submitted = S->n_submitted;
        st->completed = S->n_done;
        st->failed = S->n_failed;
        st->queued = (int64_t)S->queue.size();
        st->p50_ms = percentile(S->latencies_ms, 0.50);
        st->p99_ms = percentile(S->latencies_ms, 0.99);
        st->max_ms = S->latencies_ms.empty() ? 0.0 : *std::max_element(S->latencies_ms.begin(), S->latencies_ms.end());
        st->point_updates = S->points_done;
        st->busy_s = S->busy_s;
        st->wall_s = S->any_submit ? std::chrono::duration<double>(Clock::now() - S->t_first_submit).count() : 0.0;
        st->bytes_in_use = S->mem_in_use.load();
        st->peak_bytes = S->mem_peak.load();
    });
}

MNAD_API int mnad_server_destroy(mnad_server* S)
{
    return guard([&] {
        if (!S) return;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->stop = true;
            S->cv_work.notify_all();
        }
        if (S->worker.joinable()) S->worker.join();
        delete S;
    });
}

}  // extern "C"
