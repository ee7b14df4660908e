/*
 * mnad.h -- C ABI of the GB300 MNAD modeling / RTM library (libmnad.so).
 *
 * The library runs the time-stepping hot path of the MNAD acoustic modeling
 * and reverse-time-migration code on one NVIDIA GB300 (sm_103a): the fused
 * MNAD compact-stencil update of U and its gradient fields V = U_x, W = U_z
 * under CPML, source injection, receiver sampling, d2u snapshots with
 * illumination, and the adjoint propagation with the zero-lag
 * cross-correlation imaging condition.
 *
 * Conventions (those of the reference MATLAB code):
 *   - grids are the PML-padded nz x nx model, column-major (z fastest);
 *   - source/receiver positions are 1-based padded grid indices, passed as
 *     doubles that must hold integer values (the MATLAB drivers compute them
 *     as d_pml + metres/dx);
 *   - receiver data is nt x nr column-major FP64 (datau(tt, rr));
 *   - images and illumination are (nz-2*d_pml) x (nx-2*d_pml) column-major
 *     FP64 (the reference's Nint x 1 vectors).
 *
 * Every function returns an int status (MNAD_OK == 0).  On failure
 * mnad_last_error() returns a message for the calling thread.  Functions
 * taking a context may be called from several threads only if each thread
 * uses its own context.
 */
#ifndef MNAD_H
#define MNAD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MNAD_API __attribute__((visibility("default")))
#else
#define MNAD_API
#endif

#define MNAD_ABI_VERSION 1

/* Status codes. */
enum {
    MNAD_OK = 0,
    MNAD_E_ARG = 1,        /* invalid argument (sizes, indices, T, ...) */
    MNAD_E_OOM = 2,        /* device or host allocation failed */
    MNAD_E_CUDA = 3,       /* CUDA runtime/driver error */
    MNAD_E_TIMEOUT = 4,    /* a bounded device wait ran out */
    MNAD_E_NOTFOUND = 5,   /* no stored source wavefield for this shot id */
    MNAD_E_NUMERIC = 6,    /* non-finite values / codec saturation detected */
    MNAD_E_BUDGET = 7,     /* job does not fit the context's HBM budget */
    MNAD_E_STATE = 8       /* call not valid in the current state */
};

/* Storage codec of the source-side d2u snapshots. */
enum { MNAD_SNAP_F32 = 0, MNAD_SNAP_BF16 = 1, MNAD_SNAP_F16 = 2 };

/* Snapshot pairing of the imaging condition.
 * REFERENCE: column ncols-ttt+1 of UU, ncols = max(2*nf+1, k) as in
 *            SRC/migration/Born_adj_MNAD.m:128 (columns past k are zero).
 * ALIGNED:   column k-ttt+1 (source and receiver fields at the same time). */
enum { MNAD_PAIR_REFERENCE = 0, MNAD_PAIR_ALIGNED = 1 };

/* Step kernel choice.  AUTO picks per launch group (propagations of one grid
 * size advancing together): the persistent TMA kernel once a launch has about
 * 2.25 of its 64 x 16 tiles per resident CTA (0.7M point-updates on a 152-SM
 * GB300) -- on 64 x 8 tiles (TMA_NARROW) where the CPML strips hold under
 * 15 % of the grid's points, on 64 x 16 tiles otherwise -- and the
 * one-thread-per-point kernel (32 x 8 tiles) below.
 * TMA_NARROW is the persistent kernel on 64 x 8 tiles (128 threads per CTA,
 * 4 CTAs per SM); its outputs are bitwise those of TMA.
 * TMA2 is the persistent kernel advancing two time steps per pass (temporal
 * blocking of depth 2: each pass reads the two current time levels and writes
 * the next two, so the field traffic per step falls from 40 to about 26
 * bytes per point).  It serves whole runs of the drop-in calls and of job
 * batches (mnad_run_jobs, plans) without checkpointing, FP16 snapshots or the
 * energy diagnostic; elsewhere TMA2 runs as TMA.
 * TUNE measures the candidates -- one thread per point, TMA (64 x 16 tiles),
 * TMA_NARROW (64 x 8 tiles), and TMA2 where it applies -- on each launch
 * group of a plan or job batch at its first run (10 trial steps each, before
 * the run starts from zero state) and keeps the fastest; choices are cached in
 * the context per grid, CPML width and propagation count.  The serving loop
 * treats TUNE as AUTO. */
enum {
    MNAD_KERNEL_AUTO = 0,
    MNAD_KERNEL_DIRECT = 1,
    MNAD_KERNEL_TMA = 2,
    MNAD_KERNEL_TUNE = 3,
    MNAD_KERNEL_TMA2 = 4,
    MNAD_KERNEL_TMA_NARROW = 5
};

typedef struct mnad_options {
    int snapshot_codec;   /* MNAD_SNAP_*; default MNAD_SNAP_F32 */
    int pairing;          /* MNAD_PAIR_*; default MNAD_PAIR_REFERENCE */
    int T;                /* snapshot interval; <= 0: reference formula
                             T = floor(nt/nf/2), nf = floor(nt/(6 vmax/vmin))
                             (SRC/MNAD/fwd_PDE_exact_MNAD.m:46-47) */
    int record_vw;        /* forward also records V and W (reference keeps
                             them commented out, fwd_PDE_exact_MNAD.m:167-168) */
    int use_graphs;       /* capture the time loop in a CUDA graph (default 1) */
    int kernel;           /* MNAD_KERNEL_*; default AUTO */
    int energy_every;     /* > 0: FP64 energy diagnostic of each forward every
                             that many steps (read with mnad_context_energy) */
    int checkpoint_every; /* > 0: RTM jobs of a plan keep no snapshot history:
                             the background forward saves its state every C
                             steps (C = this value rounded up to an even
                             multiple of T), and the adjoint runs in segments,
                             each recomputing its C steps of source snapshots
                             from a checkpoint into an FP32 buffer of C/T
                             columns.  Default 0 (all snapshots kept). */
    int checkpoint_codec; /* MNAD_SNAP_F32 (exact recompute: images identical
                             to the stored-snapshot FP32 run) or MNAD_SNAP_F16
                             (states stored in FP16 with one power-of-two scale
                             per array); default MNAD_SNAP_F32 */
} mnad_options;

typedef struct mnad_context mnad_context;

/* ---- context ---------------------------------------------------------- */
MNAD_API int mnad_abi_version(void);
MNAD_API const char* mnad_last_error(void);
/* Creates a context on CUDA device `device` with its own stream.
 * hbm_budget_bytes bounds the device memory the context keeps for job
 * state and stored wavefields (0: no bound). */
MNAD_API int mnad_context_create(int device, size_t hbm_budget_bytes, mnad_context** out);
MNAD_API int mnad_context_destroy(mnad_context* ctx);
MNAD_API int mnad_context_set_options(mnad_context* ctx, const mnad_options* opt);
MNAD_API int mnad_context_get_options(const mnad_context* ctx, mnad_options* opt);
/* Bytes of device memory currently held by the context (state + wavefields). */
MNAD_API int mnad_context_memory(const mnad_context* ctx, size_t* bytes_in_use);
/* Host<->device bytes the context has copied so far (inputs, outputs). */
MNAD_API int mnad_context_transfers(const mnad_context* ctx, uint64_t* h2d_bytes, uint64_t* d2h_bytes);
/* Energy history of the last forward run by mnad_fwd_pde_exact / mnad_fwd_fields
 * with options.energy_every = K > 0: entry m (m = 0 .. floor(nt/K)-1) is, after
 * step (m+1)K, E = 1/2 sum over the image region of ((U(t+1)-U(t))^2/(v dt)^2
 * + V^2 + W^2) dx dz, accumulated in FP64 on the device (V = U_x, W = U_z are
 * the MNAD gradient fields).  *n receives the number of entries; at most max
 * are copied to out. */
MNAD_API int mnad_context_energy(const mnad_context* ctx, double* out, int max, int* n);
/* Bit set of device-side status flags seen so far (and clears them):
 * 1 = a recorded value was not finite, 2 = an FP16 snapshot saturated,
 * 4 = a bounded device wait ran out.  Every propagating entry point reads and
 * clears these flags itself at its end and fails with MNAD_E_NUMERIC (1, 2)
 * or MNAD_E_TIMEOUT (4) when one is set; the context stays usable. */
MNAD_API int mnad_context_status(mnad_context* ctx, unsigned* flags);
/* Bound of every barrier wait in the persistent step kernel, in polls of the
 * barrier (0: the default, about 4 M polls -- far longer than any tile copy
 * takes).  A wait that runs out makes the launch give up its remaining
 * tiles, and the call then returns MNAD_E_TIMEOUT.  A diagnostic for
 * watchdog tests: a limit of a few polls makes the waits run out on purpose.
 * No counterpart in the reference (its MATLAB loop has no device waits). */
MNAD_API int mnad_context_set_wait_limit(mnad_context* ctx, unsigned polls);

/* ---- drop-in entry points (reference call signatures) ------------------- */

/* data = fwd_PDE_exact_MNAD(dx,xs,xr,dz,zs,zr,v,dt,nt,w,d_pml,ss,Auu,...,Aww,indx)
 * (SRC/MNAD/fwd_PDE_exact_MNAD.m:1).  The nine sparse operators are
 * deterministic functions of (v, dx, dz, dt) and are recomputed on the
 * device, so they are not passed.  datau receives nt x nr (data{1}).
 * datav/dataw may be NULL; when non-NULL (and options.record_vw set) they
 * receive the V/W receiver traces.  With indx == 1 the d2u snapshots and the
 * illumination are kept on the device under shot id `ss` (replacing
 * ./Wavefields/UU_<ss>.mat and ./Illuminations/illum_<ss>.mat, :160-164). */
MNAD_API int mnad_fwd_pde_exact(mnad_context* ctx, double dx, double xs, const double* xr, int nr,
                                double dz, double zs, const double* zr,
                                const double* v, int nz, int nx, double dt, int nt,
                                const double* w, int d_pml, int ss, int indx,
                                double* datau, double* datav, double* dataw);

/* Forward modeling as mnad_fwd_pde_exact(..., indx=0) that also returns the
 * wavefields after the listed steps: for each 1-based step steps[k]
 * (ascending, 1..nt), fields receives nU, nV, nW of that step
 * (SRC/MNAD/fwd_PDE_exact_MNAD.m:114-116) as 3 consecutive nz x nx
 * column-major FP64 arrays (nkeep*3*nz*nx values in total). */
MNAD_API int mnad_fwd_fields(mnad_context* ctx, double dx, double xs, const double* xr, int nr,
                             double dz, double zs, const double* zr,
                             const double* v, int nz, int nx, double dt, int nt,
                             const double* w, int d_pml, int nkeep, const int* steps,
                             double* datau, double* fields);

/* Forward modeling of one shot, as mnad_fwd_pde_exact(..., indx=0) with the
 * default options, that allocates no device memory.  This entry point has no
 * counterpart in the reference.  It is for callers that cannot let a library
 * call cudaMalloc: applications whose GPU memory is already reserved by their
 * own allocator, or processes that forbid allocation after start-up.  All of
 * its working memory (wavefields, CPML memory variables, tables, the shot
 * record) lives in one static device array of 64 MiB that every GPU loading
 * the library holds until the process exits; a shot needing more (roughly a
 * 1000 x 1000 padded grid, or a long record with many receivers) is rejected
 * with MNAD_E_ARG.  The first call on a device sets up the array's device
 * address on that device, so that first call should come before any stream
 * capture on the device.  Calls share the array, clear it on entry and are
 * serialised by the library (calls that overlapped on the GPU would race on
 * it); all pointers are host pointers, as in mnad_fwd_pde_exact.  No context
 * is needed; the calling thread's current device is the same after the call
 * as before it.  Fails with MNAD_E_NUMERIC when a recorded value is not
 * finite. */
MNAD_API int mnad_fwd_pde_exact_noalloc(int device, double dx, double xs, const double* xr, int nr,
                                        double dz, double zs, const double* zr,
                                        const double* v, int nz, int nx, double dt, int nt,
                                        const double* w, int d_pml, double* datau);

/* Im = Born_adj_MNAD(dx,dz,nt,dt,v,xr,zr,data,d_pml,ss,Auu,...,Aww)
 * (SRC/migration/Born_adj_MNAD.m:1).  data is the nt x nr residual
 * (data{1} of the reference, :50); the source wavefield of shot `ss` must
 * have been stored by mnad_fwd_pde_exact(..., indx=1) or
 * mnad_wavefield_import().  im receives the Nint image, already multiplied
 * by T (:138). */
MNAD_API int mnad_born_adj(mnad_context* ctx, double dx, double dz, int nt, double dt,
                           const double* v, int nz, int nx, const double* xr, const double* zr, int nr,
                           const double* data, int d_pml, int ss, double* im);

/* ---- stored source wavefields (the ./Wavefields hand-off) -------------- */
/* nint = (nz-2d)(nx-2d); ncols = columns of the reference's UU matrix;
 * nsnap = columns actually filled (k = floor(nt/T)); T = snapshot interval. */
MNAD_API int mnad_wavefield_info(mnad_context* ctx, int ss, int64_t* nint, int* ncols, int* nsnap, int* T);
/* UU: nint x ncols FP64 (columns past nsnap are zero, as in the reference's
 * preallocated matrix); illum: nint FP64, times T.  Either may be NULL. */
MNAD_API int mnad_wavefield_export(mnad_context* ctx, int ss, double* UU, double* illum);
/* Stores a UU matrix loaded from UU_<ss>.mat (parfor may run a shot's
 * forward and adjoint in different processes).  illum may be NULL. */
MNAD_API int mnad_wavefield_import(mnad_context* ctx, int ss, int nz, int nx, int d_pml, int nt, int T,
                                   int ncols, int nsnap, const double* UU, const double* illum);
MNAD_API int mnad_wavefield_release(mnad_context* ctx, int ss);

/* ---- batched jobs (many shots per launch) ----------------------------- */
enum { MNAD_JOB_MODEL = 0, MNAD_JOB_RTM = 1 };

typedef struct mnad_job {
    int kind;                 /* MNAD_JOB_MODEL or MNAD_JOB_RTM */
    int nz, nx, d_pml, nt;    /* padded grid, CPML thickness, steps */
    double dx, dz, dt;
    const double* v;          /* true model, nz*nx column-major (host) */
    const double* vs;         /* RTM: migration (background) model */
    double zs, xs;            /* 1-based padded source indices */
    int nr;
    const double* zr;         /* 1-based padded receiver indices [nr] */
    const double* xr;
    const double* w;          /* source wavelet [nt] */
    int T;                    /* RTM snapshot interval, <= 0: formula on vs */
    double* data_out;         /* MODEL: shot gather nt x nr; RTM: scattered
                                 data data - datas (may be NULL) */
    double* image_out;        /* RTM: Nint image, times T */
    double* illum_out;        /* RTM: Nint illumination, times T (may be NULL) */
} mnad_job;

/* Runs the jobs as batches of propagations advancing together (one launch
 * per time step for every shot of a phase): MODEL = one forward; RTM = the
 * reference workflow of SRC/migration/main_Acoustic_RTM.m:221-253 per shot
 * (true-model forward, background forward with snapshots, scattered data
 * formed on the device, adjoint with imaging).  Host buffers in, host
 * buffers out. */
MNAD_API int mnad_run_jobs(mnad_context* ctx, const mnad_job* jobs, int njobs);

/* Device-resident form of mnad_run_jobs: create uploads every input and
 * allocates all state; run executes all phases on the device; download
 * copies the outputs into the jobs' host pointers. */
typedef struct mnad_plan mnad_plan;
MNAD_API int mnad_plan_create(mnad_context* ctx, const mnad_job* jobs, int njobs, mnad_plan** out);
MNAD_API int mnad_plan_run(mnad_plan* plan);
MNAD_API int mnad_plan_download(mnad_plan* plan);
MNAD_API int mnad_plan_destroy(mnad_plan* plan);
/* Grid-point updates one run performs (sum over propagations of nz*nx*nt)
 * and the algorithmic HBM bytes of those updates. */
MNAD_API int mnad_plan_work(const mnad_plan* plan, double* point_updates, double* algorithmic_bytes);
/* Device time of the last run (ms, CUDA events on the plan's stream) and the
 * device time spent in step kernels only. */
MNAD_API int mnad_plan_timing(const mnad_plan* plan, double* run_ms, double* step_ms, int* step_launches);
/* The last run split by phase: device time (ms) and algorithmic bytes of the
 * forwards (phase 1) and of the adjoints (phase 3; with checkpointing this
 * phase also holds the background recomputation). */
MNAD_API int mnad_plan_phases(const mnad_plan* plan, double* forward_ms, double* forward_bytes, double* adjoint_ms,
                              double* adjoint_bytes);
/* Step kernel (MNAD_KERNEL_DIRECT, _TMA, _TMA_NARROW or _TMA2) that the
 * forward phase and the adjoint phase of the plan run, for the launch group
 * with the most tiles (after MNAD_KERNEL_TUNE's trials, once the plan has
 * run).  -1 where a phase has no propagation. */
MNAD_API int mnad_plan_kernels(const mnad_plan* plan, int* forward_kernel, int* adjoint_kernel);
/* Stack of the plan's RTM shots after mnad_plan_run, formed in FP64 on the
 * device (SRC/migration/main_Acoustic_RTM.m:237-262): image_sum = sum of the
 * shots' images (each T*sum US.*UR), illum_sum = sum of the shots'
 * illuminations (each T*sum d2u^2), img_rtm = image_sum ./ illum_sum (the
 * reference's mean(mhh,3)./illum; the 1/ns factors cancel).  All RTM jobs
 * must share the grid.  Each output is Nint FP64 on the host, may be NULL. */
MNAD_API int mnad_plan_stack(mnad_plan* plan, double* image_sum, double* illum_sum, double* img_rtm);

/* ---- serving loop (continuous batching) -------------------------------- */
/* A server owns a worker thread and a private context on one device.  Jobs
 * (the mnad_job of mnad_run_jobs; inputs are copied at submission, outputs
 * are written into the job's host pointers before the job completes) are
 * admitted in arrival order while their device state fits the HBM budget,
 * and every admitted propagation -- of any grid and record length -- advances
 * chunk_steps time steps per tick of the worker, so jobs that arrive while
 * others run join them at the next tick.  RTM jobs run the same three
 * propagations as mnad_run_jobs (the background forward keeps its snapshots
 * on the device until the adjoint has imaged them).  A job's outputs are
 * bitwise those of the same job run alone. */
typedef struct mnad_server mnad_server;
typedef struct mnad_server_options {
    size_t hbm_budget_bytes;  /* 0: 90% of the device's free memory */
    int chunk_steps;          /* time steps per tick (rounded up to even; <= 0: 64) */
    int max_active_jobs;      /* <= 0: limited by the budget only */
    int snapshot_codec;       /* MNAD_SNAP_* of RTM snapshots */
    int kernel;               /* MNAD_KERNEL_* */
    int no_graphs;            /* 1: launch each tick's steps one by one instead of
                                 replaying a CUDA graph of the tick (the graph is
                                 captured again whenever the set of propagations
                                 changes; FP16 snapshots never use it) */
} mnad_server_options;

enum { MNAD_JOB_QUEUED = 0, MNAD_JOB_RUNNING = 1, MNAD_JOB_DONE = 2, MNAD_JOB_FAILED = 3 };

typedef struct mnad_server_stats {
    int64_t submitted, completed, failed, queued;
    double p50_ms, p99_ms, max_ms;  /* submission -> outputs on the host, completed jobs */
    double point_updates;           /* grid-point updates of the completed jobs */
    double busy_s;                  /* worker time spent in ticks */
    double wall_s;                  /* since the first submission */
    size_t bytes_in_use;            /* device memory held by the server now */
    size_t peak_bytes;              /* largest device memory the server has held */
} mnad_server_stats;

MNAD_API int mnad_server_create(int device, const mnad_server_options* opt, mnad_server** out);
/* Copies the job's inputs and queues it; *ticket identifies it.  Invalid
 * jobs fail here with MNAD_E_ARG. */
MNAD_API int mnad_server_submit(mnad_server* srv, const mnad_job* job, uint64_t* ticket);
/* *state = MNAD_JOB_*. */
MNAD_API int mnad_server_poll(mnad_server* srv, uint64_t ticket, int* state);
/* Waits until the job completes (timeout_s < 0: no limit) and returns its
 * status: MNAD_OK, the error it failed with, or MNAD_E_TIMEOUT when the
 * wait ran out (the job keeps running).  A job larger than the whole budget
 * fails with MNAD_E_BUDGET. */
MNAD_API int mnad_server_wait(mnad_server* srv, uint64_t ticket, double timeout_s);
MNAD_API int mnad_server_get_stats(mnad_server* srv, mnad_server_stats* stats);
/* Finishes every submitted job, then stops the worker and frees the server. */
MNAD_API int mnad_server_destroy(mnad_server* srv);

#ifdef __cplusplus
}
#endif
#endif /* MNAD_H */
