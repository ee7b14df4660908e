// Host-side engine of the MNAD library: context, device memory, propagations,
// batches and plans.  Internal; the public surface is include/mnad.h.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <tuple>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mnad.h"
#include "mnad_device.cuh"

namespace mnad {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void check_cuda(cudaError_t e, const char* what, const char* file, int line);
#define MNAD_CK(x) ::mnad::check_cuda((x), #x, __FILE__, __LINE__)

struct Context;

// Stream-ordered device allocation owned by a context (RAII, move-only).
class DevMem {
public:
    DevMem() = default;
    DevMem(Context* c, size_t bytes);
    ~DevMem() { reset(); }
    DevMem(DevMem&& o) noexcept { *this = std::move(o); }
    DevMem& operator=(DevMem&& o) noexcept;
    DevMem(const DevMem&) = delete;
    DevMem& operator=(const DevMem&) = delete;
    void reset();
    template <class T> T* as() const { return static_cast<T*>(p_); }
    void* get() const { return p_; }
    size_t size() const { return n_; }
private:
    Context* ctx_ = nullptr;
    void* p_ = nullptr;
    size_t n_ = 0;
};

// Source-side snapshots + illumination of one shot (the reference's
// UU_<ss>.mat / illum_<ss>.mat pair), resident on the device.
struct Wavefield {
    int nz = 0, nx = 0, d = 0, nt = 0, T = 0, nsnap = 0, ncols = 0, codec = 0;
    int held = 0;             // snapshot columns allocated: nsnap, or a segment of a checkpointed run
    size_t nint = 0;
    DevMem snap, scale, illum;
    DevMem stage, maxbits;   // FP16 codec: FP32 staging snapshot, per-snapshot max |d2u|
};

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    mnad_options opt{};
    size_t budget = 0;        // 0: unbounded
    size_t in_use = 0;
    size_t peak = 0;           // largest in_use since creation
    uint64_t h2d = 0, d2h = 0;   // bytes copied host->device / device->host
    int num_sms = 0;
    unsigned* d_status = nullptr;    // launch-wide status word, and every propagation's unless it has its own
    unsigned wait_limit = 0;         // polls of a bounded barrier wait in the step kernels (0: default)
    std::map<int, std::unique_ptr<Wavefield>> wavefields;
    // MNAD_KERNEL_TUNE: measured step kernel per (nz, nx, d_pml, propagations per launch)
    std::map<std::tuple<int, int, int, int>, int> kernel_choice;
    std::vector<double> last_energy;  // energy history of the last drop-in forward

    explicit Context(int dev, size_t budget_bytes);
    ~Context();
    void* alloc(size_t bytes);
    void release(void* p, size_t bytes);
    void sync();
    unsigned take_status();
};

// Step-kernel choice of a batch: MNAD_KERNEL_DIRECT, MNAD_KERNEL_TMA,
// MNAD_KERNEL_AUTO (per launch group: the TMA kernel once a launch has
// AUTO_TMA_TILES_PER_CTA of its tiles for each resident CTA, the direct
// kernel below) or MNAD_KERNEL_TUNE (per launch group, measured on the
// batch's own propagations at its first run; Batch::tune).
struct TileCfg {
    int kind;     // MNAD_KERNEL_*
};
TileCfg tile_cfg(int kernel);
// Measured crossover of the two step kernels on GB300 (152 SMs, 2 CTAs per
// SM; grids of 96^2 to 2048^2, 1 to 8 propagations per launch): the direct
// kernel wins up to 0.59M point-updates per launch (575 tiles, 1.9 per CTA),
// the persistent TMA kernel from 0.82M (800 tiles, 2.6 per CTA) on; its
// pipeline needs a few tiles per CTA to hide the load latency.
constexpr double AUTO_TMA_TILES_PER_CTA = 2.25;
// AUTO: the narrow (64 x 8) tiles below this share of CPML strip points in
// the grid, the 64 x 16 tiles above it (between two measured grids: 8 % and
// 22 %).
constexpr double AUTO_NARROW_STRIP_SHARE = 0.15;
constexpr int TUNE_WARMUP = 2, TUNE_STEPS = 8;

// Receivers of one propagation bucketed by TMA_TZ x TMA_TX tile and, within a
// tile, by column (stable counting sort): entries of tile t are
// tile_rec[t] .. tile_rec[t+1], those of its local column c are
// col_rec[t*TMA_TX + c] .. col_rec[t*TMA_TX + c+1].  pt: storage offsets,
// id: receiver numbers, rr: r at the receiver (mode's formula).
struct RecBuckets {
    std::vector<int> pt, id, tile_rec, col_rec;
    std::vector<double> rr;
};
void bucket_receivers(int nz, int nx, int ld, const std::vector<int>& zr, const std::vector<int>& xr,
                      const double* v, double dt, int mode, RecBuckets& out);

// Geometry and inputs of one propagation.
struct PropSpec {
    int mode = MODE_FWD;
    int nz = 0, nx = 0, d = 0, nt = 0;
    double dx = 0, dz = 0, dt = 0;
    const double* v = nullptr;         // host model, nz*nx column-major
    int zs = -1, xs = -1;              // 0-based source (forward), -1: none
    const double* w = nullptr;         // host wavelet [nt]
    std::vector<int> zr, xr;           // 0-based receivers
    bool record_vw = false;
    Wavefield* wf = nullptr;           // forward: snapshots to fill; adjoint: to image with
    int T = 0;                         // snapshot / imaging interval (0: none)
    int pairing = MNAD_PAIR_REFERENCE;
    int energy_every = 0;              // forward: FP64 energy every that many steps
    unsigned* status = nullptr;        // device status word of this propagation (null: the context's)
    bool depth2 = false;               // also keep the storage of the two-step kernel (4 field
                                       // levels, a second bank of CPML memory variables)
};

// Saved states of a forward propagation (checkpointed RTM).  Slot g - 1
// holds the state (both time levels of U, V, W and the CPML memory variables)
// after g*C steps, g = 1 .. G-1; the state after 0 steps is a fresh start.
struct Checkpoints {
    int C = 0, G = 0, codec = MNAD_SNAP_F32;
    bool saving = false;                  // save while the propagation runs
    size_t slot = 0;                      // elements per slot (fields, then mx, then mz)
    std::vector<std::pair<size_t, size_t>> blocks;   // FP16: (offset, count) of each scaled array
    DevMem data, scale, maxbits;          // data [G-1][slot]; FP16: scale, maxbits [G-1][blocks]
};

// Device state of one propagation.
struct Prop {
    PropSpec spec;
    PropDesc desc{};
    Coefs coefs{};                     // stencil polynomials of (dx, dz)
    size_t S = 0;                      // floats per field in storage
    std::vector<int> tile_rec_host;    // receiver bucket offsets per tile
    std::vector<int> col_rec_host;     // ... and per bucket column (RecBuckets::col_rec)
    DevMem fields, r, mx, mz, mx2, mz2, src_amp, rec_pt, rec_id, rec_r, tile_rec, col_rec, data, datav, dataw, image;
    DevMem energy, d_desc;             // energy history; this propagation's descriptor on the device
    DevMem inj;                        // adjoint: injection table [nt][nr] (built by reset())
    const float* r_ext = nullptr;      // set before build(): r shared with other propagations
    void build(Context& ctx);
    void reset(Context& ctx);          // zero the state of a fresh run; an adjoint also builds
                                       // its injection table from its (final) data (stream-ordered)
    void start(Context& ctx, int s_off);   // reset + seed the source; run from global step s_off (even)
    Checkpoints ckpt;
    void setup_checkpoints(Context& ctx, int C, int G, int codec);
    void save_state(Context& ctx, int g);       // state after g*C steps into slot g-1 (async)
    void restore_state(Context& ctx, int g);    // g = 0: fresh start (zero state, source seeded)
    size_t nint() const { return (size_t)(spec.nz - 2 * spec.d) * (spec.nx - 2 * spec.d); }
    double point_updates() const { return (double)spec.nz * spec.nx * spec.nt; }
    double algorithmic_bytes() const;
};

// Propagations of one geometry (dx, dz, nz, nx, d_pml) share the stencil
// coefficients that a launch carries as kernel parameters and one tiling.
struct LaunchGroup {
    Coefs coefs{};
    double dx = 0, dz = 0;
    int nz = 0, nx = 0, d = 0;
    std::vector<Prop*> props;
    int kind = MNAD_KERNEL_TMA;        // step kernel of this group
    DevMem desc, tile_prop, tmaps, tile_info;
    int ntiles = 0;                    // tiles of one launch (of the group's kernel)
    int ntz = 0, tiles_per_prop = 0;   // tiling of the group's kernel
};

// Propagations that advance together: one launch per geometry group and step
// (or, for groups on the two-step kernel, per two steps).  `depth2_ok` lets
// groups use the two-step kernel: the batch's propagations start at global
// step 0, advance without step windows and were built with depth2 storage.
class Batch {
public:
    Batch(Context& ctx, const TileCfg& tc, bool depth2_ok = false) : ctx_(ctx), tc_(tc), depth2_ok_(depth2_ok) {}
    ~Batch();
    void add(Prop* p) { props_.push_back(p); }
    void finalize();
    void run(bool use_graph);          // start() + every step, optionally as one CUDA graph (async)
    // MNAD_KERNEL_TUNE: time TUNE_STEPS steps of every launch group with
    // each step kernel (after TUNE_WARMUP untimed ones) and keep the faster
    // per group; choices are cached in the context.  The trial steps leave
    // no trace: run() starts from start(), which resets what they touched.
    void tune();
    void start();                      // zero all state and seed the sources (async)
    void advance(int s0, int s1);      // launch global steps s0..s1-1 (async)
    void refresh_descs();              // re-upload the descriptors after host-side changes
    // Global steps 0..K-1 (async), as one CUDA graph replayed tick after tick
    // when `use_graph` and no propagation needs per-step host work; callers
    // shift each propagation's s_off by -K between ticks.
    void tick(int K, bool use_graph);
    bool has_step_hooks() const;       // FP16 snapshot encodes, energy or checkpoints per step
    bool has_tma() const;              // a group runs the TMA kernel
    int launches_per_step() const;     // step-kernel launches of one time step
    int step_launches() const;         // step-kernel launches of a whole run (run())
    int group_kind_count(int kind) const;   // launch groups running that kernel
    int main_kind() const;             // kernel of the group with the most tiles (-1: no group)
    int group_kind(size_t g) const { return groups_[g]->kind; }
    size_t groups() const { return groups_.size(); }
    int steps() const { return nsteps_; }
    int tiles() const { return ntiles_; }
    const std::vector<Prop*>& props() const { return props_; }
private:
    void launch_step(int s, int slot);
    void launch_group(size_t gi, int s, int slot);
    int pick_kind(const LaunchGroup& g) const;
    bool depth2_allowed(const LaunchGroup& g) const;
    size_t reserve_counters(int nsteps);   // tile counters for nsteps steps (bytes used)
    void encode_snapshots(int s);      // FP16 codec: encode the snapshots taken at step s
    void energy_after(int s);          // energy diagnostic after step s
    void checkpoint_after(int s);      // checkpointed propagations: save the state after step s
    Context& ctx_;
    TileCfg tc_;
    bool depth2_ok_ = false;
    int trial_kind_ = -1;              // tune(): kernel forced on every group during a trial
    bool tuned_ = false;
    std::vector<Prop*> props_;
    std::vector<std::unique_ptr<LaunchGroup>> groups_;
    DevMem d_all_desc_;                // every descriptor (source seeding)
    DevMem d_counters_;                // per step and group: tiles claimed (TMA kernel)
    int ntiles_ = 0, nsteps_ = 0;
    cudaGraphExec_t graph_ = nullptr;
    cudaGraphExec_t tick_graph_ = nullptr;
    int tick_K_ = 0;
};

// r = v^2 dt^2 (forward) or (v dt)^2 (adjoint) of a host model, in padded
// storage on the device.
DevMem make_r(Context& ctx, const double* v, int nz, int nx, double dt, int mode);

// Stencil coefficient polynomials of one grid spacing (centre entries as in
// the Coef enum) and r = v^2 dt^2 as the forward / adjoint compute it.
void stencil_polys(double dx, double dz, float* al, float* be);
double r_of(double v, double dt, int mode);

// Model statistics for the reference's snapshot plan.
void model_minmax(const double* v, size_t n, double& vmin, double& vmax);
// nf of fwd_PDE_exact_MNAD.m:46 (may be 0).
int snapshot_nf(int nt, double vmin, double vmax);
// T of fwd_PDE_exact_MNAD.m:47 (throws when nf == 0).
int snapshot_T(int nt, int nf);

// Forward shot entirely inside the library's static scratch array (no device
// allocation); indices 0-based.  Throws Error(MNAD_E_ARG) when the shot does
// not fit.
void fwd_noalloc(int device, double dx, int xs, const std::vector<int>& xr, double dz, int zs,
                 const std::vector<int>& zr, const double* v, int nz, int nx, double dt, int nt, const double* w,
                 int d, double* datau);
size_t noalloc_scratch_bytes();

// Device copies of the shot records (FP64, nt x nr).
void upload(Context& ctx, void* dst, const void* src, size_t bytes);
void download(Context& ctx, void* dst, const void* src, size_t bytes);

}  // namespace mnad
