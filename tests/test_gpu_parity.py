"""GPU parity: the CUDA path (through the C ABI) against the FP64 oracle.

Tolerances (FP32 stencil vs FP64 oracle): shot gathers and wavefields
rel-L2 <= 1e-5; RTM images rel-L2 <= 1e-4 with FP32 snapshots; the BF16
snapshot codec's image error is measured and bounded separately (<= 1e-2).
"""
import os

import numpy as np
import pytest

import mnad
from mnad import _lib, workflow
from oracle import coracle
from oracle import mnad_oracle as P

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL_GATHER = 1e-5
TOL_IMAGE = 1e-4


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def ctx():
    from mnad import build
    build.build()
    with mnad.Context(0) as c:
        yield c


def test_forward_matches_golden_fixture(ctx):
    g = np.load(os.path.join(GOLDEN, "golden_fwd_small.npz"))
    args = (float(g["dx"]), int(g["xs"]), g["xr"], float(g["dz"]), int(g["zs"]), g["zr"], g["v"], float(g["dt"]),
            int(g["nt"]), g["w"], int(g["d"]))
    datau, fields = ctx.fwd_fields(*args, steps=g["steps"])
    assert rel(datau, g["datau"]) <= TOL_GATHER
    for k, t in enumerate(g["steps"]):
        nU, nV, nW = fields[int(t)]
        assert rel(nU, g["fields"][k]) <= TOL_GATHER
        assert rel(nV, g["fields_v"][k]) <= TOL_GATHER
        assert rel(nW, g["fields_w"][k]) <= TOL_GATHER
    ctx.set_options(T=int(g["T"]))
    try:
        d2 = ctx.fwd(*args, ss=77, indx=1)
        UU, illum = ctx.wavefield_export(77)
    finally:
        ctx.set_options(T=0)
    assert rel(d2, g["datau"]) <= TOL_GATHER
    assert UU.shape == g["UU"].shape
    assert rel(UU, g["UU"]) <= 1e-4           # d2u is a second difference of FP32 fields
    assert rel(illum, g["illum"].ravel(order="F")) <= 2e-4
    ctx.wavefield_release(77)


def test_rtm_image_matches_golden_fixture(ctx):
    g = np.load(os.path.join(GOLDEN, "golden_rtm_small.npz"))
    dx, dz, dt, nt, d = float(g["dx"]), float(g["dz"]), float(g["dt"]), int(g["nt"]), int(g["d"])
    xr, zr, w = g["xr"], g["zr"], g["w"]
    zs, xs = int(g["zs"]), int(g["xs"])
    data = ctx.fwd(dx, xs, xr, dz, zs, zr, g["v"], dt, nt, w, d, ss=5)
    bg = ctx.fwd(dx, xs, xr, dz, zs, zr, g["vs"], dt, nt, w, d, ss=5, indx=1)
    assert ctx.wavefield_info(5)["T"] == int(g["T"])
    assert ctx.wavefield_info(5)["ncols"] == g["UU"].shape[1]
    assert rel(data, g["datau"]) <= TOL_GATHER
    res = data - bg
    assert rel(res, g["data"]) <= 1e-4        # difference of two close gathers
    im = ctx.adj(dx, dz, nt, dt, g["vs"], xr, zr, res, d, ss=5)
    assert rel(im, g["Im"]) <= TOL_IMAGE
    # the drop-in mirror returns the reference's Nint x 1 column
    Im = mnad.Born_adj_MNAD(dx, dz, nt, dt, g["vs"], xr, zr, [res], d, 5, ctx=ctx)
    assert Im.shape == (g["Im"].size, 1)
    assert rel(Im[:, 0], g["Im"]) <= TOL_IMAGE
    ctx.wavefield_release(5)


@pytest.mark.parametrize("src", ["interior", "strip", "corner"])
def test_forward_vs_oracle_random_model(ctx, src):
    rng = np.random.default_rng({"interior": 1, "strip": 2, "corner": 3}[src])
    nz, nx, d, nt = 37, 70, 9, 200
    v = 1600 + 1200 * rng.random((nz, nx))
    dx, dz, dt = 11.0, 9.0, 1e-3
    zs, xs = {"interior": (19, 35), "strip": (d, 30), "corner": (2, 3)}[src]
    xr = rng.integers(1, nx + 1, 40)
    zr = rng.integers(1, nz + 1, 40)
    xr[:3] = xr[0]                  # duplicate receivers
    zr[:3] = zr[0]
    w = workflow.ricker(30.0, dt, nt)
    out = ctx.fwd(dx, xs, xr, dz, zs, zr, v, dt, nt, w, d, record_vw=True)
    ref = coracle.fwd(dx, xs, xr, dz, zs, zr, v, dt, nt, w, d, record_vw=True)
    assert rel(out[0], ref["datau"]) <= TOL_GATHER
    assert rel(out[1], ref["datav"]) <= TOL_GATHER
    assert rel(out[2], ref["dataw"]) <= TOL_GATHER


@pytest.mark.parametrize("pairing", ["reference", "aligned"])
def test_misaligned_snapshot_pairing(ctx, pairing):
    """D3: with ncols = 2nf+1 > k the reference pairs snapshots T steps late."""
    nz, nx, d = 30, 44, 6
    v = np.full((nz, nx), 1500.0)
    v[15:, :] = 1500.0 * 1.4          # vmax/vmin = 1.4
    nt, T = 60, 5                      # nf = floor(60/8.4) = 7: ncols = 15 > k = 12
    nf = P.snapshot_nf(v, nt)
    assert 2 * nf + 1 > nt // T
    dx = dz = 10.0
    dt = 1e-3
    w = workflow.ricker(40.0, dt, nt)
    xr = np.arange(d + 1, nx - d + 1)
    zr = np.full(xr.size, d + 1)
    ctx.set_options(T=T, pairing=pairing)
    try:
        ctx.fwd(dx, nx // 2, xr, dz, d + 1, zr, v, dt, nt, w, d, ss=9, indx=1)
        data = np.random.default_rng(5).standard_normal((nt, xr.size))
        im = ctx.adj(dx, dz, nt, dt, v, xr, zr, data, d, ss=9)
    finally:
        ctx.set_options(T=0, pairing="reference")
    ncols = max(2 * nf + 1, nt // T)
    bg = coracle.fwd(dx, nx // 2, xr, dz, d + 1, zr, v, dt, nt, w, d, indx=1, T=T, ncols=ncols)
    ref = coracle.adj(dx, dz, nt, dt, v, xr, zr, data, d, bg["UU"], T, pairing=pairing)
    assert rel(im, ref) <= TOL_IMAGE
    ctx.wavefield_release(9)


def test_constant_velocity_gather_and_snapshots(ctx):
    """Constant-velocity shot: 201x201, 2000 m/s, 20 Hz, nt=1000; gather and the wavefield
    at t = 0.3 s and 0.6 s (steps 300 and 600) against the FP64 oracle."""
    sv = workflow.constant_velocity_shot()
    sh = sv.shots[0]
    args = (sv.dx, sh.xs, sh.xr, sv.dz, sh.zs, sh.zr, sv.v, sv.dt, sv.nt, sv.w, sv.d_pml)
    datau, fields = ctx.fwd_fields(*args, steps=[300, 600])
    ref = coracle.fwd(*args, keep_steps=(300, 600))
    assert rel(datau, ref["datau"]) <= TOL_GATHER
    for t in (300, 600):
        assert rel(fields[t][0], ref["fields"][t][0]) <= TOL_GATHER


def test_bf16_snapshot_error_is_bounded(ctx):
    g = np.load(os.path.join(GOLDEN, "golden_rtm_small.npz"))
    dx, dz, dt, nt, d = float(g["dx"]), float(g["dz"]), float(g["dt"]), int(g["nt"]), int(g["d"])
    ctx.set_options(snapshot_codec="bf16")
    try:
        ctx.fwd(dx, int(g["xs"]), g["xr"], dz, int(g["zs"]), g["zr"], g["vs"], dt, nt, g["w"], d, ss=6, indx=1)
        im = ctx.adj(dx, dz, nt, dt, g["vs"], g["xr"], g["zr"], g["data"], d, ss=6)
    finally:
        ctx.set_options(snapshot_codec="f32")
    e = rel(im, g["Im"])
    print(f"BF16 snapshot image rel-L2 = {e:.3e}")
    assert e <= 1e-2
    ctx.wavefield_release(6)


def test_batched_equals_single_shot_bitwise(ctx):
    g = np.load(os.path.join(GOLDEN, "golden_rtm_small.npz"))
    dx, dz, dt, nt, d = float(g["dx"]), float(g["dz"]), float(g["dt"]), int(g["nt"]), int(g["d"])
    xr, zr, w = g["xr"], g["zr"], g["w"]
    jobs = []
    for xs in (12, 30, 47):
        jobs.append(mnad.ShotJob(kind="rtm", v=g["v"], vs=g["vs"], dx=dx, dz=dz, dt=dt, nt=nt, d_pml=d, zs=int(g["zs"]),
                                 xs=xs, zr=zr, xr=xr, w=w, keep_data=True))
    jobs.append(mnad.ShotJob(kind="model", v=g["v"], dx=dx, dz=dz, dt=dt, nt=nt, d_pml=d, zs=int(g["zs"]), xs=20,
                             zr=zr, xr=xr, w=w))
    ctx.run_jobs(jobs)
    for j in jobs[:3]:
        data = ctx.fwd(dx, j.xs, xr, dz, j.zs, zr, g["v"], dt, nt, w, d, ss=3)
        bg = ctx.fwd(dx, j.xs, xr, dz, j.zs, zr, g["vs"], dt, nt, w, d, ss=3, indx=1)
        im = ctx.adj(dx, dz, nt, dt, g["vs"], xr, zr, data - bg, d, ss=3)
        UU, illum = ctx.wavefield_export(3)
        assert np.array_equal(j.data, data - bg)
        assert np.array_equal(j.image, im)
        assert np.array_equal(j.illum.ravel(order="F"), illum)
    single = ctx.fwd(dx, 20, xr, dz, int(g["zs"]), zr, g["v"], dt, nt, w, d)
    assert np.array_equal(jobs[3].data, single)
    ctx.wavefield_release(3)


def test_plan_rerun_is_deterministic(ctx):
    g = np.load(os.path.join(GOLDEN, "golden_rtm_small.npz"))
    job = mnad.ShotJob(kind="rtm", v=g["v"], vs=g["vs"], dx=float(g["dx"]), dz=float(g["dz"]), dt=float(g["dt"]),
                       nt=int(g["nt"]), d_pml=int(g["d"]), zs=int(g["zs"]), xs=int(g["xs"]), zr=g["zr"],
                       xr=g["xr"], w=g["w"])
    plan = ctx.plan([job])
    plan.run()
    plan.download()
    first = job.image.copy()
    plan.run()
    plan.download()
    assert np.array_equal(first, job.image)
    assert rel(job.image, g["Im"]) <= TOL_IMAGE
    pts, byt = plan.work()
    assert pts == 3 * g["v"].size * int(g["nt"])
    t = plan.timing()
    assert t["run_ms"] > 0 and t["step_launches"] == 2 * int(g["nt"])
    plan.close()


def test_plan_checks_every_model_once_and_names_the_bad_one(ctx):
    """Jobs of a plan that share one model array are checked once; a job with
    its own model holding a NaN still fails the plan with E_ARG."""
    g = np.load(os.path.join(GOLDEN, "golden_rtm_small.npz"))
    common = dict(dx=float(g["dx"]), dz=float(g["dz"]), dt=float(g["dt"]), nt=int(g["nt"]), d_pml=int(g["d"]),
                  zs=int(g["zs"]), xs=int(g["xs"]), zr=g["zr"], xr=g["xr"], w=g["w"])
    v, vs = np.asfortranarray(g["v"]), np.asfortranarray(g["vs"])
    bad = vs.copy(order="F")
    bad[5, 7] = np.nan
    jobs = [mnad.ShotJob(kind="rtm", v=v, vs=vs, **common), mnad.ShotJob(kind="rtm", v=v, vs=vs, **common),
            mnad.ShotJob(kind="rtm", v=v, vs=bad, **common)]
    with pytest.raises(mnad.MnadError) as e:
        ctx.plan(jobs)
    assert e.value.code == _lib.E_ARG
    assert f"velocity must be positive and finite (entry {5 + 7 * v.shape[0]})" in str(e.value)
    plan = ctx.plan(jobs[:2])             # the two shots of one model run alike
    plan.run()
    plan.download()
    assert np.array_equal(jobs[0].image, jobs[1].image)
    assert rel(jobs[0].image, g["Im"]) <= TOL_IMAGE
    plan.close()


def test_wavefield_export_import_round_trip(ctx):
    g = np.load(os.path.join(GOLDEN, "golden_rtm_small.npz"))
    nz, nx = g["vs"].shape
    d, nt, T = int(g["d"]), int(g["nt"]), int(g["T"])
    ctx.wavefield_import(41, nz, nx, d, nt, T, g["UU"], nsnap=nt // T, illum=g["illum"].ravel(order="F"))
    UU, illum = ctx.wavefield_export(41)
    assert np.array_equal(UU, g["UU"].astype(np.float32).astype(np.float64))
    assert rel(illum, g["illum"].ravel(order="F")) < 1e-15
    im = ctx.adj(float(g["dx"]), float(g["dz"]), nt, float(g["dt"]), g["vs"], g["xr"], g["zr"], g["data"], d, ss=41)
    assert rel(im, g["Im"]) <= TOL_IMAGE
    ctx.wavefield_release(41)


def test_errors_are_reported_not_crashed(ctx):
    g = np.load(os.path.join(GOLDEN, "golden_fwd_small.npz"))
    v = g["v"]
    nz, nx = v.shape
    args = dict(dx=10.0, dz=10.0, dt=1e-3, nt=10, w=np.zeros(10), d_pml=4)
    with pytest.raises(mnad.MnadError) as e:
        ctx.fwd(10.0, nx + 1, [1], 10.0, 1, [1], v, 1e-3, 10, np.zeros(10), 4)
    assert e.value.code == _lib.E_ARG
    assert f"xs must be an integer grid index in [1, {nx}]" in str(e.value)
    with pytest.raises(mnad.MnadError) as e:
        ctx.fwd(10.0, 2.5, [1], 10.0, 1, [1], v, 1e-3, 10, np.zeros(10), 4)
    assert e.value.code == _lib.E_ARG
    with pytest.raises(mnad.MnadError) as e:
        ctx.fwd(10.0, 5, [1, nx + 3], 10.0, 5, [1, 1], v, 1e-3, 10, np.zeros(10), 4)
    assert e.value.code == _lib.E_ARG and "xr must be an integer grid index" in str(e.value)
    bad = v.copy()
    bad[3, 3] = np.nan
    with pytest.raises(mnad.MnadError) as e:
        ctx.fwd(10.0, 5, [1], 10.0, 5, [1], bad, 1e-3, 10, np.zeros(10), 4)
    assert e.value.code == _lib.E_ARG
    assert f"velocity must be positive and finite (entry {3 + 3 * nz})" in str(e.value)
    with pytest.raises(mnad.MnadError) as e:
        ctx.adj(10.0, 10.0, 10, 1e-3, v, [1], [1], np.zeros((10, 1)), 4, ss=12345)
    assert e.value.code == _lib.E_NOTFOUND
    with mnad.Context(0, hbm_budget=1 << 20) as small:
        with pytest.raises(mnad.MnadError) as e:
            small.fwd(10.0, 5, [1], 10.0, 5, [1], np.full((400, 400), 2000.0), 1e-3, 10, np.zeros(10), 4)
        assert e.value.code == _lib.E_BUDGET
    # the context stays usable after every error
    out = ctx.fwd(10.0, 5, [1, 2], 10.0, 5, [1, 2], v, 1e-3, 10, np.ones(10), 4)
    assert np.all(np.isfinite(out))


@pytest.mark.parametrize("kernel", ["direct", "tma"])
def test_step_kernels_agree(ctx, kernel):
    """Both step kernels evaluate the same per-point arithmetic."""
    g = np.load(os.path.join(GOLDEN, "golden_rtm_small.npz"))
    dx, dz, dt, nt, d = float(g["dx"]), float(g["dz"]), float(g["dt"]), int(g["nt"]), int(g["d"])
    ctx.set_options(kernel=kernel)
    try:
        data = ctx.fwd(dx, int(g["xs"]), g["xr"], dz, int(g["zs"]), g["zr"], g["v"], dt, nt, g["w"], d, ss=8)
        bg = ctx.fwd(dx, int(g["xs"]), g["xr"], dz, int(g["zs"]), g["zr"], g["vs"], dt, nt, g["w"], d, ss=8, indx=1)
        im = ctx.adj(dx, dz, nt, dt, g["vs"], g["xr"], g["zr"], data - bg, d, ss=8)
    finally:
        ctx.set_options(kernel="auto")
    assert rel(data, g["datau"]) <= TOL_GATHER
    assert rel(im, g["Im"]) <= TOL_IMAGE
    ctx.wavefield_release(8)


@pytest.mark.parametrize("kernel", ["direct", "tma"])
@pytest.mark.parametrize("nz,nx,d", [(48, 64, 0), (45, 53, 1), (66, 47, 5), (80, 80, 40)])
def test_edge_geometries(ctx, kernel, nz, nx, d):
    """No CPML, a 1-point CPML, sizes off the tile and 4-row grid, nz = 2*d_pml."""
    rng = np.random.default_rng(nz * 1000 + nx + d)
    v = 1800 + 600 * rng.random((nz, nx))
    nt = 120
    w = workflow.ricker(35.0, 1e-3, nt)
    xr = np.arange(1, nx + 1, 2)
    zr = np.full(xr.size, d + 1)      # first interior row, as the reference drivers place them
    zs, xs = nz // 2, nx // 2
    ctx.set_options(kernel=kernel)
    try:
        out = ctx.fwd(10.0, xs, xr, 10.0, zs, zr, v, 1e-3, nt, w, d)
    finally:
        ctx.set_options(kernel="auto")
    ref = coracle.fwd(10.0, xs, xr, 10.0, zs, zr, v, 1e-3, nt, w, d)["datau"]
    assert rel(out, ref) <= TOL_GATHER
    assert ctx.status() == 0
