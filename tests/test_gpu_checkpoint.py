"""GPU tests of checkpointed RTM (options.checkpoint_every): the background
forward keeps checkpoints instead of its snapshot history and the adjoint
runs in segments that recompute their snapshots.

With FP32 checkpoints the recomputation replays the same arithmetic, so the
image, illumination and scattered data are bitwise those of the run that
keeps every snapshot (FP32).  With FP16 checkpoints (one power-of-two scale
per array) the image error against the FP64 oracle is measured and bounded.
Segment edges are exercised with record lengths that are not multiples of
the segment, with both imaging pairings (the reference pairing is shifted by
one snapshot when floor(nt/T) < 2nf+1) and with jobs of different grids and
lengths in one plan."""
import os

import numpy as np
import pytest

import mnad
from mnad import workflow
from oracle import coracle
from oracle import mnad_oracle as P

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from mnad import build
    build.build()


def _job(seed, nz, nx, nt, d=12, T=0):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[:, None] * np.ones((1, nx))
    x = np.ones((nz, 1)) * np.arange(nx)[None, :]
    v = 1700.0 + 700.0 * (z > nz * 0.45) + 500.0 * (z > nz * 0.75)
    v = v + 300.0 * np.exp(-((z - 0.55 * nz) ** 2 + (x - rng.uniform(0.3, 0.7) * nx) ** 2) / (2 * (0.1 * nx) ** 2))
    vs = workflow.gaussian_smooth(v, 7)
    w = workflow.ricker(25.0, 1e-3, nt)
    xr = np.arange(d + 1, nx - d + 1, dtype=np.float64)
    zr = np.full(xr.size, d + 2.0)
    return mnad.ShotJob(kind="rtm", v=v, vs=vs, dx=10.0, dz=10.0, dt=1e-3, nt=nt, d_pml=d,
                        zs=float(d + 2), xs=float(rng.integers(d + 3, nx - d - 2)), zr=zr, xr=xr, w=w, T=T,
                        keep_data=True)


def _copy(j):
    return mnad.ShotJob(kind=j.kind, v=j.v, vs=j.vs, dx=j.dx, dz=j.dz, dt=j.dt, nt=j.nt, d_pml=j.d_pml, zs=j.zs,
                        xs=j.xs, zr=j.zr, xr=j.xr, w=j.w, T=j.T, keep_data=True)


def _run(jobs, **opts):
    out = [_copy(j) for j in jobs]
    with mnad.Context(0, **opts) as ctx:
        plan = ctx.plan(out)
        plan.run()
        plan.download()
        cp = lambda a: None if a is None else a.copy()
        first = [(cp(o.image), cp(o.illum), cp(o.data)) for o in out]
        plan.run()                                  # a rerun must give the same outputs
        plan.download()
        for o, f in zip(out, first):
            assert np.array_equal(o.data, f[2])
            if o.image is not None:
                assert np.array_equal(o.image, f[0]) and np.array_equal(o.illum, f[1])
        plan.close()
    return out


def _delta(j):
    nf, T = P.snapshot_plan(j.vs, j.nt)
    T = j.T or T
    k = j.nt // T
    return max(2 * nf + 1, k) - k, T


@pytest.mark.parametrize("pairing", ["reference", "aligned"])
def test_fp32_checkpoints_reproduce_the_stored_snapshot_run_bitwise(pairing):
    # natural T (aligned pairing), and explicit T with floor(nt/T) < 2nf+1, where
    # the reference pairing images with snapshots 36 and 20 columns later
    jobs = [_job(1, 64, 96, 430), _job(1, 64, 96, 430, T=9), _job(2, 80, 72, 377, T=7)]
    deltas = [_delta(j) for j in jobs]
    print("delta, T:", deltas)
    ref = _run(jobs, pairing=pairing)
    for every in (1, 40, 100):
        got = _run(jobs, pairing=pairing, checkpoint_every=every)
        for a, b in zip(got, ref):
            assert np.array_equal(a.image, b.image), every
            assert np.array_equal(a.illum, b.illum)
            assert np.array_equal(a.data, b.data)
            assert np.linalg.norm(a.image) > 0


def test_checkpointed_plan_with_model_jobs_and_uneven_lengths():
    jobs = [_job(3, 72, 88, 300), _job(4, 64, 64, 511)]
    m = _copy(jobs[0])
    m.kind = "model"
    m.vs = None
    m.image = m.illum = None
    ref = _run(jobs + [m])
    got = _run(jobs + [m], checkpoint_every=64)
    for a, b in zip(got, ref):
        assert np.array_equal(a.data, b.data)
        if a.kind == "rtm":
            assert np.array_equal(a.image, b.image)


def test_fp16_checkpoints_image_error_against_the_oracle():
    g = np.load(os.path.join(GOLDEN, "golden_rtm_small.npz"))
    j = mnad.ShotJob(kind="rtm", v=g["v"], vs=g["vs"], dx=float(g["dx"]), dz=float(g["dz"]), dt=float(g["dt"]),
                     nt=int(g["nt"]), d_pml=int(g["d"]), zs=float(g["zs"]), xs=float(g["xs"]), zr=g["zr"], xr=g["xr"],
                     w=g["w"], keep_data=True)
    f32 = _run([j], checkpoint_every=30)[0]
    f16 = _run([j], checkpoint_every=30, checkpoint_codec="f16")[0]
    e32, e16 = rel(f32.image, g["Im"]), rel(f16.image, g["Im"])
    print(f"image rel-L2 vs FP64 oracle: FP32 checkpoints {e32:.2e}, FP16 checkpoints {e16:.2e}")
    assert e32 <= 1e-4
    assert e16 <= 2e-3
    assert np.array_equal(f16.illum, f32.illum)     # the illumination comes from the full forward
