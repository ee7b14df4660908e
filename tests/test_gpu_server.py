"""GPU tests of the serving loop (mnad_server_*): continuous batching of
modeling and RTM jobs of uneven grids and record lengths, with admission by
HBM budget.

The bar is the one a server must meet to be a drop-in for running each shot
on its own: every job's outputs, served in a mix with jobs that arrive while
it runs, are bitwise those of the same job run alone (mnad_run_jobs of that
job only), and the RTM images also match the FP64 oracle.
"""
import time

import numpy as np
import pytest

import mnad
from mnad import workflow
from oracle import coracle
from oracle import mnad_oracle as P

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from mnad import build
    build.build()


def _job(kind, seed, nz, nx, nt, d=12, T=0):
    """Layered model with a Gaussian anomaly, smoothed migration model."""
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[:, None] * np.ones((1, nx))
    x = np.ones((nz, 1)) * np.arange(nx)[None, :]
    v = 1600.0 + 600.0 * (z > nz * 0.4) + 700.0 * (z > nz * 0.7)
    cz, cx = rng.uniform(0.3, 0.7) * nz, rng.uniform(0.3, 0.7) * nx
    v = v + 250.0 * np.exp(-((z - cz) ** 2 + (x - cx) ** 2) / (2 * (0.08 * nx) ** 2))
    vs = workflow.gaussian_smooth(v, 7)
    w = workflow.ricker(rng.uniform(15.0, 30.0), 1e-3, nt)
    xr = np.arange(d + 1, nx - d + 1, 2, dtype=np.float64)
    zr = np.full(xr.size, d + 2.0)
    xs = float(rng.integers(d + 2, nx - d - 1))
    return mnad.ShotJob(kind=kind, v=v, vs=vs if kind == "rtm" else None, dx=10.0, dz=10.0, dt=1e-3, nt=nt,
                        d_pml=d, zs=float(d + 2), xs=xs, zr=zr, xr=xr, w=w, T=T)


def _copy(j):
    return mnad.ShotJob(
        kind=j.kind, v=j.v, vs=j.vs, dx=j.dx, dz=j.dz, dt=j.dt, nt=j.nt, d_pml=j.d_pml, zs=j.zs, xs=j.xs,
        zr=j.zr, xr=j.xr, w=j.w, T=j.T)


def _alone(jobs):
    out = []
    with mnad.Context(0) as ctx:
        for j in jobs:
            a = _copy(j)
            ctx.run_jobs([a])
            out.append(a)
    return out


def _mix():
    return [_job("model", 1, 96, 128, 300), _job("rtm", 2, 80, 160, 360), _job("model", 3, 64, 64, 200),
            _job("rtm", 4, 96, 128, 240), _job("model", 5, 80, 160, 420), _job("rtm", 6, 64, 64, 300)]


def _same(a, b):
    assert np.array_equal(a.data, b.data)
    if a.kind == "rtm":
        assert np.array_equal(a.image, b.image)
        assert np.array_equal(a.illum, b.illum)
        assert np.linalg.norm(a.image) > 0


def test_served_in_a_mix_equals_alone():
    jobs = _mix()
    ref = _alone(jobs)
    with mnad.Server(0, chunk_steps=32) as srv:
        # half now, the rest while those run: they join at the next tick
        tickets = [srv.submit(j) for j in jobs[:3]]
        time.sleep(0.05)
        tickets += [srv.submit(j) for j in jobs[3:]]
        for t in tickets:
            srv.wait(t, timeout_s=300)
        st = srv.stats()
    for a, b in zip(jobs, ref):
        _same(a, b)
    assert st["completed"] == len(jobs) and st["failed"] == 0
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    expect = sum(j.v.size * j.nt * (3 if j.kind == "rtm" else 1) for j in jobs)
    assert st["point_updates"] == expect


def test_served_rtm_image_matches_the_fp64_oracle():
    j = _job("rtm", 11, 72, 120, 320)
    with mnad.Server(0, chunk_steps=16) as srv:
        srv.wait(srv.submit(j), timeout_s=300)
    nt, d = j.nt, j.d_pml
    nf, T = P.snapshot_plan(j.vs, nt)
    ncols = max(2 * nf + 1, nt // T)
    dat = coracle.fwd(j.dx, j.xs, j.xr, j.dz, j.zs, j.zr, j.v, j.dt, nt, j.w, d)["datau"]
    bg = coracle.fwd(j.dx, j.xs, j.xr, j.dz, j.zs, j.zr, j.vs, j.dt, nt, j.w, d, indx=1, T=T, ncols=ncols)
    res = dat - bg["datau"]
    im = coracle.adj(j.dx, j.dz, nt, j.dt, j.vs, j.xr, j.zr, res, d, bg["UU"], T)
    assert rel(j.data, res) <= 1e-4
    assert rel(j.image, im) <= 1e-4
    assert rel(j.illum, bg["illum"].reshape(j.illum.shape, order="F")) <= 1e-4


def test_admission_by_hbm_budget_and_oversized_jobs():
    jobs = _mix()
    ref = _alone(jobs)
    with mnad.Context(0) as ctx:
        # the device state of the largest job alone, as a bound for the budget
        big = max(jobs, key=lambda j: j.v.size * (3 if j.kind == "rtm" else 1))
        before = ctx.memory()
        plan = ctx.plan([_copy(big)])
        one = ctx.memory() - before
        plan.close()
    budget = int(one * 2.2) + (8 << 20)
    seen = []
    with mnad.Server(0, hbm_budget_bytes=budget, chunk_steps=32) as srv:
        tickets = [srv.submit(j) for j in jobs]
        huge = _job("rtm", 9, 1024, 1024, 2000)
        t_huge = srv.submit(huge)
        while srv.stats()["completed"] + srv.stats()["failed"] < len(jobs) + 1:
            seen.append(srv.stats()["bytes_in_use"])
            time.sleep(0.002)
        for t in tickets:
            srv.wait(t, timeout_s=300)
        with pytest.raises(mnad.MnadError) as e:
            srv.wait(t_huge, timeout_s=300)
        assert e.value.code == mnad._lib.E_BUDGET
        peak = srv.stats()["peak_bytes"]
    assert max(seen, default=0) <= budget
    assert 0 < peak <= budget
    for a, b in zip(jobs, ref):
        _same(a, b)


def test_one_slot_serialises_and_still_matches():
    jobs = _mix()[:3]
    ref = _alone(jobs)
    with mnad.Server(0, max_active_jobs=1, chunk_steps=64) as srv:
        tickets = [srv.submit(j) for j in jobs]
        states = [srv.poll(t) for t in tickets]
        assert states[-1] in ("queued", "running")
        for t in tickets:
            srv.wait(t, timeout_s=300)
        assert all(srv.poll(t) == "done" for t in tickets)
    for a, b in zip(jobs, ref):
        _same(a, b)


def test_invalid_jobs_fail_at_submission():
    j = _job("model", 1, 64, 64, 100)
    j.xs = 1000.0
    with mnad.Server(0) as srv:
        with pytest.raises(mnad.MnadError) as e:
            srv.submit(j)
        assert e.value.code == mnad._lib.E_ARG


def test_tick_graphs_and_direct_launches_agree():
    jobs_g, jobs_d = _mix(), _mix()
    for jobs, graphs in ((jobs_g, True), (jobs_d, False)):
        with mnad.Server(0, chunk_steps=32, graphs=graphs) as srv:
            for t in [srv.submit(j) for j in jobs]:
                srv.wait(t, timeout_s=300)
    for a, b in zip(jobs_g, jobs_d):
        _same(a, b)


def test_fp16_snapshots_served_equal_a_plan_run():
    """FP16 snapshot encodes are per-step host work, so these ticks launch
    step by step; the outputs still equal mnad_run_jobs with the same codec."""
    jobs = [j for j in _mix() if j.kind == "rtm"]
    ref = [_copy(j) for j in jobs]
    with mnad.Context(0, snapshot_codec="f16") as ctx:
        ctx.run_jobs(ref)
    with mnad.Server(0, chunk_steps=16, snapshot_codec="f16") as srv:
        for t in [srv.submit(j) for j in jobs]:
            srv.wait(t, timeout_s=300)
    for a, b in zip(jobs, ref):
        _same(a, b)
