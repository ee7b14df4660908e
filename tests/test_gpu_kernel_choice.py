"""GPU tests of the per-launch-group step-kernel choice (MNAD_KERNEL_AUTO,
and the measured choice MNAD_KERNEL_TUNE).

A plan whose propagations fall into a small launch group (fewer than 2.25
TMA tiles of 64 x 16 points per resident CTA: the direct kernel) and a large
one (the TMA kernel) must give, group by group, bitwise the outputs of the kernel the policy
picks when that kernel is forced for the whole plan.  Both forced runs are
also checked against the FP64 oracle on one shot of each group."""
import numpy as np
import pytest

import mnad
from mnad import workflow
from oracle import coracle

pytestmark = pytest.mark.gpu
TOL_GATHER = 1e-5


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from mnad import build
    build.build()


def _jobs(nz, nx, n, nt, seed, d=10):
    rng = np.random.default_rng(seed)
    v = 1800.0 + 900.0 * rng.random((nz, nx))
    w = workflow.ricker(30.0, 1e-3, nt)
    xr = np.arange(d + 1, nx - d + 1, 3, dtype=np.float64)
    zr = np.full(xr.size, d + 2.0)
    zr[::5] = nz - d - 3.0                        # some receivers deep in the grid
    out = []
    for k in range(n):
        xs = float(d + 2 + (k * 37) % (nx - 2 * d - 4))
        out.append(mnad.ShotJob(kind="model", v=v, dx=10.0, dz=10.0, dt=1e-3, nt=nt, d_pml=d, zs=float(d + 2),
                                xs=xs, zr=zr, xr=xr, w=w))
    return out


def _copies(jobs):
    return [mnad.ShotJob(kind=j.kind, v=j.v, dx=j.dx, dz=j.dz, dt=j.dt, nt=j.nt, d_pml=j.d_pml, zs=j.zs, xs=j.xs,
                         zr=j.zr, xr=j.xr, w=j.w) for j in jobs]


def _run(kernel, small, large):
    jobs = _copies(small + large)
    with mnad.Context(0, kernel=kernel) as ctx:
        ctx.run_jobs(jobs)
        assert ctx.status() == 0
    return [j.data.copy() for j in jobs]


def test_auto_picks_the_kernel_per_launch_group():
    small = _jobs(96, 112, 3, 160, 1)             # 42 tiles per launch
    large = _jobs(360, 376, 8, 160, 2)            # 1152 tiles per launch (>= 2.25 x 304 CTAs)
    ns = len(small)
    auto = _run("auto", small, large)
    direct = _run("direct", small, large)
    tma = _run("tma", small, large)
    for k in range(ns):
        assert np.array_equal(auto[k], direct[k]), f"small-group shot {k} did not run the direct kernel"
    for k in range(ns, len(auto)):
        assert np.array_equal(auto[k], tma[k]), f"large-group shot {k} did not run the TMA kernel"
    # the two kernels agree with the FP64 oracle on one shot of each group
    for k in (0, ns):
        j = (small + large)[k]
        ref = coracle.fwd(j.dx, int(j.xs), j.xr, j.dz, int(j.zs), j.zr, j.v, j.dt, j.nt, j.w, j.d_pml)["datau"]
        assert rel(direct[k], ref) <= TOL_GATHER
        assert rel(tma[k], ref) <= TOL_GATHER


def test_tuned_choice_matches_a_forced_kernel_and_is_cached():
    """TUNE runs trial steps of both kernels before the real run; the outputs
    of each group are bitwise those of one forced kernel (the trial leaves no
    trace), and a second batch of the same shape in the context reuses the
    cached choice with the same outputs."""
    small = _jobs(96, 112, 3, 160, 1)
    large = _jobs(360, 376, 8, 160, 2)
    ns = len(small)
    direct = _run("direct", small, large)
    tma = _run("tma", small, large)
    with mnad.Context(0, kernel="tune") as ctx:
        first = _copies(small + large)
        ctx.run_jobs(first)
        again = _copies(small + large)
        ctx.run_jobs(again)
        assert ctx.status() == 0
    for group in (range(ns), range(ns, len(first))):
        ks = list(group)
        same_direct = all(np.array_equal(first[k].data, direct[k]) for k in ks)
        same_tma = all(np.array_equal(first[k].data, tma[k]) for k in ks)
        assert same_direct or same_tma
        assert all(np.array_equal(first[k].data, again[k].data) for k in ks)
