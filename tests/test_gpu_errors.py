"""Device-side failures reach the caller as status codes, without a GPU fault.

* Timeout: every barrier wait of the persistent step kernel is bounded.  A
  diagnostic wait limit of one poll makes waits run out on purpose; the
  launch gives up its remaining tiles (after the copies it issued have
  landed), the call returns MNAD_E_TIMEOUT, and the same context then runs a
  correct shot.  The reference's counterpart is its error(id, msg) style
  (SRC/MNAD/acquisi.m:66-67); its MATLAB loop has no device waits.
* Numeric: a valid but unstable input (Courant number v*dt/dx = 1, above the
  reference's own 0.52 rule, SRC/migration/main_Acoustic_RTM.m:75,81) blows
  up to inf/NaN in FP32 within about 60 steps; the recorded traces are not
  finite and the call returns MNAD_E_NUMERIC -- through the drop-in call on
  both step kernels, the batched jobs, and the server, where only the
  unstable job fails.
"""
import numpy as np
import pytest

import mnad
from mnad import _lib, workflow
from oracle import coracle

pytestmark = pytest.mark.gpu
TOL_GATHER = 1e-5


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def built():
    from mnad import build
    build.build()


def _geometry(nz=200, nx=300, d=20, nt=300, cfl=None, seed=0):
    dx, dt = 10.0, 1e-3
    if cfl is None:
        rng = np.random.default_rng(seed)
        z = np.arange(nz)[:, None]
        v = np.where(z < nz // 2, 1800.0, 2500.0) + 100.0 * rng.random((nz, nx))
    else:
        v = np.full((nz, nx), cfl * dx / dt)
    w = workflow.ricker(25.0, dt, nt)
    xr = np.arange(d + 1, nx - d + 1, 3, dtype=np.float64)
    zr = np.full(xr.size, d + 3.0)
    return dict(dx=dx, dz=dx, dt=dt, v=np.asfortranarray(v), w=w, xr=xr, zr=zr, nt=nt, d=d,
                zs=float(nz // 2), xs=float(nx // 2))


def _fwd(ctx, g):
    return ctx.fwd(g["dx"], g["xs"], g["xr"], g["dz"], g["zs"], g["zr"], g["v"], g["dt"], g["nt"], g["w"], g["d"])


def _oracle(g):
    return coracle.fwd(g["dx"], g["xs"], g["xr"], g["dz"], g["zs"], g["zr"], g["v"], g["dt"], g["nt"], g["w"],
                       g["d"])["datau"]


def test_wait_that_runs_out_returns_timeout_and_the_context_recovers():
    g = _geometry()
    with mnad.Context(0, kernel="tma") as ctx:
        ctx.set_wait_limit(1)
        with pytest.raises(_lib.MnadError) as e:
            _fwd(ctx, g)
        assert e.value.code == _lib.E_TIMEOUT
        assert e.value.identifier == "mnad:timeout"
        assert ctx.status() == 0                   # the call read and cleared the flag itself
        ctx.set_wait_limit(0)
        got = _fwd(ctx, g)
        err = rel(got, _oracle(g))
        print(f"shot after the timed-out call: gather rel-L2 {err:.2e}")
        assert err <= TOL_GATHER


@pytest.mark.parametrize("kernel", ["direct", "tma"])
def test_unstable_time_step_returns_numeric(kernel):
    bad = _geometry(nz=96, nx=128, d=12, nt=200, cfl=1.0)
    good = _geometry(nz=96, nx=128, d=12, nt=200)
    with mnad.Context(0, kernel=kernel) as ctx:
        with pytest.raises(_lib.MnadError) as e:
            _fwd(ctx, bad)
        assert e.value.code == _lib.E_NUMERIC
        assert e.value.identifier == "mnad:numeric"
        assert rel(_fwd(ctx, good), _oracle(good)) <= TOL_GATHER


def _job(g, kind="model"):
    return mnad.ShotJob(kind, g["v"], g["dx"], g["dz"], g["dt"], g["nt"], g["d"], g["zs"], g["xs"], g["zr"],
                        g["xr"], g["w"], vs=g["v"] if kind == "rtm" else None, T=4 if kind == "rtm" else 0)


def test_batched_jobs_return_numeric():
    bad = _geometry(nz=96, nx=128, d=12, nt=200, cfl=1.0)
    good = _geometry(nz=96, nx=128, d=12, nt=200)
    with mnad.Context(0) as ctx:
        with pytest.raises(_lib.MnadError) as e:
            ctx.run_jobs([_job(good), _job(bad)])
        assert e.value.code == _lib.E_NUMERIC
        j = _job(good)
        ctx.run_jobs([j])
        assert rel(j.data, _oracle(good)) <= TOL_GATHER


def test_server_fails_only_the_unstable_job():
    bad = _geometry(nz=96, nx=128, d=12, nt=200, cfl=1.0)
    good = _geometry(nz=96, nx=128, d=12, nt=200)
    with mnad.Server(0, chunk_steps=32) as srv:
        tb = srv.submit(_job(bad))
        tg = srv.submit(_job(good))
        with pytest.raises(_lib.MnadError) as e:
            srv.wait(tb, timeout_s=600)
        assert e.value.code == _lib.E_NUMERIC
        j = srv.wait(tg, timeout_s=600)
        assert rel(j.data, _oracle(good)) <= TOL_GATHER
        st = srv.stats()
        assert st["failed"] == 1 and st["completed"] == 1
