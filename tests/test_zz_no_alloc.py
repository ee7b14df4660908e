"""GPU test of mnad_fwd_pde_exact_noalloc, the forward entry point that
allocates no device memory (for callers whose GPU memory is reserved by
their own allocator, or that forbid allocation after start-up).

It is called straight through the C ABI twice in a row.  Each shot record is
compared with the FP64 oracle's record of the same shot and with the
allocating entry point's record run on the persistent TMA kernel (the
no-allocation path runs the one-thread-per-point kernel), within the gather
tolerance of the parity tests; a repeat of the first call must give the same
record bit for bit.  The file is named so that pytest collects it after every
other test module.
"""
import ctypes as C

import numpy as np
import pytest

import mnad
from mnad import _lib, workflow
from oracle import coracle

pytestmark = pytest.mark.gpu
TOL_GATHER = 1e-5


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _shot(seed, nz=70, nx=96, d=12, nt=260):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[:, None]
    v = np.where(z < nz // 2, 1700.0, 2300.0) + 200.0 * rng.random((nz, nx))
    w = workflow.ricker(30.0, 1e-3, nt)
    xr = np.ascontiguousarray(np.arange(d + 1, nx - d + 1, dtype=np.float64))
    zr = np.ascontiguousarray(np.full(xr.size, d + 2, dtype=np.float64))
    return dict(v=np.asfortranarray(v), w=w, xr=xr, zr=zr, nz=nz, nx=nx, d=d, nt=nt, zs=float(d + 1),
                xs=float(nx // 2 + seed))


def _noalloc(s):
    L = _lib.lib()
    out = np.zeros((s["nt"], s["xr"].size), order="F")
    rc = L.mnad_fwd_pde_exact_noalloc(0, 10.0, s["xs"], _p(s["xr"]), s["xr"].size, 10.0, s["zs"], _p(s["zr"]),
                                      _p(s["v"]), s["nz"], s["nx"], 1e-3, s["nt"], _p(s["w"]), s["d"], _p(out))
    _lib.check(rc)
    return out


def test_noalloc_matches_the_oracle_and_the_allocating_entry_point_on_two_calls_in_a_row():
    from mnad import build
    build.build()
    shots = [_shot(1), _shot(2)]
    got = [_noalloc(s) for s in shots]           # two calls in a row share the scratch array
    with mnad.Context(0, kernel="tma") as ctx:
        for s, g in zip(shots, got):
            args = (10.0, s["xs"], s["xr"], 10.0, s["zs"], s["zr"], s["v"], 1e-3, s["nt"], s["w"], s["d"])
            ref = coracle.fwd(*args)["datau"]
            alloc = ctx.fwd(*args)
            assert np.all(np.isfinite(g))
            assert np.linalg.norm(g) > 0
            e_oracle, e_alloc = rel(g, ref), rel(g, alloc)
            print(f"no-allocation record: vs FP64 oracle {e_oracle:.2e}, vs allocating entry point {e_alloc:.2e}")
            assert e_oracle <= TOL_GATHER
            assert e_alloc <= TOL_GATHER
    # the second shot left nothing behind that changes a repeat of the first
    again = _noalloc(shots[0])
    assert np.array_equal(again, got[0])


def test_noalloc_reports_an_unstable_shot_as_numeric():
    s = _shot(4)
    s["v"] = np.full_like(s["v"], 1.0e4)         # v*dt/dx = 1: blows up to inf/NaN in FP32
    with pytest.raises(_lib.MnadError) as e:
        _noalloc(s)
    assert e.value.code == _lib.E_NUMERIC
    assert np.array_equal(_noalloc(_shot(1)), _noalloc(_shot(1)))


def test_noalloc_rejects_shots_beyond_its_scratch_size():
    s = _shot(3)
    big = np.full((1500, 1500), 2000.0, order="F")
    L = _lib.lib()
    out = np.zeros((10, s["xr"].size), order="F")
    rc = L.mnad_fwd_pde_exact_noalloc(0, 10.0, 700.0, _p(s["xr"]), s["xr"].size, 10.0, 700.0, _p(s["zr"]), _p(big),
                                      1500, 1500, 1e-3, 10, _p(s["w"]), 20, _p(out))
    assert rc == _lib.E_ARG
    assert b"working memory" in L.mnad_last_error()
