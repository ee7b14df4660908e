"""Sensitivity of the bottom-strip edge case, shown on the CPU.

The GPU test ``test_bottom_strip_when_nz_minus_d_is_not_a_multiple_of_4``
compares the step kernels with the FP64 oracle at rel-L2 1e-5.  Here the
mistake it guards against is planted in the oracle instead: the bottom
strip's damping distance counted from the storage row (nz - d rounded down
to 4) rather than from the strip edge nz - d, i.e. the profile x_b of
``SRC/MNAD/C_cof.m:35-65`` shifted by the rounding.  On the test's own
geometry the planted oracle's gathers differ from the correct ones by far
more than the GPU test's tolerance, so the GPU test would catch the mistake;
where nz - d is a multiple of 4 the two agree exactly."""
import numpy as np
import pytest

from mnad import workflow
from oracle import mnad_oracle as P


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


def _shifted_c_cof(original):
    def c_cof(R, d_pml, dx, dz, dt, nx, nz, v):
        out = original(R, d_pml, dx, dz, dt, nx, nz, v)
        d = d_pml
        shift = (nz - d) - ((nz - d) & ~3)
        if shift == 0:
            return out
        # the bottom side with X = (row - zb0 + 1) dz instead of (row - (nz - d) + 1) dz
        D = d * dz
        K = (3 * np.log(1 / R)) / (2 * D**3)
        rows = np.arange(nz - d, nz)
        Xb = (rows - (nz - d) + 1 + shift) * dz
        sig0 = K * np.asarray(v, dtype=np.float64)[rows, :]
        sig = sig0 * (Xb[:, None] ** 2)
        dsig = 2 * sig0 * Xb[:, None]
        den = 1 + sig * (dt / 2)
        for name, val in (("c1zb", (1 - sig * (dt / 2)) / den), ("c2zb", (dsig * dt) / den),
                          ("c3zb", (sig * dt) / den)):
            a = np.array(out[name], dtype=np.float64, copy=True)
            a[rows, :] = val
            out[name] = a
        return out
    return c_cof


@pytest.mark.parametrize("nz", [52, 53, 54, 55])
def test_planted_bottom_strip_shift_exceeds_the_gpu_tolerance(monkeypatch, nz):
    rng = np.random.default_rng(5)
    v = 1900.0 + 500.0 * rng.random((nz, 60))
    d, nt = 8, 220
    w = workflow.ricker(30.0, 1e-3, nt)
    xr = np.array([10, 20, 30, 40, 50, 30, 30], dtype=float)
    zr = np.array([nz - 9, nz - 7, nz - 5, nz - 3, nz - 1, nz, nz - 10], dtype=float)
    args = (10.0, 30, xr, 10.0, nz - d - 2, zr, v, 1e-3, nt, w, d)
    good = P.fwd_pde_exact_mnad(*args)["datau"]
    monkeypatch.setattr(P, "c_cof", _shifted_c_cof(P.c_cof))
    bad = P.fwd_pde_exact_mnad(*args)["datau"]
    e = rel(bad, good)
    if (nz - d) % 4 == 0:
        assert e == 0.0
    else:
        assert e > 100 * 1e-5, e
