"""Edge cases of the hot path against the FP64 C oracle: a source inside the
CPML strip next to a corner (the strip's pre-injection correction),
receivers in the strip, a bottom strip whose rows are off the 4-row storage
grid, a snapshot at every step (T = 1, so the d2u of
tt = 1 and tt = 2 take the reference's special forms), the shortest records
(nt = 1, 2) and a shot without receivers."""
import numpy as np
import pytest

import mnad
from mnad import workflow
from oracle import coracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def ctx():
    from mnad import build
    build.build()
    with mnad.Context(0) as c:
        yield c


def _model(nz=52, nx=60, seed=5):
    rng = np.random.default_rng(seed)
    return 1900.0 + 500.0 * rng.random((nz, nx))


@pytest.mark.parametrize("kernel", ["direct", "tma"])
@pytest.mark.parametrize("zs,xs", [(3, 3), (2, 57), (50, 30), (26, 2)])
def test_source_in_the_cpml_strip(ctx, kernel, zs, xs):
    v = _model()
    d, nt = 8, 150
    w = workflow.ricker(30.0, 1e-3, nt)
    xr = np.array([1, 2, 5, 9, 30, 52, 59, 60, 30], dtype=float)     # strip, interior, duplicate
    zr = np.array([1, 4, 9, 10, 12, 45, 51, 52, 12], dtype=float)
    ctx.set_options(kernel=kernel)
    try:
        out = ctx.fwd(10.0, xs, xr, 10.0, zs, zr, v, 1e-3, nt, w, d)
    finally:
        ctx.set_options(kernel="auto")
    ref = coracle.fwd(10.0, xs, xr, 10.0, zs, zr, v, 1e-3, nt, w, d)["datau"]
    assert rel(out, ref) <= 1e-5
    assert ctx.status() == 0


@pytest.mark.parametrize("kernel", ["direct", "tma"])
@pytest.mark.parametrize("nz", [53, 54, 55])
def test_bottom_strip_when_nz_minus_d_is_not_a_multiple_of_4(ctx, kernel, nz):
    """The bottom z strip's memory variables are stored from row nz - d
    rounded down to 4; the damping profile still starts at row nz - d.  A
    source just above the strip and receivers inside it see the difference
    within a few wave periods."""
    v = _model(nz=nz)
    d, nt = 8, 220
    w = workflow.ricker(30.0, 1e-3, nt)
    xr = np.array([10, 20, 30, 40, 50, 30, 30], dtype=float)
    zr = np.array([nz - 9, nz - 7, nz - 5, nz - 3, nz - 1, nz, nz - 10], dtype=float)
    ctx.set_options(kernel=kernel)
    try:
        out = ctx.fwd(10.0, 30, xr, 10.0, nz - d - 2, zr, v, 1e-3, nt, w, d)
    finally:
        ctx.set_options(kernel="auto")
    ref = coracle.fwd(10.0, 30, xr, 10.0, nz - d - 2, zr, v, 1e-3, nt, w, d)["datau"]
    assert rel(out, ref) <= 1e-5
    assert ctx.status() == 0


@pytest.mark.parametrize("kernel", ["direct", "tma"])
def test_snapshot_every_step_including_the_first_two(ctx, kernel):
    v = _model()
    d, nt, T = 8, 40, 1
    w = workflow.ricker(30.0, 1e-3, nt)
    xr = np.arange(d + 1, 60 - d + 1, dtype=float)
    zr = np.full(xr.size, d + 2.0)
    ctx.set_options(kernel=kernel, T=T)
    try:
        ctx.fwd(10.0, 30, xr, 10.0, d + 2, zr, v, 1e-3, nt, w, d, ss=4, indx=1)
        UU, illum = ctx.wavefield_export(4)
    finally:
        ctx.set_options(kernel="auto", T=0)
    ctx.wavefield_release(4)
    from oracle import mnad_oracle as P
    nf = P.snapshot_nf(v, nt)
    ref = coracle.fwd(10.0, 30, xr, 10.0, d + 2, zr, v, 1e-3, nt, w, d, indx=1, T=T, ncols=max(2 * nf + 1, nt))
    assert UU.shape == ref["UU"].shape
    for c in (0, 1, 2, nt - 1):                   # tt = 1, 2, 3 and the last step
        assert rel(UU[:, c], ref["UU"][:, c]) <= 1e-4, c
    assert rel(illum, ref["illum"]) <= 1e-4


@pytest.mark.parametrize("nt", [1, 2])
def test_shortest_records(ctx, nt):
    v = _model()
    w = workflow.ricker(30.0, 1e-3, 8)[:nt] + 0.5
    xr = np.array([30.0, 31.0])
    zr = np.array([26.0, 27.0])
    out = ctx.fwd(10.0, 30, xr, 10.0, 26, zr, v, 1e-3, nt, w, 8)
    ref = coracle.fwd(10.0, 30, xr, 10.0, 26, zr, v, 1e-3, nt, w, 8)["datau"]
    assert out.shape == (nt, 2)
    assert rel(out, ref) <= 1e-6


def test_shot_without_receivers_runs(ctx):
    v = _model()
    w = workflow.ricker(30.0, 1e-3, 50)
    out = ctx.fwd(10.0, 30, np.zeros(0), 10.0, 26, np.zeros(0), v, 1e-3, 50, w, 8)
    assert out.shape == (50, 0)
    assert ctx.status() == 0
