"""GPU results against fixtures produced by the reference's own MATLAB
sources (run under oracle/mlite.py; see tests/golden/make_reference_golden.py):
three RTM record lengths covering the shifted, aligned and grown snapshot
pairing of Born_adj_MNAD.m, and the constant-velocity 201 x 201 shot's gather."""
import os

import numpy as np
import pytest

import mnad

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL_GATHER, TOL_IMAGE = 1e-5, 1e-4


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def ctx():
    from mnad import build
    build.build()
    with mnad.Context(0) as c:
        yield c


@pytest.mark.parametrize("name", ["a", "b", "c"])
def test_rtm_shot_matches_the_reference_run(ctx, name):
    g = np.load(os.path.join(GOLDEN, "golden_ref_rtm.npz"))
    c = {k[2:]: g[k] for k in g.files if k.startswith(name + "_")}
    nt, d, dt, dx, dz = int(c["nt"]), int(c["d"]), float(c["dt"]), float(c["dx"]), float(c["dz"])
    a = (dx, float(c["xs"]), c["xr"], dz, float(c["zs"]), c["zr"])
    data = ctx.fwd(*a, c["v"], dt, nt, c["w"], d, ss=9)
    datas = ctx.fwd(*a, c["vs"], dt, nt, c["w"], d, ss=9, indx=1)
    UU, illum = ctx.wavefield_export(9)
    im = ctx.adj(dx, dz, nt, dt, c["vs"], c["xr"], c["zr"], data - datas, d, ss=9)
    ctx.wavefield_release(9)
    errs = dict(gather=rel(data, c["data"]), gather_bg=rel(datas, c["datas"]), UU=rel(UU, c["UU"]),
                illum=rel(illum, c["illum"]), image=rel(im, c["Im"]))
    print(name, nt, {k: f"{v:.2e}" for k, v in errs.items()})
    assert UU.shape == c["UU"].shape
    assert errs["gather"] <= TOL_GATHER and errs["gather_bg"] <= TOL_GATHER
    assert errs["UU"] <= TOL_IMAGE and errs["illum"] <= TOL_IMAGE
    assert errs["image"] <= TOL_IMAGE


def test_constant_velocity_gather_matches_the_reference_run(ctx):
    g = np.load(os.path.join(GOLDEN, "golden_ref_constant_velocity.npz"))
    nz, nx, nt, d = int(g["nz"]), int(g["nx"]), int(g["nt"]), int(g["d"])
    dt, dx, fc = float(g["dt"]), float(g["dx"]), float(g["fc"])
    t = np.arange(nt) * dt
    tau = np.pi * (t - 1.1 / fc) * fc
    w = (1 - 2 * tau ** 2) * np.exp(-tau ** 2)
    xr = np.arange(1, nx + 1, dtype=np.float64)
    zr = np.full(xr.size, float(g["zr"]))
    out = ctx.fwd(dx, float(g["xs"]), xr, dx, float(g["zs"]), zr, np.full((nz, nx), float(g["v0"])), dt, nt, w, d)
    e = rel(out, g["data"])
    print(f"constant-velocity gather vs reference run: {e:.2e}")
    assert e <= TOL_GATHER
