"""Pins the FP64 oracles to the reference code itself.

tests/golden/golden_ref_*.npz were produced by running the reference's own
SRC/MNAD/*.m and SRC/migration/Born_adj_MNAD.m under the MATLAB-subset
interpreter oracle/mlite.py (tests/golden/make_reference_golden.py).  Both
oracles -- the SciPy literal restatement and the C matrix-free one -- must
reproduce every gather, snapshot matrix, illumination and image of those
runs to FP64 rounding.  The interpreter's own semantics are checked on small
MATLAB snippets."""
import os

import numpy as np
import pytest

from oracle import coracle, mlite
from oracle import mnad_oracle as P

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-12


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def ref():
    return np.load(os.path.join(GOLDEN, "golden_ref_rtm.npz"))


def _case(g, n):
    return {k[2:]: g[k] for k in g.files if k.startswith(n + "_")}


@pytest.mark.parametrize("name", ["a", "b", "c"])
def test_c_oracle_reproduces_the_reference_rtm_shot(ref, name):
    c = _case(ref, name)
    nt, d, dt, dx, dz = int(c["nt"]), int(c["d"]), float(c["dt"]), float(c["dx"]), float(c["dz"])
    zs, xs = int(c["zs"]), int(c["xs"])
    nf, T = P.snapshot_plan(c["vs"], nt)
    ncols = max(2 * nf + 1, nt // T)
    assert c["UU"].shape[1] == ncols
    data = coracle.fwd(dx, xs, c["xr"], dz, zs, c["zr"], c["v"], dt, nt, c["w"], d)["datau"]
    bg = coracle.fwd(dx, xs, c["xr"], dz, zs, c["zr"], c["vs"], dt, nt, c["w"], d, indx=1, T=T, ncols=ncols)
    im = coracle.adj(dx, dz, nt, dt, c["vs"], c["xr"], c["zr"], data - bg["datau"], d, bg["UU"], T)
    assert rel(data, c["data"]) <= TOL
    assert rel(bg["datau"], c["datas"]) <= TOL
    assert rel(bg["UU"], c["UU"]) <= TOL
    assert rel(bg["illum"], c["illum"]) <= TOL
    assert rel(im, c["Im"]) <= TOL


def test_scipy_oracle_reproduces_the_reference_rtm_shot(ref):
    c = _case(ref, "a")
    nt, d, dt, dx, dz = int(c["nt"]), int(c["d"]), float(c["dt"]), float(c["dx"]), float(c["dz"])
    zs, xs = int(c["zs"]), int(c["xs"])
    data = P.fwd_pde_exact_mnad(dx, xs, c["xr"], dz, zs, c["zr"], c["v"], dt, nt, c["w"], d)["datau"]
    bg = P.fwd_pde_exact_mnad(dx, xs, c["xr"], dz, zs, c["zr"], c["vs"], dt, nt, c["w"], d, indx=1)
    im = P.born_adj_mnad(dx, dz, nt, dt, c["vs"], c["xr"], c["zr"], data - bg["datau"], d, bg["UU"])
    assert rel(data, c["data"]) <= TOL
    assert rel(bg["UU"], c["UU"]) <= TOL
    assert rel(im, c["Im"]) <= TOL


def test_c_oracle_reproduces_the_reference_constant_velocity_gather():
    g = np.load(os.path.join(GOLDEN, "golden_ref_constant_velocity.npz"))
    nz, nt, d = int(g["nz"]), int(g["nt"]), int(g["d"])
    v = np.full((nz, int(g["nx"])), float(g["v0"]))
    t = np.arange(nt) * float(g["dt"])
    fc = float(g["fc"])
    tau = np.pi * (t - 1.1 / fc) * fc
    w = (1 - 2 * tau ** 2) * np.exp(-tau ** 2)
    xr = np.arange(1, int(g["nx"]) + 1)
    zr = np.full(xr.size, int(g["zr"]))
    out = coracle.fwd(float(g["dx"]), int(g["xs"]), xr, float(g["dx"]), int(g["zs"]), zr, v, float(g["dt"]), nt, w,
                      d)["datau"]
    assert rel(out, g["data"]) <= TOL


# ---- the interpreter's MATLAB semantics --------------------------------------

def _run(src, **inputs):
    it = mlite.Interpreter([])
    it.funcs.update(mlite.Parser(mlite.lex(src)).file())
    name = next(iter(it.funcs))
    return it.call(name, [np.atleast_2d(np.asarray(v, dtype=float)) for v in inputs.values()], 4)


def test_column_major_reshape_colon_and_end():
    src = """function [a,b,c,d] = f(x)
    a = reshape(1:6,2,3) ;
    b = a(:) ;
    c = a(end,2:end) ;
    d = [10:-2.5:5, zeros(1,2)] ;
    end"""
    a, b, c, d = _run(src, x=0)
    assert np.array_equal(a, np.array([[1, 3, 5], [2, 4, 6]]))
    assert np.array_equal(b.ravel(), np.arange(1, 7))
    assert np.array_equal(c, np.array([[4, 6]]))
    assert np.array_equal(d, np.array([[10, 7.5, 5, 0, 0]]))


def test_growth_sparse_cells_and_power_precedence():
    src = """function [a,b,c,d] = f(x)
    a = zeros(2,1) ;
    a(:,3) = [7;8] ;
    S = sparse([1;2;2],[1;1;2],[1;2;3],2,2) ;
    b = S*[1;10] ;
    q{1} = a ;
    c = q{1}(2,3) + -2^2 ;
    d = rem(7,3) == 1 && ~isempty(a) ;
    end"""
    a, b, c, d = _run(src, x=0)
    assert np.array_equal(a, np.array([[0, 0, 7], [0, 0, 8]]))
    assert np.array_equal(b.ravel(), np.array([1, 32]))
    assert c[0, 0] == 4.0
    assert bool(d[0, 0])


# ---- acquisition geometry and model smoothing (the drivers' preparation) -----

@pytest.mark.parametrize("kind", ["fixspread", "onesided", "splitspread", "obn"])
def test_acquisition_matches_the_reference(kind):
    from mnad import workflow
    g = np.load(os.path.join(GOLDEN, "golden_ref_prep.npz"))
    a = {k[4:]: float(g[k]) for k in g.files if k.startswith("acq_")}
    Source, Receiver = workflow.acquisi(g["V"], a["dx"], a["dz"], a["zsc"], a["zrc"], a["h_offset"], a["ds"],
                                        a["dr"], a["slag"], a["rlag"], kind)
    assert np.array_equal(Source, g[f"{kind}_Source"])
    assert [len(x) for x, _ in Receiver] == list(g[f"{kind}_nr"])
    assert np.array_equal(np.concatenate([x for x, _ in Receiver]), g[f"{kind}_xr"])
    assert np.array_equal(np.concatenate([z for _, z in Receiver]), g[f"{kind}_zr"])


def test_v_smooth_matches_the_reference():
    from mnad import workflow
    g = np.load(os.path.join(GOLDEN, "golden_ref_prep.npz"))
    assert rel(workflow.v_smooth(g["vsm_in"], 5, 3, 2), g["vsm_out"]) <= TOL


def test_driver_grid_and_time_rules():
    """main_Acoustic_RTM.m:70-90 on its own example model (1500 / 2500 m/s,
    fc = 15 Hz, 3 s): dx = floor(1500 / 112.5) = 13, dt = 0.8 * 0.65 *
    13.33 / 2500, nt = length(0:dt:3-dt)."""
    from mnad import drivers
    V = np.full((100, 200), 1500.0)
    V[69:, :] = 2500.0
    dx, dz, dt, nt = drivers.grid_and_time(V, 15.0, 3.0)
    assert (dx, dz) == (13.0, 13.0)
    assert dt == 0.8 * ((0.65 * (1500.0 / (2.5 * 45.0))) / 2500.0)
    assert nt == len(mlite.colon(0.0, dt, 3.0 - dt).ravel())
