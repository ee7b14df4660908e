"""The MATLAB MEX gateway (mnad-modeling-rtm_gb300/matlab/mnad_mex.c), built
against a fake MATLAB C Matrix API (tests/mex) and called as MATLAB calls
it.  CPU tests cover argument marshalling and error identifiers; the GPU
tests run the reference's own call sequence for one shot (forward, forward
with indx = 1, adjoint of the scattered data) through the gateway and check
the results against the golden FP64 fixtures."""
import os

import numpy as np
import pytest

from mex import fakemex

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL_GATHER, TOL_IMAGE = 1e-5, 1e-4


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_gateway_builds_against_the_header():
    assert os.path.exists(fakemex.build())


def test_gateway_rejects_bad_calls_with_mnad_identifiers():
    with pytest.raises(fakemex.MexError) as e:
        fakemex.call("nonsense")
    assert e.value.identifier == "mnad:arg"
    with pytest.raises(fakemex.MexError) as e:
        fakemex.call("fwd", 10.0, 5.0)              # too few arguments
    assert e.value.identifier == "mnad:arg"
    with pytest.raises(fakemex.MexError) as e:
        fakemex.call("adj", *([1.0] * 7), "text", 0.0, 1.0)
    assert e.value.identifier == "mnad:arg"


def _golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.mark.gpu
def test_reference_call_sequence_through_the_gateway():
    g = _golden("golden_rtm_small.npz")
    dx, dz, dt, nt, d = float(g["dx"]), float(g["dz"]), float(g["dt"]), int(g["nt"]), int(g["d"])
    xs, zs = float(g["xs"]), float(g["zs"])
    xr, zr = g["xr"], g["zr"]
    ss = 7
    # data = fwd_PDE_exact_MNAD(dx,xs,xr,dz,zs,zr,v,dt,nt,w,d_pml,ss,...)           (main_Acoustic_RTM.m:224)
    data = fakemex.call("fwd", dx, xs, xr, dz, zs, zr, g["v"], dt, nt, g["w"], d, ss, 0.0)
    # datas = fwd_PDE_exact_MNAD(dx,xs,xr,dz,zs,zr,vs,dt,nt,w,d_pml,ss,...,1)       (:248)
    datas = fakemex.call("fwd", dx, xs, xr, dz, zs, zr, g["vs"], dt, nt, g["w"], d, ss, 1.0)
    assert isinstance(data, list) and data[0].shape == (nt, xr.size)
    assert fakemex.call("has", ss)[0, 0] == 1.0
    UU, illum = fakemex.call("export", ss, nlhs=2)
    assert rel(UU, g["UU"]) <= 1e-5
    # Im = Born_adj_MNAD(dx,dz,nt,dt,vs,xr,zr,data-datas,d_pml,ss,...)                 (:252)
    im = fakemex.call("adj", dx, dz, nt, dt, g["vs"], xr, zr, data[0] - datas[0], d, ss)
    assert im.shape == (UU.shape[0], 1)
    assert rel(data[0] - datas[0], g["data"]) <= TOL_IMAGE
    assert rel(im, g["Im"]) <= TOL_IMAGE
    # the file hand-off: export, release, import into a fresh slot, adjoint again (data as a cell)
    fakemex.call("release", ss)
    assert fakemex.call("has", ss)[0, 0] == 0.0
    fakemex.call("import", ss + 1, g["vs"].shape[0], g["vs"].shape[1], d, nt, int(g["T"]), UU, illum)
    im2 = fakemex.call("adj", dx, dz, nt, dt, g["vs"], xr, zr, [data[0] - datas[0]], d, ss + 1)
    assert rel(im2, im) <= 1e-6
    with pytest.raises(fakemex.MexError) as e:
        fakemex.call("adj", dx, dz, nt, dt, g["vs"], xr, zr, data[0], d, 999)
    assert e.value.identifier == "mnad:notfound"
    fakemex.call("reset")


@pytest.mark.gpu
def test_noalloc_through_the_gateway():
    g = _golden("golden_fwd_small.npz")
    out = fakemex.call("noalloc", float(g["dx"]), float(g["xs"]), g["xr"], float(g["dz"]), float(g["zs"]), g["zr"],
                       g["v"], float(g["dt"]), int(g["nt"]), g["w"], int(g["d"]))
    assert rel(out[0], g["datau"]) <= TOL_GATHER


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a GPU")
def test_gateway_without_a_gpu_raises_mnad_cuda():
    g = _golden("golden_fwd_small.npz")
    with pytest.raises(fakemex.MexError) as e:
        fakemex.call("fwd", float(g["dx"]), float(g["xs"]), g["xr"], float(g["dz"]), float(g["zs"]), g["zr"],
                     g["v"], float(g["dt"]), int(g["nt"]), g["w"], int(g["d"]), 1.0, 0.0)
    assert e.value.identifier == "mnad:cuda"
