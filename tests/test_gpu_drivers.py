"""The reference's RTM driver (main_Acoustic_RTM.m) as mnad.drivers.acoustic_rtm
on its own example model, compared with the same workflow run shot by shot
on the FP64 C oracle, and the modeling driver's gathers likewise."""
import numpy as np
import pytest

from mnad import drivers, workflow
from oracle import coracle
from oracle import mnad_oracle as P

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _example_model():
    V = np.full((100, 200), 1500.0)        # main_Acoustic_RTM.m: V(70:end,:) = 2500
    V[69:, :] = 2500.0
    return V


@pytest.fixture(scope="module", autouse=True)
def _built():
    from mnad import build
    build.build()


def test_rtm_driver_matches_the_oracle_workflow():
    V = _example_model()
    # 1.5 s: reflections from the interface at 910 m are recorded; sources every 40 dx
    out = drivers.acoustic_rtm(V, fc=15.0, T_max=1.5, d_pml=40, acquisition=dict(ds=40))
    pf = out["profile"]
    d, nt, dt, dx, dz = pf["d_pml"], pf["nt"], pf["dt"], pf["dx"], pf["dz"]
    v = workflow.pad_model(V, d)
    vs = workflow.pad_model(workflow.v_smooth(V, 3, 3, 3), d)
    xs, zs, xr, zr = workflow.padded_indices(pf["Source"], pf["Receiver"], dx, dz, d)
    nf, T = P.snapshot_plan(vs, nt)
    ncols = max(2 * nf + 1, nt // T)
    im_sum = 0.0
    il_sum = 0.0
    for k in range(pf["ns"]):
        a = (dx, xs[k], xr[k], dz, zs[k], zr[k])
        data = coracle.fwd(*a, v, dt, nt, pf["w"], d)["datau"]
        bg = coracle.fwd(*a, vs, dt, nt, pf["w"], d, indx=1, T=T, ncols=ncols)
        im = coracle.adj(dx, dz, nt, dt, vs, xr[k], zr[k], data - bg["datau"], d, bg["UU"], T)
        im_sum = im_sum + im.reshape(V.shape, order="F")     # both already x T, as the reference's outputs
        il_sum = il_sum + bg["illum"]
    img = (im_sum / pf["ns"]) / (il_sum / pf["ns"])
    print(f"ns {pf['ns']}, nt {nt}, dx {dx}, dt {dt:.3e}: stack rel-L2 {rel(out['image_sum'], im_sum):.2e}, "
          f"img_RTM {rel(out['img_RTM'], img):.2e}")
    assert np.linalg.norm(im_sum) > 0
    assert rel(out["image_sum"], im_sum) <= 1e-4
    assert rel(out["illum"], il_sum / pf["ns"]) <= 1e-4
    assert rel(out["img_RTM"], img) <= 1e-4


def test_modeling_driver_gathers_match_the_oracle():
    V = _example_model()
    data, pf = drivers.acoustic_data(V, fc=10.0, T_max=0.4, d_pml=30, acquisition=dict(ds=40))
    d, nt, dt, dx, dz = pf["d_pml"], pf["nt"], pf["dt"], pf["dx"], pf["dz"]
    v = workflow.pad_model(V, d)
    xs, zs, xr, zr = workflow.padded_indices(pf["Source"], pf["Receiver"], dx, dz, d)
    for k in range(pf["ns"]):
        ref = coracle.fwd(dx, xs[k], xr[k], dz, zs[k], zr[k], v, dt, nt, pf["w"], d)["datau"]
        assert rel(data[k], ref) <= 1e-5
