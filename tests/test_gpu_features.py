"""GPU tests of the image stack, the FP16 snapshot codec and the FP64 energy
diagnostic, against the FP64 oracle."""
import os

import numpy as np
import pytest

import mnad
from mnad import workflow
from oracle import coracle
from oracle import mnad_oracle as P

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def ctx():
    from mnad import build
    build.build()
    with mnad.Context(0) as c:
        yield c


@pytest.fixture(scope="module")
def rtm():
    return np.load(os.path.join(GOLDEN, "golden_rtm_small.npz"))


def _oracle_shot(g, xs):
    dx, dz, dt, nt, d = float(g["dx"]), float(g["dz"]), float(g["dt"]), int(g["nt"]), int(g["d"])
    T = int(g["T"])
    ncols = max(2 * P.snapshot_nf(g["vs"], nt) + 1, nt // T)
    data = coracle.fwd(dx, xs, g["xr"], dz, int(g["zs"]), g["zr"], g["v"], dt, nt, g["w"], d)["datau"]
    bg = coracle.fwd(dx, xs, g["xr"], dz, int(g["zs"]), g["zr"], g["vs"], dt, nt, g["w"], d, indx=1, T=T,
                     ncols=ncols)
    im = coracle.adj(dx, dz, nt, dt, g["vs"], g["xr"], g["zr"], data - bg["datau"], d, bg["UU"], T)
    return im, bg["illum"].ravel(order="F")


def test_image_stack_and_illumination_normalisation(ctx, rtm):
    """img_RTM = mean(mhh,3)./illum over shots (main_Acoustic_RTM.m:237-262)."""
    g = rtm
    shots = (14, 30, 46)
    jobs = [mnad.ShotJob(kind="rtm", v=g["v"], vs=g["vs"], dx=float(g["dx"]), dz=float(g["dz"]), dt=float(g["dt"]),
                         nt=int(g["nt"]), d_pml=int(g["d"]), zs=int(g["zs"]), xs=xs, zr=g["zr"], xr=g["xr"], w=g["w"])
            for xs in shots]
    plan = ctx.plan(jobs)
    plan.run()
    plan.download()
    im_sum, il_sum, img = plan.stack()
    plan.close()
    ref = [_oracle_shot(g, xs) for xs in shots]
    ref_im = sum(r[0] for r in ref)
    ref_il = sum(r[1] for r in ref)
    assert rel(im_sum, ref_im) <= 1e-4
    assert rel(il_sum, ref_il) <= 2e-4
    ref_img = (ref_im / len(shots)) / (ref_il / len(shots))
    assert rel(img, ref_img) <= 2e-4
    # the stack equals the sum of the per-job outputs
    assert np.allclose(im_sum, sum(j.image for j in jobs), rtol=1e-12, atol=0)


@pytest.mark.parametrize("codec,bound", [("f16", 2e-3), ("bf16", 1e-2)])
def test_scaled_snapshot_codecs(ctx, rtm, codec, bound):
    """FP16 uses a per-snapshot power-of-two scale; both codecs' image errors
    are measured against the FP64 oracle and bounded."""
    g = rtm
    dx, dz, dt, nt, d = float(g["dx"]), float(g["dz"]), float(g["dt"]), int(g["nt"]), int(g["d"])
    ctx.set_options(snapshot_codec=codec)
    try:
        ctx.fwd(dx, int(g["xs"]), g["xr"], dz, int(g["zs"]), g["zr"], g["vs"], dt, nt, g["w"], d, ss=21, indx=1)
        UU, illum = ctx.wavefield_export(21)
        im = ctx.adj(dx, dz, nt, dt, g["vs"], g["xr"], g["zr"], g["data"], d, ss=21)
    finally:
        ctx.set_options(snapshot_codec="f32")
    e_snap = rel(UU, g["UU"])
    e_img = rel(im, g["Im"])
    print(f"{codec}: snapshot rel-L2 {e_snap:.2e}, image rel-L2 {e_img:.2e}")
    assert e_snap <= bound
    assert e_img <= bound
    assert rel(illum, g["illum"].ravel(order="F")) <= 2e-4      # illumination stays FP64
    ctx.wavefield_release(21)


def test_f16_import_round_trip(ctx, rtm):
    g = rtm
    nz, nx = g["vs"].shape
    d, nt, T = int(g["d"]), int(g["nt"]), int(g["T"])
    ctx.set_options(snapshot_codec="f16")
    try:
        ctx.wavefield_import(22, nz, nx, d, nt, T, g["UU"], nsnap=nt // T)
        UU, _ = ctx.wavefield_export(22)
    finally:
        ctx.set_options(snapshot_codec="f32")
    assert rel(UU, g["UU"]) <= 1e-3
    ctx.wavefield_release(22)


def _energy_oracle(sv, sh, steps, every):
    """1/2 sum over the image region ((U(t+1)-U(t))^2/r + V^2 + W^2) dx dz."""
    keep = sorted(set([t for t in steps] + [t - 1 for t in steps if t > 1]))
    o = coracle.fwd(sv.dx, sh.xs, sh.xr, sv.dz, sh.zs, sh.zr, sv.v, sv.dt, max(steps), sv.w, sv.d_pml,
                    keep_steps=tuple(keep))
    d = sv.d_pml
    r = (sv.v * sv.dt) ** 2
    sl = (slice(d, sv.nz - d), slice(d, sv.nx - d))
    out = []
    for t in steps:
        un, vn, wn = o["fields"][t]
        uo = o["fields"][t - 1][0] if t > 1 else np.zeros_like(un)
        e = 0.5 * sv.dx * sv.dz * np.sum(((un - uo) ** 2 / r + vn ** 2 + wn ** 2)[sl])
        out.append(e)
    return np.array(out)


def test_energy_diagnostic_matches_oracle_and_is_absorbed(ctx):
    sv = workflow.constant_velocity_shot(nt=700)
    sh = sv.shots[0]
    every = 50
    ctx.set_options(energy_every=every)
    try:
        ctx.fwd(sv.dx, sh.xs, sh.xr, sv.dz, sh.zs, sh.zr, sv.v, sv.dt, sv.nt, sv.w, sv.d_pml)
        e = ctx.energy()
    finally:
        ctx.set_options(energy_every=0)
    assert e.size == sv.nt // every
    steps = [every * (m + 1) for m in range(e.size)]
    ref = _energy_oracle(sv, sh, [steps[2], steps[5], steps[-1]], every)
    got = e[[2, 5, e.size - 1]]
    assert np.allclose(got, ref, rtol=2e-4, atol=0), (got, ref)
    # physics: no growth beyond the source-driven peak, and the CPML absorbs
    # the wave once it has left the image region
    peak = e.max()
    assert np.all(np.isfinite(e))
    assert e[-1] < 0.05 * peak
