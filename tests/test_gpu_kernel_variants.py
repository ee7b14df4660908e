"""The variants of the persistent kernel: two steps per pass (temporal
blocking of depth 2, MNAD_KERNEL_TMA2) and 64 x 8 tiles (MNAD_KERNEL_TMA_NARROW).

Per point both run the arithmetic of the one-step 64 x 16 kernel, so their
outputs must equal that kernel's exactly, for every event the reference's time
loop has (SRC/MNAD/fwd_PDE_exact_MNAD.m:92-157, SRC/migration/Born_adj_MNAD.m:
85-136): CPML strips on all sides and in corners, a source inside a strip and
on tile edges, receivers on tile edges (the two-step kernel's adjoint injects
them in the ring a pass computes around its tile; the narrow kernel reads half
of a receiver bucket), snapshots on either sub-step (odd T), the tt = 1, 2
snapshot formulas, odd record lengths (the two-step kernel's last pass runs one
step), no CPML, several grids and record lengths in one plan.  One RTM shot per
variant is also checked against the FP64 oracle.
"""
import numpy as np
import pytest

import mnad
from mnad import workflow
from oracle import coracle
from oracle import mnad_oracle as P

pytestmark = pytest.mark.gpu
TOL_GATHER, TOL_IMAGE = 1e-5, 1e-4


@pytest.fixture(scope="module", autouse=True)
def built():
    from mnad import build
    build.build()


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def model(nz, nx, seed=0):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[:, None]
    v = np.where(z < nz // 3, 1600.0, np.where(z < 2 * nz // 3, 2100.0, 2700.0)) + 150.0 * rng.random((nz, nx))
    return np.asfortranarray(v)


def shot(nz=150, nx=100, d=12, nt=301, zs=None, xs=None, seed=0):
    """Receivers on tile edges (rows 63/64, columns 15/16/31/32) and inside
    the top strip; 1-based indices."""
    v = model(nz, nx, seed)
    xr = np.array([1, 2, 15, 16, 17, 32, 33, nx - 1, nx, 40, 41, 48, 49], dtype=float)
    zr = np.array([d + 2, 3, 64, 65, d + 2, 64, 65, d + 2, 10, 128, 129, 64, 1], dtype=float)
    keep = (xr <= nx) & (zr <= nz)          # receivers of the grid only
    xr, zr = xr[keep], zr[keep]
    return dict(v=v, vs=np.asfortranarray(v * 0.97 + 40.0), dx=10.0, dz=10.0, dt=1e-3, nt=nt, d=d,
                zs=float(zs if zs is not None else d // 2 + 1), xs=float(xs if xs is not None else 17),
                xr=xr, zr=zr, w=workflow.ricker(28.0, 1e-3, nt))


def fwd(kernel, s, indx=0, ss=1, codec="f32", T=0, ctx=None):
    own = ctx is None
    ctx = ctx or mnad.Context(0, kernel=kernel, snapshot_codec=codec, T=T)
    try:
        return ctx.fwd(s["dx"], s["xs"], s["xr"], s["dz"], s["zs"], s["zr"], s["v"], s["dt"], s["nt"], s["w"],
                       s["d"], ss=ss, indx=indx, record_vw=True)
    finally:
        if own:
            ctx.close()


VARIANTS = ["tma2", "tma_narrow"]


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("geom", [dict(), dict(nt=300), dict(zs=64, xs=16), dict(zs=1, xs=1), dict(zs=150, xs=100),
                                  dict(d=0), dict(nz=64, nx=16, d=6, nt=120, xs=9), dict(nz=200, nx=97, d=40),
                                  dict(xs=8), dict(xs=9)])
def test_forward_equals_the_one_step_kernel(geom, variant):
    s = shot(**geom)
    a = fwd("tma", s)
    b = fwd(variant, s)
    for x, y, name in zip(a, b, ("U", "V", "W")):
        assert np.linalg.norm(x) > 0
        assert np.array_equal(x, y), f"{name} traces differ ({geom}): rel {rel(y, x):.2e}"


def rtm(kernel, s, codec, T):
    with mnad.Context(0, kernel=kernel, snapshot_codec=codec, T=T) as ctx:
        d_true = fwd(None, s, ctx=ctx)[0]
        s_bg = dict(s, v=s["vs"])
        d_bg = fwd(None, s_bg, indx=1, ss=7, ctx=ctx)[0]
        UU, illum = ctx.wavefield_export(7)
        im = ctx.adj(s["dx"], s["dz"], s["nt"], s["dt"], s["vs"], s["xr"], s["zr"], d_true - d_bg, s["d"], ss=7)
        ctx.wavefield_release(7)
    return d_true, d_bg, UU, illum, im


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("codec,T", [("f32", 3), ("bf16", 4), ("f32", 1)])
def test_rtm_equals_the_one_step_kernel(codec, T, variant):
    """Snapshots and imaging on both sub-steps (odd T), at every step (T = 1:
    the tt = 1 and 2 formulas), and the adjoint's injection of receivers on
    tile edges and inside the top strip."""
    s = shot(nt=241)
    a = rtm("tma", s, codec, T)
    b = rtm(variant, s, codec, T)
    for x, y, name in zip(a, b, ("gather", "background gather", "UU", "illum", "image")):
        assert np.linalg.norm(x) > 0, name
        assert np.array_equal(x, y), f"{name} differs ({codec}, T={T}): rel {rel(y, x):.2e}"


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("nt", [1, 2, 3])
def test_shortest_records(nt, variant):
    s = shot(nt=nt)
    for x, y in zip(rtm("tma", s, "f32", 1), rtm(variant, s, "f32", 1)):
        assert np.array_equal(x, y)


def _jobs():
    out = []
    for k, (nz, nx, nt, kind) in enumerate([(150, 100, 200, "rtm"), (150, 100, 203, "model"), (96, 80, 157, "rtm"),
                                            (150, 100, 161, "rtm")]):
        s = shot(nz=nz, nx=nx, nt=nt, seed=k, xs=20 + 3 * k)
        out.append(mnad.ShotJob(kind, s["v"], s["dx"], s["dz"], s["dt"], s["nt"], s["d"], s["zs"], s["xs"], s["zr"],
                                s["xr"], s["w"], vs=s["vs"] if kind == "rtm" else None, T=3, keep_data=True))
    return out


def _plan(kernel):
    jobs = _jobs()
    with mnad.Context(0, kernel=kernel) as ctx:
        plan = ctx.plan(jobs)
        plan.run()
        plan.run()                         # a second run starts from zero state again
        plan.download()
        launches = plan.timing()["step_launches"]
        plan.close()
    return jobs, launches


@pytest.mark.parametrize("variant", VARIANTS)
def test_plan_of_mixed_grids_and_lengths_equals_the_one_step_kernel(variant):
    a, la = _plan("tma")
    b, lb = _plan(variant)
    if variant == "tma2":
        assert lb < la                      # the two-step kernel ran: one launch per two steps
    for ja, jb in zip(a, b):
        assert np.array_equal(ja.data, jb.data)
        if ja.kind == "rtm":
            assert np.linalg.norm(ja.image) > 0
            assert np.array_equal(ja.image, jb.image)
            assert np.array_equal(ja.illum, jb.illum)


@pytest.mark.parametrize("variant", VARIANTS)
def test_rtm_shot_against_the_oracle(variant):
    s = shot(nz=181, nx=241, d=20, nt=600, zs=21, xs=121)
    T = 4
    nf = P.snapshot_nf(s["vs"], s["nt"])
    ncols = max(2 * nf + 1, s["nt"] // T)
    a = (s["dx"], s["xs"], s["xr"], s["dz"], s["zs"], s["zr"])
    data = coracle.fwd(*a, s["v"], s["dt"], s["nt"], s["w"], s["d"])["datau"]
    bg = coracle.fwd(*a, s["vs"], s["dt"], s["nt"], s["w"], s["d"], indx=1, T=T, ncols=ncols)
    im = coracle.adj(s["dx"], s["dz"], s["nt"], s["dt"], s["vs"], s["xr"], s["zr"], data - bg["datau"], s["d"],
                     bg["UU"], T)
    g, gb, UU, illum, img = rtm(variant, s, "f32", T)
    errs = dict(gather=rel(g, data), gather_bg=rel(gb, bg["datau"]), illum=rel(illum, bg["illum"]),
                image=rel(img, im))
    print(f"{variant} kernel vs FP64 oracle: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert errs["gather"] <= TOL_GATHER and errs["gather_bg"] <= TOL_GATHER
    assert errs["illum"] <= TOL_IMAGE and errs["image"] <= TOL_IMAGE


def shot_layout(layout):
    """Receivers of shot() plus, for 'scan', receivers at several depths in
    columns 20 and 41 (a vertical line: several entries in one bucket column
    of the adjoint's injection scan), or, for 'duplicates', second receivers
    at the points (65, 16) and (65, 33) (two injections at one point, added in
    entry order)."""
    s = shot(nt=241)
    extra = {"scan": ([20, 20, 20, 41], [30, 70, 100, 90]), "duplicates": ([16, 33], [65, 65])}[layout]
    return dict(s, xr=np.concatenate([s["xr"], extra[0]]), zr=np.concatenate([s["zr"], extra[1]]))


@pytest.mark.parametrize("layout", ["scan", "duplicates"])
@pytest.mark.parametrize("variant", VARIANTS)
def test_adjoint_injection_forms_equal_the_one_step_kernel(layout, variant):
    s = shot_layout(layout)
    a = rtm("tma", s, "f32", 3)
    b = rtm(variant, s, "f32", 3)
    for x, y, name in zip(a, b, ("gather", "background gather", "UU", "illum", "image")):
        assert np.linalg.norm(x) > 0, name
        assert np.array_equal(x, y), f"{name} differs ({layout}): rel {rel(y, x):.2e}"


@pytest.mark.parametrize("layout", ["scan", "duplicates"])
@pytest.mark.parametrize("kernel", ["tma", "direct"])
def test_adjoint_injection_forms_against_the_oracle(layout, kernel):
    s = shot_layout(layout)
    T = 3
    nf = P.snapshot_nf(s["vs"], s["nt"])
    ncols = max(2 * nf + 1, s["nt"] // T)
    a = (s["dx"], s["xs"], s["xr"], s["dz"], s["zs"], s["zr"])
    data = coracle.fwd(*a, s["v"], s["dt"], s["nt"], s["w"], s["d"])["datau"]
    bg = coracle.fwd(*a, s["vs"], s["dt"], s["nt"], s["w"], s["d"], indx=1, T=T, ncols=ncols)
    im = coracle.adj(s["dx"], s["dz"], s["nt"], s["dt"], s["vs"], s["xr"], s["zr"], data - bg["datau"], s["d"],
                     bg["UU"], T)
    img = rtm(kernel, s, "f32", T)[4]
    err = rel(img, im)
    print(f"{layout} receivers, {kernel} kernel: image rel-L2 {err:.2e}")
    assert err <= TOL_IMAGE
