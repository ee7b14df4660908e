"""Full-size parity of the benchmark configurations against the FP64 C
oracle: the layered single-shot RTM (381 x 681 padded, 3 s, T = 4), one
shot of the 64-shot random-field survey (481 x 1281 padded, 4 s, snapshot
interval by the reference formula) with FP32 and BF16 snapshots, and one
checkpointed shot on the faulted-salt survey's 1281 x 4081 grid (1 s) with FP32
and FP16 checkpoints; at that survey's full 6 s the checkpointed runs are
checked against the stored-snapshot run.  Each error is printed so the run log
states it for every gather, snapshot set and image."""
import numpy as np
import pytest

import mnad
from mnad import workflow
from oracle import coracle
from oracle import mnad_oracle as P

pytestmark = pytest.mark.gpu
TOL_GATHER, TOL_IMAGE, TOL_BF16, TOL_F16 = 1e-5, 1e-4, 1e-2, 2e-3


def rel(a, b):
    a, b = np.ravel(np.asarray(a), order="F"), np.ravel(np.asarray(b), order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def ctx():
    from mnad import build
    build.build()
    with mnad.Context(0) as c:
        yield c


def _oracle_rtm(sv, sh, T):
    nf = P.snapshot_nf(sv.vs, sv.nt)
    T = T or P.snapshot_plan(sv.vs, sv.nt)[1]
    ncols = max(2 * nf + 1, sv.nt // T)
    a = (sv.dx, sh.xs, sh.xr, sv.dz, sh.zs, sh.zr)
    data = coracle.fwd(*a, sv.v, sv.dt, sv.nt, sv.w, sv.d_pml)["datau"]
    bg = coracle.fwd(*a, sv.vs, sv.dt, sv.nt, sv.w, sv.d_pml, indx=1, T=T, ncols=ncols)
    im = coracle.adj(sv.dx, sv.dz, sv.nt, sv.dt, sv.vs, sh.xr, sh.zr, data - bg["datau"], sv.d_pml, bg["UU"], T)
    return data, bg, im, T


def _gpu_rtm(ctx, sv, sh, codec):
    ctx.set_options(snapshot_codec=codec, T=sv.T)
    try:
        a = (sv.dx, sh.xs, sh.xr, sv.dz, sh.zs, sh.zr)
        data = ctx.fwd(*a, sv.v, sv.dt, sv.nt, sv.w, sv.d_pml, ss=1)
        datas = ctx.fwd(*a, sv.vs, sv.dt, sv.nt, sv.w, sv.d_pml, ss=1, indx=1)
        UU, illum = ctx.wavefield_export(1)
        im = ctx.adj(sv.dx, sv.dz, sv.nt, sv.dt, sv.vs, sh.xr, sh.zr, data - datas, sv.d_pml, ss=1)
        ctx.wavefield_release(1)
    finally:
        ctx.set_options(snapshot_codec="f32", T=0)
    return data, datas, UU, illum, im


def _check(name, ctx, sv, shot, codecs, oracle=None):
    data, bg, im_ref, T = oracle or _oracle_rtm(sv, shot, sv.T)
    for codec in codecs:
        d, ds, UU, illum, im = _gpu_rtm(ctx, sv, shot, codec)
        errs = dict(gather=rel(d, data), gather_bg=rel(ds, bg["datau"]), snapshots=rel(UU, bg["UU"]),
                    illum=rel(illum, bg["illum"]), image=rel(im, im_ref))
        print(f"{name} T={T} {codec}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
        assert errs["gather"] <= TOL_GATHER and errs["gather_bg"] <= TOL_GATHER
        assert errs["illum"] <= TOL_IMAGE
        assert errs["image"] <= (TOL_IMAGE if codec == "f32" else TOL_BF16)


@pytest.mark.parametrize("kernel", ["direct", "tma"])
def test_layered_single_shot_full_size(ctx, kernel):
    """381 - 40 is not a multiple of 4: the bottom CPML strip's storage rows
    start one row above the strip, which the damping profile must not see."""
    sv = workflow.layered_anomaly_shot()
    ctx.set_options(kernel=kernel)
    try:
        _check(f"layered 381x681 {kernel}", ctx, sv, sv.shots[0], ("f32", "bf16"))
    finally:
        ctx.set_options(kernel="auto")


@pytest.fixture(scope="module")
def random_field_shot32():
    """The random-field survey with the FP64 oracle of shot 32 (about 45 s of CPU)."""
    sv = workflow.random_field_survey(nshots=64)
    data, bg, im_ref, T = _oracle_rtm(sv, sv.shots[32], sv.T)
    return sv, dict(scattered=data - bg["datau"], illum=bg["illum"], image=im_ref, T=T,
                    raw=(data, bg, im_ref, T))


def test_random_field_shot_full_size(ctx, random_field_shot32):
    sv, ref = random_field_shot32
    _check("random field 481x1281 shot 32", ctx, sv, sv.shots[32], ("f32", "bf16"), oracle=ref["raw"])


@pytest.mark.parametrize("codec", ["bf16", "f32"])
def test_random_field_batched_tma_plan_against_the_oracle(random_field_shot32, codec):
    """The benchmarked path at its size: shots 30-33 of the random-field survey
    (481 x 1281 padded, 4 s) as one batched plan on the persistent TMA kernel
    (8 forwards in one launch per step, then 4 adjoints), scattered data
    formed on the device, BF16 (the benchmark's codec) and FP32 snapshots.
    Shot 32's scattered gather, illumination and image against the oracle."""
    sv, ref = random_field_shot32
    shots = sv.shots[30:34]
    jobs = workflow.shot_jobs(sv, "rtm", shots=shots, keep_data=True)
    with mnad.Context(0, kernel="tma", snapshot_codec=codec) as c:
        plan = c.plan(jobs)
        plan.run()
        plan.download()
        plan.close()
    j = jobs[2]
    errs = dict(scattered=rel(j.data, ref["scattered"]), illum=rel(j.illum, ref["illum"]),
                image=rel(j.image, ref["image"]))
    print(f"random field batched TMA plan, shot 32, T={ref['T']}, {codec} snapshots: " +
          ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert errs["scattered"] <= 10 * TOL_GATHER        # a difference of two gathers
    assert errs["illum"] <= TOL_IMAGE
    assert errs["image"] <= (TOL_IMAGE if codec == "f32" else TOL_BF16)


def _faulted_plan(sv, stack=False, **opts):
    jobs = workflow.shot_jobs(sv, "rtm", keep_data=True)
    with mnad.Context(0, **opts) as c:
        plan = c.plan(jobs)
        plan.run()
        plan.download()
        stacks = plan.stack() if stack else None
        assert c.status() == 0
        plan.close()
    return (jobs, stacks) if stack else jobs[0]


def test_faulted_salt_checkpointed_stack_against_the_oracle():
    """The faulted-salt survey's full 1281 x 4081 grid, shots 219-222 of 256
    (222's first reflector is the shallowest of the line, 600 m), cut to 1 s
    so that the FP64 oracle's propagations take about a minute per shot (T = 9
    by the reference formula).  One plan of the 4 shots; the adjoint runs in
    segments from checkpoints every 360 steps, FP32 and FP16 codecs.  Shot
    222's outputs and the FP64 stacks formed on the device
    (main_Acoustic_RTM.m:237-262) against the oracle's.  A 16-shot version
    spread over the line is tests/faulted_salt_subset.py."""
    sv = workflow.faulted_salt_survey(nshots=256, nt=1000, first=219, count=4)
    im_sum = il_sum = 0.0
    for k, sh in enumerate(sv.shots):
        data, bg, im_ref, T = _oracle_rtm(sv, sh, sv.T)
        im_sum = im_sum + im_ref.reshape(bg["illum"].shape, order="F")     # Nint vector -> image region
        il_sum = il_sum + bg["illum"]
        if k == 3:
            ref222 = dict(scattered=data - bg["datau"], illum=bg["illum"], image=im_ref)
    mask = il_sum > 1e-6 * il_sum.max()
    for codec, tol in (("f32", TOL_IMAGE), ("f16", TOL_F16)):
        jobs, (im, il, img) = _faulted_plan(sv, stack=True, checkpoint_every=360, checkpoint_codec=codec)
        j = jobs[3]
        errs = dict(scattered=rel(j.data, ref222["scattered"]), illum=rel(j.illum, ref222["illum"]),
                    image=rel(j.image, ref222["image"]), image_sum=rel(im, im_sum), illum_sum=rel(il, il_sum),
                    img_rtm=rel(img[mask], im_sum[mask] / il_sum[mask]))
        print(f"faulted salt shots 219-222 (222 alone, then the stack), nt 1000, T={T}, {codec} checkpoints: " +
              ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
        assert errs["scattered"] <= 10 * TOL_GATHER
        assert errs["illum"] <= TOL_IMAGE and errs["illum_sum"] <= TOL_IMAGE
        assert errs["image"] <= tol and errs["image_sum"] <= tol and errs["img_rtm"] <= tol


def test_faulted_salt_full_length_checkpoints_match_stored_snapshots():
    """One faulted-salt shot at its full 6 s: FP32 checkpoints replay the stored-
    snapshot run bitwise (image, illumination, scattered data); FP16
    checkpoints stay within the FP16 bar of it."""
    sv = workflow.faulted_salt_survey(nshots=256, first=128, count=1)
    stored = _faulted_plan(sv)
    ck32 = _faulted_plan(sv, checkpoint_every=360)
    ck16 = _faulted_plan(sv, checkpoint_every=360, checkpoint_codec="f16")
    assert np.linalg.norm(stored.image) > 0
    assert np.array_equal(ck32.image, stored.image)
    assert np.array_equal(ck32.illum, stored.illum)
    assert np.array_equal(ck32.data, stored.data)
    e16 = rel(ck16.image, stored.image)
    print(f"faulted salt shot 128, 6 s: FP16 checkpoints vs stored FP32 snapshots, image {e16:.2e}")
    assert e16 <= TOL_F16
