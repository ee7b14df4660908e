"""Large-grid RTM against the FP64 oracle on a 16-shot subset.

The faulted-salt survey (1201 x 4001 at 12.5 m, 1281 x 4081 padded, 256
shots over the line, 25 Hz) is imaged on the GPU with checkpoint-and-
recompute (states every 360 steps, FP32 and FP16 checkpoints) for 16 shots
spread along the line (every 16th shot, from shot 8), at a 1 s record (the
full 6 s would take the FP64 oracle about 45 CPU-minutes per shot).  The
image and illumination stacks formed on the device (the reference's
SRC/migration/main_Acoustic_RTM.m:237-262: image = sum of the shots' T*Im,
illumination = sum of their T*illum, img_RTM = image ./ illumination) are
compared with the same stacks of the FP64 C/OpenMP oracle.

The oracle part is CPU-bound (16 x 3 propagations of 5.2 M points x 1000
steps, about 95 minutes on 8 host cores), so the three parts run apart:

  python tests/faulted_salt_subset.py gpu <gpu.npz>        (on a GB300)
  python tests/faulted_salt_subset.py oracle <oracle.npz>  (any host)
  python tests/faulted_salt_subset.py compare <gpu.npz> <oracle.npz>

The GPU stacks are stored in FP32 (rounding 6e-8, far below the errors
measured); the oracle's in FP64.  tests/test_gpu_configs.py runs a 4-shot
version of the same comparison as a GPU test.
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "mnad-modeling-rtm_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

from mnad import workflow  # noqa: E402

SHOTS = list(range(8, 256, 16))
NT = 1000
CHECKPOINT_EVERY = 360


def survey():
    return workflow.faulted_salt_survey(nshots=256, nt=NT)


def gpu_stacks(sv, shots, codec):
    """(image_sum, illum_sum, img_rtm) of the shots from one checkpointed plan."""
    import mnad
    jobs = workflow.shot_jobs(sv, "rtm", shots=shots)
    with mnad.Context(0, checkpoint_every=CHECKPOINT_EVERY, checkpoint_codec=codec) as c:
        plan = c.plan(jobs)
        plan.run()
        out = plan.stack()
        plan.close()
    return out


def oracle_stacks(sv, shots, log=print):
    """FP64 oracle stacks of the shots: sum of images, sum of illuminations."""
    from oracle import coracle
    from oracle import mnad_oracle as P
    nf = P.snapshot_nf(sv.vs, sv.nt)
    T = sv.T or P.snapshot_plan(sv.vs, sv.nt)[1]
    ncols = max(2 * nf + 1, sv.nt // T)
    nzi, nxi = sv.nz - 2 * sv.d_pml, sv.nx - 2 * sv.d_pml
    im_sum = np.zeros(nzi * nxi)
    il_sum = np.zeros(nzi * nxi)
    for k, sh in enumerate(shots):
        t = time.perf_counter()
        a = (sv.dx, sh.xs, sh.xr, sv.dz, sh.zs, sh.zr)
        data = coracle.fwd(*a, sv.v, sv.dt, sv.nt, sv.w, sv.d_pml)["datau"]
        bg = coracle.fwd(*a, sv.vs, sv.dt, sv.nt, sv.w, sv.d_pml, indx=1, T=T, ncols=ncols)
        im = coracle.adj(sv.dx, sv.dz, sv.nt, sv.dt, sv.vs, sh.xr, sh.zr, data - bg["datau"], sv.d_pml, bg["UU"], T)
        im_sum += np.ravel(im, order="F")
        il_sum += np.ravel(bg["illum"], order="F")
        log(f"oracle shot {k + 1}/{len(shots)} ({time.perf_counter() - t:.0f} s)")
    shape = (nzi, nxi)
    return im_sum.reshape(shape, order="F"), il_sum.reshape(shape, order="F")


def rel(a, b):
    a, b = np.ravel(np.asarray(a, dtype=np.float64)), np.ravel(np.asarray(b, dtype=np.float64))
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def errors(im, il, im_ref, il_ref):
    """rel-L2 of the stacked image and illumination, and of img_RTM where
    the oracle's illumination is above 1e-6 of its maximum."""
    mask = np.asarray(il_ref) > 1e-6 * float(np.max(il_ref))
    img = np.asarray(im, dtype=np.float64)[mask] / np.asarray(il, dtype=np.float64)[mask]
    img_ref = np.asarray(im_ref)[mask] / np.asarray(il_ref)[mask]
    return {"image_sum": rel(im, im_ref), "illum_sum": rel(il, il_ref), "img_rtm": rel(img, img_ref)}


def main(argv):
    if len(argv) < 3 or argv[1] not in ("gpu", "oracle", "compare"):
        sys.exit(__doc__)
    sv = survey()
    shots = [sv.shots[k] for k in SHOTS]
    if argv[1] == "gpu":
        out = {}
        for codec in ("f32", "f16"):
            t = time.perf_counter()
            im, il, _ = gpu_stacks(sv, shots, codec)
            out[f"image_{codec}"] = im.astype(np.float32)
            if codec == "f32":
                out["illum"] = il.astype(np.float32)   # the forward phase does not depend on the checkpoint codec
            print(f"gpu {codec} checkpoints: {len(shots)} shots in {time.perf_counter() - t:.1f} s", flush=True)
        np.savez_compressed(argv[2], shots=np.array(SHOTS), nt=NT, **out)
    elif argv[1] == "oracle":
        im, il = oracle_stacks(sv, shots, log=lambda m: print(m, flush=True))
        np.savez(argv[2], shots=np.array(SHOTS), nt=NT, image=im, illum=il)
    else:
        g = np.load(argv[2])
        o = np.load(argv[3])
        assert list(g["shots"]) == list(o["shots"]) and int(g["nt"]) == int(o["nt"])
        for codec in ("f32", "f16"):
            e = errors(g[f"image_{codec}"], g["illum"], o["image"], o["illum"])
            print(f"{len(SHOTS)} shots, 1281x4081, nt {NT}, {codec} checkpoints every {CHECKPOINT_EVERY} steps: " +
                  ", ".join(f"{k} {v:.2e}" for k, v in e.items()))


if __name__ == "__main__":
    main(sys.argv)
