"""The multi-GPU replica path on CPU: two gloo ranks each image their share
of the shots (with the FP64 oracle standing in for the GPU) and reduce their
stacks; the result equals the single-process stack of all shots.  A rank
that fails before the reduction makes the other rank's reduction fail with
an error instead of hanging."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from mnad import shards, workflow
from oracle import coracle
from oracle import mnad_oracle as P


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _survey():
    nz, nx, d, nt = 44, 60, 10, 160
    z = np.arange(nz)[:, None] * np.ones((1, nx))
    v = 1800.0 + 600.0 * (z > nz / 2)
    vs = workflow.gaussian_smooth(v, 7)
    xr = np.arange(d + 1, nx - d + 1, dtype=np.float64)
    zr = np.full(xr.size, d + 2.0)
    shots = [d + 6 + 8 * k for k in range(5)]
    return dict(v=v, vs=vs, d=d, nt=nt, xr=xr, zr=zr, shots=shots, w=workflow.ricker(25.0, 1e-3, nt))


def _shot_stack(sv, xs):
    nf, T = P.snapshot_plan(sv["vs"], sv["nt"])
    ncols = max(2 * nf + 1, sv["nt"] // T)
    a = (10.0, xs, sv["xr"], 10.0, sv["d"] + 2, sv["zr"])
    data = coracle.fwd(*a, sv["v"], 1e-3, sv["nt"], sv["w"], sv["d"])["datau"]
    bg = coracle.fwd(*a, sv["vs"], 1e-3, sv["nt"], sv["w"], sv["d"], indx=1, T=T, ncols=ncols)
    im = coracle.adj(10.0, 10.0, sv["nt"], 1e-3, sv["vs"], sv["xr"], sv["zr"], data - bg["datau"], sv["d"], bg["UU"], T)
    shape = bg["illum"].shape
    return T * im.reshape(shape, order="F"), T * bg["illum"]


def _worker(rank, world, port, fail_rank, q, timeout_s):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import datetime
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=timeout_s))
    try:
        sv = _survey()
        mine = shards.shard(sv["shots"], rank, world)
        parts = [_shot_stack(sv, xs) for xs in mine]
        im = sum(p[0] for p in parts)
        il = sum(p[1] for p in parts)
        if rank == fail_rank:
            raise RuntimeError("rank failed before the reduction")
        out = shards.reduce_stack(im, il)
        q.put((rank, "ok", [x.copy() for x in out], mine))
    except Exception as e:
        q.put((rank, "error", repr(e), None))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(world, fail_rank=-1, timeout_s=60):
    """Run the ranks; `timeout_s` bounds every collective (a generous bound
    when all ranks are healthy -- their oracle shots may run on a loaded host --
    and a short one where a failed rank must be detected)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, fail_rank, q, timeout_s)) for r in range(world)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(world):
        r, status, payload, mine = q.get(timeout=120)
        res[r] = (status, payload, mine)
    for p in procs:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    return res


def test_shard_covers_every_shot_once():
    items = list(range(11))
    parts = [shards.shard(items, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == items
    assert max(map(len, parts)) - min(map(len, parts)) <= 1
    with pytest.raises(ValueError):
        shards.shard(items, 3, 3)


def test_two_gloo_ranks_reduce_to_the_single_process_stack():
    res = _run(2)
    assert all(v[0] == "ok" for v in res.values()), res
    sv = _survey()
    parts = [_shot_stack(sv, xs) for xs in sv["shots"]]
    im = sum(p[0] for p in parts)
    il = sum(p[1] for p in parts)
    assert sorted(res[0][2] + res[1][2]) == sorted(sv["shots"])
    for r in (0, 1):
        got_im, got_il, got_img = res[r][1]
        assert np.allclose(got_im, im, rtol=1e-12, atol=0)
        assert np.allclose(got_il, il, rtol=1e-12, atol=0)
        assert np.allclose(got_img, im / il, rtol=1e-12, atol=0)
    assert np.array_equal(res[0][1][0], res[1][1][0])   # identical on every rank


def test_a_failed_rank_makes_the_reduction_fail_not_hang():
    res = _run(2, fail_rank=1, timeout_s=8)
    assert res[1][0] == "error"
    assert res[0][0] == "error"          # the surviving rank's collective errors out (timeout or peer loss)
