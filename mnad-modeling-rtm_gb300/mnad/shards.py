"""Multi-GPU replicas: shots are independent, so N processes (one per GPU)
each run their own share of the shots and the only exchange is the final
FP64 sum of the per-shot images and illuminations
(SRC/migration/main_Acoustic_RTM.m:256-262: img = mean(mhh,3)./illum).

The reduction runs over ``torch.distributed`` (NCCL between GPUs, gloo on
CPU); nothing else crosses ranks.
"""
from __future__ import annotations

from typing import Sequence, TypeVar

import numpy as np

T = TypeVar("T")


def shard(items: Sequence[T], rank: int, world: int) -> list:
    """Round-robin share of ``items`` for ``rank`` of ``world`` (every item
    lands on exactly one rank; shares differ in length by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    return list(items[rank::world])


def reduce_stack(image_sum: np.ndarray, illum_sum: np.ndarray, group=None):
    """Sum every rank's FP64 image and illumination stacks and form
    ``img = image_sum ./ illum_sum`` (the reference's mean(mhh,3)./illum; the
    1/ns factors cancel).  Returns (image_sum, illum_sum, img), identical on
    every rank."""
    import torch
    import torch.distributed as dist
    shape = np.shape(image_sum)
    both = np.ascontiguousarray(np.stack([np.ravel(image_sum, order="F"), np.ravel(illum_sum, order="F")]),
                                dtype=np.float64)
    t = torch.from_numpy(both)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    out = t.cpu().numpy()
    im = out[0].reshape(shape, order="F")
    il = out[1].reshape(shape, order="F")
    with np.errstate(divide="ignore", invalid="ignore"):
        img = im / il
    return im, il, img
