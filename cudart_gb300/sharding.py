"""Splitting a render over several GPUs, one process per GPU.

The path tracer shards without any exchange on the data path: every rank
holds the whole scene and renders its own units of work, and the only
collective is one sum of float accumulators at the end (or none, for
batched views, where each rank owns whole views).

* sample_range(spp, rank, world): the contiguous samples [s0, s1) a rank
  renders of every pixel.  Samples are keyed by their global index in the
  Philox counter, so the union over ranks is exactly the single-GPU render's
  sample set.
* view_shard(views, rank, world): whole views per rank, balanced by their
  sample counts (largest first onto the least-loaded rank).
* reduce_accumulators(acc, group): the sum of the ranks' FP32 accumulators
  (torch.distributed all_reduce; NCCL on GPUs, gloo on CPU tensors).
"""
from __future__ import annotations

from typing import List, Sequence, Tuple


def sample_range(spp: int, rank: int, world: int) -> Tuple[int, int]:
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(spp, world)
    s0 = rank * base + min(rank, extra)
    return s0, s0 + base + (1 if rank < extra else 0)


def view_shard(view_samples: Sequence[int], rank: int, world: int) -> List[int]:
    """Indices of the views rank `rank` renders; view_samples[k] is view k's
    pixel count x spp.  Deterministic: every rank computes the same split."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    load = [0] * world
    owner = [0] * len(view_samples)
    for k in sorted(range(len(view_samples)), key=lambda k: (-view_samples[k], k)):
        r = min(range(world), key=lambda r: (load[r], r))
        owner[k] = r
        load[r] += view_samples[k]
    return [k for k in range(len(view_samples)) if owner[k] == rank]


def reduce_accumulators(acc, group=None):
    """Sum the ranks' accumulators in place (a torch tensor)."""
    import torch.distributed as dist
    dist.all_reduce(acc, op=dist.ReduceOp.SUM, group=group)
    return acc
