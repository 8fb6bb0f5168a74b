"""One batch of independent TTs split over the processes of a job, one
process per GPU.

The reference rounds TTs one after another (round/tt_round.hpp:60-63); TTs
share nothing, so a batch splits without any exchange step.  Every rank
computes the same partition from the shapes alone (shard_plan: longest
estimated rounding cost first, each TT to the least-loaded rank), rounds
its own part on its own GPU, and the results travel to one rank through
host memory (torch.distributed.gather_object; give it a gloo group to keep
the transfer off the GPUs).

Within one process, round_batch(..., devices=[...]) and
eval_batch(..., devices=[...]) split over several devices directly.
"""
from __future__ import annotations

from . import round_batch, shard_plan


def my_part(tts, rank: int, world: int) -> list[int]:
    """Indices (in input order) of the TTs that rank `rank` of `world` rounds."""
    part_of, _ = shard_plan(tts, world)
    return [i for i in range(len(tts)) if int(part_of[i]) == rank]


def round_batch_distributed(tts, opts=None, group=None, dst: int = 0, worker=None):
    """Round `tts` split over the ranks of `group` (default: the world).

    Every rank passes the whole batch (only shapes of the other ranks' TTs
    are read).  Returns the rounded TTs in input order on rank `dst`, None
    on the others.  `worker(list_of_tts) -> list_of_tts` rounds one part;
    the default is this library's round_batch with `opts` on the rank's
    current CUDA device."""
    import torch.distributed as dist
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    mine = my_part(tts, rank, world)
    if worker is None:
        def worker(part):
            return round_batch(part, opts) if part else []
    ys = worker([tts[i] for i in mine])
    if len(ys) != len(mine):
        raise RuntimeError("round_batch_distributed: the worker returned "
                           f"{len(ys)} results for {len(mine)} TTs")
    gathered = [None] * world if rank == dst else None
    dist.gather_object(list(zip(mine, ys)), gathered, dst=dst, group=group)
    if rank != dst:
        return None
    out = [None] * len(tts)
    for part in gathered:
        for i, y in part:
            out[i] = y
    if any(y is None for y in out):
        raise RuntimeError("round_batch_distributed: a TT was rounded by no rank")
    return out
