"""Stream sharding across ranks (one process per GPU).

The reference hands 143-frame groups to GPU ``index % NUM_GPU``
(software/aphids/vdif_in_databuf_cuda.cu:48-84) and each GPU works alone; the
only shared value is the threshold, which in per-stream mode is local.  Here
whole packet streams go round-robin to ranks; no data moves between GPUs.  The
only collective is a bookkeeping gather of per-rank work counts.
"""
from __future__ import annotations


def streams_for_rank(streams, rank: int, world: int):
    """Round-robin assignment, as ``index % NUM_GPU``."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return [s for i, s in enumerate(streams) if i % world == rank]


def allgather_counts(n: int):
    """Gather one integer per rank (no-op when torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return [n]
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([n], dtype=torch.int64, device=dev)
    out = [torch.zeros_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(out, t)
    return [int(x.item()) for x in out]


def process_shard(streams, run, rank: int, world: int):
    """Run ``run(index, stream)`` on this rank's streams (round-robin) and
    gather the results of every rank: returns ``{index: result}`` for all
    streams on every rank (results must be picklable, e.g. digests of the
    payloads).  Without torch.distributed (world 1) it is a plain loop."""
    import torch.distributed as dist

    mine = {i: run(i, s) for i, s in enumerate(streams) if i % world == rank}
    if not (dist.is_available() and dist.is_initialized()) or world == 1:
        return mine
    parts = [None] * world
    dist.all_gather_object(parts, mine)
    out = {}
    for p in parts:
        out.update(p)
    return out
