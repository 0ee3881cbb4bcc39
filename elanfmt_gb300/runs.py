"""Independent runs spread over processes, one GPU each.

The time loop does not exchange data between runs: the 6 elementary moment-tensor runs of an
inversion, the models of a batch and the source positions of a surrogate's training set are
separate solves.  Several GPUs therefore take disjoint shares of the run list (contiguous
blocks, so every rank's share is a batch of similar problems) and the only communication is a
host-side gather of the seismograms to rank 0 at the end -- no collective touches device data.

    from elanfmt_gb300 import runs
    mine = runs.shard(len(units), rank, world)
    traces = {u: solve(units[u]) for u in mine}          # this rank's GPU
    everything = runs.gather(traces, dist)                # rank 0: {unit: traces}, others: None
"""
from __future__ import annotations

import numpy as np


def shard(n_units: int, rank: int, world: int) -> range:
    """The contiguous block of unit indices owned by `rank` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def gather(local: dict, dist=None) -> dict | None:
    """Collects every rank's {unit index: array} on rank 0 (host memory, gloo or NCCL object
    gather); returns the merged dict on rank 0 and None elsewhere.  Without an initialised process
    group it returns `local` unchanged."""
    if dist is None or not dist.is_initialized():
        return dict(local)
    world = dist.get_world_size()
    rank = dist.get_rank()
    payload = {int(k): np.asarray(v) for k, v in local.items()}
    out = [None] * world if rank == 0 else None
    dist.gather_object(payload, out, dst=0)
    if rank != 0:
        return None
    merged: dict = {}
    for part in out:
        overlap = merged.keys() & part.keys()
        if overlap:
            raise ValueError(f"units {sorted(overlap)[:5]} reported by two ranks")
        merged.update(part)
    return merged


def run_sharded(units: list, solve, rank: int = 0, world: int = 1, dist=None) -> dict | None:
    """Runs solve(unit) for this rank's share of `units` and gathers {index: result} on rank 0."""
    mine = {u: solve(units[u]) for u in shard(len(units), rank, world)}
    return gather(mine, dist)
