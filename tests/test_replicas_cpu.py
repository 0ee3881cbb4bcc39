"""Several processes: bench.py's replicas (every rank runs the whole workload, the job's time is
the slowest rank's) and elanfmt_gb300.runs (independent runs sharded over ranks, seismograms
gathered on rank 0).  Two gloo ranks on the CPU check both."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(10.0 + 5.0 * rank, dist)
        dist.barrier()
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: 15.0, 1: 15.0}


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5) == 3.5


def _shard_rank(rank: int, world: int, port: int, out):
    import numpy as np
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    from elanfmt_gb300 import runs

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = list(range(7))
        got = runs.run_sharded(units, lambda u: np.full((2, 3), float(u * 10 + rank)), rank, world, dist)
        out.put((rank, None if got is None else {k: v.tolist() for k, v in got.items()}))
    finally:
        dist.destroy_process_group()


def test_runs_sharded_and_gathered_on_rank0():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res[1] is None
    got = res[0]
    assert sorted(got) == list(range(7))
    # units 0-3 ran on rank 0, 4-6 on rank 1 (contiguous shares)
    for u in range(7):
        assert got[u] == [[float(u * 10 + (0 if u < 4 else 1))] * 3] * 2


def test_shard_covers_every_unit_once():
    sys.path.insert(0, ROOT)
    from elanfmt_gb300 import runs

    for n in (0, 1, 5, 22, 100):
        for world in (1, 2, 3, 8):
            parts = [list(runs.shard(n, r, world)) for r in range(world)]
            assert sorted(sum(parts, [])) == list(range(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1
    with pytest.raises(ValueError):
        runs.shard(4, 2, 2)
