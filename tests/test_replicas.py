"""The N>1 path of bench.py on CPU: two gloo ranks (127.0.0.1) deal the
batched instances round-robin with no overlap and agree on the max-over-ranks
time, with no data-path collective."""
from __future__ import annotations

import os
import socket

import pytest

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ids = bench.replica_ids(96, rank, world)
    t = bench._max_over_ranks(float(10 + rank), dist)
    out[rank] = (ids, t)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    ids0, t0 = out[0]
    ids1, t1 = out[1]
    assert t0 == t1 == 11.0
    assert sorted(ids0 + ids1) == list(range(96)) and not set(ids0) & set(ids1)


def test_replica_ids_cover_everything():
    import sys
    sys.path.insert(0, str(ROOT))
    import bench
    for world in (1, 2, 3, 8):
        seen = sorted(i for r in range(world) for i in bench.replica_ids(96, r, world))
        assert seen == list(range(96))
    pytest.importorskip("torch")
