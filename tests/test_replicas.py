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


def test_bench_gpus_flag_spawns_ranks():
    """`bench.py --gpus 2` without a launcher starts two local ranks itself:
    the reference arm (CPU) prints one line from rank 0 with n_gpus 2, and
    the other rank exits 0 without work."""
    import json
    import subprocess
    import sys
    env = {k: v for k, v in os.environ.items()
           if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT")}
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--impl",
                        "reference", "--workload", "sphere17", "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, env=env, timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["cpu_baseline"]["measured_fraction"] == 1.0 and line["value"] > 0


def test_bench_rejects_a_mismatched_launcher():
    import subprocess
    import sys
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--impl",
                        "reference", "--workload", "sphere17"], capture_output=True, text=True,
                       env=env, timeout=300, cwd=str(ROOT))
    assert r.returncode != 0 and "does not match WORLD_SIZE" in r.stderr
