"""The N>1 replica path of bench.py on CPU: two gloo ranks (no GPU).

The pressure solve does not shard, so N GPUs run N independent replicas;
the only cross-rank traffic is the timing barrier and the max over ranks.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import REPO


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import bench
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(dist)
    m = bench.max_over_ranks(dist, float(rank + 1) * 1.5)
    out.put((rank, m))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in (0, 1)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 3.0, 1: 3.0}


def test_reference_arm_two_ranks_prints_one_line():
    """torchrun with two ranks: rank 0 times the reference's CPU algorithm
    and prints the one JSON line; rank 1 exits 0 without work."""
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(free_port()), os.path.join(REPO, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--grid", "16", "--steps", "1",
           "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600,
                       cwd=REPO)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
