"""The N > 1 path of bench.py on CPU: world-size-2 gloo process groups.

The engine's multi-GPU mode is replicas (independent disks per GPU, no
data-path collective); what crosses ranks is the timing, reduced with MAX, and
the reference arm, which rank 0 alone runs.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    vals = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 5.0], dist, torch, "cpu")
    out.put((rank, vals))
    dist.barrier()
    dist.destroy_process_group()


def test_timings_reduce_to_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got[0] == got[1] == [2.0, 10.0, 5.0]
    assert bench_identity_without_group(torch) == [3.0, 4.0]


def bench_identity_without_group(torch):
    sys.path.insert(0, REPO)
    import bench
    return bench.max_over_ranks([3.0, 4.0], None, torch, "cpu")


def test_reference_arm_under_torchrun_prints_one_line():
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={port}", "bench.py", "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--config", "c1",
           "--cpu-seconds", "0.3"]
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
