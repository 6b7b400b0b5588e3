"""The multi-GPU path of bench.py (replicas only): world-size-2 gloo ranks on the CPU.

Each rank times its own replica; the reported time is the slowest rank's and the throughput counts the units
of every rank. The reference arm under torchrun runs on rank 0 only and the other ranks exit 0.
"""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    import bench

    r = bench.Replicas(ws)
    r.barrier()
    seconds = 1.0 + rank  # rank 1 is the slow one
    out.put((rank, r.max(seconds), r.throughput(100.0, seconds)))
    r.close()


def test_replicas_max_and_throughput_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's time; 2 replicas x 100 units in 2 s
    assert got == [(0, 2.0, 100.0), (1, 2.0, 100.0)]


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--cells", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1 and '"impl": "reference"' in lines[0]
