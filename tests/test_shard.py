"""The replica ensemble split over the ranks of a multi-GPU run (ffea_ci_demo_gb300.shard; bench.py's batch
workload under torchrun): each rank steps a batch of its own blobs, with no exchange on the data path.

* The split covers every blob exactly once, balances the ranks' element totals to within the largest blob, and is
  the same on every rank (each rank computes it from the seeded ensemble).
* world-size-2 gloo ranks on the CPU: each takes its shard, the reported time is the slowest rank's, and the
  throughput counts every rank's nodes.
"""
import os
import sys

import pytest

from ffea_ci_demo_gb300.mesh import ensemble_cells
from ffea_ci_demo_gb300.shard import partition_by_elements
from test_replicas import ROOT, free_port


def ensemble_elements(n=256):
    return [6 * int(c) ** 3 for c in ensemble_cells(n)]


@pytest.mark.parametrize("nranks", [1, 2, 3, 4, 8])
def test_partition_covers_and_balances(nranks):
    el = ensemble_elements()
    parts = partition_by_elements(el, nranks)
    flat = sorted(b for p in parts for b in p)
    assert flat == list(range(len(el)))
    loads = [sum(el[b] for b in p) for p in parts]
    assert max(loads) - min(loads) <= max(el)
    assert parts == partition_by_elements(el, nranks)
    assert all(p == sorted(p) for p in parts)


def test_partition_refuses_bad_counts():
    with pytest.raises(ValueError):
        partition_by_elements([10, 20], 3)
    with pytest.raises(ValueError):
        partition_by_elements([10], 0)


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    import bench

    el = ensemble_elements()
    mine = partition_by_elements(el, ws)[rank]
    r = bench.Replicas(ws)
    r.barrier()
    seconds = sum(el[b] for b in mine) * 1e-7  # a rank's time grows with its elements
    slowest = r.max(seconds)
    nodes_all = sum((int(round((e / 6) ** (1 / 3))) + 1) ** 3 for e in el)
    out.put((rank, tuple(mine), slowest, nodes_all / slowest))
    r.close()


def test_sharded_ensemble_over_two_gloo_ranks():
    pytest.importorskip("torch")
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
    el = ensemble_elements()
    (r0, s0, t0, v0), (r1, s1, t1, v1) = got
    assert sorted(s0 + s1) == list(range(len(el))) and not set(s0) & set(s1)
    assert t0 == t1 == max(sum(el[b] for b in s0), sum(el[b] for b in s1)) * 1e-7
    assert v0 == v1
