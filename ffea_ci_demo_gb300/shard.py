"""A replica ensemble split over the ranks of a multi-GPU run.

The reference advances a World's blobs one after another (`World::run`, src/World.cpp:1788-2059; with OpenMP over
blobs in its multi-blob build, :2032-2059); the blobs never interact on this path, so an ensemble splits over GPUs
with no exchange at all: each rank builds a batch of its own blobs and steps it. The work of a blob is about
proportional to its element count (element phase, assembly) times its CG iterations (unknown before the run), so
the split balances element counts: longest-processing-time first, each blob to the least-loaded rank, ties to the
lower rank, blobs of a rank kept in ensemble order.
"""
from __future__ import annotations


def partition_by_elements(elements: list[int], nranks: int) -> list[list[int]]:
    """Blob indices of each rank, balancing the ranks' element totals."""
    if nranks < 1:
        raise ValueError("at least one rank")
    if len(elements) < nranks:
        raise ValueError("fewer blobs than ranks")
    load = [0] * nranks
    parts: list[list[int]] = [[] for _ in range(nranks)]
    for b in sorted(range(len(elements)), key=lambda i: (-elements[i], i)):
        r = min(range(nranks), key=lambda k: (load[k], k))
        parts[r].append(b)
        load[r] += elements[b]
    return [sorted(p) for p in parts]
