"""Sharding independent cells across GPUs (one process per GPU).

Cells of a batch or of a surrogate dataset share nothing, so N ranks split them with no per-step
exchange: each rank runs its own batch, and the only collective is one gather of the results at
the end. The split is longest-processing-time-first bin packing on each cell's tetra count (the
work of a step is proportional to it): cells in decreasing size go to the currently lightest
rank, which keeps the largest rank load within 4/3 of the optimum.
"""

from __future__ import annotations

import heapq
from typing import Sequence


def lpt_partition(weights: Sequence[float], n_ranks: int) -> list[list[int]]:
    """Indices of the cells each rank runs (every index exactly once, each list ascending)."""
    if n_ranks < 1:
        raise ValueError("n_ranks must be >= 1")
    order = sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i))
    heap = [(0.0, r) for r in range(n_ranks)]
    parts: list[list[int]] = [[] for _ in range(n_ranks)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + float(weights[i]), r))
    return [sorted(p) for p in parts]


def rank_loads(weights: Sequence[float], parts: list[list[int]]) -> list[float]:
    return [float(sum(weights[i] for i in p)) for p in parts]


def gather_results(dist, local: dict[int, object], n_total: int) -> list[object] | None:
    """Gather {cell index: result} from every rank; rank 0 receives the list in cell order (other
    ranks None). `dist` is torch.distributed with an initialised process group, or None for one
    process."""
    if dist is None:
        return [local[i] for i in range(n_total)]
    world = dist.get_world_size()
    out = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(local, out, dst=0)
    if dist.get_rank() != 0:
        return None
    merged: dict[int, object] = {}
    for part in out:
        for k, v in part.items():
            if k in merged:
                raise RuntimeError(f"cell {k} came back from two ranks")
            merged[k] = v
    missing = [i for i in range(n_total) if i not in merged]
    if missing:
        raise RuntimeError(f"cells {missing[:8]} came back from no rank")
    return [merged[i] for i in range(n_total)]
