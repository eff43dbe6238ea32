"""Sharding cells across ranks: LPT balance, and the one gather of results, with two gloo
ranks on the CPU (the multi-GPU path of batches and surrogate datasets)."""

import os
import socket

import numpy as np
import pytest

from nofluidx3d_gb300.shard import gather_results, lpt_partition, rank_loads


def test_lpt_partition_covers_and_balances():
    rng = np.random.default_rng(0)
    w = np.exp(rng.uniform(np.log(5e3), np.log(1.6e6), 256))  # tetra counts of the batched population
    for n in (1, 2, 4, 8):
        parts = lpt_partition(w, n)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(256))
        loads = rank_loads(w, parts)
        assert max(loads) <= (4 / 3) * max(w.sum() / n, w.max()) + 1e-6
    assert lpt_partition([3, 3, 2, 2, 2], 2) in ([[0, 2, 3], [1, 4]], [[0, 2], [1, 3, 4]], [[0, 3], [1, 2, 4]],
                                                 [[0, 2, 4], [1, 3]], [[0, 4], [1, 2, 3]], [[0, 3, 4], [1, 2]])


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, weights, out_path):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        parts = lpt_partition(weights, world)
        local = {i: ("cell", i, rank, float(weights[i]) ** 0.5) for i in parts[rank]}
        res = gather_results(dist, local, len(weights))
        if rank == 0:
            np.save(out_path, np.array([r[1] for r in res] + [r[2] for r in res]))
        else:
            assert res is None
    finally:
        dist.destroy_process_group()


def test_gather_over_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    weights = [float(x) for x in np.linspace(1e4, 1e6, 37)]
    out = str(tmp_path / "gathered.npy")
    mp.spawn(_rank_main, args=(2, _free_port(), weights, out), nprocs=2, join=True)
    g = np.load(out)
    ids, ranks = g[:37], g[37:]
    assert list(ids) == list(range(37))  # every cell once, in cell order
    parts = lpt_partition(weights, 2)
    for r in (0, 1):
        assert sorted(np.flatnonzero(ranks == r)) == parts[r]
