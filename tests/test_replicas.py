"""Replicas over two CPU ranks (gloo, world size 2): the round-robin deal
of sweep points, the host-side gather back into point order, and the
timing reduction (slowest rank, summed pairs) -- the multi-process logic
that bench.py --gpus N and multi-GPU sweeps use, without a GPU: the
per-rank solve is a stand-in that returns known values."""
import os
import socket
import tempfile
from types import SimpleNamespace

import numpy as np
import pytest

from tailor_gb300 import replicas


def fake_solve(cases, points, **kw):
    """Deterministic stand-in for api.sweep: lambda from the point's alpha."""
    a = np.array([p[1] for p in points])
    lam = np.stack([a + 1j * k for k in range(3)], axis=1)
    return SimpleNamespace(lam=lam, residual=np.full(lam.shape, 1e-12),
                           status=np.zeros(len(points), dtype=np.int32),
                           diag={"wall_ms": 10.0 * len(points)})


POINTS = [(i % 2, 0.5 + 0.1 * i) for i in range(7)]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        r = replicas.sweep(None, POINTS, solve=fake_solve)
        ms, pairs = replicas.reduce_timing(10.0 * (rank + 1), rank + 3)
        np.savez(os.path.join(out, f"rank{rank}.npz"), lam=r["lam"], residual=r["residual"],
                 status=r["status"], wall=r["wall_ms"], world=r["world"], ms=ms, pairs=pairs)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition():
    assert replicas.partition(7, 0, 2) == [0, 2, 4, 6]
    assert replicas.partition(7, 1, 2) == [1, 3, 5]
    assert sorted(replicas.partition(10, 0, 3) + replicas.partition(10, 1, 3)
                  + replicas.partition(10, 2, 3)) == list(range(10))
    with pytest.raises(ValueError):
        replicas.partition(4, 2, 2)


def test_single_rank_is_the_plain_sweep():
    r = replicas.sweep(None, POINTS, solve=fake_solve)
    ref = fake_solve(None, POINTS)
    assert r["world"] == 1 and np.array_equal(r["lam"], ref.lam)
    assert replicas.reduce_timing(5.0, 4) == (5.0, 4)


def test_two_gloo_ranks_gather_in_point_order():
    import torch.multiprocessing as mp
    serial = fake_solve(None, POINTS)
    with tempfile.TemporaryDirectory() as out:
        mp.spawn(_rank, args=(2, _free_port(), out), nprocs=2, join=True)
        for rank in range(2):
            r = np.load(os.path.join(out, f"rank{rank}.npz"))
            assert int(r["world"]) == 2
            assert np.array_equal(r["lam"], serial.lam)  # every rank holds the full result
            assert np.all(r["residual"] == 1e-12) and np.all(r["status"] == 0)
            assert float(r["wall"]) == 40.0  # slowest rank: 4 of the 7 points
            assert float(r["ms"]) == 20.0 and int(r["pairs"]) == 7
