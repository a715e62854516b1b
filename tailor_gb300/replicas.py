"""Replicas across processes: one process per GPU, no data-path collective.

The path does not shard within an instance (the sparse LU couples every
unknown), so several GPUs run independent instances.  Sweep points are
dealt round-robin to the ranks, every rank solves its share with the
single-GPU sweep, and the results are gathered on the host (one
``all_gather_object`` of small arrays at the end); timings reduce to the
slowest rank and converged pairs to their sum.  ``torch.distributed``
carries only this host-side bookkeeping (gloo on CPU, or NCCL/gloo when the
caller initialised it); without an initialised process group everything
runs as a single rank.
"""
from __future__ import annotations

import numpy as np


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover - torch is part of the image
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def rank_world() -> tuple[int, int]:
    d = _dist()
    return (d.get_rank(), d.get_world_size()) if d else (0, 1)


def barrier() -> None:
    d = _dist()
    if d:
        d.barrier()


def partition(npoints: int, rank: int, world: int) -> list[int]:
    """Point indices of one rank: round-robin, so every grid class is spread."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    return list(range(rank, npoints, world))


def reduce_timing(ms: float, pairs: int) -> tuple[float, int]:
    """(slowest rank's time, total converged pairs) over all ranks."""
    d = _dist()
    if not d:
        return float(ms), int(pairs)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    g = torch.tensor([float(pairs)], dtype=torch.float64)
    d.all_reduce(g)
    return float(t.item()), int(round(g.item()))


def sweep(cases, points, solve=None, **kw):
    """The sweep of ``api.sweep`` spread over the ranks of the process group.

    Every rank solves points[rank::world] with ``solve`` (``api.sweep`` by
    default, on the rank's own GPU) and receives the full result: lam
    [points][nev], residual [points][nev], status [points] in the original
    point order, plus per-rank diagnostics and the slowest rank's wall time.
    """
    if solve is None:
        from . import api
        solve = api.sweep
    rank, world = rank_world()
    mine = partition(len(points), rank, world)
    local = solve(cases, [points[i] for i in mine], **kw) if mine else None
    part = {"idx": mine,
            "lam": None if local is None else np.asarray(local.lam),
            "residual": None if local is None else np.asarray(local.residual),
            "status": None if local is None else np.asarray(local.status),
            "diag": None if local is None else dict(local.diag)}
    d = _dist()
    parts = [part]
    if d:
        parts = [None] * world
        d.all_gather_object(parts, part)
    nev = next((p["lam"].shape[1] for p in parts if p["lam"] is not None), 0)
    lam = np.zeros((len(points), nev), dtype=np.complex128)
    res = np.full((len(points), nev), -1.0)
    status = np.zeros(len(points), dtype=np.int32)
    for p in parts:
        if p["lam"] is None:
            continue
        lam[p["idx"]] = p["lam"]
        res[p["idx"]] = p["residual"]
        status[p["idx"]] = p["status"]
    walls = [p["diag"]["wall_ms"] for p in parts if p["diag"]]
    return {"lam": lam, "residual": res, "status": status,
            "wall_ms": max(walls) if walls else 0.0,
            "rank_diag": [p["diag"] for p in parts], "world": world}
