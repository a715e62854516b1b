"""Neutral-curve sweep at the largest grid: (alpha, Re) points on one grid.

    python -m tailor_gb300.neutral_sweep --ny 300 --nz 192 --plain-points 2

Grid Ny x Nz (FD-q q=10 / q=6), bump amplitude 0.05, Mach 0.7, target
lambda_s = 0, nev 8, tol 1e-10; points on an 8 x 4 grid of alpha in
[0.5, 3.5] and Re in [800, 2400], in snake order.  The mixed + batched
form (complex64 fronts with tensor-core Schur updates and FP64
refinement, the sweep engine's shared symbolic analysis and autotuned
kernels, --workers concurrent instances each taking a contiguous run of
the points, every point but a run's first warm-started from its
predecessor's Ritz vectors) solves every point; the plain FP64 form
solves the first --plain-points points one at a time, and their
eigenvalues are compared.  Prints one JSON line with
eigenpairs at resid <= 1e-10 per wall second for each form and the
per-point factor size.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import api
from .case import Physics, make_case


C5_GRID = (300, 192)


def c5_case(ny: int = C5_GRID[0], nz: int = C5_GRID[1], nev: int = 8) -> "Case":
    """The neutral-curve case: wavy wall (bump 0.05), Mach 0.7, target
    lambda 0, nev 8, tol 1e-10 (alpha and Re are set per point)."""
    ph = Physics(alpha=1.0, mach=0.7, omega=0j, nev=nev, tol=1e-10)
    return make_case(ny, nz, amplitude=0.05, physics=ph)


def c5_points(snake: bool = False):
    """The 8 x 4 (alpha, Re) grid as (class 0, alpha, Re) points, Re-major.
    snake: alpha runs up on even Re rows and down on odd ones, so that
    consecutive points are neighbours (warm starts)."""
    alphas = [float(a) for a in np.linspace(0.5, 3.5, 8)]
    pts = []
    for r, re in enumerate(np.linspace(800, 2400, 4)):
        row = alphas if (not snake or r % 2 == 0) else alphas[::-1]
        pts += [(0, a, float(re)) for a in row]
    return pts


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ny", type=int, default=300)
    ap.add_argument("--nz", type=int, default=192)
    ap.add_argument("--nev", type=int, default=8)
    ap.add_argument("--workers", type=int, default=4)
    ap.add_argument("--plain-points", type=int, default=2)
    ap.add_argument("--ncv", type=int, default=64)
    a = ap.parse_args()
    case = c5_case(a.ny, a.nz, a.nev)
    points = c5_points(snake=True)
    out = {"grid": [a.ny, a.nz], "points": len(points), "nev": a.nev, "ncv": a.ncv,
           "mach": 0.7}
    t = time.perf_counter()
    r = api.sweep([case], points, nev=a.nev, ncv=a.ncv, precision=1, workers=a.workers,
                  autotune=True, raise_on_error=False, warm_start=True)
    wall = time.perf_counter() - t
    good = int(np.sum((r.residual >= 0) & (r.residual <= 1e-10)))
    fb = [d["factor_bytes"] for d in r.point_diag if d["factor_bytes"] > 0]
    out["mixed_batched"] = {"wall_s": wall, "eigenpairs": good, "value": good / wall,
                            "failed_points": r.diag["failed"], "workers": r.diag["workers"],
                            "factor_gb_per_instance": (max(fb) / 1e9) if fb else None,
                            "solve_block": r.diag["solve_block"],
                            "tensor_core_schur": [1 - c for c in r.diag["cuda_core_schur"]]}
    if a.plain_points > 0:
        sub = points[:a.plain_points]
        t = time.perf_counter()
        p = api.sweep([case], sub, nev=a.nev, ncv=a.ncv, precision=0, workers=1,
                      autotune=False, raise_on_error=False)
        wall_p = time.perf_counter() - t
        good_p = int(np.sum((p.residual >= 0) & (p.residual <= 1e-10)))
        out["plain_fp64"] = {"wall_s": wall_p, "points": len(sub), "eigenpairs": good_p,
                             "value": good_p / wall_p,
                             "max_abs_dlambda_rel": float(max(
                                 np.min(np.abs(r.lam[i] - lam)) / abs(lam)
                                 for i in range(len(sub)) for lam in p.lam[i]))}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
