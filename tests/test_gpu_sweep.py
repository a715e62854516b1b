"""Batched alpha-sweep (tlr_sweep) against one-at-a-time FP64 solves.

Two grid classes of uneven size, ten points, three workers, mixed form with
autotuned kernels: every point's eigenvalues match the plain FP64 solve of
the same (grid, alpha) to |dlambda|/|lambda| <= 1e-8 with relative residual
<= 1e-10, and a point with an invalid class is rejected before any work."""
import numpy as np
import pytest

from tailor_gb300 import api
from tailor_gb300.case import Physics, make_case

pytestmark = pytest.mark.gpu


def _cases():
    ph = Physics(alpha=1.0, omega=0j, nev=6)
    return [make_case(24, 16, physics=ph), make_case(60, 32, physics=ph)]


def test_sweep_matches_plain(gpu_lib):
    cases = _cases()
    rng = np.random.default_rng(4)
    points = [(i % 2, float(rng.uniform(0.8, 3.0))) for i in range(10)]
    out = api.sweep(cases, points, nev=6, precision=1, workers=3, autotune=True)
    assert out.diag["failed"] == 0
    assert out.diag["converged_pairs"] == 60
    assert all(b in (128, 256) for b in out.diag["solve_block"])
    for i, (c, a) in enumerate(points):
        case = cases[c]
        with api.Problem(case) as p:
            p.set_alpha(a)
            api.run_pipeline(p)
            plain = api.EigenSolver(p).solve(nev=6, precision=0)
        for lam in out.lam[i]:
            assert np.min(np.abs(plain.lam - lam)) <= 1e-8 * abs(lam), (i, lam, plain.lam)
        assert np.all(out.residual[i] <= 1e-10)


def test_sweep_rejects_bad_class(gpu_lib):
    with pytest.raises(api.TailorError):
        api.sweep(_cases(), [(0, 1.0), (5, 2.0)], nev=6)
