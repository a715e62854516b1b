"""The concurrent chains of bench.py: which sweep points each chain visits.
With the default 32 steps the timed pass and the end-to-end pass each cover
the 32 points of the sweep exactly once, every chain walks contiguous
neighbours of the snake (so every point can start from its predecessor's
Ritz vectors), and each chain warms up on the points just before its own
stretch."""
import importlib.util
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
bench = importlib.util.module_from_spec(spec)
spec.loader.exec_module(bench)


@pytest.mark.parametrize("width", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("warmup", [1, 3])
def test_timed_and_e2e_passes_cover_the_sweep_once(width, warmup):
    seqs, nstep, nnext = bench.chain_sequences(32, 32, width, warmup)
    assert sum(nstep) == 32 and sum(nnext) == 32
    timed = sorted(i for w, s in enumerate(seqs) for i in s[warmup:warmup + nstep[w]])
    e2e = sorted(i for w, s in enumerate(seqs)
                 for i in s[warmup + nstep[w]:warmup + nstep[w] + nnext[w]])
    assert timed == list(range(32)) and e2e == list(range(32))


@pytest.mark.parametrize("width", [1, 3])
def test_chains_walk_neighbours(width):
    seqs, _, _ = bench.chain_sequences(32, 32, width, 3, offset=5)
    for s in seqs:
        assert all((b - a) % 32 == 1 for a, b in zip(s, s[1:]))


def test_fewer_steps_than_points():
    seqs, nstep, _ = bench.chain_sequences(32, 10, 3, 3)
    assert nstep == [4, 3, 3]
    timed = [i for w, s in enumerate(seqs) for i in s[3:3 + nstep[w]]]
    assert sorted(timed) == list(range(3, 13))


def test_snake_order_visits_neighbours():
    """c5_points(snake=True): the 8 x 4 (alpha, Re) grid, alpha running up on
    even Re rows and down on odd ones, so consecutive points differ in one
    coordinate by one grid step (the warm start's neighbour)."""
    import numpy as np
    from tailor_gb300.neutral_sweep import c5_points
    pts = c5_points(snake=True)
    assert len(pts) == 32 and len(set(pts)) == 32
    alphas = np.linspace(0.5, 3.5, 8)
    res = np.linspace(800, 2400, 4)
    for (_, a0, r0), (_, a1, r1) in zip(pts, pts[1:]):
        da = abs(np.searchsorted(alphas, a1 - 1e-9) - np.searchsorted(alphas, a0 - 1e-9))
        dr = abs(np.searchsorted(res, r1 - 1e-9) - np.searchsorted(res, r0 - 1e-9))
        assert (da, dr) in ((1, 0), (0, 1))
