"""Learned shift / start-vector proposal.

* the GPU MLP's forward pass and gradients agree with an FP64 NumPy MLP
  (oracle/mlp_oracle.py) -- FP32 arithmetic, tolerance 1e-4 relative;
* BF16 inference stays within 2e-2 of FP32 inference;
* trained on eigenpairs the solver produced at 48 (alpha, Re, Mach) points
  of a 24x16 grid, the proposal solves 10 held-out points: the start-vector
  solves return the plain solve's eigenvalues (|dlambda|/|lambda| <= 1e-8)
  at residual <= 1e-10 with fewer operator applications in total, and the
  shift-mode solves return the plain eigenvalues whether they are accepted
  or fall back."""
import math

import numpy as np
import pytest

from oracle import mlp_oracle
from tailor_gb300 import api, learned
from tailor_gb300.case import Physics, make_case, target_lambda

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(3, 32, 2, 10), (3, 256, 4, 80)])
def test_mlp_gradients_match_fp64(gpu_lib, shape):
    net = learned.MLP(*shape, seed=7)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((64, shape[0])).astype(np.float32)
    Y = rng.standard_normal((64, shape[3])).astype(np.float32)
    loss, g = net.gradients(X, Y)
    p = net.get_params().astype(np.float64)
    loss_ref, g_ref = mlp_oracle.loss_and_grad(p, X, Y, shape)
    assert abs(loss - loss_ref) <= 1e-4 * abs(loss_ref)
    assert np.linalg.norm(g - g_ref) <= 1e-4 * np.linalg.norm(g_ref)
    y32 = net.forward(X)
    y_ref, _, _ = mlp_oracle.forward(p, X, shape)
    assert np.linalg.norm(y32 - y_ref) <= 1e-5 * np.linalg.norm(y_ref)
    y16 = net.forward(X, bf16=True)
    assert np.linalg.norm(y16 - y_ref) <= 2e-2 * np.linalg.norm(y_ref)
    net.close()


def test_mlp_training_reduces_loss(gpu_lib):
    rng = np.random.default_rng(5)
    X = rng.uniform(-1, 1, (512, 3)).astype(np.float32)
    Y = np.stack([np.sin(2 * X[:, 0]) * X[:, 1], X[:, 2] ** 2], 1).astype(np.float32)
    net = learned.MLP(3, 64, 2, 2, seed=2)
    hist = net.train(X, Y, epochs=300, batch=128, lr=3e-3)
    assert hist[-1] < 0.05 * hist[0]
    net.close()


def test_learned_proposal_gain(gpu_lib):
    base = Physics(alpha=1.5, omega=0j, nev=6)
    case = make_case(24, 16, physics=base)
    rng = np.random.default_rng(11)

    def points(k):
        return [(float(rng.uniform(1.0, 2.0)), float(10 ** rng.uniform(math.log10(800), math.log10(1600))),
                 float(rng.uniform(0.4, 0.6))) for _ in range(k)]

    train_pts, test_pts = points(48), points(10)
    tgt = target_lambda(base.omega)
    with api.Problem(case) as prob:
        samples = learned.generate(prob, train_pts, nev=6, precision=0)
        prop = learned.Proposal.fit(samples, tgt, epochs=2000, batch=48, lr=2e-3, width=128, depth=4)
        plain_solves = learned_solves = 0
        log = []
        for pt in test_pts:
            prob.set_physics(learned.physics_at(base, *pt, 6))
            plain = learned.plain_solve(prob, 6, precision=0)
            for shift in (False, True):
                sol, used, stats = learned.learned_solve(prob, prop, 6, precision=0, shift=shift)
                for lam in sol.lam:
                    assert np.min(np.abs(plain.lam - lam)) <= 1e-8 * abs(lam)
                assert np.all(sol.residual <= 1e-10)
                if not shift:
                    assert used
                    plain_solves += plain.diag["solves"]
                    learned_solves += stats["solves"]
                log.append((shift, used, plain.diag["solves"], stats.get("solves")))
        assert learned_solves < plain_solves, (learned_solves, plain_solves, log)
    prop.mlp.close()
