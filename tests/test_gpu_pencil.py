"""Explicit generalized pencils on the GPU (the reference's EigenSolver
overload for small known problems, EigenSolver.hpp:60-67): the 10 x 10
pencil of test_eigen_solver.cpp:17-57 (eigenvalues -0.5+0.7i and
-1.2-0.4i near the target, 2e-10), an order that is not a multiple of
the 5 x 5 block size, and a dense 300 x 300 pencil against SciPy's QZ."""
import numpy as np
import pytest
import scipy.linalg as sl

from tailor_gb300 import api, output
from test_eigen_oracle import known_pencil

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_known_pencil(gpu_lib, precision):
    A, B = known_pencil()
    omega = complex(-0.65, -0.45)  # lambda_s = -0.45 + 0.65i
    sol = api.solve_pencil(A, B, omega=omega, nev=2, precision=precision, ncv=8)
    assert sol.diag["converged"] >= 2
    assert abs(complex(sol.diag["target_re"], sol.diag["target_im"]) - (-0.45 + 0.65j)) == 0
    for expected in (-0.5 + 0.7j, -1.2 - 0.4j):
        assert np.min(np.abs(sol.lam - expected)) <= 2e-10, sol.lam
    assert np.all(sol.residual <= 2e-10)
    for lam, v in zip(sol.lam, sol.modes):
        m = output.fix_mode_phase(v)
        r = np.linalg.norm(A @ m - lam * (B @ m)) / abs(lam)
        assert r <= 2e-10


@pytest.mark.parametrize("n,precision", [(12, 0), (12, 1), (300, 0), (300, 1)])
def test_random_pencil_against_qz(gpu_lib, n, precision):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    B = np.zeros((n, n), dtype=complex)
    for s in range(0, n, 5):  # block diagonal, well conditioned
        k = min(5, n - s)
        B[s:s + k, s:s + k] = np.eye(k) + 0.1 * rng.standard_normal((k, k))
    ref = sl.eig(A, B, right=False)
    omega = complex(0.3, 0.2)
    sigma = complex(omega.imag, -omega.real)
    nev = 4
    sol = api.solve_pencil(A, B, omega=omega, nev=nev, precision=precision,
                           ncv=min(24, n - 1))
    near = ref[np.argsort(np.abs(ref - sigma))[:nev]]
    assert np.all(sol.residual <= 1e-10)
    for lam in sol.lam:
        assert np.min(np.abs(near - lam)) <= 1e-8 * abs(lam), (lam, near)
