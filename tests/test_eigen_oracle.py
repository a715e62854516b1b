"""The reference's known generalized eigenproblem (test_eigen_solver.cpp:
17-57, 90-159) through the FP64 shift-invert oracle."""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl


def known_pencil():
    lam = np.array([1 + 0.2j, -0.5 + 0.7j, 2 - 0.3j, -1.2 - 0.4j, 3 + 1j, -3 - 1j,
                    4 + 2j, -4 - 2j, 5 + 3j, -5 - 3j])
    d = np.array([1.0, 2.0, 1.5, 1.0, 0.8, 1.2, 1.1, 0.9, 1.4, 1.3])
    A = np.diag(d * lam).astype(complex)
    A[0, 1] = 0.7 - 0.2j; A[0, 3] = -0.3 + 0.5j; A[1, 2] = 1.1 + 0.4j
    A[2, 3] = 0.2 - 0.8j
    for r in range(3, 9):
        A[r, r + 1] = 0.05 * r - 0.03j * r
    return A, np.diag(d).astype(complex)


def test_known_pencil_shift_invert():
    A, B = known_pencil()
    omega = complex(-0.65, -0.45)
    sigma = complex(omega.imag, -omega.real)
    assert abs(sigma - complex(-0.45, 0.65)) <= 2e-10
    lu = spl.splu(sp.csc_matrix(A - sigma * B))
    op = spl.LinearOperator((10, 10), matvec=lambda v: lu.solve(B @ v), dtype=complex)
    theta, vecs = spl.eigs(op, k=2, which="LM", ncv=6, tol=1e-12)
    lam = sigma + 1 / theta
    for expected in (-0.5 + 0.7j, -1.2 - 0.4j):
        assert np.min(np.abs(lam - expected)) <= 2e-10
    for t in range(2):
        x = vecs[:, t]
        res = np.linalg.norm(A @ x - lam[t] * (B @ x)) / (abs(lam[t]) * np.linalg.norm(x))
        assert res <= 2e-10
