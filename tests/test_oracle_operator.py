"""Oracle assembly against the reference's structural and matrix-free
checks (test_global_operator.cpp:105-296) and its boundary-row checks
(test_boundary_conditions.cpp:80-183, test_boundary_uniform.py)."""
import numpy as np
import pytest

from oracle.oracle import boundary_rows, to_complex_blocks
from tailor_gb300.case import make_case
from tests.helpers import deterministic_vector, matrix_free_action


@pytest.fixture(scope="module")
def small(oracle):
    case = make_case(24, 16)
    return case, oracle.full(case)


def test_structure(small):
    case, r = small
    S = (case.qy + 1) * (case.qz + 1)
    assert r["row_ptr"][-1] == case.nodes * S
    for n in range(case.nodes):
        cols = r["col"][r["row_ptr"][n]:r["row_ptr"][n + 1]]
        assert np.all(np.diff(cols) > 0)
    assert r["spatial"].shape[0] == case.nodes * S


def test_matrix_free_action(small, oracle):
    case, r = small
    x = deterministic_vector(case.ny, case.nz)
    mref, lref = matrix_free_action(case, r["metrics"], r["derivs"], oracle, x)
    nb = case.nodes
    ident = np.arange(nb + 1, dtype=np.int32)
    m = oracle.spmv(ident, ident[:-1], r["mass"], x)
    l = oracle.spmv(r["row_ptr"], r["col"], r["spatial"], x)
    assert np.linalg.norm(m - mref) <= 2e-13 * max(1.0, np.linalg.norm(mref))
    assert np.linalg.norm(l - lref) <= 2e-11 * max(1.0, np.linalg.norm(lref))


def test_boundary_rows_oracle(small):
    case, r = small
    mass = to_complex_blocks(r["mass"]); sp = to_complex_blocks(r["spatial"])
    A, B, info = boundary_rows(case, r["metrics"], r["row_ptr"], r["col"], mass, sp)
    ny = case.ny
    # 1 incoming (u_n - c) and 3 neutral modes per far-field node for V=W=0
    assert info["per_node"] == [1] * case.nz
    assert info["neutral"] == 3 * case.nz
    for j in range(case.nz):
        node = j * ny
        ks = slice(r["row_ptr"][node], r["row_ptr"][node + 1])
        assert np.array_equal(A[ks, 0, :], -sp[ks, 0, :])   # continuity row kept
        for c in range(1, 5):
            row = A[ks, c, :].copy()
            k_own = np.where(r["col"][ks] == node)[0][0]
            row[k_own, c] -= 1.0
            assert np.all(row == 0)
        assert np.all(B[node, 1:, :] == 0)
    interior = 1
    ks = slice(r["row_ptr"][interior], r["row_ptr"][interior + 1])
    assert np.array_equal(A[ks], -sp[ks])


def test_uniform_flow_counts(oracle):
    # test_boundary_uniform.py: (rho, U, V, W, T) = (1, 1, 0, 0, 1)
    case = make_case(24, 16)
    case.baseflow[:] = 0.0
    case.baseflow[:, 0, 0] = 1.0
    case.baseflow[:, 1, 0] = 1.0
    case.baseflow[:, 4, 0] = 1.0
    r = oracle.full(case)
    A, B, info = boundary_rows(case, r["metrics"], r["row_ptr"], r["col"],
                               to_complex_blocks(r["mass"]), to_complex_blocks(r["spatial"]))
    assert info["per_node"] == [1] * case.nz
    assert info["neutral"] == 3 * case.nz
