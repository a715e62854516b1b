"""GPU metrics -> derivatives -> assembly -> boundary rows -> SpMV against
the CPU oracle, entrywise, through the C ABI.

The parity bar is the reference's: assembled M_Gamma and L entrywise to
1e-13 relative (|gpu - oracle| <= 1e-13 |oracle|, and exact zeros where the
oracle has zeros).  Metrics and derivatives use the same bar.  Both sides
evaluate the same expressions without fused multiply-add, so in practice
the arrays agree bit for bit; the test reports the bitwise fraction too.
"""
import numpy as np
import pytest

from oracle.oracle import boundary_rows, to_complex_blocks
from tailor_gb300 import api
from tailor_gb300.case import make_case
from tests.helpers import deterministic_vector, matrix_free_action

pytestmark = pytest.mark.gpu

TOL = 1e-13


def entrywise_ok(gpu, ref, tol=TOL):
    gpu = np.asarray(gpu); ref = np.asarray(ref)
    zero = ref == 0
    if np.any(gpu[zero] != 0):
        return False
    nz = ~zero
    return bool(np.all(np.abs(gpu[nz] - ref[nz]) <= tol * np.abs(ref[nz])))


CASES = [(12, 8, 0.05, 0), (24, 16, 0.05, 0), (60, 32, 0.08, 7), (100, 50, 0.05, 0)]


@pytest.fixture(scope="module", params=CASES, ids=lambda c: f"{c[0]}x{c[1]}")
def run(request, gpu_lib, oracle):
    ny, nz, amp, seed = request.param
    case = make_case(ny, nz, amplitude=amp, seed=seed)
    ref = oracle.full(case)
    prob = api.Problem(case)
    diags = api.run_pipeline(prob)
    yield case, ref, prob, diags
    prob.close()


def test_metrics_parity(run):
    case, ref, prob, d = run
    m = prob.copy_out(api.OUT_METRICS)
    assert entrywise_ok(m, ref["metrics"])
    md = d["metrics"]
    assert md["min_jacobian"] == ref["metric_diag"][0]
    assert md["max_jacobian"] == ref["metric_diag"][1]
    assert np.allclose(md["norms"], ref["metric_diag"][3:], rtol=1e-12)


def test_derivative_parity(run):
    case, ref, prob, d = run
    der = prob.copy_out(api.OUT_DERIVS)
    assert entrywise_ok(der, ref["derivs"])
    assert np.allclose(d["derivatives"]["norms"], ref["deriv_diag"][1:], rtol=1e-12)


def test_operator_parity(run):
    case, ref, prob, d = run
    assert np.array_equal(prob.copy_out(api.OUT_ROW_PTR), ref["row_ptr"])
    assert np.array_equal(prob.copy_out(api.OUT_COL), ref["col"])
    M = prob.copy_out(api.OUT_M)
    Lv = prob.copy_out(api.OUT_L)
    assert entrywise_ok(M, ref["mass"])
    assert entrywise_ok(Lv, ref["spatial"])
    op = d["operator"]
    S = (case.qy + 1) * (case.qz + 1)
    assert op["spatial_used_blocks"] == case.nodes * S
    assert op["mass_used_blocks"] == case.nodes
    assert op["rows"] == 5 * case.nodes and op["block_size"] == 5
    assert np.isclose(op["spatial_frobenius_norm"], np.linalg.norm(ref["spatial"]), rtol=1e-12)
    assert np.isclose(op["mass_frobenius_norm"], np.linalg.norm(ref["mass"]), rtol=1e-12)


def _rowspace_ok(X_gpu, X_ref, tol=1e-10):
    """X_gpu = T X_ref for an invertible 5x5 T (rows of one node)."""
    T, *_ = np.linalg.lstsq(X_ref.T, X_gpu.T, rcond=None)
    T = T.T
    resid = np.linalg.norm(X_gpu - T @ X_ref) / max(1.0, np.linalg.norm(X_gpu))
    sv = np.linalg.svd(T, compute_uv=False)
    return resid <= tol and sv[-1] > 1e-8 * sv[0]


def test_boundary_rows_parity(run):
    case, ref, prob, d = run
    ny, nz = case.ny, case.nz
    rp, col = ref["row_ptr"], ref["col"]
    sp = to_complex_blocks(ref["spatial"]); mass = to_complex_blocks(ref["mass"])
    A_ref, B_ref, info = boundary_rows(case, ref["metrics"], rp, col, mass, sp)
    A = to_complex_blocks(prob.copy_out(api.OUT_A))
    B = to_complex_blocks(prob.copy_out(api.OUT_B))
    bc = d["bc"]
    assert bc["incoming_modes"] == info["incoming"]
    assert bc["neutral_modes"] == info["neutral"]
    assert bc["wall_nodes"] == nz and bc["farfield_nodes"] == nz
    assert bc["min_incoming_per_node"] == min(info["per_node"])
    assert bc["max_incoming_per_node"] == max(info["per_node"])
    far = set(j * ny + ny - 1 for j in range(nz))
    for node in range(case.nodes):
        ks = slice(rp[node], rp[node + 1])
        if node in far:
            Xg = np.concatenate([A[ks].transpose(1, 0, 2).reshape(5, -1), B[node]], 1)
            Xr = np.concatenate([A_ref[ks].transpose(1, 0, 2).reshape(5, -1), B_ref[node]], 1)
            assert _rowspace_ok(Xg, Xr), (node, np.round(B[node].real, 4).tolist(),
                                          np.round(B_ref[node].real, 4).tolist())
            # incoming rows: zero B row and only the node's own columns
            nzero_b = np.where(np.abs(B[node]).sum(1) == 0)[0]
            assert len(nzero_b) == info["per_node"][node // ny]
            for m in nzero_b:
                other = col[ks] != node
                assert np.all(A[ks][other, m, :] == 0)
        else:
            assert np.array_equal(A[ks], A_ref[ks]), node
            assert np.array_equal(B[node], B_ref[node]), node


def test_spmv_parity(run, oracle):
    case, ref, prob, d = run
    x = deterministic_vector(case.ny, case.nz)
    for which, rp, col, val in [(api.TLR_MAT_L, ref["row_ptr"], ref["col"], ref["spatial"])]:
        y = prob.spmv(which, x)
        yo = oracle.spmv(rp, col, val, x)
        assert np.linalg.norm(y - yo) <= 1e-13 * np.linalg.norm(yo)
    nb = case.nodes
    ident = np.arange(nb + 1, dtype=np.int32)
    y = prob.spmv(api.TLR_MAT_M, x)
    yo = oracle.spmv(ident, ident[:-1], ref["mass"], x)
    assert np.linalg.norm(y - yo) <= 1e-14 * np.linalg.norm(yo)
    if case.nodes <= 400:
        mref, lref = matrix_free_action(case, ref["metrics"], ref["derivs"], oracle, x)
        assert np.linalg.norm(prob.spmv(api.TLR_MAT_L, x) - lref) <= 2e-11 * np.linalg.norm(lref)


def test_c2_size_parity(gpu_lib, oracle):
    """Full C2 size (Ny=200, Nz=128): 1 971 200 blocks of L entrywise."""
    case = make_case(200, 128, amplitude=0.08)
    ref = oracle.full(case)
    with api.Problem(case) as prob:
        api.run_pipeline(prob)
        assert entrywise_ok(prob.copy_out(api.OUT_L), ref["spatial"])
        assert entrywise_ok(prob.copy_out(api.OUT_M), ref["mass"])
