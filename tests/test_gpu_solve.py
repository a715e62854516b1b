"""Shift-and-invert Krylov-Schur on the GPU against the FP64 oracle
(SuperLU + ARPACK on the oracle's own A_bc, B_bc): every reported
eigenvalue within |dlambda|/|lambda| <= 1e-8 of an oracle eigenvalue and
with relative residual ||A x - lambda B x|| / (|lambda| ||x||) <= 1e-10
(EigenSolver.cpp:77-82), for the FP64 drop-in form and for the mixed
form (complex64 factorisation + FP64 refinement)."""
import numpy as np
import pytest

from oracle.oracle import boundary_rows, eigen_oracle, to_complex_blocks
from tailor_gb300 import api
from tailor_gb300.case import Physics, make_case

pytestmark = pytest.mark.gpu


def _oracle_eigs(oracle, case, sigma, nev):
    ref = oracle.full(case)
    A, B, _ = boundary_rows(case, ref["metrics"], ref["row_ptr"], ref["col"],
                            to_complex_blocks(ref["mass"]), to_complex_blocks(ref["spatial"]))
    lam, _, res = eigen_oracle(ref["row_ptr"], ref["col"], A, B, case.nodes, sigma, nev)
    return lam, res


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("shape", [(24, 16), (60, 32)], ids=["24x16", "60x32"])
def test_eigen_parity(gpu_lib, oracle, precision, shape):
    ny, nz = shape
    case = make_case(ny, nz, physics=Physics(alpha=1.2, omega=complex(0.3, 0.01), nev=6))
    sigma = complex(case.physics.omega.imag, -case.physics.omega.real)
    lam_ref, res_ref = _oracle_eigs(oracle, case, sigma, 10)
    with api.Problem(case) as prob:
        api.run_pipeline(prob)
        sol = api.EigenSolver(prob).solve(precision=precision)
    d = sol.diag
    assert d["converged"] >= 6 and d["reason"] == 1
    assert abs(complex(d["target_re"], d["target_im"]) - sigma) == 0
    assert np.all(sol.residual <= 1e-10), sol.residual
    for lam in sol.lam:
        err = np.min(np.abs(lam_ref - lam)) / abs(lam)
        assert err <= 1e-8, (lam, err, lam_ref)
    # the nev eigenvalues nearest the target, like EPS_TARGET_MAGNITUDE
    dist = np.sort(np.abs(lam_ref - sigma))[:6]
    assert np.allclose(np.sort(np.abs(sol.lam - sigma)), dist, rtol=1e-8)


@pytest.mark.parametrize("kw", [dict(persistent_solve=True), dict(cuda_core_schur=True),
                                dict(precision=0, persistent_solve=True), dict(solve_block=512),
                                dict(solve_block=128), dict(refinement="gmres")],
                         ids=["persistent", "cuda-core-schur", "fp64-persistent", "block512",
                              "block128", "gmres-ir"])
def test_solver_variants_agree(gpu_lib, kw):
    """The persistent (cooperative, grid-barrier) triangular solve, the
    CUDA-core Schur update and the other diagonal-block sizes give the
    default path's eigenvalues."""
    case = make_case(60, 32, physics=Physics(alpha=1.2, omega=complex(0.3, 0.01), nev=6))
    prec = kw.pop("precision", 1)
    with api.Problem(case) as prob:
        api.run_pipeline(prob)
        ref = api.EigenSolver(prob).solve(precision=prec)
        alt = api.EigenSolver(prob).solve(precision=prec, **kw)
    assert np.all(alt.residual <= 1e-10)
    for lam in alt.lam:
        assert np.min(np.abs(ref.lam - lam)) <= 1e-8 * abs(lam)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_cluster_panel_is_bitwise_the_single_cta_panel(gpu_lib, precision):
    """The 8-CTA cluster panel picks the same pivots and does the same
    arithmetic as the one-CTA panel: identical eigenvalues to the bit."""
    case = make_case(60, 32, physics=Physics(alpha=1.2, omega=complex(0.3, 0.01), nev=6))
    with api.Problem(case) as prob:
        api.run_pipeline(prob)
        a = api.EigenSolver(prob).solve(precision=precision, cluster_panel=-1)
        b = api.EigenSolver(prob).solve(precision=precision, cluster_panel=1)
    assert np.array_equal(a.lam, b.lam)
