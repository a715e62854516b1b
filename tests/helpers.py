"""Shared helpers for the parity tests."""
from __future__ import annotations

import numpy as np

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


def read_lns_gold() -> np.ndarray:
    v = np.loadtxt(GOLDEN / "lns_coefficients_gold.txt")
    return v.reshape(2, 11, 5, 5)


def read_transform_gold():
    v = np.loadtxt(GOLDEN / "lns_transform_gold.txt")
    c = (v[:, 0] + 1j * v[:, 1]).reshape(2, 14, 5, 5)
    return c[:, :7], c[:, 7:]


def transform_inputs():
    from tests.golden.make_golden import transform_parameters, transform_physical
    alphas, phys, mets = [], [], []
    for point in (1, 2):
        a, m = transform_parameters(point)
        alphas.append(a)
        phys.append(transform_physical(point))
        mets.append(m)
    return np.array(alphas), np.array(phys), np.array(mets)


def rel_close(a, b, tol, floor=1.0):
    """|a-b| <= tol * max(floor, |b|) entrywise (the reference's fixture rule)."""
    a = np.asarray(a); b = np.asarray(b)
    return np.all(np.abs(a - b) <= tol * np.maximum(floor, np.abs(b)))


def max_rel_err(a, b, floor=0.0):
    a = np.asarray(a); b = np.asarray(b)
    den = np.maximum(np.abs(b), floor)
    den = np.where(den == 0, 1.0, den)
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0


def deterministic_vector(ny: int, nz: int) -> np.ndarray:
    """fillDeterministicVector (test_global_operator.cpp:77-102)."""
    x = np.zeros((nz, ny, 5), dtype=np.complex128)
    i = np.arange(ny)[None, :, None]
    j = np.arange(nz)[:, None, None]
    c = np.arange(5)[None, None, :]
    phase = 0.017 * (i + 1) + 0.031 * (j + 1) + 0.11 * (c + 1)
    x[:] = (np.sin(phase) + 0.07 * c) + 1j * (0.3 * np.cos(1.7 * phase) - 0.02 * c)
    return x.reshape(-1)


def matrix_free_action(case, metrics, derivs, oracle_obj, x):
    """computeReferenceAction (test_global_operator.cpp:105-222): the
    stencil-by-stencil action of M_Gamma and L on x, independent of BSR."""
    ny, nz = case.ny, case.nz
    xi, eta = case.xi, case.eta
    sx, se = xi.q + 1, eta.q + 1
    X = x.reshape(nz, ny, 5)
    ph = oracle_obj.physics(case.physics)
    mass = np.zeros_like(X)
    spatial = np.zeros_like(X)
    lib = oracle_obj.lib
    for j in range(nz):
        for i in range(ny):
            n = j * ny + i
            q = np.zeros(50)
            q[0:5] = case.baseflow[n, :, 0]
            d = derivs[n]
            q[10:15] = d[0:5]; q[15:20] = d[5:10]; q[25:30] = d[10:15]
            q[30:35] = d[15:20]; q[45:50] = d[20:25]
            st, phys = oracle_obj.lns_physical(ph, q.reshape(10, 5))
            assert st == 0
            st, _, curv = oracle_obj.transform(complex(case.physics.alpha), phys,
                                               metrics[n])
            assert st == 0
            G, K0, Kxi, Keta, Vxx, Vxe, Vee = curv
            dxi = np.zeros(5, complex); dxx = np.zeros(5, complex)
            de = np.zeros(5, complex); dee = np.zeros(5, complex)
            dxe = np.zeros(5, complex)
            for s in range(sx):
                col = i + xi.offsets[i, s]
                dxi += xi.weights[1, i, s] * X[j, col]
                dxx += xi.weights[2, i, s] * X[j, col]
            for s in range(se):
                row = (j + eta.offsets[j, s]) % nz
                de += eta.weights[1, j, s] * X[row, i]
                dee += eta.weights[2, j, s] * X[row, i]
                for t in range(sx):
                    col = i + xi.offsets[i, t]
                    dxe += eta.weights[1, j, s] * xi.weights[1, i, t] * X[row, col]
            mass[j, i] = G @ X[j, i]
            spatial[j, i] = (K0 @ X[j, i] + Kxi @ dxi + Keta @ de - Vxx @ dxx
                             - Vee @ dee - Vxe @ dxe)
    return mass.reshape(-1), spatial.reshape(-1)
