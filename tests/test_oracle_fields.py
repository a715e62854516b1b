"""Oracle metrics and derivatives against independent NumPy recomputations.

Restates the reference's regression checks test_metrics.py:73-135 (metrics
by the chain rule, Jacobian range, ten component norms at rtol 5e-11 /
5e-10) and test_baseflow_derivatives.py:61-158 (25 derivative norms at
5e-10), on the synthetic case and on manufactured curved/skewed periodic
grids, plus the input-fault checks of test_metrics.py:268-357 and
test_baseflow_derivatives.py:322-424.
"""
import math

import numpy as np
import pytest

from tailor_gb300.case import make_case


def d_xi(v, rule):   # v [nz, ny]
    return np.einsum("jis,is->ji", v[:, rule.indices], rule.weights[1])


def d_xi2(v, rule):
    return np.einsum("jis,is->ji", v[:, rule.indices], rule.weights[2])


def d_eta(v, rule, translation=0.0, order=1):
    nz = v.shape[0]
    sampled = v[rule.indices, :]                        # [nz, s, ny]
    if translation:
        rows = np.arange(nz)[:, None]
        wraps = (rows + rule.offsets - rule.indices) // nz
        sampled = sampled + wraps[:, :, None] * translation
    return np.einsum("jsi,js->ji", sampled, rule.weights[order])


def numpy_metrics(case):
    ny, nz = case.ny, case.nz
    y = case.grid[:, 1, 0].reshape(nz, ny)
    z = case.grid[:, 2, 0].reshape(nz, ny)
    y_xi, z_xi = d_xi(y, case.xi), d_xi(z, case.xi)
    y_eta = d_eta(y, case.eta)
    z_eta = d_eta(z, case.eta, case.spanwise_period)
    jac = y_xi * z_eta - y_eta * z_xi
    xy, xz, ey, ez = z_eta / jac, -y_eta / jac, -z_xi / jac, y_xi / jac
    dx = lambda v: d_xi(v, case.xi)
    de = lambda v: d_eta(v, case.eta)
    m = [xy, xz, ey, ez,
         xy * dx(xy) + ey * de(xy), xz * dx(xz) + ez * de(xz),
         xz * dx(xy) + ez * de(xy), xy * dx(ey) + ey * de(ey),
         xz * dx(ez) + ez * de(ez), xz * dx(ey) + ez * de(ey)]
    return jac, np.stack([a.reshape(-1) for a in m], 1)


def numpy_derivatives(case, metrics):
    ny, nz = case.ny, case.nz
    out = np.zeros((ny * nz, 25))
    M = [metrics[:, k].reshape(nz, ny) for k in range(10)]
    xy, xz, ey, ez, xyy, xzz, xyz, eyy, ezz, eyz = M
    for f in range(5):
        v = case.baseflow[:, f, 0].reshape(nz, ny)
        vx, vxx = d_xi(v, case.xi), d_xi2(v, case.xi)
        ve, vee = d_eta(v, case.eta), d_eta(v, case.eta, order=2)
        vxe = d_eta(d_xi(v, case.xi), case.eta)
        vals = [xy * vx + ey * ve, xz * vx + ez * ve,
                xy * xy * vxx + 2 * xy * ey * vxe + ey * ey * vee + xyy * vx + eyy * ve,
                xz * xz * vxx + 2 * xz * ez * vxe + ez * ez * vee + xzz * vx + ezz * ve,
                xy * xz * vxx + (xy * ez + ey * xz) * vxe + ey * ez * vee + xyz * vx + eyz * ve]
        for d in range(5):
            out[:, d * 5 + f] = vals[d].reshape(-1)
    return out


def skewed_curved_case(ny=24, nz=16):
    """make_skewed_curved_grid (test_metrics.py:237-265) on our rules."""
    case = make_case(ny, nz)
    xi = case.xi.nodes
    eta = case.eta.nodes
    X, E = np.meshgrid(xi, eta, indexing="xy")
    theta = 2 * math.pi * (E - eta[0]) / case.eta.period
    phase = (E - eta[0]) / case.eta.period
    y = 2.0 * X + 0.03 * X ** 2 + 0.12 * np.sin(theta) + 0.05 * X * np.sin(theta)
    z = case.spanwise_period * phase - 0.15 * X + 0.08 * np.cos(theta) + 0.04 * X * np.cos(theta)
    case.grid[:, 1, 0] = y.reshape(-1)
    case.grid[:, 2, 0] = z.reshape(-1)
    # varying base flow (test_baseflow_derivatives.py:248-319 style)
    case.baseflow[:, 0, 0] = (1.0 + 0.1 * np.sin(y) * np.cos(z)).reshape(-1)
    case.baseflow[:, 1, 0] = np.tanh(y).reshape(-1)
    case.baseflow[:, 2, 0] = (0.01 * np.sin(z) * np.exp(-y * y)).reshape(-1)
    case.baseflow[:, 3, 0] = (0.02 * np.cos(z) * np.exp(-y * y)).reshape(-1)
    case.baseflow[:, 4, 0] = (1.0 + 0.2 * np.exp(-y * y) * (1 + 0.1 * np.cos(z))).reshape(-1)
    return case


@pytest.mark.parametrize("maker", [lambda: make_case(24, 16),
                                   lambda: make_case(60, 32, amplitude=0.08, seed=3),
                                   skewed_curved_case])
def test_oracle_metrics_and_derivatives_match_numpy(oracle, maker):
    case = maker()
    st, m, diag = oracle.metrics(case)
    assert st == 0
    jac, ref = numpy_metrics(case)
    assert math.isclose(diag[0], jac.min(), rel_tol=5e-11)
    assert math.isclose(diag[1], jac.max(), rel_tol=5e-11)
    assert np.allclose(diag[3:], np.linalg.norm(ref, axis=0), rtol=5e-10)
    assert np.allclose(m, ref, rtol=1e-11, atol=1e-11 * np.abs(ref).max())
    st, d, ddiag = oracle.derivatives(case, m)
    assert st == 0
    dref = numpy_derivatives(case, m)
    assert np.allclose(ddiag[1:], np.linalg.norm(dref, axis=0), rtol=5e-10, atol=5e-10)


def test_oracle_metric_faults(oracle):
    case = make_case(24, 16)
    case.grid[:, 1, 0] = 0.0
    case.grid[:, 2, 0] = 0.0
    assert oracle.metrics(case)[0] == 3          # degenerate Jacobian
    case = make_case(24, 16)
    case.grid[5, 1, 1] = 1e-6
    assert oracle.metrics(case)[0] == 4          # complex grid
    case = make_case(24, 16)
    case.grid[7, 2, 0] = np.nan
    assert oracle.metrics(case)[0] == 2          # non-finite


def test_oracle_baseflow_faults(oracle):
    case = make_case(24, 16)
    st, m, _ = oracle.metrics(case)
    bad = make_case(24, 16); bad.baseflow[3, 0, 0] = -1.0
    assert oracle.derivatives(bad, m)[0] == 6    # non-positive density
    bad = make_case(24, 16); bad.baseflow[3, 4, 0] = 0.0
    assert oracle.derivatives(bad, m)[0] == 6    # non-positive temperature
    bad = make_case(24, 16); bad.baseflow[9, 2, 0] = np.nan
    assert oracle.derivatives(bad, m)[0] == 2
    bad = make_case(24, 16); bad.baseflow[9, 1, 1] = 1e-9
    assert oracle.derivatives(bad, m)[0] == 4    # complex base flow
