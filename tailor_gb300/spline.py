"""Quintic interpolation operators for case preparation.

Every spline the preparation step needs is linear in the sampled data and
depends only on the source and target coordinates, which are shared by all
components of the grid and the base flow.  So each axis is turned once into
a dense interpolation matrix W (targets x sources), and a whole field is
interpolated by two matrix products, W_z . F . W_y^T.

Two spline spaces are used, both of degree 5:

* bounded axes: the interpolating spline with "not-a-knot" ends, i.e. simple
  knots at every source node except the two next to each end, and the end
  knots repeated six times.  The collocation system is solved once;
* periodic axes with uniformly spaced source nodes: the periodic spline with
  simple knots at the nodes.  Its collocation matrix is circulant (the
  centred quintic B-spline takes 1/120, 26/120, 66/120, 26/120, 1/120 at
  the integers), so its inverse comes from one FFT.

The interpolants are unique, so any routine that interpolates in the same
spline spaces (SciPy's ``make_interp_spline``, FITPACK) returns the same
functions up to rounding.  B-spline values are computed with the
triangular recursion of de Boor / Cox (Piegl & Tiller, The NURBS Book,
2nd ed., algorithm A2.2).
"""
from __future__ import annotations

import numpy as np

DEGREE = 5


class SplineError(ValueError):
    """Coordinates that admit no quintic interpolation operator."""


def _nonzero_basis(knots: np.ndarray, span: np.ndarray, x: np.ndarray, k: int) -> np.ndarray:
    """Values of the k + 1 B-splines of degree k that are non-zero on the
    knot interval [knots[span], knots[span + 1]) at x; column r belongs to
    B_{span - k + r}.  Vectorised over the points."""
    m = x.size
    vals = np.zeros((m, k + 1))
    vals[:, 0] = 1.0
    left = np.zeros((m, k + 1))
    right = np.zeros((m, k + 1))
    for j in range(1, k + 1):
        left[:, j] = x - knots[span + 1 - j]
        right[:, j] = knots[span + j] - x
        carry = np.zeros(m)
        for r in range(j):
            t = vals[:, r] / (right[:, r + 1] + left[:, j - r])
            vals[:, r] = carry + right[:, r + 1] * t
            carry = left[:, j - r] * t
        vals[:, j] = carry
    return vals


def _check_axis(x: np.ndarray, what: str) -> np.ndarray:
    x = np.asarray(x, dtype=np.float64)
    if x.ndim != 1:
        raise SplineError(f"{what} coordinates must be a 1-D array")
    if not np.all(np.isfinite(x)):
        raise SplineError(f"{what} coordinates must be finite")
    return x


def bounded_matrix(x_old, x_new) -> np.ndarray:
    """W [len(x_new), len(x_old)]: samples at the strictly increasing x_old
    -> values of their not-a-knot quintic interpolant at x_new (inside
    [x_old[0], x_old[-1]])."""
    x_old = _check_axis(x_old, "source")
    x_new = _check_axis(x_new, "target")
    n, k = x_old.size, DEGREE
    if n < k + 1:
        raise SplineError(f"a quintic spline needs 6 or more source nodes per axis, got {n}")
    if np.any(np.diff(x_old) <= 0.0):
        raise SplineError("source coordinates must increase strictly")
    knots = np.concatenate((np.full(k + 1, x_old[0]), x_old[3:n - 3], np.full(k + 1, x_old[-1])))

    def collocation(x):
        span = np.clip(np.searchsorted(knots, x, side="right") - 1, k, n - 1)
        vals = _nonzero_basis(knots, span, x, k)
        a = np.zeros((x.size, n))
        rows = np.repeat(np.arange(x.size), k + 1)
        cols = (span[:, None] - k + np.arange(k + 1)).ravel()
        np.add.at(a, (rows, cols), vals.ravel())
        return a

    # coefficients = A_old^{-1} samples, values = A_new coefficients
    return np.linalg.solve(collocation(x_old).T, collocation(x_new).T).T


def periodic_matrix(n_old: int, phase_new) -> np.ndarray:
    """W [len(phase_new), n_old]: samples at the uniform periodic nodes
    phase = j / n_old (j = 0 .. n_old - 1, in units of the period) -> values
    of their periodic quintic interpolant at phase_new (any real numbers;
    read modulo 1)."""
    phase_new = _check_axis(phase_new, "target")
    if n_old < DEGREE + 1:
        raise SplineError(f"a quintic spline needs 6 or more source nodes per axis, got {n_old}")
    # node value of the centred quintic B-spline at offsets 0, +-1, +-2
    stencil = np.zeros(n_old)
    stencil[0] = 66.0 / 120.0
    stencil[1] = stencil[-1] = 26.0 / 120.0
    stencil[2] = stencil[-2] = 1.0 / 120.0
    symbol = np.fft.fft(stencil).real          # >= 16/120 > 0: always solvable
    inv_col = np.fft.ifft(1.0 / symbol).real   # first column of the inverse
    cinv = inv_col[(np.arange(n_old)[:, None] - np.arange(n_old)[None, :]) % n_old]

    # evaluation: u = phase * n in node units; the six B-splines centred at
    # floor(u) - 2 .. floor(u) + 3 cover the interval [floor(u), floor(u) + 1)
    u = np.mod(phase_new * n_old, n_old)
    base = np.floor(u)
    frac = u - base
    knots = np.arange(-DEGREE, DEGREE + 2, dtype=np.float64)    # -5 .. 6
    span = np.full(u.size, DEGREE)                               # interval [0, 1)
    vals = _nonzero_basis(knots, span, frac, DEGREE)             # B-splines starting at -5..0
    e = np.zeros((u.size, n_old))
    rows = np.repeat(np.arange(u.size), DEGREE + 1)
    # the B-spline whose knots start at s (s = -5..0) is centred at s + 3
    centres = (base.astype(np.int64)[:, None] + np.arange(-DEGREE, 1)[None, :] + 3) % n_old
    np.add.at(e, (rows, centres.ravel()), vals.ravel())
    return e @ cinv


def tensor_apply(w_z: np.ndarray, values: np.ndarray, w_y: np.ndarray) -> np.ndarray:
    """values [nz_old, ny_old, ...] -> [nz_new, ny_new, ...] through the two
    axis operators (real and complex data alike)."""
    return np.einsum("zZ,Zy...,Yy->zY...", w_z, values, w_y, optimize=True)
