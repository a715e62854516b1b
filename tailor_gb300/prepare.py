"""Case preparation: structured samples onto FD-q nodes, and prepared-case files.

Two entry points mirror the reference's preparation layer:

* ``prepare_sample(path, q_y, q_z, physics)`` -- the reference's
  ``prepare_fdq_case`` (src/Python/interpolate.py:501-585) without its
  HDF5 cache: read a structured source sample (interpolate.py:170-215),
  take (or generate) the bounded y and periodic z FD-q rules, interpolate
  every grid and base-flow component in the reference's spline spaces
  (quintic, periodic along z and not-a-knot along y; interpolate.py:82-157,
  220-246) and check the result (the checks of interpolate.py:249-337);
* ``load_prepared(path, q_y, q_z, physics)`` -- ``Prepare::initialize``
  (src/CPlusPlus/Prepare.cpp:443-687): read a prepared schema-2 FD-q case
  (attributes, the two rules under /discretization, the natural-order grid
  and base-flow vectors) with the reference's checks and messages.

Both return a :class:`tailor_gb300.case.Case` ready for ``api.Problem``.
The splines are this package's own interpolation operators (``spline``):
each axis becomes one dense matrix and every component is interpolated by
two matrix products.  The spline spaces are the reference's, and the
interpolants are unique, so prepared fields agree with the reference's to
rounding.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import h5, spline
from .case import Case, Physics
from .rules import Rule, RuleError, load_rule, validate_rule


PrepareError = RuleError  # rule and case preparation share one error type


# ---- structured source samples --------------------------------------------

def read_structured_sample(path: str | Path):
    """grid [nz, ny, 3], baseflow [nz, ny, 5] (complex), ny, nz and the
    spanwise period of a structured sample (interpolate.py:170-215)."""
    with h5.File(path) as f:
        if "grid" not in f or "baseflow" not in f:
            raise PrepareError("sample HDF5 must contain /grid and /baseflow")
        try:
            ny, nz = int(f.attrs["Ny"]), int(f.attrs["Nz"])
        except KeyError as e:
            raise PrepareError("sample HDF5 must define root attributes Ny and Nz") from e
        if int(f.attrs.get("spanwise_periodic", 0)) != 1:
            raise PrepareError("sample HDF5 must declare spanwise_periodic=1")
        if "spanwise_period" not in f.attrs:
            raise PrepareError("sample HDF5 must define spanwise_period")
        period = float(f.attrs["spanwise_period"])
        grid_parts = np.asarray(f["grid"][...], dtype=np.float64)
        base_parts = np.asarray(f["baseflow"][...], dtype=np.float64)
    if ny < 6 or nz < 6:
        raise PrepareError("sample Ny and Nz must both be at least 6")
    if not np.isfinite(period) or period <= 0.0:
        raise PrepareError("sample spanwise_period must be finite and positive")
    if grid_parts.shape != (nz, ny, 3, 2):
        raise PrepareError(f"/grid must have shape {(nz, ny, 3, 2)}; got {grid_parts.shape}")
    if base_parts.shape != (nz, ny, 5, 2):
        raise PrepareError(f"/baseflow must have shape {(nz, ny, 5, 2)}; got {base_parts.shape}")
    if not (np.all(np.isfinite(grid_parts)) and np.all(np.isfinite(base_parts))):
        raise PrepareError("sample grid and baseflow must contain only finite values")
    grid = grid_parts[..., 0] + 1j * grid_parts[..., 1]
    base = base_parts[..., 0] + 1j * base_parts[..., 1]
    if np.any(base[..., 0].real <= 0.0):
        raise PrepareError("sample density must be strictly positive")
    if np.any(base[..., 4].real <= 0.0):
        raise PrepareError("sample temperature must be strictly positive")
    return grid, base, ny, nz, period


def _uniform_periodic_phase(z_old: np.ndarray, period: float) -> np.ndarray:
    """Phases (in units of the period) of periodic source nodes, which must
    be uniformly spaced and must not repeat the wrap-around node."""
    n = z_old.size
    h = period / n
    if z_old[-1] - z_old[0] >= period:
        raise PrepareError("periodic source nodes repeat the wrap-around node "
                           "(give the open interval only)")
    if float(np.max(np.abs(np.diff(z_old) - h))) > 5e-13 * max(1.0, abs(h)):
        raise PrepareError("periodic source nodes are not uniformly spaced "
                           f"(expected spacing {h!r})")
    return (z_old - z_old[0]) / period


def tensor_interpolate(z_old, y_old, values, z_new, y_new, period: float = 2.0,
                       shift=0.0) -> np.ndarray:
    """Fields [nz_old, ny_old, ...] on a periodic (z) x bounded (y) tensor grid
    onto (z_new, y_new) with quintic splines: periodic along z, not-a-knot
    along y (spline.periodic_matrix, spline.bounded_matrix).  A component
    that grows by ``shift`` over one period (the spanwise coordinate) is
    interpolated as its periodic part plus the linear growth."""
    z_old = np.asarray(z_old, dtype=np.float64)
    z_new = np.asarray(z_new, dtype=np.float64)
    field = np.asarray(values)
    try:
        w_y = spline.bounded_matrix(y_old, y_new)
        if z_old.ndim != 1 or z_new.ndim != 1:
            raise spline.SplineError("z coordinates must be 1-D arrays")
        if z_old.size < spline.DEGREE + 1:
            raise spline.SplineError("a quintic spline needs 6 or more source nodes per axis, "
                                     f"got {z_old.size}")
    except spline.SplineError as e:
        raise PrepareError(str(e)) from e
    if field.shape[:2] != (z_old.size, w_y.shape[1]):
        raise PrepareError(f"values have shape {field.shape}; the source grid needs "
                           f"({z_old.size}, {w_y.shape[1]}, ...)")
    if not (np.isfinite(period) and period > 0.0):
        raise PrepareError("the spanwise period must be finite and positive")
    if not (np.all(np.isfinite(field)) and np.all(np.isfinite(z_old))
            and np.all(np.isfinite(z_new))):
        raise PrepareError("interpolation inputs must be finite")
    if np.any(np.diff(z_old) <= 0.0):
        raise PrepareError("source coordinates must increase strictly")
    phase_old = _uniform_periodic_phase(z_old, period)
    phase_new = (z_new - z_old[0]) / period
    w_z = spline.periodic_matrix(z_old.size, phase_new)
    growth = np.broadcast_to(np.asarray(shift), field.shape[2:])
    lift = phase_old.reshape((-1,) + (1,) * (field.ndim - 1)) * growth[None, None]
    out = spline.tensor_apply(w_z, field - lift, w_y)
    return out + phase_new.reshape((-1,) + (1,) * (field.ndim - 1)) * growth[None, None]


def _d1_operator(rule: Rule):
    """(D, c): the rule's first-derivative matrix and, for a periodic rule,
    the per-row derivative of the wrap count, so that a field that grows by
    p over one period has the derivative D f + c p."""
    n = rule.n
    d = np.zeros((n, n))
    rows = np.repeat(np.arange(n), rule.indices.shape[1])
    np.add.at(d, (rows, rule.indices.ravel()), rule.weights[1].ravel())
    if not rule.periodic:
        return d, np.zeros(n)
    laps = (np.arange(n)[:, None] + rule.offsets - rule.indices) // n
    return d, np.sum(rule.weights[1] * laps, axis=1)


def check_prepared_fields(src_grid, src_base, grid, base, y_rule: Rule, z_rule: Rule,
                          period: float, y_old, z_old) -> float:
    """Checks on an interpolated case; returns the smallest grid Jacobian.

    * every value finite, density and temperature positive;
    * wherever a target node coincides with a source node (the wall and the
      far field, and any shared spanwise station) the source value is kept,
      within 2e-11 of the field's scale;
    * the Jacobian y_xi z_eta - y_eta z_xi of the target grid, from the
      FD-q first-derivative rules, is finite and positive everywhere."""
    fields = {"grid": (src_grid, grid), "baseflow": (src_base, base)}
    for name, (_, tgt) in fields.items():
        if not np.all(np.isfinite(tgt)):
            raise PrepareError(f"the interpolated {name} has non-finite values")
    for comp, label in ((0, "density"), (4, "temperature")):
        if np.any(base[..., comp].real <= 0.0):
            raise PrepareError(f"the interpolated {label} is not positive everywhere")
    sy = [(int(j), int(np.argmin(np.abs(np.asarray(y_old) - v))))
          for j, v in enumerate(y_rule.nodes)
          if np.min(np.abs(np.asarray(y_old) - v)) <= 1e-14]
    sz = [(int(k), int(np.argmin(np.abs(np.asarray(z_old) - v))))
          for k, v in enumerate(z_rule.nodes)
          if np.min(np.abs(np.asarray(z_old) - v)) <= 1e-14]
    if sy and sz:
        (tj, sj), (tk, sk) = zip(*sy), zip(*sz)
        tj, sj, tk, sk = list(tj), list(sj), list(tk), list(sk)
        for name, (src, tgt) in fields.items():
            a = tgt[np.ix_(tk, tj)]
            b = src[np.ix_(sk, sj)]
            scale = max(1.0, float(np.max(np.abs(b))))
            dev = float(np.max(np.abs(a - b)))
            if dev > 2e-11 * scale:
                raise PrepareError(f"the interpolated {name} moved a source node value by "
                                   f"{dev:.3e}")
    y, z = grid[..., 1].real, grid[..., 2].real      # [nz, ny]
    dxi, _ = _d1_operator(y_rule)
    deta, laps = _d1_operator(z_rule)
    y_xi, z_xi = y @ dxi.T, z @ dxi.T
    y_eta = deta @ y
    z_eta = deta @ z + laps[:, None] * period
    jac = y_xi * z_eta - y_eta * z_xi
    if not np.all(np.isfinite(jac)):
        raise PrepareError("the interpolated grid's Jacobian has non-finite values")
    jmin = float(np.min(jac))
    if jmin <= 0.0:
        raise PrepareError(f"the interpolated grid's Jacobian is not positive "
                           f"(smallest value {jmin:.6e})")
    return jmin


def _interleave(a: np.ndarray) -> np.ndarray:
    """[nz, ny, c] complex -> natural-order [N][c][2] float64."""
    nz, ny, c = a.shape
    out = np.empty((nz * ny, c, 2))
    out[..., 0] = a.real.reshape(-1, c)
    out[..., 1] = a.imag.reshape(-1, c)
    return out


def prepare_sample(path: str | Path, q_y: int = 10, q_z: int = 6,
                   physics: Physics | None = None) -> Case:
    """A structured source sample interpolated onto FD-q nodes
    (interpolate.py:501-585, without the HDF5 cache)."""
    grid, base, ny, nz, period = read_structured_sample(path)
    for name, q in (("q_y", q_y), ("q_z", q_z)):
        if isinstance(q, bool) or not isinstance(q, int):
            raise TypeError(f"{name} must be an integer polynomial degree")
    if not 2 <= q_y <= ny - 1:
        raise PrepareError(f"q_y must satisfy 2 <= q_y <= {ny - 1}")
    if not 2 <= q_z <= nz - 1:
        raise PrepareError(f"q_z must satisfy 2 <= q_z <= {nz - 1}")
    if q_z % 2:
        raise PrepareError("periodic q_z must be even")
    y_rule = load_rule(ny, q_y, periodic=False)
    z_rule = load_rule(nz, q_z, periodic=True)
    y_old = np.linspace(-1.0, 1.0, ny)
    z_old = -1.0 + 2.0 * np.arange(nz) / nz
    g = tensor_interpolate(z_old, y_old, grid, z_rule.nodes, y_rule.nodes, 2.0,
                           np.array([0.0, 0.0, period]))
    b = tensor_interpolate(z_old, y_old, base, z_rule.nodes, y_rule.nodes, 2.0)
    check_prepared_fields(grid, base, g, b, y_rule, z_rule, period, y_old, z_old)
    return Case(ny, nz, q_y, q_z, y_rule, z_rule, period, _interleave(g), _interleave(b),
                physics or Physics())


# ---- prepared schema-2 case files -----------------------------------------

def _dataset(group, gpath: str, name: str, shape: tuple[int, ...]) -> np.ndarray:
    """A rule dataset with the reference's messages (Prepare.cpp:78-111)."""
    path = f"{gpath}/{name}"
    try:
        a = np.asarray(group[name][...])
    except KeyError as e:
        raise PrepareError(f"Failed to load FD-q discretization: Missing HDF5 dataset: "
                           f"{path}") from e
    if a.shape != shape:
        raise PrepareError(f"Failed to load FD-q discretization: Unexpected shape for HDF5 "
                           f"dataset: {path}")
    return a


def _rule_from(group, gpath: str, node_count: int, q: int, periodic: bool,
               period: float) -> Rule:
    s = q + 1
    nodes = _dataset(group, gpath, "nodes", (node_count,)).astype(np.float64)
    idx = _dataset(group, gpath, "stencil_indices", (node_count, s))
    off = _dataset(group, gpath, "stencil_offsets", (node_count, s))
    w = np.stack([_dataset(group, gpath, f"weights/d{k}", (node_count, s)).astype(np.float64)
                  for k in range(3)])
    return Rule(n=node_count, q=q, periodic=periodic, period=period, nodes=nodes,
                indices=np.ascontiguousarray(idx, dtype=np.int32),
                offsets=np.ascontiguousarray(off, dtype=np.int32),
                weights=np.ascontiguousarray(w))


def load_prepared(path: str | Path, q_y: int | None = None, q_z: int | None = None,
                  physics: Physics | None = None) -> Case:
    """A prepared FD-q case file (Prepare.cpp:443-687).  q_y / q_z are the
    configuration's degrees (checked against the file when given)."""
    with h5.File(path) as f:
        a = f.attrs
        try:
            ny, nz = int(a["Ny"]), int(a["Nz"])
            schema, fq_y, fq_z = int(a["schema_version"]), int(a["q_y"]), int(a["q_z"])
            periodic, period = int(a["spanwise_periodic"]), float(a["spanwise_period"])
            ordering = a["ordering"]
        except KeyError as e:
            raise PrepareError(f"Failed to read FD-q metadata: missing attribute {e}") from e
        if ny <= 0 or nz <= 0:
            raise PrepareError("HDF5 attributes Ny and Nz must be positive")
        if schema != 2:
            raise PrepareError(f"Unsupported FD-q schema version {schema}")
        if ordering != "k_j_dof":
            raise PrepareError("FD-q ordering must be k_j_dof")
        if periodic != 1:
            raise PrepareError("FD-q input must declare spanwise_periodic=1")
        if not np.isfinite(period) or period <= 0.0:
            raise PrepareError("FD-q spanwise_period must be finite and positive")
        q_y = fq_y if q_y is None else q_y
        q_z = fq_z if q_z is None else q_z
        if fq_y != q_y or fq_z != q_z:
            raise PrepareError("FD-q q_y/q_z attributes do not match the YAML configuration")
        try:
            gy, gz = f["discretization/y"], f["discretization/z"]
        except KeyError as e:
            raise PrepareError("Failed to load FD-q discretization: missing group") from e
        if int(gy.attrs["node_count"]) != ny or int(gy.attrs["q"]) != q_y:
            raise PrepareError("The /discretization/y metadata is inconsistent")
        if int(gz.attrs["node_count"]) != nz or int(gz.attrs["q"]) != q_z:
            raise PrepareError("The /discretization/z metadata is inconsistent")
        if gy.attrs.get("topology") != "bounded" or gz.attrs.get("topology") != "periodic":
            raise PrepareError("Failed to load FD-q discretization: Expected bounded y and "
                               "periodic z FD-q topologies")
        xi = _rule_from(gy, "/discretization/y", ny, q_y, False, float(gy.attrs["period"]))
        eta = _rule_from(gz, "/discretization/z", nz, q_z, True, float(gz.attrs["period"]))
        validate_rule("xi", xi)
        validate_rule("eta", eta)
        if "baseflow" not in f:
            raise PrepareError("HDF5 dataset /baseflow is missing")
        if "grid" not in f:
            raise PrepareError("HDF5 dataset /grid is missing")
        base = np.asarray(f["baseflow"][...], dtype=np.float64)
        grid = np.asarray(f["grid"][...], dtype=np.float64)
    if base.size != ny * nz * 5 * 2:
        raise PrepareError(f"Unexpected baseflow size: expected {ny * nz * 5}, "
                           f"got {base.size // 2}")
    if grid.size != ny * nz * 3 * 2:
        raise PrepareError(f"Unexpected grid size: expected {ny * nz * 3}, got {grid.size // 2}")
    return Case(ny, nz, q_y, q_z, xi, eta, period, grid.reshape(ny * nz, 3, 2),
                base.reshape(ny * nz, 5, 2), physics or Physics())
