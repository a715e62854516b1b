"""Case preparation: structured samples onto FD-q nodes, and prepared-case files.

Two entry points mirror the reference's preparation layer:

* ``prepare_sample(path, q_y, q_z, physics)`` -- the reference's
  ``prepare_fdq_case`` (src/Python/interpolate.py:501-585) without its
  HDF5 cache: read a structured source sample (interpolate.py:170-215),
  take (or generate) the bounded y and periodic z FD-q rules, interpolate
  every grid and base-flow component with the periodic quintic tensor
  spline (interpolate.py:82-157, 220-246) and validate the result
  (interpolate.py:249-337);
* ``load_prepared(path, q_y, q_z, physics)`` -- ``Prepare::initialize``
  (src/CPlusPlus/Prepare.cpp:443-687): read a prepared schema-2 FD-q case
  (attributes, the two rules under /discretization, the natural-order grid
  and base-flow vectors) with the reference's checks and messages.

Both return a :class:`tailor_gb300.case.Case` ready for ``api.Problem``.
The spline itself is SciPy's interpolating B-spline (``make_interp_spline``,
degree 5; not-a-knot along y, periodic along z), the routine the reference
calls, so prepared fields agree with the reference's to rounding.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import h5
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


def quintic_tensor_spline(z_old, y_old, values, z_new, y_new):
    """One real or complex field on a bounded tensor grid onto (z_new, y_new)
    with the exact (s = 0) degree-5 tensor-product spline
    (interpolate.py:31-79, SciPy's RectBivariateSpline as there)."""
    from scipy.interpolate import RectBivariateSpline

    z_old, y_old = np.asarray(z_old, dtype=np.float64), np.asarray(y_old, dtype=np.float64)
    z_new, y_new = np.asarray(z_new, dtype=np.float64), np.asarray(y_new, dtype=np.float64)
    field = np.asarray(values)
    if z_old.ndim != 1 or y_old.ndim != 1:
        raise PrepareError("source logical coordinates must be one-dimensional")
    if z_new.ndim != 1 or y_new.ndim != 1:
        raise PrepareError("target logical coordinates must be one-dimensional")
    if z_old.size < 6 or y_old.size < 6:
        raise PrepareError("quintic B-spline interpolation requires at least 6 nodes per axis")
    if field.shape != (z_old.size, y_old.size):
        raise PrepareError(f"values must have shape ({z_old.size}, {y_old.size}); "
                           f"got {field.shape}")
    if not all(np.all(np.isfinite(a)) for a in (z_old, y_old, z_new, y_new, field)):
        raise PrepareError("spline coordinates and values must be finite")
    if np.any(np.diff(z_old) <= 0.0) or np.any(np.diff(y_old) <= 0.0):
        raise PrepareError("source logical coordinates must be strictly increasing")

    def real(v):
        sp = RectBivariateSpline(z_old, y_old, np.asarray(v, dtype=np.float64), kx=5, ky=5, s=0.0)
        return np.asarray(sp(z_new, y_new, grid=True), dtype=np.float64)

    if np.iscomplexobj(field):
        return real(field.real) + 1j * real(field.imag)
    return real(field)


def periodic_quintic_spline(z_old, y_old, values, z_new, y_new, z_period=2.0,
                            value_translation=0.0):
    """One component [nz_old, ny_old] onto (z_new, y_new): quintic not-a-knot
    spline along y, then a periodic quintic spline along z; a field that is
    periodic up to a constant shift (the spanwise coordinate) is interpolated
    as the periodic remainder plus the shift's linear part
    (interpolate.py:82-157)."""
    from scipy.interpolate import make_interp_spline

    z_old = np.asarray(z_old, dtype=np.float64)
    y_old = np.asarray(y_old, dtype=np.float64)
    z_new = np.asarray(z_new, dtype=np.float64)
    y_new = np.asarray(y_new, dtype=np.float64)
    field = np.asarray(values)
    if z_old.ndim != 1 or y_old.ndim != 1:
        raise PrepareError("source logical coordinates must be one-dimensional")
    if z_new.ndim != 1 or y_new.ndim != 1:
        raise PrepareError("target logical coordinates must be one-dimensional")
    if z_old.size < 6 or y_old.size < 6:
        raise PrepareError("periodic quintic interpolation requires at least 6 nodes per axis")
    if field.shape != (z_old.size, y_old.size):
        raise PrepareError(f"values must have shape {(z_old.size, y_old.size)}; got {field.shape}")
    if not np.isfinite(z_period) or z_period <= 0.0:
        raise PrepareError("z_period must be finite and positive")
    if not all(np.all(np.isfinite(a)) for a in (z_old, y_old, z_new, y_new, field)):
        raise PrepareError("periodic spline coordinates and values must be finite")
    if np.any(np.diff(z_old) <= 0.0) or np.any(np.diff(y_old) <= 0.0):
        raise PrepareError("source logical coordinates must be strictly increasing")
    spacing = z_period / z_old.size
    if float(np.max(np.abs(np.diff(z_old) - spacing))) > 5e-13 * max(1.0, abs(spacing)):
        raise PrepareError("periodic source logical nodes must be uniformly spaced")
    if z_old[-1] >= z_old[0] + z_period:
        raise PrepareError("periodic source nodes must not include the repeated endpoint")
    src_phase = (z_old - z_old[0]) / z_period
    tgt_phase = (z_new - z_old[0]) / z_period
    periodic = field - src_phase[:, None] * value_translation

    def scalar(v):
        along_y = np.asarray(make_interp_spline(y_old, np.asarray(v, dtype=np.float64), k=5,
                                                axis=1)(y_new), dtype=np.float64)
        ext_z = np.concatenate((z_old, [z_old[0] + z_period]))
        ext_v = np.concatenate((along_y, along_y[:1]), axis=0)
        return np.asarray(make_interp_spline(ext_z, ext_v, k=5, bc_type="periodic",
                                             axis=0)(z_new), dtype=np.float64)

    if np.iscomplexobj(periodic):
        out = scalar(periodic.real) + 1j * scalar(periodic.imag)
    else:
        out = scalar(periodic)
    return out + tgt_phase[:, None] * value_translation


def _interpolate(values, z_old, y_old, z_new, y_new, translations=None):
    out = np.empty((z_new.size, y_new.size, values.shape[2]), dtype=np.complex128)
    tr = np.zeros(values.shape[2], dtype=np.complex128) if translations is None else \
        np.asarray(translations, dtype=np.complex128)
    for c in range(values.shape[2]):
        out[..., c] = periodic_quintic_spline(z_old, y_old, values[..., c], z_new, y_new,
                                              2.0, tr[c])
    return out


def _first_derivative(values, rule: Rule, axis: int, translation: float = 0.0):
    """FD-q first derivative along one tensor axis (interpolate.py:249-268)."""
    w = rule.weights[1]
    if axis == 1:
        return np.einsum("zij,ij->zi", values[:, rule.indices], w)
    sampled = values[rule.indices, :]
    if rule.periodic and translation != 0.0:
        rows = np.arange(rule.n)[:, None]
        wraps = (rows + rule.offsets - rule.indices) // rule.n
        sampled = sampled + wraps[:, :, None] * translation
    return np.einsum("izj,iz->ij", sampled, w)


def validate_interpolated(src_grid, src_base, grid, base, y_rule: Rule, z_rule: Rule,
                          period: float) -> float:
    """Positivity, corner preservation and a positive grid Jacobian
    (interpolate.py:271-337); returns the minimum Jacobian."""
    if not (np.all(np.isfinite(grid)) and np.all(np.isfinite(base))):
        raise PrepareError("interpolated grid and baseflow must be finite")
    if np.any(base[..., 0].real <= 0.0):
        raise PrepareError("interpolated density is not strictly positive")
    if np.any(base[..., 4].real <= 0.0):
        raise PrepareError("interpolated temperature is not strictly positive")
    for src, tgt, name in ((src_grid, grid, "grid"), (src_base, base, "baseflow")):
        sc = np.asarray([src[0, 0], src[0, -1], src[-1, 0], src[-1, -1]])
        tc = np.asarray([tgt[0, 0], tgt[0, -1], tgt[-1, 0], tgt[-1, -1]])
        scale = max(1.0, float(np.max(np.abs(sc))))
        err = float(np.max(np.abs(tc - sc)))
        if err > 2e-11 * scale:
            raise PrepareError(f"{name} corner preservation failed: error={err:.3e}")
    py, pz = grid[..., 1].real, grid[..., 2].real
    jac = (_first_derivative(py, y_rule, 1) * _first_derivative(pz, z_rule, 0, period)
           - _first_derivative(py, z_rule, 0) * _first_derivative(pz, y_rule, 1))
    if not np.all(np.isfinite(jac)):
        raise PrepareError("interpolated grid Jacobian contains non-finite values")
    jmin = float(np.min(jac))
    if jmin <= 0.0:
        raise PrepareError(f"interpolated grid Jacobian must be strictly positive; "
                           f"minimum={jmin:.6e}")
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
    g = _interpolate(grid, z_old, y_old, z_rule.nodes, y_rule.nodes, [0.0, 0.0, period])
    b = _interpolate(base, z_old, y_old, z_rule.nodes, y_rule.nodes)
    validate_interpolated(grid, base, g, b, y_rule, z_rule, period)
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
