"""HDF5 files the reference writes: prepared FD-q cases and eigen results.

* ``write_prepared(path, case, source)`` -- the prepared schema-2 case of
  interpolate.py:355-437 (root attributes, natural-order complex /grid and
  /baseflow in PETSc's layout [N][components][2] with ``complex = 1``, and
  both rules under /discretization), readable by ``prepare.load_prepared``
  and by the reference's ``Prepare::initialize``.  The rule digests are
  SHA-256 of the rule arrays (the reference hashes its own rule cache
  files, which this package does not keep).
* ``write_eigen_output(path, ...)`` -- the result schema 1 of
  EigenOutput.cpp:85-304: root attributes, /grid, /baseflow, /spectrum
  (lambda, omega = i lambda, residual) and /modes/mode_NNN in natural order,
  each mode normalised to unit 2-norm and rotated so that its largest entry
  (the first one, on ties) is real and positive (EigenOutput.cpp:36-82).
"""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np

from . import h5
from .case import Case
from .rules import Rule

_CPLX = {"complex": np.uint8(1)}


def _sha256(data: bytes) -> str:
    return hashlib.sha256(data).hexdigest()


def _rule_group(w: h5.WGroup, name: str, rule: Rule, log_error=None) -> None:
    g = w.group(f"discretization/{name}")
    g.attrs.update({"N": rule.n - (0 if rule.periodic else 1), "q": rule.q,
                    "node_count": rule.n, "topology": "periodic" if rule.periodic else "bounded",
                    "period": float(rule.period)})
    g.dataset("nodes", np.asarray(rule.nodes, dtype=np.float64))
    g.dataset("stencil_indices", np.asarray(rule.indices, dtype=np.int64))
    g.dataset("stencil_offsets", np.asarray(rule.offsets, dtype=np.int64))
    for k in range(3):
        g.dataset(f"weights/d{k}", np.asarray(rule.weights[k], dtype=np.float64))
    g.dataset("diagnostics/log_error",
              np.zeros(rule.n) if log_error is None else np.asarray(log_error, dtype=np.float64))


def _rule_digest(rule: Rule) -> str:
    parts = [np.asarray(rule.nodes, dtype="<f8"), np.asarray(rule.indices, dtype="<i8"),
             np.asarray(rule.offsets, dtype="<i8"), np.asarray(rule.weights, dtype="<f8")]
    return _sha256(b"".join(p.tobytes() for p in parts))


def write_prepared(path: str | Path, case: Case, source: str | Path | None = None) -> Path:
    """Prepared schema-2 FD-q case (interpolate.py:355-437)."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    w = h5.Writer()
    src = Path(source) if source else None
    w.attrs.update({
        "schema_version": 2,
        "interpolation_method": "bounded_y_periodic_z_quintic_bspline",
        "interpolation_version": 3,
        "source_file": src.name if src else "",
        "source_sha256": _sha256(src.read_bytes()) if src and src.is_file() else "",
        "y_rule_sha256": _rule_digest(case.xi),
        "z_rule_sha256": _rule_digest(case.eta),
        "ordering": "k_j_dof",
        "Ny": case.ny, "Nz": case.nz, "q_y": case.qy, "q_z": case.qz,
        "spanwise_periodic": 1,
        "spanwise_period": float(case.spanwise_period),
    })
    w.dataset("grid", np.asarray(case.grid, dtype=np.float64), _CPLX)
    w.dataset("baseflow", np.asarray(case.baseflow, dtype=np.float64), _CPLX)
    _rule_group(w, "y", case.xi)
    _rule_group(w, "z", case.eta)
    w.write(path)
    return path


def fix_mode_phase(mode: np.ndarray) -> np.ndarray:
    """Unit 2-norm, largest entry (first on ties) real and positive."""
    v = np.asarray(mode, dtype=np.complex128)
    nrm = np.linalg.norm(v)
    if not np.isfinite(nrm) or nrm <= 0:
        raise ValueError("Cannot normalize a zero or non-finite eigenmode")
    v = v / nrm
    pivot = v[int(np.argmax(np.abs(v)))]
    if abs(pivot) <= 0:
        raise ValueError("Could not select a deterministic mode phase")
    return v * (np.conj(pivot) / abs(pivot))


def _complex_vec(a: np.ndarray, width: int | None = None) -> np.ndarray:
    a = np.asarray(a, dtype=np.complex128)
    out = np.stack([a.real, a.imag], axis=-1)
    return out.reshape(-1, width, 2) if width else out.reshape(-1, 2)


def write_eigen_output(path: str | Path, case: Case, case_title: str, lam: np.ndarray,
                       residual: np.ndarray, modes: np.ndarray, requested: int,
                       target_lambda: complex) -> Path:
    """Result schema 1 (EigenOutput.cpp:85-304); modes [k][5 N] natural order."""
    k = len(lam)
    if k <= 0:
        raise ValueError("No converged modes are available for output")
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    ph = case.physics
    w = h5.Writer()
    w.attrs.update({
        "schema_version": 1, "case": case_title, "ordering": "k_j_dof",
        "mode_dof": "[rho,u,v,w,T]",
        "lambda_convention": "lambda=-i*omega; A_bc*q=lambda*B_bc*q",
        "xi_boundary": "isothermal_no_slip_wall|characteristic_farfield",
        "eta_boundary": "periodic",
        "Ny": case.ny, "Nz": case.nz, "q_y": case.qy, "q_z": case.qz,
        "alpha_real": float(complex(ph.alpha).real), "alpha_imag": float(complex(ph.alpha).imag),
        "search_center_omega_real": float(complex(ph.omega).real),
        "search_center_omega_imag": float(complex(ph.omega).imag),
        "search_center_lambda_real": float(target_lambda.real),
        "search_center_lambda_imag": float(target_lambda.imag),
        "spanwise_period": float(case.spanwise_period),
        "requested_modes": int(requested), "converged_modes": int(k),
    })
    w.dataset("grid", np.asarray(case.grid, dtype=np.float64), _CPLX)
    w.dataset("baseflow", np.asarray(case.baseflow, dtype=np.float64), _CPLX)
    lam = np.asarray(lam, dtype=np.complex128)
    w.dataset("spectrum/lambda", _complex_vec(lam), _CPLX)
    w.dataset("spectrum/omega", _complex_vec(1j * lam), _CPLX)
    w.dataset("spectrum/residual", _complex_vec(np.asarray(residual, dtype=np.float64)), _CPLX)
    for i in range(k):
        w.dataset(f"modes/mode_{i:03d}", _complex_vec(fix_mode_phase(modes[i]), 5), _CPLX)
    w.write(path)
    with h5.File(path) as f:  # the reference's validateFile checks
        ok = all(x in f for x in ("grid", "baseflow", "spectrum/lambda", "spectrum/omega",
                                  "spectrum/residual", "modes/mode_000"))
        if not ok or "lambda_convention" not in f.attrs or "converged_modes" not in f.attrs:
            raise OSError(f"HDF5 validation failed for {path}")
    return path
