"""FD-q differentiation rules: shipped data tables, or generated on demand.

Tables for the benchmark grids ship with the package; any other size is
generated by the library's host generator (``tlr_fdq_rule``, the
reference's fdq_nodes.py:280-353 construction).  ``save_rule`` /
``load_rule_file`` / ``load_or_create_rule`` keep rules in the reference's
HDF5 rule-cache format (schema 2, fdq_nodes.py:458-627), and
``validate_rule`` applies the checks the reference's C++ loader runs on
every rule (Prepare.cpp:328-437).  A rule mirrors the reference's ``FDQRuleData`` (ProblemData.hpp:26-96):
``nodes[n]``, ``stencil_indices[n][q+1]`` (wrapped node index),
``stencil_offsets[n][q+1]`` (unwrapped displacement) and
``weights[3][n][q+1]`` (d0, d1, d2), all row-major over (row, slot).
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
SCHEMA_VERSION = 2


class RuleError(ValueError):
    pass


@dataclass(frozen=True)
class Rule:
    n: int
    q: int
    periodic: bool
    period: float
    nodes: np.ndarray
    indices: np.ndarray
    offsets: np.ndarray
    weights: np.ndarray

    @property
    def stencil_size(self) -> int:
        return self.q + 1


def rule_name(node_count: int, q: int, periodic: bool) -> str:
    """Table name: bounded rules are named by interval count N = nodes - 1."""
    if periodic:
        return f"N{node_count}_q{q}p"
    return f"N{node_count - 1}_q{q}"


def generate_rule(node_count: int, q: int, periodic: bool, period: float = 2.0,
                  with_log_error: bool = False):
    """Generate the rule with the library's host generator (tlr_fdq_rule).

    Bounded rules have ``node_count - 1`` intervals on [-1, 1]; periodic
    rules ``node_count`` uniform nodes on [-period/2, period/2).  Raises
    ``ValueError`` for invalid sizes and ``RuntimeError`` when the node
    solve or the rule checks fail.  With ``with_log_error`` the equal-error
    amplitudes are returned too.
    """
    import ctypes
    from .. import _lib
    lib = _lib.load()
    s = q + 1
    nodes = np.zeros(node_count)
    idx = np.zeros((node_count, s), dtype=np.int32)
    off = np.zeros((node_count, s), dtype=np.int32)
    w = np.zeros((3, node_count, s))
    le = np.zeros(node_count)
    rc = lib.tlr_fdq_rule(int(node_count), int(q), int(bool(periodic)), float(period),
                          nodes.ctypes.data, idx.ctypes.data, off.ctypes.data, w.ctypes.data,
                          le.ctypes.data)
    if rc:
        msg = lib.tlr_last_error(None).decode()
        raise (ValueError if rc == 1 else RuntimeError)(f"FD-q rule N{node_count}_q{q}: {msg}")
    rule = Rule(n=node_count, q=q, periodic=bool(periodic),
                period=float(period) if periodic else 2.0, nodes=nodes,
                indices=idx, offsets=off, weights=w)
    return (rule, le) if with_log_error else rule


def load_rule(node_count: int, q: int, periodic: bool) -> Rule:
    """The rule for ``node_count`` nodes of degree ``q``: the shipped table
    when there is one, else a freshly generated rule."""
    path = _HERE / f"{rule_name(node_count, q, periodic)}.npz"
    if not path.exists():
        return generate_rule(node_count, q, periodic)
    data = np.load(path)
    nodes = np.asarray(data["nodes"], dtype=np.float64)
    rule = Rule(
        n=int(nodes.size), q=q, periodic=bool(int(data["periodic"])),
        period=float(data["period"]), nodes=nodes,
        indices=np.ascontiguousarray(data["stencil_indices"], dtype=np.int32),
        offsets=np.ascontiguousarray(data["stencil_offsets"], dtype=np.int32),
        weights=np.ascontiguousarray(data["weights"], dtype=np.float64))
    if rule.n != node_count or rule.periodic != periodic:
        raise ValueError(f"rule table {path.name} does not match request")
    return rule


def available() -> list[str]:
    return sorted(p.stem for p in _HERE.glob("*.npz"))


def validate_rule(name: str, r: Rule) -> None:
    """The rule checks of Prepare.cpp:328-437 with its messages: metadata,
    node order, stencil indices and offsets, finite weights, the evaluation
    node in every stencil, and exactness on 1, x, x^2 (5e-9 x max(1, |exact|))."""
    n, s = r.n, r.q + 1
    if not (n >= 3 and 2 <= r.q < n):
        raise RuleError(f"{name} FD-q metadata must satisfy node_count > q >= 2")
    if not np.isfinite(r.period) or r.period <= 0:
        raise RuleError(f"{name} FD-q period must be finite and positive")
    if r.periodic and r.q % 2:
        raise RuleError(f"{name} periodic FD-q degree must be even")
    for row in range(n):
        x = r.nodes[row]
        if not np.isfinite(x):
            raise RuleError(f"{name} FD-q node {row} is not finite")
        if row > 0 and not x > r.nodes[row - 1]:
            raise RuleError(f"{name} FD-q nodes must be strictly increasing")
        cols, offs = r.indices[row], r.offsets[row]
        for c, o in zip(cols, offs):
            if not 0 <= c < n:
                raise RuleError(f"{name} FD-q row {row} contains out-of-range index {c}")
            if (row + o) % n != c if r.periodic else row + o != c:
                kind = "periodic" if r.periodic else "bounded"
                raise RuleError(f"{name} {kind} row {row} has inconsistent stencil index/offset")
        if not np.all(np.isfinite(r.weights[:, row])):
            raise RuleError(f"{name} FD-q weight is not finite at row {row}")
        if row not in cols:
            raise RuleError(f"{name} FD-q stencil row {row} does not contain its evaluation node")
        xs = x + offs * (r.period / n) if r.periodic else r.nodes[cols]
        for d in range(3):
            for pw in range(3):
                approx = float(np.sum(r.weights[d, row] * xs ** pw))
                exact = [[1.0, x, x * x], [0.0, 1.0, 2.0 * x], [0.0, 0.0, 2.0]][d][pw]
                if abs(approx - exact) > 5e-9 * max(1.0, abs(exact)):
                    raise RuleError(f"{name} FD-q order-{d} weights fail degree-{pw} "
                                       f"polynomial check at row {row}")


def save_rule(rule: Rule, path: str | Path, log_error=None) -> Path:
    """Write a rule in the reference's HDF5 cache format, schema 2
    (fdq_nodes.py:470-512), after validating it; written atomically."""
    from .. import h5
    validate_rule("eta" if rule.periodic else "xi", rule)
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    w = h5.Writer()
    w.attrs.update({"schema_version": SCHEMA_VERSION,
                    "N": rule.n if rule.periodic else rule.n - 1, "q": rule.q,
                    "node_count": rule.n, "stencil_size": rule.q + 1,
                    "topology": "periodic" if rule.periodic else "bounded",
                    "period": float(rule.period)})
    w.dataset("nodes", np.asarray(rule.nodes, dtype=np.float64))
    w.dataset("stencil_indices", np.asarray(rule.indices, dtype=np.int64))
    w.dataset("stencil_offsets", np.asarray(rule.offsets, dtype=np.int64))
    for k in range(3):
        w.dataset(f"weights/d{k}", np.asarray(rule.weights[k], dtype=np.float64))
    w.dataset("diagnostics/log_error",
              np.zeros(rule.n) if log_error is None else np.asarray(log_error, dtype=np.float64))
    w.write(path)
    return path


def load_rule_file(path: str | Path) -> Rule:
    """Read and validate an HDF5 rule cache (fdq_nodes.py:515-564)."""
    from .. import h5
    with h5.File(path) as f:
        a = f.attrs
        ver = int(a.get("schema_version", -1))
        if ver != SCHEMA_VERSION:
            raise RuleError(f"unsupported FD-q schema version {ver}; expected {SCHEMA_VERSION}")
        n_int, q, nc = int(a["N"]), int(a["q"]), int(a["node_count"])
        topology, period = str(a["topology"]), float(a["period"])
        periodic = topology == "periodic"
        if nc != (n_int if periodic else n_int + 1):
            raise RuleError("HDF5 node_count attribute is inconsistent")
        if int(a["stencil_size"]) != q + 1:
            raise RuleError("HDF5 stencil_size attribute is inconsistent with q")
        rule = Rule(n=nc, q=q, periodic=periodic, period=period,
                    nodes=np.asarray(f["nodes"][...], dtype=np.float64),
                    indices=np.ascontiguousarray(f["stencil_indices"][...], dtype=np.int32),
                    offsets=np.ascontiguousarray(f["stencil_offsets"][...], dtype=np.int32),
                    weights=np.stack([np.asarray(f[f"weights/d{k}"][...], dtype=np.float64)
                                      for k in range(3)]))
    s = q + 1
    if rule.nodes.shape != (nc,) or rule.indices.shape != (nc, s) or \
            rule.offsets.shape != (nc, s) or rule.weights.shape != (3, nc, s):
        raise RuleError("HDF5 rule arrays have the wrong shape")
    validate_rule("eta" if periodic else "xi", rule)
    return rule


def load_or_create_rule(node_count: int, q: int, periodic: bool, directory: str | Path,
                        period: float = 2.0) -> Rule:
    """The cached rule ``N<N>_q<q>[p].h5`` in directory, or a generated one
    written there when the cache is missing or stale (fdq_nodes.py:567-624)."""
    import sys
    path = Path(directory) / f"{rule_name(node_count, q, periodic)}.h5"
    if path.exists():
        try:
            rule = load_rule_file(path)
            if rule.n != node_count or rule.q != q or rule.periodic != periodic or \
                    (periodic and not np.isclose(rule.period, period)):
                raise RuleError("cached rule metadata does not match")
            return rule
        except (KeyError, OSError, ValueError) as e:
            print(f"FD-q rule cache stale, rebuilding {path}: {e}", file=sys.stderr)
    rule, le = generate_rule(node_count, q, periodic, period, with_log_error=True)
    save_rule(rule, path, le)
    return rule

