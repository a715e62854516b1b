"""FD-q differentiation rules: shipped data tables, or generated on demand.

Tables for the benchmark grids ship with the package; any other size is
generated by the library's host generator (``tlr_fdq_rule``, the
reference's fdq_nodes.py:280-353 construction).  A rule mirrors the reference's ``FDQRuleData`` (ProblemData.hpp:26-96):
``nodes[n]``, ``stencil_indices[n][q+1]`` (wrapped node index),
``stencil_offsets[n][q+1]`` (unwrapped displacement) and
``weights[3][n][q+1]`` (d0, d1, d2), all row-major over (row, slot).
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent


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
