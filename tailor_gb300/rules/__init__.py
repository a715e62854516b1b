"""FD-q differentiation rules shipped as data tables.

A rule mirrors the reference's ``FDQRuleData`` (ProblemData.hpp:26-96):
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


def load_rule(node_count: int, q: int, periodic: bool) -> Rule:
    """Load the rule for ``node_count`` nodes of degree ``q``."""
    path = _HERE / f"{rule_name(node_count, q, periodic)}.npz"
    if not path.exists():
        raise FileNotFoundError(
            f"no FD-q rule table {path.name}; generate it with make_rules.py")
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
