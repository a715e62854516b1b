"""Generate the FD-q rule tables shipped with the package.

The tables are produced by the reference project's own rule generator
(src/Python/fdq_nodes.py: ``calculate_fdq_rule`` for the bounded wall-normal
direction, fdq_nodes.py:280-304, and ``calculate_periodic_fdq_rule`` for the
periodic spanwise direction, fdq_nodes.py:307-353).  The generator's HDF5
cache layer is not used, so ``h5py`` is replaced by an empty stub module.

Usage (in a checkout that has the reference sources)::

    python tailor_gb300/rules/make_rules.py /path/to/reference [N_q ...]

Each table is written as ``N<N>_q<q>.npz`` (bounded, N+1 nodes) or
``N<N>_q<q>p.npz`` (periodic, N nodes) with the arrays ``nodes``,
``stencil_indices``, ``stencil_offsets`` and ``weights`` (d0, d1, d2).
"""
import sys
import time
import types
from pathlib import Path

import numpy as np

BOUNDED = [(11, 10), (15, 10), (23, 10), (59, 10), (99, 10), (149, 10),
           (199, 10), (299, 10), (15, 4)]
PERIODIC = [(8, 6), (10, 6), (12, 6), (16, 6), (32, 6), (50, 6), (64, 6),
            (128, 6), (192, 6), (12, 4)]


def main() -> None:
    reference = Path(sys.argv[1])
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    sys.path.insert(0, str(reference))
    from src.Python import fdq_nodes  # noqa: E402

    out = Path(__file__).resolve().parent
    wanted = set(sys.argv[2:])
    for n, q in PERIODIC:
        name = f"N{n}_q{q}p"
        if wanted and name not in wanted:
            continue
        rule = fdq_nodes.calculate_periodic_fdq_rule(n, q)
        _save(out / f"{name}.npz", rule)
    for n, q in BOUNDED:
        name = f"N{n}_q{q}"
        if wanted and name not in wanted:
            continue
        t0 = time.time()
        rule = fdq_nodes.calculate_fdq_rule(n, q)
        _save(out / f"{name}.npz", rule)
        print(f"{name}: {time.time() - t0:.1f} s", flush=True)


def _save(path: Path, rule) -> None:
    np.savez_compressed(
        path,
        nodes=np.asarray(rule.nodes, dtype=np.float64),
        stencil_indices=np.asarray(rule.stencil_indices, dtype=np.int64),
        stencil_offsets=np.asarray(rule.stencil_offsets, dtype=np.int64),
        weights=np.asarray(rule.weights, dtype=np.float64),
        periodic=np.int64(1 if rule.topology == "periodic" else 0),
        period=np.float64(rule.period),
    )


if __name__ == "__main__":
    main()
