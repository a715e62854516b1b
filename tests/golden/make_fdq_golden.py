"""Regenerate the FD-q fixtures of tests/golden/ from the reference sources.

Run in a checkout that has the reference project (its Python package is
imported; its HDF5 cache layer is not used, so ``h5py`` is replaced by an
empty stub module):

    python tests/golden/make_fdq_golden.py /path/to/reference

Writes
    fdq_n100_q10_notebook.txt  the 101 nodes the reference's own test pins
                               (tests/Python/test_fdq_nodes.py:24-27,
                               NOTEBOOK_N100_Q10, checked there to 2e-9)
    fdq_reference_rules.npz    rules produced by the reference generator
                               (fdq_nodes.py:280-353) for sizes that have
                               no shipped table: bounded N10_q4, N8_q8,
                               N40_q6 and periodic N10_q4p, N24_q6p
                               (nodes, stencil_indices, stencil_offsets,
                               weights, log_error per rule, prefixed by name)
"""
from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BOUNDED = [(10, 4), (8, 8), (40, 6)]
PERIODIC = [(10, 4), (24, 6)]


def main() -> None:
    reference = Path(sys.argv[1])
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    sys.path.insert(0, str(reference))
    from src.Python import fdq_nodes  # noqa: E402
    sys.path.insert(0, str(reference / "tests" / "Python"))
    import test_fdq_nodes  # noqa: E402

    nodes = np.asarray(test_fdq_nodes.NOTEBOOK_N100_Q10, dtype=np.float64)
    (HERE / "fdq_n100_q10_notebook.txt").write_text(
        "".join(f"{v:.17g}\n" for v in nodes))
    arrays = {}
    for n, q in BOUNDED:
        _put(arrays, f"N{n}_q{q}", fdq_nodes.calculate_fdq_rule(n, q))
    for n, q in PERIODIC:
        _put(arrays, f"N{n}_q{q}p", fdq_nodes.calculate_periodic_fdq_rule(n, q))
    np.savez_compressed(HERE / "fdq_reference_rules.npz", **arrays)


def _put(arrays: dict, name: str, rule) -> None:
    arrays[f"{name}_nodes"] = np.asarray(rule.nodes, dtype=np.float64)
    arrays[f"{name}_stencil_indices"] = np.asarray(rule.stencil_indices, dtype=np.int64)
    arrays[f"{name}_stencil_offsets"] = np.asarray(rule.stencil_offsets, dtype=np.int64)
    arrays[f"{name}_weights"] = np.asarray(rule.weights, dtype=np.float64)
    arrays[f"{name}_log_error"] = np.asarray(rule.log_error, dtype=np.float64)


if __name__ == "__main__":
    main()
