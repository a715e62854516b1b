"""Regenerate the FP64 eigenvalue fixtures of the benchmarked configurations.

The reference stores no spectrum for any case, so the eigenvalues the GPU
forms are judged against come from the CPU oracle: the C restatement of the
assembly, the boundary rows with LAPACK zggev, and SuperLU + ARPACK shift-
and-invert in FP64 (oracle/oracle.py).  Run from the repository root:

    python tests/golden/make_eig_golden.py c1     # 100 x 50, nev 8
    python tests/golden/make_eig_golden.py c2     # 200 x 128, nev 16

Writes <name>_eigs.txt: one "re im residual" line per eigenvalue, nearest
the target first.

* c1: Ny 100 (q 10) x Nz 50 (q 6), bump 0.05, Re 1000, Mach 0.5,
  alpha 2.43, omega 0 (target lambda 0), nev 8;
* c2: Ny 200 x Nz 128, bump 0.08, Re 1000, Mach 0.5, alpha 1.8,
  omega 0.3 + 0.01i (target 0.01 - 0.3i), nev 16.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

CONFIGS = {
    "c1": dict(ny=100, nz=50, amplitude=0.05, alpha=2.43, omega=0j, nev=8),
    "c2": dict(ny=200, nz=128, amplitude=0.08, alpha=1.8, omega=complex(0.3, 0.01), nev=16),
}


def case_of(name: str):
    from tailor_gb300.case import Physics, make_case
    c = CONFIGS[name]
    ph = Physics(alpha=c["alpha"], omega=c["omega"], nev=c["nev"], tol=1e-10)
    return make_case(c["ny"], c["nz"], amplitude=c["amplitude"], physics=ph)


def main() -> None:
    from oracle.oracle import Oracle, boundary_rows, eigen_oracle, to_complex_blocks
    from tailor_gb300.case import target_lambda
    name = sys.argv[1]
    case = case_of(name)
    t = time.time()
    r = Oracle().full(case)
    A, B, _ = boundary_rows(case, r["metrics"], r["row_ptr"], r["col"],
                            to_complex_blocks(r["mass"]), to_complex_blocks(r["spatial"]))
    lam, _, res = eigen_oracle(r["row_ptr"], r["col"], A, B, case.nodes,
                               target_lambda(case.physics.omega), case.physics.nev)
    ny, nz = case.ny, case.nz
    with open(HERE / f"{name}_{ny}x{nz}_eigs.txt", "w") as f:
        for l, e in zip(lam, res):
            f.write(f"{l.real:.17g} {l.imag:.17g} {e:.3e}\n")
    print(f"{name}: {time.time() - t:.1f} s, max residual {max(res):.2e}")


if __name__ == "__main__":
    main()
