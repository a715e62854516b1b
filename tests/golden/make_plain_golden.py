"""Regenerate the plain-FP64 eigenvalue fixtures of the sweep workloads.

At the sizes of the sweeps (300 x 192, 288 000 unknowns per point) the CPU
oracle (SuperLU + ARPACK) does not finish in useful time, so their
reference eigenvalues come from this library's plain FP64 form -- the
drop-in form, whose eigenvalues are pinned to the CPU oracle at 100 x 50
and 200 x 128 (tests/golden/c1_100x50_eigs.txt, c2_200x128_eigs.txt) and on
the reference's shipped case.  Needs a CUDA GPU.  Run from the repository
root:

    python tests/golden/make_plain_golden.py c5     # 32 points, ~12 min

Writes c5_300x192_plain_eigs.txt: per point one line
"alpha reynolds re_1 im_1 res_1 ... re_8 im_8 res_8", nearest the target
first.  The points and the case are those of tailor_gb300.neutral_sweep
(Mach 0.7, alpha on 8 values in [0.5, 3.5], Re on 4 values in
[800, 2400], nev 8, tol 1e-10, target lambda 0).
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))


def main() -> None:
    from tailor_gb300 import api
    from tailor_gb300.neutral_sweep import c5_case, c5_points
    name = sys.argv[1]
    if name != "c5":
        raise SystemExit("usage: make_plain_golden.py c5")
    case = c5_case()
    rows = []
    t = time.time()
    with api.Problem(case) as p:
        for (_, alpha, re) in c5_points():
            p.set_physics(type(case.physics)(**{**case.physics.__dict__, "alpha": alpha,
                                                "reynolds": re}))
            api.run_pipeline(p)
            sol = api.EigenSolver(p).solve(nev=8, ncv=32, precision=0)
            order = np.argsort(np.abs(sol.lam))
            row = [alpha, re]
            for k in order:
                row += [sol.lam[k].real, sol.lam[k].imag, sol.residual[k]]
            rows.append(row)
            print(f"alpha {alpha:.4f} Re {re:.1f}: {time.time() - t:.1f} s", flush=True)
    with open(HERE / "c5_300x192_plain_eigs.txt", "w") as f:
        for row in rows:
            f.write(" ".join(f"{v:.17g}" for v in row) + "\n")


if __name__ == "__main__":
    main()
