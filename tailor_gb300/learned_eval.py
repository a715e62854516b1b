"""Held-out evaluation of the learned start-vector / shift proposal.

    python -m tailor_gb300.learned_eval --ny 100 --nz 50 --train 256 --eval 64

Training and evaluation points are drawn with fixed seeds: alpha uniform
on [0.5, 4], Re log-uniform on [500, 3000], Mach uniform on [0.2, 0.9].
Training solves are the solver's own (mixed form by default); the network
is trained on the GPU by the library's MLP kernels.  For every held-out
point the plain solve (pseudo-random start, shift at the target) and the
learned solves (start mode; shift mode with its provable acceptance test
and plain fallback) run on the same assembled operator, and the script
prints one JSON line with Krylov-Schur iterations, operator applications
(K^-1 solves, refinement included) and wall time, per mode and in total,
and the largest eigenvalue deviation of the learned answers from the plain
ones.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import api, learned
from .case import Physics, make_case, target_lambda


def draw(n, seed):
    rng = np.random.default_rng(seed)
    return [(float(rng.uniform(0.5, 4.0)), float(10 ** rng.uniform(math.log10(500), math.log10(3000))),
             float(rng.uniform(0.2, 0.9))) for _ in range(n)]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ny", type=int, default=100)
    ap.add_argument("--nz", type=int, default=50)
    ap.add_argument("--train", type=int, default=256)
    ap.add_argument("--eval", type=int, default=64)
    ap.add_argument("--nev", type=int, default=8)
    ap.add_argument("--precision", type=int, default=1)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--modes", default="start,shift",
                    help="learned modes to evaluate (comma-separated: start, shift)")
    ap.add_argument("--out", default="", help="also write the JSON result to this file")
    a = ap.parse_args()
    modes = [m for m in a.modes.split(",") if m]
    base = Physics(alpha=2.43, omega=0j, nev=a.nev)
    case = make_case(a.ny, a.nz, physics=base)
    tgt = target_lambda(base.omega)
    out = {"grid": [a.ny, a.nz], "train_points": a.train, "eval_points": a.eval, "nev": a.nev,
           "precision": a.precision}
    with api.Problem(case) as prob:
        t = time.perf_counter()
        samples = learned.generate(prob, draw(a.train, 11), nev=a.nev, precision=a.precision)
        out["train_solve_s"] = time.perf_counter() - t
        t = time.perf_counter()
        prop = learned.Proposal.fit(samples, tgt, epochs=a.epochs, batch=min(256, a.train),
                                    lr=1e-3, width=256, depth=4)
        out["fit_s"] = time.perf_counter() - t
        out["final_loss"] = float(prop.history[-1])
        tot = {k: {"iterations": 0, "solves": 0, "wall_s": 0.0, "factorizations": 0}
               for k in ["plain"] + modes}
        accepted = 0
        maxdev = 0.0
        for pt in draw(a.eval, 12):
            prob.set_physics(learned.physics_at(base, *pt, a.nev))
            t = time.perf_counter()
            plain = learned.plain_solve(prob, a.nev, a.precision)
            tot["plain"]["wall_s"] += time.perf_counter() - t
            tot["plain"]["iterations"] += plain.diag["iterations"]
            tot["plain"]["solves"] += plain.diag["solves"]
            tot["plain"]["factorizations"] += 1
            for mode in modes:
                t = time.perf_counter()
                sol, used, st = learned.learned_solve(prob, prop, a.nev, a.precision,
                                                      shift=(mode == "shift"))
                tot[mode]["wall_s"] += time.perf_counter() - t
                tot[mode]["iterations"] += st.get("iterations", 0) + st.get("iterations_plain", 0)
                tot[mode]["solves"] += st.get("solves", 0) + st.get("solves_plain", 0)
                # start mode factors once at the target, like the plain solve;
                # shift mode factors at sigma' and, when rejected, again at
                # the target
                tot[mode]["factorizations"] += (1 if mode == "start" else
                                                (1 if used else 2))
                if mode == "shift":
                    accepted += int(used)
                for lam in sol.lam:
                    maxdev = max(maxdev, float(np.min(np.abs(plain.lam - lam)) / abs(lam)))
        out["modes"] = tot
        out["shift_accepted"] = accepted
        out["max_rel_deviation_from_plain"] = maxdev
    for mode in modes:
        out[f"iterations_saved_{mode}"] = tot["plain"]["iterations"] - tot[mode]["iterations"]
        out[f"solves_saved_{mode}"] = tot["plain"]["solves"] - tot[mode]["solves"]
    if "shift" in modes:
        # a point solved by the plain method needs one factorisation at the
        # target; shift mode needs one at sigma' and, on fallback, a second
        out["refactorizations_saved_shift"] = (tot["plain"]["factorizations"]
                                               - tot["shift"]["factorizations"])
    print(json.dumps(out))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
