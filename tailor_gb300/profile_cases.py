"""Run one stage of the hot path on one synthetic grid (profiling driver).

    python -m tailor_gb300.profile_cases --stage assemble --ny 100 --nz 50
    python -m tailor_gb300.profile_cases --stage solve --ny 100 --nz 50 --precision 1

--stage assemble runs metrics, derivatives and --repeat assemblies;
--stage bc adds the boundary rows; --stage spmv adds --repeat SpMVs of A_bc;
--stage solve adds one shift-and-invert eigen solve (nev from --nev,
Krylov basis --ncv, block size --block); with --warm the solve is repeated
at alpha + 0.43 from the first solve's Ritz vectors (a neighbouring sweep
point).  Prints one JSON line with the stage timings reported by the library.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import api
from .case import Physics, make_case


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--stage", default="assemble", choices=["assemble", "bc", "spmv", "solve"])
    ap.add_argument("--ny", type=int, default=100)
    ap.add_argument("--nz", type=int, default=50)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--precision", type=int, default=0)
    ap.add_argument("--nev", type=int, default=8)
    ap.add_argument("--alpha", type=float, default=2.43)
    ap.add_argument("--omega-re", type=float, default=0.0)
    ap.add_argument("--omega-im", type=float, default=0.0)
    ap.add_argument("--mach", type=float, default=0.5)
    ap.add_argument("--reynolds", type=float, default=1000.0)
    ap.add_argument("--ncv", type=int, default=0)
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--schur-kernel", type=int, default=0,
                    help="tlr_solve_opts.cuda_core_schur: 0 fastest, 1 CUDA cores, 2 other")
    ap.add_argument("--warm", action="store_true")
    a = ap.parse_args()
    case = make_case(a.ny, a.nz, physics=Physics(alpha=a.alpha, nev=a.nev, mach=a.mach,
                                                 reynolds=a.reynolds,
                                                 omega=complex(a.omega_re, a.omega_im)))
    out = {"ny": a.ny, "nz": a.nz, "stage": a.stage}
    with api.Problem(case) as p:
        api.Metrics(p).compute()
        api.BaseFlowDerivatives(p).compute()
        out["assemble_ms"] = [api.GlobalOperator(p).assemble()["assemble_ms"]
                              for _ in range(a.repeat)]
        if a.stage in ("bc", "spmv", "solve"):
            api.BoundaryConditions(p).apply()
        if a.stage == "spmv":
            x = np.random.default_rng(0).standard_normal(5 * case.nodes) + 0j
            for _ in range(a.repeat):
                p.spmv(api.TLR_MAT_A, x)
        if a.stage == "solve":
            keys = ("factor_ms", "krylov_ms", "solves", "iterations", "max_relative_error",
                    "solve_ms", "factor_bytes", "factor_flops", "trisolve_ms", "trisolves")
            kw = dict(precision=a.precision, ncv=a.ncv, block=a.block,
                      cuda_core_schur=a.schur_kernel)
            sol = api.EigenSolver(p).solve(**kw)
            out["solve"] = {k: sol.diag[k] for k in keys}
            if a.warm:
                p.set_alpha(a.alpha + 0.43)
                api.run_pipeline(p)
                sol = api.EigenSolver(p).solve(warm_start=True, **kw)
                out["warm_solve"] = {k: sol.diag[k] for k in keys}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
