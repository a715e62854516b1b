"""Case launcher: config.yaml -> prepared FD-q case -> GPU eigen solve -> HDF5.

    python -m tailor_gb300.run -c case/config.yaml [--prepare-only]
                               [--precision 0|1] [--output PATH]

The reference's launcher (src/Python/main.py:232-332) prepares the FD-q
case (interpolate.py, cached under <source dir>/FD-q/) and then starts the
C++ solver on the configuration.  Here the same two steps run in one
process: the configuration is parsed and validated (``config``), the
prepared file is reused when it exists and is valid, otherwise the sample
is interpolated and the prepared file written (``prepare``, ``output``);
unless --prepare-only, the case runs through the GPU stages (metrics,
derivatives, assembly, boundary rows, shift-and-invert Krylov-Schur) and
the spectrum and phased modes are written in the reference's result
schema.  --precision 1 selects the mixed form (complex64 factors,
tensor-core Schur updates, FP64 refinement); the default is the FP64 form
the reference runs.  Exit status 0 on success, 1 on a configuration or
preparation error, 2 on a solver error.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

from . import config, output, prepare


def prepared_case(cfg: config.Config, verbose: bool = True):
    """The configuration's prepared case: the cached file when it is valid,
    otherwise a fresh interpolation of the source sample (written back)."""
    if cfg.input_file.is_file():
        try:
            case = prepare.load_prepared(cfg.input_file, cfg.q_y, cfg.q_z, cfg.physics)
            if verbose:
                print(f"FD-q cache hit: {cfg.input_file}")
            return case
        except (ValueError, OSError, KeyError) as e:
            if verbose:
                print(f"FD-q cache invalid, rebuilding: {e}", file=sys.stderr)
    case = prepare.prepare_sample(cfg.source_file, cfg.q_y, cfg.q_z, cfg.physics)
    try:
        output.write_prepared(cfg.input_file, case, cfg.source_file)
        if verbose:
            print(f"FD-q cache generated: {cfg.input_file}\n"
                  f"  Ny={case.ny}, q_y={case.qy}; Nz={case.nz}, q_z={case.qz}")
    except OSError as e:  # a read-only case folder: keep the case in memory
        if verbose:
            print(f"FD-q cache not written ({e}); continuing", file=sys.stderr)
    return case


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m tailor_gb300.run")
    ap.add_argument("-c", "--config", required=True)
    ap.add_argument("--prepare-only", action="store_true")
    ap.add_argument("--precision", type=int, choices=(0, 1), default=0)
    ap.add_argument("--output", default=None, help="result file (default: the config's)")
    a = ap.parse_args(argv)
    try:
        cfg = config.load_config(a.config)
        print(f"Tailor FD-q preprocessing\n  config: {Path(a.config).absolute()}\n"
              f"  source: {cfg.source_file}\n  output: {cfg.input_file}\n"
              f"  q_y: {cfg.q_y}\n  q_z: {cfg.q_z}", flush=True)
        case = prepared_case(cfg)
    except (ValueError, OSError, TypeError) as e:
        print(f"Tailor preprocessing error: {e}", file=sys.stderr)
        return 1
    if a.prepare_only:
        return 0
    from . import api
    try:
        with api.Problem(case) as prob:
            api.run_pipeline(prob)
            sol = api.EigenSolver(prob).solve(precision=a.precision, modes=True)
        d = sol.diag
        target = complex(d["target_re"], d["target_im"])
        out = output.write_eigen_output(a.output or cfg.output_file, case, cfg.case_title,
                                        sol.lam, sol.residual, sol.modes, d["requested"],
                                        target)
    except (RuntimeError, ValueError, OSError) as e:
        print(f"Tailor solver error: {e}", file=sys.stderr)
        return 2
    print(f"converged {d['converged']} of {d['requested']} eigenpairs "
          f"(factor {d['factor_ms']:.1f} ms, Krylov {d['krylov_ms']:.1f} ms); wrote {out}")
    for lam, res in zip(sol.lam, sol.residual):
        print(f"  lambda = {lam.real:+.12e} {lam.imag:+.12e}i   residual {res:.2e}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
