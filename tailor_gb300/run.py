"""Case launcher: config.yaml -> prepared FD-q case -> GPU eigen solve -> HDF5.

    python -m tailor_gb300.run -c case/config.yaml [--prepare-only]
                               [--assemble-only] [--precision 0|1] [--output PATH]

The reference's launcher (src/Python/main.py:232-332) prepares the FD-q
case (interpolate.py, cached under <source dir>/FD-q/) and then starts the
C++ solver on the configuration.  Here the same two steps run in one
process: the configuration is parsed and validated (``config``), the
prepared file is reused when it exists and is valid, otherwise the sample
is interpolated and the prepared file written (``prepare``, ``output``);
unless --prepare-only, the case runs through the GPU stages (metrics,
derivatives, assembly, boundary rows, shift-and-invert Krylov-Schur) and
the spectrum and phased modes are written in the reference's result
schema.  The printed stage report is the reference driver's, line for line
(Process.cpp:62-176).  --precision 1 selects the mixed form (complex64 factors,
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


METRIC_NAMES = ("xi_y", "xi_z", "eta_y", "eta_z", "xi_yy", "xi_zz", "xi_yz", "eta_yy",
                "eta_zz", "eta_yz")
DERIVATIVE_NAMES = ("dy", "dz", "dyy", "dzz", "dyz")


def _g(x) -> str:
    return f"{float(x):.16g}"


def report(cfg: config.Config, case, stages: dict) -> str:
    """The stage report of the reference's driver (Process.cpp:62-152), line
    for line, from the stage diagnostics of ``api.run_pipeline``: scripts that
    parse Tailor's output (Jacobian range, metric and derivative norms,
    operator and boundary statistics) read this one unchanged."""
    import numpy as np
    md, dd, od, bd = stages["metrics"], stages["derivatives"], stages["operator"], stages["bc"]
    ph = case.physics
    a = complex(ph.alpha)
    width = max(int(np.max(np.abs(case.xi.offsets))), int(np.max(np.abs(case.eta.offsets))))
    out = [f"Prepared case '{cfg.case_title}'",
           f"  input: {cfg.input_file}",
           f"  Ny x Nz: {case.ny} x {case.nz}",
           f"  alpha: {a.real:.16g} {a.imag:+.16g}i",
           f"  FD-q degrees: y={case.qy}, z={case.qz}; DMDA stencil width: {width}",
           f"  xi rule: {case.xi.n} nodes, {case.xi.q + 1}-point stencil",
           f"  eta rule: {case.eta.n} nodes, {case.eta.q + 1}-point stencil",
           f"  ||baseflow||2: {_g(np.linalg.norm(case.baseflow))}, "
           f"||grid||2: {_g(np.linalg.norm(case.grid))}",
           f"  Jacobian range: [{_g(md['min_jacobian'])}, {_g(md['max_jacobian'])}]",
           f"  max |Im(grid y/z)|: {_g(md['max_grid_imaginary'])}"]
    out += [f"  metric norm {n}: {_g(v)}" for n, v in zip(METRIC_NAMES, md["norms"])]
    out.append(f"  base-flow derivative components: 25; max |Im(baseflow)|: "
               f"{_g(dd['max_baseflow_imaginary'])}")
    for k, n in enumerate(DERIVATIVE_NAMES):
        out.append(f"  base-flow derivative norm {n}: "
                   + " ".join(_g(v) for v in dd["norms"][5 * k:5 * k + 5]))
    out += [f"  global matrices: {od['rows']} x {od['columns']}, block size {od['block_size']}",
            f"  M_Gamma blocks used/allocated: {od['mass_used_blocks']:.0f} / "
            f"{od['mass_allocated_blocks']:.0f}; ||M_Gamma||F: {_g(od['mass_frobenius_norm'])}",
            f"  L blocks used/allocated: {od['spatial_used_blocks']:.0f} / "
            f"{od['spatial_allocated_blocks']:.0f}; ||L||F: {_g(od['spatial_frobenius_norm'])}",
            "  eigenvalue convention: (-L) q = lambda M_Gamma q, lambda = -i omega",
            f"  boundaries: wall nodes={bd['wall_nodes']}, far-field nodes={bd['farfield_nodes']}",
            f"  far-field incoming modes={bd['incoming_modes']} (per node "
            f"{bd['min_incoming_per_node']}..{bd['max_incoming_per_node']}), "
            f"neutral modes={bd['neutral_modes']}",
            f"  max characteristic |imag(c)|: {_g(bd['max_characteristic_imaginary'])}; "
            f"max cond(R): {_g(bd['max_eigenvector_condition'])}",
            f"  ||A_bc||F: {_g(bd['eigen_frobenius_norm'])}; "
            f"||B_bc||F: {_g(bd['eigen_mass_frobenius_norm'])}"]
    return "\n".join(out)


def solve_report(d: dict, output_file, modes: int) -> str:
    """The eigensolver lines of Process.cpp:161-175."""
    return (f"  eigensolver: requested={d['requested']}, converged={d['converged']}, "
            f"iterations={d['iterations']}\n"
            f"  lambda target: {d['target_re']:.16g} {d['target_im']:+.16g}i; "
            f"max relative error: {_g(d['max_relative_error'])}\n"
            f"  output: {output_file} ({modes} modes)")


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m tailor_gb300.run")
    ap.add_argument("-c", "--config", required=True)
    ap.add_argument("--prepare-only", action="store_true")
    ap.add_argument("--precision", type=int, choices=(0, 1), default=0)
    ap.add_argument("--output", default=None, help="result file (default: the config's)")
    ap.add_argument("--assemble-only", action="store_true",
                    help="stop after the boundary rows (the reference's -tailor_assemble_only)")
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
            stages = api.run_pipeline(prob)
            print(report(cfg, case, stages), flush=True)
            if a.assemble_only:
                print("  assemble-only: boundary matrices validated; EPSSolve skipped")
                return 0
            sol = api.EigenSolver(prob).solve(precision=a.precision, modes=True)
        d = sol.diag
        target = complex(d["target_re"], d["target_im"])
        out = output.write_eigen_output(a.output or cfg.output_file, case, cfg.case_title,
                                        sol.lam, sol.residual, sol.modes, d["requested"],
                                        target)
    except (RuntimeError, ValueError, OSError) as e:
        print(f"Tailor solver error: {e}", file=sys.stderr)
        return 2
    print(solve_report(d, out, len(sol.lam)))
    for lam, res in zip(sol.lam, sol.residual):
        print(f"  lambda = {lam.real:+.12e} {lam.imag:+.12e}i   residual {res:.2e}")
    print(f"  factorisation {d['factor_ms']:.1f} ms, Krylov-Schur {d['krylov_ms']:.1f} ms")
    return 0


if __name__ == "__main__":
    sys.exit(main())
