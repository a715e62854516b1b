"""Regenerate the shipped-sample fixtures of tests/golden/.

The reference ships one case: case/config.yaml with the structured sample
case/data/sample.h5 and its prepared FD-q file
case/data/FD-q/fdq_sample_qy10_qz6.h5 (201 x 50 nodes, Re 32500, Mach 6,
alpha 2.43, nev 8 nearest lambda = 0).  Run in a checkout that has the
reference project:

    python tests/golden/make_sample_golden.py /path/to/reference [--fields-only]

Writes
    sample_201x50_source.npz  the structured source sample (grid [Nz][Ny][3]
                              and base flow [Nz][Ny][5], real parts; the
                              imaginary parts are zero, checked) and its
                              spanwise period, so the interpolation can be
                              checked against the reference's prepared file
                              without the reference checkout
    sample_201x50_fields.npz  the prepared grid [N][3] and base flow [N][5]
                              read from the reference's prepared file (all
                              imaginary parts are zero there, checked), so
                              the GPU test can run the case without the
                              reference checkout
    sample_201x50_eigs.txt    the oracle's eigenvalues nearest the target
                              (FP64: C oracle assembly, boundary rows,
                              SuperLU + ARPACK), one "re im residual" line
                              per eigenvalue
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))


def main() -> None:
    from oracle.oracle import Oracle, boundary_rows, eigen_oracle, to_complex_blocks
    from tailor_gb300 import config, prepare

    ref = Path(sys.argv[1])
    cfg = config.load_config(ref / "case" / "config.yaml", require_input=True)
    grid, base, _, _, period = prepare.read_structured_sample(cfg.source_file)
    assert np.all(grid.imag == 0) and np.all(base.imag == 0)
    np.savez_compressed(HERE / "sample_201x50_source.npz", grid=grid.real, baseflow=base.real,
                        spanwise_period=np.float64(period))
    case = prepare.load_prepared(cfg.input_file, cfg.q_y, cfg.q_z, cfg.physics)
    assert np.all(case.grid[..., 1] == 0) and np.all(case.baseflow[..., 1] == 0)
    np.savez_compressed(HERE / "sample_201x50_fields.npz", grid=case.grid[..., 0],
                        baseflow=case.baseflow[..., 0],
                        spanwise_period=np.float64(case.spanwise_period))
    if "--fields-only" in sys.argv:
        return
    t = time.time()
    o = Oracle()
    r = o.full(case)
    A, B, _ = boundary_rows(case, r["metrics"], r["row_ptr"], r["col"],
                            to_complex_blocks(r["mass"]), to_complex_blocks(r["spatial"]))
    om = cfg.physics.omega
    sigma = complex(om.imag, -om.real)
    lam, _, res = eigen_oracle(r["row_ptr"], r["col"], A, B, case.nodes, sigma, 12)
    with open(HERE / "sample_201x50_eigs.txt", "w") as f:
        for l, e in zip(lam, res):
            f.write(f"{l.real:.17g} {l.imag:.17g} {e:.3e}\n")
    print(f"oracle: {time.time() - t:.1f} s")


if __name__ == "__main__":
    main()
