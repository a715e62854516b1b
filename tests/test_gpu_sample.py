"""The reference's shipped case on the GPU: case/config.yaml with its
prepared 201 x 50 FD-q file (Re 32500, Mach 6, alpha 2.43, nev 8 nearest
lambda = 0), read from the committed fixture of the prepared fields
(tests/golden/sample_201x50_fields.npz, made by make_sample_golden.py).
Every GPU eigenvalue, in the FP64 and the mixed form, lies within
|dlambda|/|lambda| <= 1e-8 of the FP64 oracle's (sample_201x50_eigs.txt)
with relative residual <= 1e-10, and the result file written in the
reference's schema reads back."""
from pathlib import Path

import numpy as np
import pytest

from tailor_gb300 import api, h5, output
from tailor_gb300.case import Case, Physics
from tailor_gb300.rules import load_rule

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"

# case/config.yaml of the reference
PHYSICS = dict(reynolds=32500.0, mach=6.0, prandtl=0.72, gas_constant=287.05, gamma=1.4,
               reference_viscosity=1.716e-5, reference_temperature=63.334,
               sutherland_constant=110.4, alpha=2.43 + 0j, omega=0j, nev=8, tol=1e-10,
               max_it=1000)


def sample_case() -> Case:
    fx = np.load(GOLDEN / "sample_201x50_fields.npz")
    n = fx["grid"].shape[0]
    grid = np.zeros((n, 3, 2))
    base = np.zeros((n, 5, 2))
    grid[..., 0] = fx["grid"]
    base[..., 0] = fx["baseflow"]
    return Case(201, 50, 10, 6, load_rule(201, 10, False), load_rule(50, 6, True),
                float(fx["spanwise_period"]), grid, base, Physics(**PHYSICS))


def golden_eigs():
    g = np.loadtxt(GOLDEN / "sample_201x50_eigs.txt", ndmin=2)
    return g[:, 0] + 1j * g[:, 1]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_shipped_sample(gpu_lib, precision, tmp_path):
    case = sample_case()
    ref = golden_eigs()
    with api.Problem(case) as prob:
        api.run_pipeline(prob)
        sol = api.EigenSolver(prob).solve(precision=precision, modes=True)
    d = sol.diag
    assert d["converged"] >= 8 and np.all(sol.residual <= 1e-10), sol.residual
    for lam in sol.lam:
        err = np.min(np.abs(ref - lam)) / abs(lam)
        assert err <= 1e-8, (lam, err, ref)
    p = output.write_eigen_output(tmp_path / "sample_eigenmodes.h5", case, "Sample", sol.lam,
                                  sol.residual, sol.modes, d["requested"], 0j)
    with h5.File(p) as f:
        assert f.attrs["converged_modes"] == len(sol.lam)
        lam = f["spectrum/lambda"][...]
        assert np.array_equal(lam[:, 0] + 1j * lam[:, 1], sol.lam)
        assert f["modes/mode_000"][...].shape == (case.nodes, 5, 2)


def test_launcher_end_to_end(gpu_lib, tmp_path, capsys):
    """python -m tailor_gb300.run on the shipped case: the prepared file is
    found, the GPU stages run, the reference driver's report is printed and
    the result file is written in the reference's schema."""
    from tailor_gb300 import run
    case = sample_case()
    data = tmp_path / "data"
    output.write_prepared(data / "FD-q" / "fdq_sample_qy10_qz6.h5", case)
    (data / "sample.h5").write_bytes(b"")  # the source is not read on a cache hit
    cfg = """CaseTitle: Sample
Folder: data
File: sample.h5
Q-Value:
    y: 10
    z: 6
Stability:
    Alpha:
        Real: 2.43
        Imag: 0.0
EigenSolver:
    SearchCenterOmega:
        Real: 0.0
        Imag: 0.0
    NumberOfEigenvalues: 8
    Tolerance: 1.0e-10
    MaximumIterations: 1000
Output:
    File: data/results/sample_eigenmodes.h5
Physics:
    Targets:
        ReynoldsNumber: 32500
        MachNumber: 6.0
    Gas:
        PrandtlNumber: 0.72
        GasConstant: 287.05
        RatioOfSpecificHeats: 1.4
    Transport:
        ReferenceMu: 1.716E-5
        ReferenceTemperature: 63.3340
        SutherlandConstant: 110.4
"""
    (tmp_path / "config.yaml").write_text(cfg)
    assert run.main(["-c", str(tmp_path / "config.yaml")]) == 0
    text = capsys.readouterr().out
    assert "FD-q cache hit" in text and "Prepared case 'Sample'" in text
    assert "  Ny x Nz: 201 x 50" in text and "eigensolver: requested=8, converged=" in text
    ref = golden_eigs()
    with h5.File(data / "results" / "sample_eigenmodes.h5") as f:
        assert f.attrs["case"] == "Sample" and f.attrs["converged_modes"] >= 8
        lam = f["spectrum/lambda"][...]
        for l in lam[:, 0] + 1j * lam[:, 1]:
            assert np.min(np.abs(ref - l)) / abs(l) <= 1e-8
