"""Input-fault and stage-order checks on the GPU path, mirroring the
reference's fault-injection tests (test_metrics.py:268-357,
test_baseflow_derivatives.py:322-424): each bad input is built on the
host and must produce the reference's error category and message; no
device fault is involved, and the context stays usable."""
import numpy as np
import pytest

from tailor_gb300 import api
from tailor_gb300.case import make_case

pytestmark = pytest.mark.gpu


def _expect(fn, status, text):
    with pytest.raises(api.TailorError) as e:
        fn()
    assert e.value.status == status
    assert text in e.value.message


def test_metric_faults(gpu_lib):
    case = make_case(24, 16)
    case.grid[:, 1:, 0] = 0.0
    with api.Problem(case) as p:
        _expect(api.Metrics(p).compute, 6, "Grid Jacobian must be positive and nonsingular")
    case = make_case(24, 16)
    case.grid[11, 1, 1] = 1e-7
    with api.Problem(case) as p:
        _expect(api.Metrics(p).compute, 7, "Grid y/z coordinates must be real")
    case = make_case(24, 16)
    case.grid[13, 2, 0] = np.nan
    with api.Problem(case) as p:
        _expect(api.Metrics(p).compute, 5, "not finite")
        # the context survives: reload good fields and continue
        good = make_case(24, 16)
        p.load_fields(good.grid, good.baseflow)
        api.Metrics(p).compute()


def test_baseflow_faults(gpu_lib):
    for f, v, st, text in [(0, -1.0, 8, "density and temperature must both be positive"),
                           (4, 0.0, 8, "density and temperature must both be positive"),
                           (2, np.nan, 5, "Base-flow values are not finite")]:
        case = make_case(24, 16)
        case.baseflow[17, f, 0] = v
        with api.Problem(case) as p:
            api.Metrics(p).compute()
            _expect(api.BaseFlowDerivatives(p).compute, st, text)
    case = make_case(24, 16)
    case.baseflow[5, 1, 1] = 1e-8
    with api.Problem(case) as p:
        api.Metrics(p).compute()
        _expect(api.BaseFlowDerivatives(p).compute, 7, "Base-flow values must be real")


def test_stage_order(gpu_lib):
    case = make_case(24, 16)
    with api.Problem(case) as p:
        _expect(api.BaseFlowDerivatives(p).compute, 2, "Metrics must be computed")
        _expect(api.GlobalOperator(p).assemble, 2, "Metrics are required")
        _expect(api.BoundaryConditions(p).apply, 2, "must be assembled")
        api.Metrics(p).compute()
        _expect(api.GlobalOperator(p).assemble, 2, "derivatives are required")


def test_rule_validation(gpu_lib):
    case = make_case(24, 16)
    bad = case.xi
    import dataclasses
    idx = bad.indices.copy(); idx[3, 2] += 1
    case.xi = dataclasses.replace(bad, indices=idx)
    with pytest.raises(api.TailorError) as e:
        api.Problem(case)
    assert e.value.status == 4


@pytest.mark.parametrize("which", [0, 1], ids=["mbarrier", "grid-barrier"])
def test_bounded_waits_report_timeouts(gpu_lib, which):
    """The GPU's only waits (the tensor-core kernel's mbarrier wait, the
    persistent solve's grid barrier) give up after their poll limit and set
    an error flag the host reads; the context stays usable afterwards."""
    import ctypes
    t = ctypes.c_int(-1)
    assert gpu_lib.tlr_wait_selftest(which, 200000, ctypes.byref(t)) == 0
    assert t.value == 1
    case = make_case(24, 16)
    with api.Problem(case) as prob:
        api.run_pipeline(prob)
        sol = api.EigenSolver(prob).solve(nev=4, precision=1)
    assert np.all(sol.residual <= 1e-10)
