"""GB300-native BiGlobal linear-stability hot path (Tailor operator API).

The compute path is libtailor_gb300.so (hand-written sm_103a CUDA kernels
behind the C ABI of include/tailor_gb300.h); this package holds the
host-side mirror of the reference's stage objects, the synthetic case
generator and the shipped FD-q rule tables.
"""
from .case import Case, Physics, make_case, target_lambda  # noqa: F401
from .api import (  # noqa: F401
    BaseFlowDerivatives, BoundaryConditions, EigenSolver, GlobalOperator,
    Metrics, Problem, TailorError, lns_points, run_pipeline, transform_points)
