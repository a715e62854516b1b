"""ctypes binding of libtailor_gb300.so (the C ABI in include/tailor_gb300.h).

The library is loaded from the package's lib/ folder.  There is no CPU
fallback: a missing or unloadable library raises immediately.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "lib" / "libtailor_gb300.so"
_lib = None

c_double_p = ctypes.POINTER(ctypes.c_double)


class Recipe(ctypes.Structure):
    _fields_ = [("q_y", ctypes.c_int), ("q_z", ctypes.c_int),
                ("mach", ctypes.c_double), ("reynolds", ctypes.c_double),
                ("prandtl", ctypes.c_double), ("gas_constant", ctypes.c_double),
                ("gamma", ctypes.c_double),
                ("reference_viscosity", ctypes.c_double),
                ("reference_temperature", ctypes.c_double),
                ("sutherland_constant", ctypes.c_double),
                ("alpha_re", ctypes.c_double), ("alpha_im", ctypes.c_double),
                ("omega_re", ctypes.c_double), ("omega_im", ctypes.c_double),
                ("nev", ctypes.c_int), ("tol", ctypes.c_double),
                ("max_it", ctypes.c_int)]


class Rule(ctypes.Structure):
    _fields_ = [("node_count", ctypes.c_int), ("q", ctypes.c_int),
                ("periodic", ctypes.c_int), ("period", ctypes.c_double),
                ("nodes", ctypes.c_void_p), ("stencil_indices", ctypes.c_void_p),
                ("stencil_offsets", ctypes.c_void_p), ("weights", ctypes.c_void_p)]


class MetricDiag(ctypes.Structure):
    _fields_ = [("min_jacobian", ctypes.c_double), ("max_jacobian", ctypes.c_double),
                ("max_grid_imaginary", ctypes.c_double),
                ("norms", ctypes.c_double * 10)]


class DerivDiag(ctypes.Structure):
    _fields_ = [("max_baseflow_imaginary", ctypes.c_double),
                ("norms", ctypes.c_double * 25)]


class OperatorDiag(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_long), ("columns", ctypes.c_long),
                ("block_size", ctypes.c_long),
                ("mass_used_blocks", ctypes.c_double),
                ("mass_allocated_blocks", ctypes.c_double),
                ("spatial_used_blocks", ctypes.c_double),
                ("spatial_allocated_blocks", ctypes.c_double),
                ("mass_frobenius_norm", ctypes.c_double),
                ("spatial_frobenius_norm", ctypes.c_double),
                ("assemble_ms", ctypes.c_float)]


class BcDiag(ctypes.Structure):
    _fields_ = [("wall_nodes", ctypes.c_int), ("farfield_nodes", ctypes.c_int),
                ("incoming_modes", ctypes.c_int), ("neutral_modes", ctypes.c_int),
                ("min_incoming_per_node", ctypes.c_int),
                ("max_incoming_per_node", ctypes.c_int),
                ("max_characteristic_imaginary", ctypes.c_double),
                ("max_eigenvector_condition", ctypes.c_double),
                ("eigen_frobenius_norm", ctypes.c_double),
                ("eigen_mass_frobenius_norm", ctypes.c_double)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("nev", ctypes.c_int), ("ncv", ctypes.c_int),
                ("tol", ctypes.c_double), ("max_it", ctypes.c_int),
                ("precision", ctypes.c_int), ("sigma_re", ctypes.c_double),
                ("sigma_im", ctypes.c_double), ("use_sigma", ctypes.c_int),
                ("start", ctypes.c_void_p), ("cuda_core_schur", ctypes.c_int),
                ("solve_block", ctypes.c_int), ("refinement", ctypes.c_int),
                ("panel_width", ctypes.c_int), ("cluster_panel", ctypes.c_int),
                ("persistent_solve", ctypes.c_int), ("block", ctypes.c_int),
                ("nstart", ctypes.c_int), ("warm_start", ctypes.c_int),
                ("ring_slack_percent", ctypes.c_int), ("conv_check", ctypes.c_int),
                ("solve_wave", ctypes.c_int), ("fp64_acceptance", ctypes.c_int)]


class EigDiag(ctypes.Structure):
    _fields_ = [("requested", ctypes.c_int), ("converged", ctypes.c_int),
                ("iterations", ctypes.c_int), ("reason", ctypes.c_int),
                ("target_re", ctypes.c_double), ("target_im", ctypes.c_double),
                ("max_relative_error", ctypes.c_double),
                ("factorizations", ctypes.c_int), ("solves", ctypes.c_int),
                ("refinement_steps", ctypes.c_int),
                ("factor_ms", ctypes.c_double), ("krylov_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("factor_flops", ctypes.c_double),
                ("solve_ms", ctypes.c_double), ("factor_bytes", ctypes.c_double),
                ("trisolve_ms", ctypes.c_double), ("trisolves", ctypes.c_int),
                ("ortho_ms", ctypes.c_double), ("dense_ms", ctypes.c_double),
                ("residual_ms", ctypes.c_double), ("refine_res", ctypes.c_double * 3),
                ("block", ctypes.c_int), ("conv_checks", ctypes.c_int)]


class GridClass(ctypes.Structure):
    _fields_ = [("recipe", ctypes.c_void_p), ("xi", ctypes.c_void_p), ("eta", ctypes.c_void_p),
                ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("spanwise_period", ctypes.c_double), ("grid", ctypes.c_void_p),
                ("baseflow", ctypes.c_void_p)]


class SweepPoint(ctypes.Structure):
    _fields_ = [("grid_class", ctypes.c_int), ("alpha_re", ctypes.c_double),
                ("alpha_im", ctypes.c_double), ("start", ctypes.c_void_p),
                ("reynolds", ctypes.c_double)]


class SweepOpts(ctypes.Structure):
    _fields_ = [("solve", SolveOpts), ("workers", ctypes.c_int), ("autotune", ctypes.c_int),
                ("device", ctypes.c_int)]


class SweepDiag(ctypes.Structure):
    _fields_ = [("wall_ms", ctypes.c_double), ("points", ctypes.c_int),
                ("failed", ctypes.c_int), ("workers", ctypes.c_int),
                ("converged_pairs", ctypes.c_int),
                ("cuda_core_schur", ctypes.c_int * 16), ("solve_block", ctypes.c_int * 16),
                ("tune_factor_ms", (ctypes.c_double * 2) * 16),
                ("tune_trisolve_ms", (ctypes.c_double * 2) * 16),
                ("panel_width", ctypes.c_int * 16), ("tune_wide_factor_ms", ctypes.c_double * 16)]


class SymbolicInfo(ctypes.Structure):
    _fields_ = [("fronts", ctypes.c_int), ("levels", ctypes.c_int),
                ("max_front_order", ctypes.c_int), ("max_pivots", ctypes.c_int),
                ("flops", ctypes.c_double), ("factor_elems", ctypes.c_longlong),
                ("pool_elems", ctypes.c_longlong)]


# Exported symbols and their signatures (argtypes, restype).
_P = ctypes.c_void_p
_I = ctypes.c_int
SIGNATURES = {
    "tlr_ctx_create": ([_P, _P, _P, _I, _I, ctypes.c_double, _I, _P], _I),
    "tlr_ctx_destroy": ([_P], None),
    "tlr_set_alpha": ([_P, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                       ctypes.c_double], _I),
    "tlr_set_physics": ([_P, _P], _I),
    "tlr_load_fields": ([_P, _P, _P], _I),
    "tlr_metrics": ([_P, _P], _I),
    "tlr_baseflow_derivatives": ([_P, _P], _I),
    "tlr_assemble": ([_P, _P], _I),
    "tlr_apply_bc": ([_P, _P], _I),
    "tlr_spmv": ([_P, _I, _P, _P, _I], _I),
    "tlr_copy_out": ([_P, _I, _P, ctypes.c_size_t], _I),
    "tlr_out_bytes": ([_P, _I], ctypes.c_size_t),
    "tlr_lns_points": ([_P, _I, _P, _P, _P], _I),
    "tlr_transform_points": ([_I, _P, _P, _P, _P, _P, _P], _I),
    "tlr_solve": ([_P, _P, _P, _P, _P, _P], _I),
    "tlr_stream": ([_P], ctypes.c_void_p),
    "tlr_kernel_launches": ([], ctypes.c_longlong),
    "tlr_sweep": ([_P, _I, _P, _I, _P, _P, _P, _P, _P, _P], _I),
    "tlr_schur_update_c64": ([_P, _I, _I, _I, _I, ctypes.c_uint, ctypes.c_uint, _P], _I),
    "tlr_factor_solve": ([_P, _I, _P, _P, _I], _I),
    "tlr_wait_selftest": ([_I, ctypes.c_uint, _P], _I),
    "tlr_pencil_create": ([_P, _I, _P, _P, _I, _P], _I),
    "tlr_fdq_rule": ([_I, _I, _I, ctypes.c_double, _P, _P, _P, _P, _P], _I),
    "tlr_symbolic_analyze": ([_P, _P, _I, _I, _P, _P, _P, _P, _I], _I),
    "tlr_frobenius_noalloc": ([_P, ctypes.c_size_t, _P, _P], _I),
    "tlr_mlp_create": ([_I, _I, _I, _I, ctypes.c_ulonglong, _P], _I),
    "tlr_mlp_destroy": ([_P], None),
    "tlr_mlp_num_params": ([_P], ctypes.c_longlong),
    "tlr_mlp_params": ([_P, _P, _I], _I),
    "tlr_mlp_gradients": ([_P, _P, _P, _I, _P, _P], _I),
    "tlr_mlp_train": ([_P, _P, _P, _I, _I, _I, ctypes.c_float, _P], _I),
    "tlr_mlp_forward": ([_P, _P, _I, _P, _I], _I),
    "tlr_status_string": ([_I], ctypes.c_char_p),
    "tlr_last_error": ([_P], ctypes.c_char_p),
}


def lib_path() -> Path:
    return _LIB_PATH


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(
                f"{_LIB_PATH} is missing: build it with tailor_gb300.build.build() "
                "(the CUDA library is required; there is no CPU fallback)")
        lib = ctypes.CDLL(str(_LIB_PATH))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib
