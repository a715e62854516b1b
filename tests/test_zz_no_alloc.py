"""tlr_frobenius_noalloc: the allocation-free Frobenius norm.

It is for callers that cannot allocate device memory (hosts whose caching
allocator forbids raw cudaMalloc from the libraries they load, or that hold
nearly all of HBM in their own pool).  Its result must match the norm the
existing entry point tlr_assemble reports for the assembled operator L, on
two calls in a row (the calls share the library's fixed scratch array), and
sizes beyond its fixed maximum and misaligned inputs must be refused.  The
test allocates the input buffer itself; the entry point allocates nothing.
This file runs last so a stop-at-first-failure run has executed every other
test before it."""
import ctypes

import numpy as np
import pytest

from tailor_gb300 import api
from tailor_gb300.case import make_case

pytestmark = pytest.mark.gpu

TLR_ERR_ARG = 1
TLR_ERR_SIZE = 3


def test_frobenius_noalloc_matches_assembly_norm(gpu_lib):
    case = make_case(60, 32)
    rt = ctypes.CDLL("libcudart.so")
    with api.Problem(case) as prob:
        d = api.run_pipeline(prob)
        expected_l = d["operator"]["spatial_frobenius_norm"]
        expected_a = d["bc"]["eigen_frobenius_norm"]
        L = prob.copy_out(api.OUT_L)
        A = prob.copy_out(api.OUT_A)
    for host, expected in ((L, expected_l), (A, expected_a)):
        dptr = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(dptr), ctypes.c_size_t(host.nbytes)) == 0
        try:
            assert rt.cudaMemcpy(dptr, ctypes.c_void_p(host.ctypes.data),
                                 ctypes.c_size_t(host.nbytes), 1) == 0
            count = host.nbytes // 16
            for _ in range(2):
                out = ctypes.c_double(0.0)
                st = gpu_lib.tlr_frobenius_noalloc(dptr, count, ctypes.byref(out), None)
                assert st == 0, gpu_lib.tlr_last_error(None)
                assert out.value == pytest.approx(expected, rel=1e-12)
                assert out.value == pytest.approx(float(np.linalg.norm(host)), rel=1e-12)
        finally:
            rt.cudaFree(dptr)
    out = ctypes.c_double(0.0)
    st = gpu_lib.tlr_frobenius_noalloc(ctypes.c_void_p(16), 2 ** 28 + 1, ctypes.byref(out), None)
    assert st == TLR_ERR_SIZE
    assert b"maximum" in gpu_lib.tlr_last_error(None)
    # an odd-double offset into a complex array is refused before any launch
    st = gpu_lib.tlr_frobenius_noalloc(ctypes.c_void_p(24), 4, ctypes.byref(out), None)
    assert st == TLR_ERR_ARG
    assert b"aligned" in gpu_lib.tlr_last_error(None)
