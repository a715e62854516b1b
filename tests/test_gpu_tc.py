"""Tensor-core (tcgen05, 3xTF32) Schur-complement update of a complex64 front
against NumPy: F22 -= L21 U12 over one panel step, partial tiles included.
The 3xTF32 product carries FP32 accuracy: relative error <= 2e-6 of the
product's norm, and every entry outside F22 is unchanged."""
import ctypes

import numpy as np
import pytest

from tailor_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _run(lib, A, p, k0, w, lbo=0, sbo=0):
    m = A.shape[0]
    front = np.ascontiguousarray(A.T.astype(np.complex64)).view(np.float32).reshape(-1)
    out = np.zeros_like(front)
    st = lib.tlr_schur_update_c64(front.ctypes.data, m, p, k0, w, lbo, sbo, out.ctypes.data)
    return st, out.view(np.complex64).reshape(m, m).T


@pytest.mark.parametrize("m,p,k0,w", [(300, 200, 64, 64), (200, 120, 0, 64), (129, 100, 64, 64),
                                      (77, 40, 32, 32)])
def test_schur_update_tc(gpu_lib, m, p, k0, w):
    rng = np.random.default_rng(m + k0)
    A = (rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))).astype(np.complex64)
    ww = min(w, p - k0)
    b = k0 + ww
    ref = A.astype(np.complex128)
    prod = ref[b:, k0:b] @ ref[k0:b, b:]
    expect = ref.copy()
    expect[b:, b:] -= prod
    results = {}
    for lbo, sbo in [(0, 0), (256, 128)]:
        st, got = _run(gpu_lib, A, p, k0, w, lbo, sbo)
        err = float(np.linalg.norm(got[b:, b:] - expect[b:, b:]) / max(np.linalg.norm(prod), 1e-30))
        results[(lbo, sbo)] = (st, err)
        if (lbo, sbo) == (0, 0) and st == 0 and err <= 2e-6:
            outside = got.copy()
            outside[b:, b:] = 0
            untouched = A.copy()
            untouched[b:, b:] = 0
            assert np.array_equal(outside, untouched)
            return
    pytest.fail(f"tensor-core update mismatch (status, error) per (lbo, sbo): {results}")
