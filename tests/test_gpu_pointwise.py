"""GPU pointwise physics against the reference's Fortran fixtures and the
oracle (LNSCoefficients.cpp:173-404; StreamwiseFourier.cpp:16-44;
CurvilinearTransform.cpp:62-101)."""
import numpy as np
import pytest

from tailor_gb300 import api
from tests.golden.make_golden import lns_points
from tests.helpers import read_lns_gold, read_transform_gold, rel_close, transform_inputs
from tests.test_oracle_golden import CANON

pytestmark = pytest.mark.gpu


def test_gpu_lns_points_match_gold_and_oracle(gpu_lib, oracle):
    gold = read_lns_gold()
    q = lns_points()
    st, blocks = api.lns_points(CANON, q)
    assert list(st) == [0, 0]
    for p in range(2):
        assert rel_close(blocks[p], gold[p], 5e-13)
        ost, ob = oracle.lns_physical(oracle.physics(CANON), q[p])
        assert ost == 0
        assert np.array_equal(blocks[p], ob)          # same expressions, no FMA


def test_gpu_lns_points_status(gpu_lib):
    q = np.repeat(lns_points()[:1], 4, axis=0)
    q[1, 0, 0] = -1.0
    q[2, 0, 4] = -0.5
    q[3, 5, 1] = np.nan
    st, _ = api.lns_points(CANON, q)
    assert list(st) == [0, 2, 3, 1]


def test_gpu_transforms_match_gold_and_oracle(gpu_lib, oracle):
    gf, gc = read_transform_gold()
    alphas, phys, mets = transform_inputs()
    st, four, curv = api.transform_points(alphas, phys.reshape(2, 275), mets)
    assert list(st) == [0, 0]
    for p in range(2):
        assert rel_close(four[p], gf[p], 5e-13)
        assert rel_close(curv[p], gc[p], 5e-13)
        _, of, oc = oracle.transform(alphas[p], phys[p], mets[p])
        assert np.array_equal(four[p], of) and np.array_equal(curv[p], oc)


def test_gpu_identity_transform_bitwise(gpu_lib):
    _, phys, _ = transform_inputs()
    ident = np.array([[1.0, 0, 0, 1.0, 0, 0, 0, 0, 0, 0]])
    st, four, curv = api.transform_points(np.array([1.2 - 0.3j]),
                                          phys[:1].reshape(1, 275), ident)
    assert st[0] == 0 and np.array_equal(four, curv)
    st, _, _ = api.transform_points(np.array([complex(np.nan, 0)]),
                                    phys[:1].reshape(1, 275), ident)
    assert st[0] == 1
