"""Pin the CPU oracle's pointwise physics to the reference's fixtures.

test_lns_coefficients.cpp:78-139 and test_lns_transforms.cpp:139-227
compare LNSCoefficients / StreamwiseFourier / CurvilinearTransform with
Fortran-generated gold at 5e-13 * max(1, |x|); the same comparison here
pins the oracle (tests/golden/make_golden.py restates the generators).
"""
import numpy as np

from tailor_gb300.case import Physics
from tests.helpers import read_lns_gold, read_transform_gold, rel_close, transform_inputs
from tests.golden.make_golden import lns_points

CANON = Physics(reynolds=32500.0, mach=6.0, prandtl=0.72, gamma=1.4,
                reference_temperature=63.334, sutherland_constant=110.4)


def test_lns_oracle_matches_fortran_gold(oracle):
    gold = read_lns_gold()
    ph = oracle.physics(CANON)
    for p, q in enumerate(lns_points()):
        st, blocks = oracle.lns_physical(ph, q)
        assert st == 0
        assert rel_close(blocks, gold[p], 5e-13), np.max(np.abs(blocks - gold[p]))


def test_transform_oracle_matches_fortran_gold(oracle):
    gf, gc = read_transform_gold()
    alphas, phys, mets = transform_inputs()
    for p in range(2):
        st, four, curv = oracle.transform(alphas[p], phys[p], mets[p])
        assert st == 0
        assert rel_close(four, gf[p], 5e-13)
        assert rel_close(curv, gc[p], 5e-13)


def test_identity_metrics_reproduce_fourier_blocks_bitwise(oracle):
    # test_lns_transforms.cpp:171-203
    _, phys, _ = transform_inputs()
    ident = np.array([1.0, 0, 0, 1.0, 0, 0, 0, 0, 0, 0])
    st, four, curv = oracle.transform(complex(1.2, -0.3), phys[0], ident)
    assert st == 0
    assert np.array_equal(four, curv)


def test_non_finite_inputs_rejected(oracle):
    _, phys, mets = transform_inputs()
    st, _, _ = oracle.transform(complex(np.nan, 0.0), phys[0], mets[0])
    assert st == 1
    bad = mets[0].copy(); bad[6] = np.nan
    st, _, _ = oracle.transform(complex(1.0, 0.0), phys[0], bad)
    assert st == 1
    ph = oracle.physics(CANON)
    q = lns_points()[0].copy(); q[0, 0] = -1.0
    assert oracle.lns_physical(ph, q)[0] == 2
    q = lns_points()[0].copy(); q[0, 4] = 0.0
    assert oracle.lns_physical(ph, q)[0] == 3
    q = lns_points()[0].copy(); q[3, 2] = np.inf
    assert oracle.lns_physical(ph, q)[0] == 1
