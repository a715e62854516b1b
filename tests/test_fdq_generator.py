"""Host FD-q rule generator (tlr_fdq_rule) against the reference's rules.

Golden data: the shipped tables and tests/golden/fdq_reference_rules.npz
were produced by the reference's generator (fdq_nodes.py:280-353; the
scripts are tailor_gb300/rules/make_rules.py and
tests/golden/make_fdq_golden.py), and fdq_n100_q10_notebook.txt is the node
vector the reference's own test pins (test_fdq_nodes.py:24-27, 70-76).
The reference's node solve stops at a least-squares tolerance, so bounded
nodes are compared to 1e-13 and weights relative to their row scale to
1e-11; periodic rules have no solve and must match bit for bit.  No GPU.
"""
import re
import time
from pathlib import Path

import numpy as np
import pytest

from tailor_gb300 import build as tb
from tailor_gb300 import rules

from conftest import REFERENCE

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module", autouse=True)
def _lib():
    tb.build()


def _compare(g, nodes, idx, off, w, periodic):
    assert np.array_equal(g.indices, idx) and np.array_equal(g.offsets, off)
    if periodic:
        assert np.array_equal(g.nodes, nodes) and np.array_equal(g.weights, w)
        return
    assert np.max(np.abs(g.nodes - nodes)) < 1e-13
    for k in range(3):
        scale = np.max(np.abs(w[k]), axis=1, keepdims=True)
        assert np.max(np.abs(g.weights[k] - w[k]) / scale) < 1e-11, k


@pytest.mark.parametrize("name", rules.available())
def test_generated_matches_shipped_table(name):
    m = re.match(r"N(\d+)_q(\d+)(p?)", name)
    n, q, per = int(m.group(1)), int(m.group(2)), m.group(3) == "p"
    nc = n if per else n + 1
    r = rules.load_rule(nc, q, per)
    g = rules.generate_rule(nc, q, per, r.period)
    _compare(g, r.nodes, r.indices, r.offsets, r.weights, per)


@pytest.mark.parametrize("name", ["N10_q4", "N8_q8", "N40_q6", "N10_q4p", "N24_q6p"])
def test_generated_matches_reference_generator(name):
    ref = np.load(GOLDEN / "fdq_reference_rules.npz")
    m = re.match(r"N(\d+)_q(\d+)(p?)", name)
    n, q, per = int(m.group(1)), int(m.group(2)), m.group(3) == "p"
    g, le = rules.generate_rule(n if per else n + 1, q, per, with_log_error=True)
    _compare(g, ref[f"{name}_nodes"], ref[f"{name}_stencil_indices"],
             ref[f"{name}_stencil_offsets"], ref[f"{name}_weights"], per)
    # equal-error amplitudes: flat, and at the reference's level
    assert np.max(np.abs(np.diff(le))) < 1e-9
    assert np.max(np.abs(le - ref[f"{name}_log_error"])) < 1e-9


def test_notebook_nodes_n100_q10():
    """The reference test's pinned N=100, q=10 nodes (atol 2e-9 there)."""
    want = np.loadtxt(GOLDEN / "fdq_n100_q10_notebook.txt")
    g = rules.generate_rule(101, 10, False)
    assert np.max(np.abs(g.nodes - want)) < 2e-9


def test_full_stencil_limit_is_cgl():
    """q = N gives the Chebyshev-Gauss-Lobatto nodes (test_fdq_nodes.py:62-68)."""
    for n in (4, 8, 12):
        g = rules.generate_rule(n + 1, n, False)
        cgl = -np.cos(np.arange(n + 1) * np.pi / n)
        assert np.max(np.abs(g.nodes - cgl)) < 2e-11


def test_bounded_shapes_and_invariants():
    g, le = rules.generate_rule(11, 4, False, with_log_error=True)
    assert g.nodes.shape == (11,) and g.indices.shape == (11, 5) and g.weights.shape == (3, 11, 5)
    assert g.nodes[0] == -1.0 and g.nodes[-1] == 1.0 and np.all(np.diff(g.nodes) > 0)
    assert np.max(np.abs(g.nodes + g.nodes[::-1])) < 5e-12
    assert np.max(np.abs(np.diff(le))) < 1e-9


def test_periodic_half_open_and_wraps():
    g = rules.generate_rule(10, 4, True)
    assert g.nodes[0] == -1.0 and g.nodes[-1] < 1.0
    assert list(g.offsets[0]) == [-2, -1, 0, 1, 2]
    assert list(g.indices[0]) == [8, 9, 0, 1, 2]


def test_periodic_derivatives_converge():
    errs = []
    for nc in (24, 48):
        g = rules.generate_rule(nc, 6, True)
        v = np.sin(np.pi * g.nodes)
        d = np.sum(g.weights[1] * v[g.indices], axis=1)
        errs.append(np.max(np.abs(d - np.pi * np.cos(np.pi * g.nodes))))
    assert errs[1] < errs[0] / 40.0


@pytest.mark.parametrize("nc,q,per,period", [
    (2, 2, False, 2.0), (5, 1, False, 2.0), (5, 5, False, 2.0),   # N < 2, q < 2, q > N
    (2, 2, True, 2.0), (10, 3, True, 2.0), (10, 10, True, 2.0),   # n < 3, odd q, q >= n
    (10, 4, True, 0.0), (10, 4, True, float("nan"))])
def test_argument_checks(nc, q, per, period):
    with pytest.raises(ValueError):
        rules.generate_rule(nc, q, per, period)


def test_unshipped_size_is_generated_on_demand():
    assert "N40_q10" not in rules.available()
    t = time.perf_counter()
    r = rules.load_rule(41, 10, False)
    assert time.perf_counter() - t < 5.0
    assert r.n == 41 and r.nodes[0] == -1.0 and r.nodes[-1] == 1.0


# ---- HDF5 rule caches (fdq_nodes.py:458-627; test_fdq_nodes.py:143-219)

def test_rule_cache_round_trip(tmp_path):
    for nc, q, per in ((16, 4, False), (24, 6, True)):
        g, le = rules.generate_rule(nc, q, per, with_log_error=True)
        p = rules.save_rule(g, tmp_path / f"{rules.rule_name(nc, q, per)}.h5", le)
        r = rules.load_rule_file(p)
        assert (r.n, r.q, r.periodic) == (nc, q, per)
        for a, b in ((r.nodes, g.nodes), (r.indices, g.indices), (r.offsets, g.offsets),
                     (r.weights, g.weights)):
            assert np.array_equal(a, b)
        from tailor_gb300 import h5
        with h5.File(p) as f:
            assert f.attrs["schema_version"] == 2 and f.attrs["stencil_size"] == q + 1
            assert np.array_equal(f["diagnostics/log_error"][...], le)


def test_load_or_create_uses_and_rebuilds_the_cache(tmp_path):
    from tailor_gb300 import h5
    r1 = rules.load_or_create_rule(21, 6, False, tmp_path)
    path = tmp_path / "N20_q6.h5"
    assert path.is_file()
    stamp = path.stat().st_mtime_ns
    r2 = rules.load_or_create_rule(21, 6, False, tmp_path)  # cache hit
    assert path.stat().st_mtime_ns == stamp and np.array_equal(r1.nodes, r2.nodes)
    # a stale schema is rebuilt
    w = h5.Writer()
    with h5.File(path) as f:
        w.attrs.update(f.attrs)
        w.attrs["schema_version"] = 1
    w.write(path)
    with pytest.raises(rules.RuleError, match="unsupported FD-q schema version 1"):
        rules.load_rule_file(path)
    r3 = rules.load_or_create_rule(21, 6, False, tmp_path)
    assert np.array_equal(r3.nodes, r1.nodes) and rules.load_rule_file(path).n == 21


@pytest.mark.skipif(REFERENCE is None or not (REFERENCE / "fdqNodes" / "N200_q10.h5").is_file(),
                    reason="TAILOR_REFERENCE (a reference checkout) not set")
def test_reference_rule_caches_load():
    ref = REFERENCE / "fdqNodes"
    r = rules.load_rule_file(ref / "N200_q10.h5")
    g = rules.generate_rule(201, 10, False)
    assert np.max(np.abs(r.nodes - g.nodes)) < 1e-14
    p = rules.load_rule_file(ref / "N50_q6p.h5")
    assert p.periodic and np.array_equal(p.weights, rules.generate_rule(50, 6, True).weights)
    with pytest.raises(rules.RuleError, match="schema version 1"):
        rules.load_rule_file(ref / "N100_q10.h5")  # the older cache schema


def test_validate_rule_rejects_broken_rules():
    g = rules.generate_rule(16, 4, False)
    import dataclasses
    bad = dataclasses.replace(g, weights=g.weights.copy())
    bad.weights[1, 3, 2] += 1e-3
    with pytest.raises(rules.RuleError, match="order-1 weights fail degree-0 polynomial check at row 3"):
        rules.validate_rule("xi", bad)
    pr = rules.generate_rule(24, 6, True)
    nodes = pr.nodes.copy()
    nodes[5] = nodes[4]  # periodic moments use x + offset h, so row 5 fails on order first
    with pytest.raises(rules.RuleError, match="eta FD-q nodes must be strictly increasing"):
        rules.validate_rule("eta", dataclasses.replace(pr, nodes=nodes))


@pytest.mark.parametrize("q", [2, 3, 4, 5, 6, 7, 8, 9, 10, 12])
def test_generator_sweep_passes_the_loader_checks(q):
    """Every degree with node counts from the full-stencil limit (q + 1
    nodes) to 400 bounded and 500 periodic nodes converges and passes the
    C++ loader's rule checks (Prepare.cpp:328-437)."""
    for n in sorted({q + 1, q + 2, q + 3, 2 * q, 3 * q + 1, 25, 40, 64, 101, 150, 257, 400}):
        r = rules.generate_rule(n, q, False)
        rules.validate_rule("xi", r)
        assert r.n == n and np.all(np.diff(r.nodes) > 0)
    if q % 2 == 0:
        for n in (q + 1, q + 2, 16, 33, 64, 128, 192, 500):
            rules.validate_rule("eta", rules.generate_rule(n, q, True))
