"""Host symbolic analysis (tlr_symbolic_analyze), checked on the CPU.

The reference leaves ordering and symbolic factorisation to MUMPS behind
PCLU (EigenSolver.cpp:61-71); the solver here factors along a geometric
nested-dissection tree.  These tests restate, independently in NumPy, what
makes that tree a valid multifrontal structure for the operator's block
pattern (GlobalOperator.cpp:209-283: the tensor product of the two FD-q
stencils at every node):

* the elimination order is a permutation and each front eliminates a
  contiguous run of it, fronts in postorder;
* every coupling (u, v) of the pattern, u eliminated first, lands in a front
  on the path from u's front to the root, so no update is lost;
* front borders, flops and stored entries recomputed from the tree and the
  pattern equal the library's counts.

The default ordering's counts at 200 x 128 are pinned to the ones tlr_solve
reported for that grid's factorisation, so the analysis the solver runs is
the one checked here.
"""
import ctypes

import numpy as np
import pytest

from tailor_gb300 import _lib as L
from tailor_gb300 import api, rules

pytestmark = pytest.mark.timeout(300)


def _grid_rules(ny, nz):
    return rules.load_rule(ny, 10, False), rules.load_rule(nz, 6, True)


def _pattern(xi, eta):
    """Directed block couplings (row node, column node) of A_bc."""
    ny, nz = xi.n, eta.n
    i = np.arange(ny * nz) % ny
    j = np.arange(ny * nz) // ny
    cols = (eta.indices[j][:, :, None] * ny + xi.indices[i][:, None, :]).reshape(ny * nz, -1)
    rows = np.repeat(np.arange(ny * nz), cols.shape[1])
    pairs = np.unique(np.stack([rows, cols.ravel()], 1), axis=0)
    return pairs[:, 0], pairs[:, 1]


def _check_tree(xi, eta, res):
    nn = xi.n * eta.n
    rank, front, parent = res["node_rank"], res["node_front"], res["front_parent"]
    nf = res["fronts"]
    assert np.array_equal(np.sort(rank), np.arange(nn))
    # each front eliminates a contiguous run of ranks, fronts in rank order
    order = np.argsort(rank)
    f_by_rank = front[order]
    assert np.all(np.diff(f_by_rank) >= 0)
    assert np.array_equal(np.unique(f_by_rank), np.arange(nf))
    # postorder: parents after children, subtrees contiguous
    assert parent[-1] == -1 and np.all(parent[:-1] > np.arange(nf - 1))
    size = np.ones(nf, dtype=np.int64)
    for t in range(nf - 1):
        size[parent[t]] += size[t]
    lo = np.arange(nf) - size + 1
    for t in range(nf - 1):
        p = parent[t]
        assert lo[p] <= lo[t] and t < p
    # every coupling reaches an ancestor-or-self front of the earlier node
    u, v = _pattern(xi, eta)
    for a, b in ((u, v), (v, u)):
        first = rank[a] < rank[b]
        fa, fb = front[a[first]], front[b[first]]
        assert np.all((lo[fb] <= fa) & (fa <= fb)), "a coupling escapes the elimination tree"
    return u, v, size


def _recount(xi, eta, res, u, v):
    """Borders bottom-up from the pattern; flops and storage as the solver
    counts them (5 unknowns per node, 8 real flops per complex MAC)."""
    nn = xi.n * eta.n
    rank, front, parent = res["node_rank"], res["node_front"], res["front_parent"]
    nf = res["fronts"]
    a = np.concatenate([u, v])
    b = np.concatenate([v, u])
    ptr = np.searchsorted(a[np.argsort(a, kind="stable")], np.arange(nn + 1))
    nbr = b[np.argsort(a, kind="stable")]
    piv = [[] for _ in range(nf)]
    for node in np.argsort(rank):
        piv[front[node]].append(node)
    children = [[] for _ in range(nf)]
    for t in range(nf - 1):
        children[parent[t]].append(t)
    border = [None] * nf
    flops, factor, pool, max_m = 0.0, 0, 0, 0
    for t in range(nf):
        rmax = rank[piv[t][-1]]
        cand = [nbr[ptr[x]:ptr[x + 1]] for x in piv[t]] + [border[c] for c in children[t]]
        c = np.unique(np.concatenate(cand))
        border[t] = c[rank[c] > rmax]
        p, bb = 5 * len(piv[t]), 5 * len(border[t])
        flops += 8.0 * (p ** 3 / 3.0 + p * p * bb + p * bb * bb)
        factor += p * (p + 2 * bb)
        pool += (p + bb) ** 2
        max_m = max(max_m, p + bb)
    return flops, factor, pool, max_m


@pytest.mark.parametrize("ny,nz,leaf,slack", [(60, 32, 0, 0), (60, 32, 16, 0),
                                              (150, 64, 0, 0), (200, 128, 0, 0),
                                              (200, 128, 0, 120), (400, 64, 0, 120)])
def test_tree_is_a_valid_multifrontal_structure(ny, nz, leaf, slack):
    xi, eta = _grid_rules(ny, nz)
    res = api.symbolic_analysis(xi, eta, leaf, slack)
    u, v, _ = _check_tree(xi, eta, res)
    flops, factor, pool, max_m = _recount(xi, eta, res, u, v)
    assert res["factor_elems"] == factor
    assert res["pool_elems"] == pool
    assert res["max_front_order"] == max_m
    assert flops == pytest.approx(res["flops"], rel=1e-12)


def test_default_ordering_is_the_solvers():
    """200 x 128 (128 000 unknowns): the flops and complex64 factor bytes
    tlr_solve reports for this grid's factorisation (ring slack 110)."""
    xi, eta = _grid_rules(200, 128)
    res = api.symbolic_analysis(xi, eta)
    assert res["flops"] == pytest.approx(5428264403333.333, rel=1e-12)
    assert res["factor_elems"] * 8 == 3784518000
    assert res["fronts"] == 673 and res["levels"] == 11
    same = api.symbolic_analysis(xi, eta, 48, 110)
    assert np.array_equal(same["node_rank"], res["node_rank"])


def test_ring_slack_trades_separators():
    """Accepting xi-cuts of ring boxes up to 1.1x the ring cut (the solver's
    ordering) lowers the 200 x 128 factorisation by about 9% against the
    smallest separators, and leaves 60 x 32 unchanged."""
    xi, eta = _grid_rules(200, 128)
    base = api.symbolic_analysis(xi, eta, 0, 100)
    wide = api.symbolic_analysis(xi, eta)
    assert wide["flops"] < 0.92 * base["flops"]
    assert wide["factor_elems"] < base["factor_elems"]
    xs, es = _grid_rules(60, 32)
    assert np.array_equal(api.symbolic_analysis(xs, es)["node_rank"],
                          api.symbolic_analysis(xs, es, 0, 100)["node_rank"])


def test_argument_errors():
    xi, eta = _grid_rules(60, 32)
    with pytest.raises(api.TailorError, match="ring_slack_percent") as e:
        api.symbolic_analysis(xi, eta, 0, 50)
    assert e.value.status == 1
    with pytest.raises(api.TailorError, match="bounded"):
        api.symbolic_analysis(eta, xi)
    with pytest.raises(api.TailorError, match="leaf_nodes"):
        api.symbolic_analysis(xi, eta, -1)
    lib = L.load()
    holder = api.Problem.__new__(api.Problem)
    holder._keep = []
    rx, re_ = holder._rule(xi), holder._rule(eta)
    info = L.SymbolicInfo()
    parent = np.zeros(4, dtype=np.int32)
    st = lib.tlr_symbolic_analyze(ctypes.byref(rx), ctypes.byref(re_), 0, 0, ctypes.byref(info),
                                  None, None, parent.ctypes.data, 4)
    assert st == 3 and info.fronts > 4  # TLR_ERR_SIZE, info filled for sizing
    assert lib.tlr_symbolic_analyze(None, ctypes.byref(re_), 0, 0, ctypes.byref(info),
                                    None, None, None, 0) == 1


@pytest.mark.parametrize("seed", range(24))
def test_random_grids(seed):
    """Random grid sizes, stencil degrees (odd and even bounded q, even
    periodic q), leaf sizes and ring slack: the tree stays valid and the
    counts match the independent recount."""
    rng = np.random.default_rng(seed)
    qy = int(rng.integers(2, 11))
    qz = int(rng.choice([2, 4, 6, 8]))
    ny = int(rng.integers(qy + 1, 90))
    nz = int(rng.integers(qz + 2, 70))
    xi, eta = rules.generate_rule(ny, qy, False), rules.generate_rule(nz, qz, True)
    leaf = int(rng.choice([0, 1, 8, 32, 200]))
    slack = int(rng.choice([0, 100, 150, 400]))
    res = api.symbolic_analysis(xi, eta, leaf, slack)
    u, v, _ = _check_tree(xi, eta, res)
    flops, factor, pool, max_m = _recount(xi, eta, res, u, v)
    assert (res["factor_elems"], res["pool_elems"], res["max_front_order"]) == (factor, pool, max_m)
    assert flops == pytest.approx(res["flops"], rel=1e-12)
