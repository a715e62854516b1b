"""Shipped FD-q rules (polynomial exactness, like Prepare.cpp:328-437's
moment checks) and the C ABI library surface (loads, exports every
function declared in include/tailor_gb300.h) -- no GPU needed."""
import os
import re
from pathlib import Path

import numpy as np
import pytest

from tailor_gb300 import rules
from tailor_gb300 import build as tb

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("name", rules.available())
def test_rule_polynomial_exactness(name):
    m = re.match(r"N(\d+)_q(\d+)(p?)", name)
    n, q, per = int(m.group(1)), int(m.group(2)), m.group(3) == "p"
    r = rules.load_rule(n if per else n + 1, q, per)
    x = r.nodes
    for i in range(r.n):
        if per:
            xs = x[i] + (r.offsets[i] * (r.period / r.n))
        else:
            xs = x[r.indices[i]]
        h = xs - x[i]
        scale = np.max(np.abs(h))
        for k in range(0, min(q, 6) + 1):
            p = (h / scale) ** k
            d1 = np.dot(r.weights[1, i], p) * scale
            d2 = np.dot(r.weights[2, i], p) * scale * scale
            e1 = 1.0 if k == 1 else 0.0
            e2 = 2.0 if k == 2 else 0.0
            assert abs(d1 - e1) < 5e-9 * max(1, np.abs(r.weights[1, i]).sum() * scale)
            assert abs(d2 - e2) < 5e-7 * max(1, np.abs(r.weights[2, i]).sum() * scale ** 2)
        assert np.all(r.indices[i] == ((i + r.offsets[i]) % r.n if per else i + r.offsets[i]))


def test_library_exports_header_symbols():
    lib_path = tb.build()
    header = (ROOT / "include" / "tailor_gb300.h").read_text()
    declared = set(re.findall(r"^(?:int|void|size_t|const char \*)\s*\*?(tlr_\w+)\(",
                              header, re.M))
    assert len(declared) >= 15
    import ctypes
    lib = ctypes.CDLL(str(lib_path))
    for name in sorted(declared):
        assert hasattr(lib, name), name
    lib.tlr_status_string.restype = ctypes.c_char_p
    assert lib.tlr_status_string(0) == b"success"
    assert lib.tlr_status_string(6) == b"non-positive Jacobian"


def test_no_product_import_of_oracle():
    for p in (ROOT / "tailor_gb300").rglob("*.py"):
        txt = p.read_text()
        assert "import oracle" not in txt and "from oracle" not in txt, p


def test_sweep_argument_checks_without_gpu():
    """tlr_sweep rejects malformed sweeps before touching the device."""
    import ctypes
    from tailor_gb300 import _lib as L
    tb.build()
    lib = L.load()
    gcs = (L.GridClass * 1)()
    pts = (L.SweepPoint * 2)(L.SweepPoint(0, 1.0, 0.0, None, 0.0),
                             L.SweepPoint(3, 2.0, 0.0, None, 0.0))
    opts = L.SweepOpts()
    lam = np.zeros(64)
    res = np.zeros(32)
    st = np.zeros(2, dtype=np.int32)
    rc = lib.tlr_sweep(gcs, 1, pts, 2, ctypes.byref(opts), lam.ctypes.data, res.ctypes.data,
                       st.ctypes.data, None, None)
    assert rc == 1 and b"invalid grid class" in lib.tlr_last_error(None)
    rc = lib.tlr_sweep(gcs, 0, pts, 2, ctypes.byref(opts), lam.ctypes.data, res.ctypes.data,
                       st.ctypes.data, None, None)
    assert rc == 1 and b"invalid sweep arguments" in lib.tlr_last_error(None)


def test_noalloc_norm_argument_checks_without_gpu():
    """tlr_frobenius_noalloc refuses null, misaligned and oversized inputs
    before it touches a device, so these calls launch no kernel."""
    import ctypes
    from tailor_gb300 import _lib as L
    tb.build()
    lib = L.load()
    out = ctypes.c_double(0.0)
    rc = lib.tlr_frobenius_noalloc(None, 4, ctypes.byref(out), None)
    assert rc == 1 and b"null" in lib.tlr_last_error(None)
    # base + 1 double: an odd-double offset into a complex128 array
    rc = lib.tlr_frobenius_noalloc(ctypes.c_void_p(4096 + 8), 4, ctypes.byref(out), None)
    assert rc == 1 and b"16-byte aligned" in lib.tlr_last_error(None)
    rc = lib.tlr_frobenius_noalloc(ctypes.c_void_p(4096), 2 ** 28 + 1, ctypes.byref(out), None)
    assert rc == 3 and b"maximum" in lib.tlr_last_error(None)
    # a count above LLONG_MAX is still a size error, not a launch failure
    rc = lib.tlr_frobenius_noalloc(ctypes.c_void_p(4096), 2 ** 63 + 5, ctypes.byref(out), None)
    assert rc == 3 and b"maximum" in lib.tlr_last_error(None)


def test_rebuilt_baseflow_matches_synthetic_case():
    """Mach changes reload the Crocco-Busemann base flow (api.Problem.set_physics)."""
    from tailor_gb300.case import Physics, make_case, rebuild_baseflow
    c = make_case(24, 16, physics=Physics(mach=0.5), amplitude=0.08)
    assert np.array_equal(rebuild_baseflow(c), c.baseflow)
    c.physics = Physics(mach=0.85)
    assert np.array_equal(rebuild_baseflow(c),
                          make_case(24, 16, physics=Physics(mach=0.85), amplitude=0.08).baseflow)


def test_pencil_argument_checks_without_gpu():
    """tlr_pencil_create rejects malformed pencils before touching the device."""
    from tailor_gb300 import api
    tb.build()
    A = np.eye(6, dtype=complex)
    B = np.eye(6, dtype=complex)
    B[0, 5] = 0.5  # couples two 5 x 5 blocks
    with pytest.raises(api.TailorError, match="block diagonal"):
        api.PencilProblem(A, B)
    B = np.eye(6, dtype=complex)
    A[2, 3] = np.nan
    with pytest.raises(api.TailorError, match="non-finite"):
        api.PencilProblem(A, B)
    with pytest.raises(ValueError, match="square"):
        api.PencilProblem(np.eye(3), np.eye(4))


def test_mixed_solve_falls_back_to_fp64_without_gpu():
    """EigenSolver.solve repeats a failed mixed-form solve in FP64 (a stand-in
    library reports "not converged" for precision 1)."""
    from types import SimpleNamespace
    from tailor_gb300 import api
    from tailor_gb300.case import Physics

    class FakeLib:
        def __init__(self, fail_status):
            self.calls, self.fail_status = [], fail_status

        def tlr_solve(self, ctx, opts, lam, res, vec, diag):
            prec = opts._obj.precision
            self.calls.append(prec)
            if prec == 1:
                return self.fail_status
            diag._obj.converged = 2
            diag._obj.requested = 2
            return 0

        def tlr_last_error(self, ctx):
            return b"Krylov-Schur failed to converge"

    for status, falls_back in ((13, True), (1, False)):
        p = api.Problem.__new__(api.Problem)
        p.lib, p.ctx, p._keep = FakeLib(status), None, []
        p.case = SimpleNamespace(physics=Physics(nev=2), nodes=2)
        if falls_back:
            sol = api.EigenSolver(p).solve(precision=1)
            assert p.lib.calls == [1, 0] and sol.diag["fallback"] == 1
        else:  # an argument error is not retried
            with pytest.raises(api.TailorError):
                api.EigenSolver(p).solve(precision=1)
            assert p.lib.calls == [1]
    p = api.Problem.__new__(api.Problem)
    p.lib, p.ctx, p._keep = FakeLib(13), None, []
    p.case = SimpleNamespace(physics=Physics(nev=2), nodes=2)
    with pytest.raises(api.TailorError):
        api.EigenSolver(p).solve(precision=1, fallback=False)


def test_sweep_argument_errors_are_not_hidden_by_the_fallback():
    """An argument error of tlr_sweep (no point solved) still raises."""
    from tailor_gb300 import api
    from tailor_gb300.case import make_case
    tb.build()
    with pytest.raises(api.TailorError, match="invalid grid class"):
        api.sweep([make_case(24, 16)], [(0, 1.0), (5, 2.0)], nev=6)


def test_proposal_save_load_without_gpu(tmp_path, monkeypatch):
    """Proposal.save / load round trip (a stand-in network keeps it on the CPU);
    a tampered parameter file is rejected by its digest."""
    from tailor_gb300 import learned

    class FakeMLP:
        def __init__(self, n_in=3, width=8, depth=2, n_out=4, seed=1):
            self.shape = (n_in, width, depth, n_out)
            self.n_params = 10
            self.p = np.arange(10, dtype=np.float32) * seed

        def get_params(self):
            return self.p.copy()

        def set_params(self, p):
            self.p = np.asarray(p, dtype=np.float32).copy()

    monkeypatch.setattr(learned, "MLP", FakeMLP)
    prop = learned.Proposal(FakeMLP(seed=3), np.ones(3), np.ones(3), np.zeros(4), np.ones(4),
                            np.eye(6, 2, dtype=complex), 0.01 - 0.3j, 2, np.array([1.0, 0.5]))
    prop.save(tmp_path / "p.npz")
    back = learned.Proposal.load(tmp_path / "p.npz")
    assert np.array_equal(back.mlp.p, prop.mlp.p) and back.mlp.shape == prop.mlp.shape
    assert back.target == prop.target and back.n_lam == 2
    assert np.array_equal(back.basis, prop.basis) and np.array_equal(back.history, prop.history)
    z = dict(np.load(tmp_path / "p.npz"))
    z["params"] = z["params"] + 1
    np.savez(tmp_path / "bad.npz", **z)
    with pytest.raises(ValueError, match="digest"):
        learned.Proposal.load(tmp_path / "bad.npz")


def test_header_is_c11_and_the_library_links_from_c(tmp_path):
    """include/tailor_gb300.h compiles as strict C11 and a plain C program
    linked against libtailor_gb300.so calls it (here the host FD-q generator,
    which needs no GPU) -- what a cgo / FFI binding of the path relies on."""
    import shutil
    import subprocess
    lib = tb.build()
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "t.c"
    src.write_text(r'''
#include <stdio.h>
#include "tailor_gb300.h"
int main(void) {
  double nodes[11], w[3 * 11 * 5], le[11];
  int idx[11 * 5], off[11 * 5];
  int rc = tlr_fdq_rule(11, 4, 0, 2.0, nodes, idx, off, w, le);
  if (rc) return rc;
  rc = tlr_fdq_rule(2, 4, 0, 2.0, nodes, idx, off, w, NULL);
  printf("%s|%s|%.17g\n", tlr_status_string(rc), tlr_last_error(NULL), nodes[0]);
  return 0;
}
''')
    exe = tmp_path / "t"
    cuda_lib = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parents[1] / "lib64"
    subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                    str(src), "-L", str(lib.parent), "-ltailor_gb300", "-o", str(exe)], check=True)
    env = dict(os.environ, LD_LIBRARY_PATH=f"{lib.parent}:{cuda_lib}:" +
               os.environ.get("LD_LIBRARY_PATH", ""))
    out = subprocess.run([str(exe)], capture_output=True, text=True, env=env, check=True).stdout
    status, message, x0 = out.strip().split("|")
    assert status == "invalid argument" and "N must be at least 2" in message
    assert float(x0) == -1.0


def test_no_gpu_means_an_error_not_a_fallback():
    """Without a CUDA device the product path stops with TLR_ERR_CUDA and the
    driver's message; nothing computes on the CPU in its place."""
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a CUDA device is present")
    from tailor_gb300 import api
    from tailor_gb300.case import make_case
    with pytest.raises(api.TailorError) as e:
        api.Problem(make_case(24, 16))
    assert e.value.status == 11 and "CUDA" in e.value.message
    with pytest.raises(api.TailorError) as e:
        api.solve_pencil(np.eye(10, dtype=complex), np.eye(10, dtype=complex), 0.5j, nev=2)
    assert e.value.status == 11


def test_shift_mode_answer_is_checked_against_the_plain_one(monkeypatch):
    """learned_solve in shift mode keeps a shifted answer only when every
    eigenvalue within R of the target lies inside the disk the shifted solve
    covered and every kept residual meets 1e-10; otherwise the plain solve
    runs and is returned.  Stand-ins replace the GPU solver and the network."""
    from types import SimpleNamespace
    from tailor_gb300 import api, learned

    target = 0.0 + 0.0j
    plain_lam = np.array([0.10 + 0.0j, -0.20j])
    calls = []

    class FakeSolver:
        def __init__(self, problem):
            pass

        def solve(self, nev=0, precision=1, sigma=None, start=None, fallback=True, **kw):
            calls.append(("shift" if sigma is not None else "plain", nev))
            if sigma is None:
                return api.EigenSolution(plain_lam.copy(), np.full(2, 1e-12), None,
                                         {"iterations": 5, "solves": 50})
            return shifted(nev)

    class FakeProposal:
        target = 0.0 + 0.0j

        def propose(self, point, nev):
            return sigma_p, np.ones(4, complex), np.zeros(8, complex)

    monkeypatch.setattr(api, "EigenSolver", FakeSolver)
    monkeypatch.setattr(api, "run_pipeline", lambda p: {})
    prob = SimpleNamespace(case=SimpleNamespace(physics=SimpleNamespace(alpha=1.0, reynolds=1e3,
                                                                        mach=0.5)))

    def covering(nev):  # nev + 2 values around sigma, far ones beyond the target disk
        lam = np.array([0.10 + 0.0j, -0.20j, 0.9 + 0.0j, -0.9 + 0.0j])[:nev]
        return api.EigenSolution(lam, np.full(nev, 1e-12), None, {"iterations": 3, "solves": 30})

    # covered: |target - sigma| + R <= r' with sigma near the target
    sigma_p, shifted = 0.01 + 0.0j, covering
    sol, used, st = learned.learned_solve(prob, FakeProposal(), nev=2, shift=True, extra=2)
    assert used and calls == [("shift", 4)]
    assert np.allclose(np.sort_complex(sol.lam), np.sort_complex(plain_lam))

    # not covered: sigma far from the target; the nev + 2 values nearest it
    # span a disk that misses the target's neighbourhood
    calls.clear()
    sigma_p = 5.0 + 0.0j

    def around_sigma(nev):
        lam = sigma_p + np.array([-0.1, 0.1, 0.15j, -0.2])[:nev]
        return api.EigenSolution(lam, np.full(nev, 1e-12), None, {"iterations": 3, "solves": 30})
    shifted = around_sigma
    sol, used, st = learned.learned_solve(prob, FakeProposal(), nev=2, shift=True, extra=2)
    assert not used and st["fallback"] and calls == [("shift", 4), ("plain", 2)]
    assert np.array_equal(sol.lam, plain_lam)

    # a kept pair above the residual bar
    calls.clear()
    sigma_p = 0.01 + 0.0j

    def loose(nev):
        s = covering(nev)
        s.residual[0] = 1e-8
        return s
    shifted = loose
    sol, used, st = learned.learned_solve(prob, FakeProposal(), nev=2, shift=True, extra=2)
    assert not used and calls[-1] == ("plain", 2)

    # the shifted solve fails outright
    calls.clear()

    def failing(nev):
        raise api.TailorError(13, "not converged")
    shifted = failing
    sol, used, st = learned.learned_solve(prob, FakeProposal(), nev=2, shift=True, extra=2)
    assert not used and calls == [("shift", 4), ("plain", 2)]
