"""CPU oracle for the Tailor hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module.  The product (``tailor_gb300``) never does.

Pieces:

* ``Oracle`` -- ctypes binding of ``tlr_oracle.c`` (built by the Makefile
  beside it): metrics, base-flow derivatives, pointwise LNS blocks, the
  Fourier/curvilinear transforms, BSR pattern and numeric assembly, SpMV.
* ``boundary_rows`` -- BoundaryConditions.cpp:152-548 restated in NumPy,
  calling LAPACK ``zggev`` through ``scipy.linalg.lapack`` exactly as the
  reference calls ``LAPACKggev_`` (BoundaryConditions.cpp:198-224), with the
  reference's pivoted Gauss-Jordan inverse (92-140) and row combination
  (combineRows, 366-387).
* ``eigen_oracle`` -- FP64 shift-invert eigen solve of (A_bc, B_bc): SuperLU
  (``scipy.sparse.linalg.splu``) factors A - sigma B and ARPACK
  (``eigs``) iterates on (A - sigma B)^-1 B in the Euclidean inner product,
  lambda = sigma + 1/theta, nev nearest the target -- the arithmetic of
  SLEPc's STSINVERT + PCLU (EigenSolver.cpp:61-67).
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "build" / "libtlr_oracle.so"

EPS = np.finfo(np.float64).eps


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(_HERE)], check=True)
    return _LIB_PATH


class _Rule(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("q", ctypes.c_int),
                ("periodic", ctypes.c_int),
                ("idx", ctypes.c_void_p), ("off", ctypes.c_void_p),
                ("w0", ctypes.c_void_p), ("w1", ctypes.c_void_p),
                ("w2", ctypes.c_void_p)]


class _Physics(ctypes.Structure):
    _fields_ = [("reynolds", ctypes.c_double), ("mach", ctypes.c_double),
                ("prandtl", ctypes.c_double), ("gamma", ctypes.c_double),
                ("sutherland_ratio", ctypes.c_double),
                ("alpha_re", ctypes.c_double), ("alpha_im", ctypes.c_double)]


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


class Oracle:
    def __init__(self):
        if not _LIB_PATH.exists():
            build()
        self.lib = ctypes.CDLL(str(_LIB_PATH))
        self._keep = []

    # -- helpers -------------------------------------------------------
    def _rule(self, rule) -> _Rule:
        w = np.ascontiguousarray(rule.weights, dtype=np.float64)
        idx = np.ascontiguousarray(rule.indices, dtype=np.int32)
        off = np.ascontiguousarray(rule.offsets, dtype=np.int32)
        self._keep += [w, idx, off]
        return _Rule(rule.n, rule.q, int(rule.periodic), idx.ctypes.data,
                     off.ctypes.data, w[0].ctypes.data, w[1].ctypes.data,
                     w[2].ctypes.data)

    @staticmethod
    def physics(ph, alpha=None) -> _Physics:
        a = complex(ph.alpha if alpha is None else alpha)
        return _Physics(ph.reynolds, ph.mach, ph.prandtl, ph.gamma,
                        ph.sutherland_constant / ph.reference_temperature,
                        a.real, a.imag)

    # -- stages --------------------------------------------------------
    def metrics(self, case):
        n = case.nodes
        grid = np.ascontiguousarray(case.grid, dtype=np.float64)
        m = np.zeros((n, 10))
        diag = np.zeros(13)
        st = self.lib.orc_metrics(
            case.ny, case.nz, ctypes.c_double(case.spanwise_period),
            ctypes.byref(self._rule(case.xi)), ctypes.byref(self._rule(case.eta)),
            _ptr(grid), _ptr(m), _ptr(diag))
        return st, m, diag

    def derivatives(self, case, metrics):
        n = case.nodes
        base = np.ascontiguousarray(case.baseflow, dtype=np.float64)
        d = np.zeros((n, 25))
        diag = np.zeros(26)
        st = self.lib.orc_baseflow_derivatives(
            case.ny, case.nz, ctypes.byref(self._rule(case.xi)),
            ctypes.byref(self._rule(case.eta)), _ptr(base),
            _ptr(np.ascontiguousarray(metrics)), _ptr(d), _ptr(diag))
        return st, d, diag

    def lns_physical(self, physics, q):
        """q: [10][5] (value, dx, dy, dz, dxx, dyy, dzz, dxy, dxz, dyz)."""
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(50)
        out = np.zeros((11, 5, 5))
        st = self.lib.orc_lns_physical(ctypes.byref(physics), _ptr(q), _ptr(out))
        return st, out

    def lns_inviscid(self, physics, state):
        state = np.ascontiguousarray(state, dtype=np.float64)
        out = np.zeros((3, 5, 5))
        st = self.lib.orc_lns_inviscid(ctypes.byref(physics), _ptr(state), _ptr(out))
        return st, out

    def transform(self, alpha: complex, phys, metrics):
        phys = np.ascontiguousarray(phys, dtype=np.float64).reshape(275)
        m = np.ascontiguousarray(metrics, dtype=np.float64)
        out = np.zeros((7, 25, 2))
        four = np.zeros((7, 25, 2))
        st = self.lib.orc_transform(ctypes.c_double(alpha.real),
                                    ctypes.c_double(alpha.imag), _ptr(phys),
                                    _ptr(m), _ptr(out), _ptr(four))
        c = lambda a: (a[..., 0] + 1j * a[..., 1]).reshape(7, 5, 5)
        return st, c(four), c(out)

    def pattern(self, case):
        s = (case.qy + 1) * (case.qz + 1)
        n = case.nodes
        row_ptr = np.zeros(n + 1, dtype=np.int32)
        col = np.zeros(n * s, dtype=np.int32)
        self.lib.orc_pattern(case.ny, case.nz, ctypes.byref(self._rule(case.xi)),
                             ctypes.byref(self._rule(case.eta)), _ptr(row_ptr),
                             _ptr(col))
        return row_ptr, col

    def assemble(self, case, metrics, derivs, alpha=None):
        s = (case.qy + 1) * (case.qz + 1)
        n = case.nodes
        mass = np.zeros((n, 5, 5, 2))
        spatial = np.zeros((n * s, 5, 5, 2))
        ph = self.physics(case.physics, alpha)
        st = self.lib.orc_assemble(
            case.ny, case.nz, ctypes.byref(self._rule(case.xi)),
            ctypes.byref(self._rule(case.eta)), ctypes.byref(ph),
            _ptr(np.ascontiguousarray(case.baseflow, dtype=np.float64)),
            _ptr(np.ascontiguousarray(derivs)), _ptr(np.ascontiguousarray(metrics)),
            _ptr(mass), _ptr(spatial))
        return st, mass, spatial

    def spmv(self, row_ptr, col, val, x):
        """val: [nnzb][5][5][2] float64; x: complex [nrows*5]."""
        xr = np.ascontiguousarray(np.stack([x.real, x.imag], -1).reshape(-1))
        y = np.zeros_like(xr)
        self.lib.orc_bsr_spmv(len(row_ptr) - 1, _ptr(row_ptr), _ptr(col),
                              _ptr(np.ascontiguousarray(val)), _ptr(xr), _ptr(y))
        return y[0::2] + 1j * y[1::2]

    def full(self, case, alpha=None):
        """Metrics -> derivatives -> pattern -> assembly, all on the CPU."""
        st, m, md = self.metrics(case)
        assert st == 0, f"oracle metrics failed: {st}"
        st, d, dd = self.derivatives(case, m)
        assert st == 0, f"oracle derivatives failed: {st}"
        row_ptr, col = self.pattern(case)
        st, mass, spatial = self.assemble(case, m, d, alpha)
        assert st == 0, f"oracle assembly failed: {st}"
        return dict(metrics=m, metric_diag=md, derivs=d, deriv_diag=dd,
                    row_ptr=row_ptr, col=col, mass=mass, spatial=spatial)


def to_complex_blocks(v: np.ndarray) -> np.ndarray:
    return v[..., 0] + 1j * v[..., 1]


def bsr_to_scipy(row_ptr, col, blocks_c, n_block_rows):
    import scipy.sparse as sp
    return sp.bsr_matrix((blocks_c, col, row_ptr),
                         shape=(5 * n_block_rows, 5 * n_block_rows)).tocsr()


# ------------------------------------------------- boundary conditions
def _gauss_jordan_inverse(a: np.ndarray):
    """BoundaryConditions.cpp:92-140 (pivoted Gauss-Jordan, 5x5)."""
    m = a.astype(np.complex128).copy()
    inv = np.eye(5, dtype=np.complex128)
    for k in range(5):
        p = k
        mag = abs(m[p, k])
        for r in range(k + 1, 5):
            if abs(m[r, k]) > mag:
                mag, p = abs(m[r, k]), r
        if not np.isfinite(mag) or mag <= 100.0 * EPS:
            return None
        if p != k:
            m[[p, k]] = m[[k, p]]
            inv[[p, k]] = inv[[k, p]]
        piv = m[k, k]
        m[k] /= piv
        inv[k] /= piv
        for r in range(5):
            if r == k:
                continue
            f = m[r, k]
            m[r] -= f * m[k]
            inv[r] -= f * inv[k]
    return inv


def characteristics(physics, state, metrics):
    """computeCharacteristics (BoundaryConditions.cpp:152-280) with zggev."""
    from scipy.linalg.lapack import zggev
    ph = physics
    pe = 1.0 / (ph.gamma * ph.mach * ph.mach)
    g2 = 1.0 / ((ph.gamma - 1.0) * ph.mach * ph.mach)
    rho, V, W, T = state[0], state[2], state[3], state[4]
    G = np.zeros((5, 5)); Bc = np.zeros((5, 5)); Cc = np.zeros((5, 5))
    G[0, 0] = 1.0; G[1, 1] = G[2, 2] = G[3, 3] = rho
    G[4, 0] = -pe * T; G[4, 4] = rho * g2 - pe * rho
    Bc[0, 0] = V; Bc[0, 2] = rho; Bc[1, 1] = rho * V; Bc[2, 0] = pe * T
    Bc[2, 2] = rho * V; Bc[2, 4] = pe * rho; Bc[3, 3] = rho * V
    Bc[4, 0] = -pe * V * T; Bc[4, 4] = rho * V * g2 - rho * V * pe
    Cc[0, 0] = W; Cc[0, 3] = rho; Cc[1, 1] = rho * W; Cc[2, 2] = rho * W
    Cc[3, 0] = pe * T; Cc[3, 3] = rho * W; Cc[3, 4] = pe * rho
    Cc[4, 0] = -pe * W * T; Cc[4, 4] = rho * W * g2 - rho * W * pe
    mag = np.sqrt(metrics[0] * metrics[0] + metrics[1] * metrics[1])
    ny_, nz_ = metrics[0] / mag, metrics[1] / mag
    normal = (ny_ * Bc + nz_ * Cc).astype(np.complex128)
    alpha, beta, _, vr, _, info = zggev(np.asfortranarray(normal),
                                        np.asfortranarray(G.astype(np.complex128)),
                                        compute_vl=0, compute_vr=1)
    assert info == 0
    if np.any(np.abs(beta) <= 100 * EPS):
        raise ValueError("infinite characteristic speed")
    speeds = alpha / beta
    smax = max(1.0, float(np.max(np.abs(speeds))))
    max_im = float(np.max(np.abs(speeds.imag)))
    if max_im > 1000 * EPS * smax:
        raise ValueError("complex characteristic speed")
    R = np.array(vr)
    Rinv = _gauss_jordan_inverse(R)
    Ginv = _gauss_jordan_inverse(G)
    P = Rinv @ Ginv
    cond = np.max(np.abs(R).sum(1)) * np.max(np.abs(Rinv).sum(1))
    tol = 1000 * EPS * smax
    incoming = speeds.real < -tol
    neutral = np.abs(speeds.real) <= tol
    return dict(speeds=speeds, R=R, Rinv=Rinv, P=P, incoming=incoming,
                neutral=neutral, cond=cond, max_im=max_im, G=G)


def boundary_rows(case, metrics, row_ptr, col, mass_c, spatial_c):
    """BoundaryConditions::apply (353-548) restated on BSR arrays.

    mass_c, spatial_c: complex blocks [nnzb][5][5].  Returns (A_bc, B_bc,
    info) with A_bc on L's pattern and B_bc on M's (block-diagonal) pattern.
    """
    ny, nz = case.ny, case.nz
    A = -spatial_c.copy()
    B = mass_c.copy()
    base = case.baseflow[..., 0]
    info = dict(incoming=0, neutral=0, per_node=[], cond=0.0, max_im=0.0)
    for j in range(nz):
        node = j * ny
        for k in range(row_ptr[node], row_ptr[node + 1]):
            diag = col[k] == node
            for c in range(1, 5):
                A[k, c, :] = 0.0
                if diag:
                    A[k, c, c] = 1.0
        for c in range(1, 5):
            B[node, c, :] = 0.0
    for j in range(nz):
        node = j * ny + ny - 1
        ch = characteristics(case.physics, base[node], metrics[node])
        nin = int(ch["incoming"].sum())
        info["incoming"] += nin
        info["neutral"] += int(ch["neutral"].sum())
        info["per_node"].append(nin)
        info["cond"] = max(info["cond"], ch["cond"])
        info["max_im"] = max(info["max_im"], ch["max_im"])
        ks = range(row_ptr[node], row_ptr[node + 1])
        oldA = A[row_ptr[node]:row_ptr[node + 1]].copy()
        oldB = B[node].copy()
        for m in range(5):
            if ch["incoming"][m]:
                for k in ks:
                    A[k, m, :] = ch["Rinv"][m, :] if col[k] == node else 0.0
                B[node, m, :] = 0.0
            else:
                newA = np.zeros((len(ks), 5), dtype=np.complex128)
                newB = np.zeros(5, dtype=np.complex128)
                for s in range(5):
                    sc = ch["P"][m, s]
                    if sc == 0:
                        continue
                    newA += sc * oldA[:, s, :]
                    newB += sc * oldB[s, :]
                for t, k in enumerate(ks):
                    A[k, m, :] = newA[t]
                B[node, m, :] = newB
    return A, B, info


# --------------------------------------------------------- eigen oracle
def eigen_oracle(row_ptr, col, A_c, B_c, nb, sigma: complex, nev: int,
                 tol: float = 1e-12):
    """nev eigenvalues of A x = lambda B x nearest sigma, with residuals."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    A = sp.bsr_matrix((A_c, col, row_ptr), shape=(5 * nb, 5 * nb)).tocsc()
    Bd = sp.bsr_matrix((B_c, np.arange(nb, dtype=np.int32),
                        np.arange(nb + 1, dtype=np.int32)),
                       shape=(5 * nb, 5 * nb)).tocsc()
    A.eliminate_zeros(); Bd.eliminate_zeros()
    lu = spl.splu((A - sigma * Bd).tocsc())
    n = A.shape[0]
    op = spl.LinearOperator((n, n), matvec=lambda v: lu.solve(Bd @ v),
                            dtype=np.complex128)
    ncv = max(2 * nev, nev + 15)
    theta, vecs = spl.eigs(op, k=nev, which="LM", ncv=min(ncv, n - 1), tol=tol)
    lam = sigma + 1.0 / theta
    order = np.argsort(np.abs(lam - sigma))
    lam, vecs = lam[order], vecs[:, order]
    res = []
    for t in range(len(lam)):
        x = vecs[:, t]
        r = A @ x - lam[t] * (Bd @ x)
        res.append(np.linalg.norm(r) / (abs(lam[t]) * np.linalg.norm(x)))
    return lam, vecs, np.asarray(res)
