"""Python mirror of the reference's operator stages over the C ABI.

The reference runs, in Process::run (Process.cpp:50-56), the stage objects
Metrics, BaseFlowDerivatives, GlobalOperator, BoundaryConditions and
EigenSolver on one ProblemData.  ``Problem`` plays ProblemData's role (it
owns one device context); the stage classes keep the reference's method
names (compute / assemble / apply / solve), diagnostics fields and error
messages.  Errors raise ``TailorError`` carrying the status code and the
reference's message text.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .case import Case, rebuild_baseflow

TLR_MAT_M, TLR_MAT_L, TLR_MAT_A, TLR_MAT_B = 0, 1, 2, 3
(OUT_METRICS, OUT_DERIVS, OUT_ROW_PTR, OUT_COL, OUT_M, OUT_L, OUT_A,
 OUT_B) = range(8)


class TailorError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status
        self.message = message


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def _diag_dict(d) -> dict:
    out = {}
    for name, _ in d._fields_:
        v = getattr(d, name)
        out[name] = list(v) if isinstance(v, ctypes.Array) else v
    return out


def make_recipe(case: Case) -> L.Recipe:
    ph = case.physics
    return L.Recipe(case.qy, case.qz, ph.mach, ph.reynolds, ph.prandtl,
                    ph.gas_constant, ph.gamma, ph.reference_viscosity,
                    ph.reference_temperature, ph.sutherland_constant,
                    complex(ph.alpha).real, complex(ph.alpha).imag,
                    complex(ph.omega).real, complex(ph.omega).imag,
                    ph.nev, ph.tol, ph.max_it)


class Problem:
    """Device-resident problem data (the reference's ProblemData)."""

    def __init__(self, case: Case, device: int = -1, load: bool = True):
        self.lib = L.load()
        self.case = case
        self._keep = []
        recipe = make_recipe(case)
        xi, eta = self._rule(case.xi), self._rule(case.eta)
        ctx = ctypes.c_void_p()
        st = self.lib.tlr_ctx_create(ctypes.byref(recipe), ctypes.byref(xi),
                                     ctypes.byref(eta), case.ny, case.nz,
                                     case.spanwise_period, device,
                                     ctypes.byref(ctx))
        if st:
            raise TailorError(st, self.lib.tlr_last_error(None).decode())
        self.ctx = ctx
        if load:
            self.load_fields(case.grid, case.baseflow)

    def _rule(self, r) -> L.Rule:
        nodes = np.ascontiguousarray(r.nodes, dtype=np.float64)
        idx = np.ascontiguousarray(r.indices, dtype=np.int32)
        off = np.ascontiguousarray(r.offsets, dtype=np.int32)
        w = np.ascontiguousarray(r.weights, dtype=np.float64)
        self._keep += [nodes, idx, off, w]
        return L.Rule(r.n, r.q, int(r.periodic), r.period, nodes.ctypes.data,
                      idx.ctypes.data, off.ctypes.data, w.ctypes.data)

    def check(self, st: int) -> None:
        if st:
            raise TailorError(st, self.lib.tlr_last_error(self.ctx).decode())

    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.lib.tlr_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ----------------------------------------------------------- data
    def load_fields(self, grid: np.ndarray, baseflow: np.ndarray) -> None:
        g = np.ascontiguousarray(grid, dtype=np.float64)
        b = np.ascontiguousarray(baseflow, dtype=np.float64)
        self.check(self.lib.tlr_load_fields(self.ctx, _ptr(g), _ptr(b)))

    def set_alpha(self, alpha: complex, omega: complex | None = None) -> None:
        omega = self.case.physics.omega if omega is None else omega
        self.check(self.lib.tlr_set_alpha(self.ctx, complex(alpha).real,
                                          complex(alpha).imag,
                                          complex(omega).real,
                                          complex(omega).imag))

    def set_physics(self, physics) -> None:
        """New Re / Mach / alpha / target on the same grid (re-run the stages
        after).  The synthetic base flow depends on Mach (Crocco-Busemann
        temperature), so a new Mach reloads it."""
        mach_changed = physics.mach != self.case.physics.mach
        self.case.physics = physics
        if mach_changed:
            self.case.baseflow = rebuild_baseflow(self.case)
            self.load_fields(self.case.grid, self.case.baseflow)
        r = make_recipe(self.case)
        self.check(self.lib.tlr_set_physics(self.ctx, ctypes.byref(r)))

    def copy_out(self, what: int) -> np.ndarray:
        nbytes = self.lib.tlr_out_bytes(self.ctx, what)
        nn = self.case.nodes
        if what == OUT_METRICS:
            a = np.empty((nn, 10))
        elif what == OUT_DERIVS:
            a = np.empty((nn, 25))
        elif what in (OUT_ROW_PTR, OUT_COL):
            a = np.empty(nbytes // 4, dtype=np.int32)
        else:
            a = np.empty((nbytes // 400, 5, 5, 2))
        self.check(self.lib.tlr_copy_out(self.ctx, what, _ptr(a), nbytes))
        return a

    def spmv(self, which: int, x: np.ndarray) -> np.ndarray:
        xr = np.ascontiguousarray(np.stack([x.real, x.imag], -1), dtype=np.float64)
        y = np.empty_like(xr)
        self.check(self.lib.tlr_spmv(self.ctx, which, _ptr(xr), _ptr(y), 0))
        return y[..., 0] + 1j * y[..., 1]


class Metrics:
    """Metrics::compute (Metrics.hpp:59-87)."""

    def __init__(self, problem: Problem):
        self.p = problem

    def compute(self) -> dict:
        d = L.MetricDiag()
        self.p.check(self.p.lib.tlr_metrics(self.p.ctx, ctypes.byref(d)))
        return _diag_dict(d)


class BaseFlowDerivatives:
    """BaseFlowDerivatives::compute (BaseFlowDerivatives.hpp:83-111)."""

    def __init__(self, problem: Problem):
        self.p = problem

    def compute(self) -> dict:
        d = L.DerivDiag()
        self.p.check(self.p.lib.tlr_baseflow_derivatives(self.p.ctx, ctypes.byref(d)))
        return _diag_dict(d)


class GlobalOperator:
    """GlobalOperator::assemble (GlobalOperator.hpp:41-71)."""

    def __init__(self, problem: Problem):
        self.p = problem

    def assemble(self) -> dict:
        d = L.OperatorDiag()
        self.p.check(self.p.lib.tlr_assemble(self.p.ctx, ctypes.byref(d)))
        return _diag_dict(d)


class BoundaryConditions:
    """BoundaryConditions::apply (BoundaryConditions.hpp:46-65)."""

    def __init__(self, problem: Problem):
        self.p = problem

    def apply(self) -> dict:
        d = L.BcDiag()
        self.p.check(self.p.lib.tlr_apply_bc(self.p.ctx, ctypes.byref(d)))
        return _diag_dict(d)


@dataclass
class EigenSolution:
    lam: np.ndarray
    residual: np.ndarray
    modes: np.ndarray | None
    diag: dict

    @property
    def omega(self) -> np.ndarray:
        return 1j * self.lam


# statuses after which a mixed-form solve is repeated in FP64: not converged,
# a timed-out bounded device wait, a singular (perturbed) factorisation
_FALLBACK_STATUS = (13, 14, 15)


class EigenSolver:
    """EigenSolver::solve (EigenSolver.hpp:48-72): shift-invert
    Krylov-Schur on (A_bc, B_bc) with lambda target Im w - i Re w."""

    def __init__(self, problem: Problem):
        self.p = problem

    def solve(self, nev: int = 0, ncv: int = 0, tol: float = 0.0,
              max_it: int = 0, precision: int = 0, sigma: complex | None = None,
              start: np.ndarray | None = None, modes: bool = False,
              cuda_core_schur: int = 0, persistent_solve: bool = False,
              solve_block: int = 0, refinement: str = "ir",
              panel_width: int = 0, cluster_panel: int = 0,
              fallback: bool = True, block: int = 0,
              warm_start: bool = False, ring_slack_percent: int = 0,
              conv_check: int = 0, solve_wave: bool = False,
              fp64_acceptance: bool = False) -> EigenSolution:
        """With fallback, a mixed-form solve (precision 1) that fails to
        converge (or hits a singular pivot or a timed-out device wait) is
        repeated in the plain FP64 form; diag["fallback"] is 1 then.

        start: one start vector [5N], or several [k][5N] (up to the block
        size); block: Krylov block size (1, 2, 4 or 8; 0 = 1); warm_start:
        without start, begin from the previous solve's Ritz vectors on this
        problem.  ring_slack_percent: the factor's nested-dissection
        ordering (tlr_solve_opts; 0: the solver's); conv_check: operator
        applications between convergence tests inside an expansion (0: the
        solver's 4; -1: only when the basis is full); solve_wave: one
        dependency-driven launch per level of the triangular solves instead
        of one launch per block step (the same bits, measured slower);
        fp64_acceptance: accept each refined application on an FP64
        residual instead of a float-float one (mixed form)."""
        kw = dict(nev=nev, ncv=ncv, tol=tol, max_it=max_it, sigma=sigma, start=start,
                  modes=modes, cuda_core_schur=cuda_core_schur,
                  persistent_solve=persistent_solve, solve_block=solve_block,
                  refinement=refinement, panel_width=panel_width, cluster_panel=cluster_panel,
                  block=block, warm_start=warm_start, ring_slack_percent=ring_slack_percent,
                  conv_check=conv_check, solve_wave=solve_wave,
                  fp64_acceptance=fp64_acceptance)
        if precision == 1 and fallback:
            try:
                sol = self._solve(precision=1, **kw)
            except TailorError as e:
                if e.status not in _FALLBACK_STATUS:
                    raise
                sol = self._solve(precision=0, **kw)
                sol.diag["fallback"] = 1
                return sol
        else:
            sol = self._solve(precision=precision, **kw)
        sol.diag["fallback"] = 0
        return sol

    def _solve(self, nev, ncv, tol, max_it, precision, sigma, start, modes, cuda_core_schur,
               persistent_solve, solve_block, refinement, panel_width,
               cluster_panel, block=0, warm_start=False,
               ring_slack_percent=0, conv_check=0, solve_wave=False,
               fp64_acceptance=False) -> EigenSolution:
        ph = self.p.case.physics
        k = nev or ph.nev
        opts = L.SolveOpts(nev, ncv, tol, max_it, precision,
                           0.0 if sigma is None else complex(sigma).real,
                           0.0 if sigma is None else complex(sigma).imag,
                           0 if sigma is None else 1, None,
                           # False/True, or 2: tile-staged tcgen05 update
                           int(cuda_core_schur),
                           int(solve_block), 1 if refinement == "gmres" else 0,
                           int(panel_width), int(cluster_panel),
                           int(bool(persistent_solve)), int(block), 0,
                           int(bool(warm_start)), int(ring_slack_percent), int(conv_check),
                           int(bool(solve_wave)), int(bool(fp64_acceptance)))
        if start is not None:
            st = np.atleast_2d(np.asarray(start, dtype=np.complex128))
            s = np.ascontiguousarray(np.stack([st.real, st.imag], -1), dtype=np.float64)
            self.p._keep.append(s)
            opts.start = s.ctypes.data
            opts.nstart = st.shape[0]
        lam = np.zeros((k, 2))
        res = np.zeros(k)
        vec = np.zeros((k, 5 * self.p.case.nodes, 2)) if modes else None
        d = L.EigDiag()
        st = self.p.lib.tlr_solve(self.p.ctx, ctypes.byref(opts), _ptr(lam),
                                  _ptr(res), None if vec is None else _ptr(vec),
                                  ctypes.byref(d))
        self.p.check(st)
        nconv = min(d.converged, k)
        lam_c = lam[:nconv, 0] + 1j * lam[:nconv, 1]
        vec_c = None if vec is None else vec[:nconv, :, 0] + 1j * vec[:nconv, :, 1]
        return EigenSolution(lam_c, res[:nconv], vec_c, _diag_dict(d))


class PencilProblem(Problem):
    """An explicit generalized pencil A x = lambda B x in place of the
    assembled operators: the reference's EigenSolver overload for small
    independently known problems (EigenSolver.hpp:60-67).  B must be block
    diagonal in 5 x 5 blocks.  ``physics`` supplies omega (the search
    centre), nev, tol and max_it; ``EigenSolver(p).solve(...)`` runs as for
    a grid problem and ``solve_pencil`` trims the modes to n entries."""

    def __init__(self, A, B, physics=None, device: int = -1):
        from types import SimpleNamespace
        from .case import Physics
        self.lib = L.load()
        self._keep = []
        self.ctx = None
        A = np.asarray(A, dtype=np.complex128)
        B = np.asarray(B, dtype=np.complex128)
        if A.ndim != 2 or A.shape[0] != A.shape[1] or B.shape != A.shape:
            raise ValueError("A and B must be square matrices of the same order")
        self.n = A.shape[0]
        ph = physics or Physics()
        self.case = SimpleNamespace(nodes=(self.n + 4) // 5, physics=ph)
        recipe = L.Recipe(0, 0, ph.mach, ph.reynolds, ph.prandtl, ph.gas_constant, ph.gamma,
                          ph.reference_viscosity, ph.reference_temperature,
                          ph.sutherland_constant, complex(ph.alpha).real,
                          complex(ph.alpha).imag, complex(ph.omega).real,
                          complex(ph.omega).imag, ph.nev, ph.tol, ph.max_it)
        # column-major, interleaved (re, im)
        a = np.ascontiguousarray(np.stack([A.T.real, A.T.imag], axis=-1))
        b = np.ascontiguousarray(np.stack([B.T.real, B.T.imag], axis=-1))
        ctx = ctypes.c_void_p()
        st = self.lib.tlr_pencil_create(ctypes.byref(recipe), self.n, a.ctypes.data,
                                        b.ctypes.data, device, ctypes.byref(ctx))
        if st:
            raise TailorError(st, self.lib.tlr_last_error(None).decode())
        self.ctx = ctx


def solve_pencil(A, B, omega: complex = 0j, nev: int = 2, tol: float = 1e-10,
                 max_it: int = 1000, precision: int = 0, modes: bool = True,
                 **kw) -> EigenSolution:
    """The nev eigenpairs of A x = lambda B x nearest lambda_s = Im(omega) -
    i Re(omega) (EigenSolver.cpp:46-48), on the GPU."""
    from .case import Physics
    with PencilProblem(A, B, Physics(omega=omega, nev=nev, tol=tol, max_it=max_it)) as p:
        sol = EigenSolver(p).solve(nev=nev, tol=tol, max_it=max_it, precision=precision,
                                   modes=modes, **kw)
        if sol.modes is not None:
            sol.modes = sol.modes[:, :p.n]
    return sol


@dataclass
class SweepResult:
    lam: np.ndarray        # [points][nev] complex (0 where not converged)
    residual: np.ndarray   # [points][nev] (-1 where not solved)
    status: np.ndarray     # [points] tlr status
    diag: dict             # sweep diagnostics
    point_diag: list       # per point solve diagnostics


def sweep(cases, points, nev: int = 0, precision: int = 1, workers: int = 0,
          autotune: bool = True, tol: float = 0.0, ncv: int = 0, max_it: int = 0,
          starts=None, device: int = 0, raise_on_error: bool = True,
          fallback: bool = True, block: int = 0, warm_start: bool = False,
          ring_slack_percent: int = 0, conv_check: int = 0) -> SweepResult:
    """Batched alpha-sweep (tlr_sweep): points are (class index, alpha) or
    (class index, alpha, Re); each class is a Case (grid, base flow,
    physics) whose alpha (and Re when given) is overridden.  With fallback,
    points that fail in the mixed form are solved again, one at a time, in
    the plain FP64 form (diag["fallback_points"] counts them).  block: the
    Krylov block size of every solve; warm_start: each worker takes a
    contiguous run of the points and starts every point but the run's first
    from its predecessor's Ritz vectors (starts[i], when given, wins);
    ring_slack_percent, conv_check: as for EigenSolver.solve, for every point."""
    lib = L.load()
    keep = []
    holder = Problem.__new__(Problem)  # reuse the rule marshalling
    holder._keep = keep
    gcs = (L.GridClass * len(cases))()
    for c, case in enumerate(cases):
        r = make_recipe(case)
        xi, eta = holder._rule(case.xi), holder._rule(case.eta)
        g = np.ascontiguousarray(case.grid, dtype=np.float64)
        b = np.ascontiguousarray(case.baseflow, dtype=np.float64)
        keep += [r, xi, eta, g, b]
        gcs[c] = L.GridClass(ctypes.addressof(r), ctypes.addressof(xi), ctypes.addressof(eta),
                             case.ny, case.nz, case.spanwise_period, _ptr(g), _ptr(b))
    npts = len(points)
    pts = (L.SweepPoint * max(npts, 1))()
    for i, pt in enumerate(points):
        c, a = pt[0], pt[1]
        re_ov = float(pt[2]) if len(pt) > 2 else 0.0
        s = None
        if starts is not None and starts[i] is not None:
            v = np.ascontiguousarray(np.stack([starts[i].real, starts[i].imag], -1),
                                     dtype=np.float64)
            keep.append(v)
            s = v.ctypes.data
        pts[i] = L.SweepPoint(int(c), complex(a).real, complex(a).imag, s, re_ov)
    k = nev or cases[0].physics.nev
    opts = L.SweepOpts(L.SolveOpts(k, ncv, tol, max_it, precision, 0.0, 0.0, 0, None, 0, 0, 0, 0,
                                   0, 0, int(block), 0, int(bool(warm_start)),
                                   int(ring_slack_percent), int(conv_check)),
                       workers, int(bool(autotune)), device)
    lam = np.zeros((max(npts, 1), k, 2))
    res = np.zeros((max(npts, 1), k))
    st = np.zeros(max(npts, 1), dtype=np.int32)
    pd = (L.EigDiag * max(npts, 1))()
    d = L.SweepDiag()
    rc = lib.tlr_sweep(gcs, len(cases), pts, npts, ctypes.byref(opts), _ptr(lam), _ptr(res),
                       st.ctypes.data, pd, ctypes.byref(d))
    message = lib.tlr_last_error(None).decode() if rc else ""
    point_diag = [_diag_dict(pd[i]) for i in range(npts)]
    fallbacks = 0
    failed = np.flatnonzero(st[:npts]) if rc else []
    if fallback and precision == 1 and len(failed):
        fallbacks = _fallback_points(cases, points, failed, k, ncv, tol, max_it, starts,
                                     device, lam, res, st, point_diag)
        if not np.any(st[:npts]):  # every failed point recovered in FP64
            rc = 0
    if rc and raise_on_error:
        raise TailorError(rc, message)
    nc = len(cases)
    diag = {"wall_ms": d.wall_ms, "points": d.points, "failed": d.failed,
            "workers": d.workers, "converged_pairs": d.converged_pairs,
            "cuda_core_schur": list(d.cuda_core_schur[:nc]),
            "solve_block": list(d.solve_block[:nc]),
            "tune_factor_ms": [list(d.tune_factor_ms[c]) for c in range(nc)],
            "tune_trisolve_ms": [list(d.tune_trisolve_ms[c]) for c in range(nc)],
            "panel_width": list(d.panel_width[:nc]),
            "tune_wide_factor_ms": list(d.tune_wide_factor_ms[:nc]),
            "fallback_points": fallbacks}
    return SweepResult(lam[:npts, :, 0] + 1j * lam[:npts, :, 1], res[:npts], st[:npts], diag,
                       point_diag)


def _fallback_points(cases, points, failed, k, ncv, tol, max_it, starts, device, lam, res, st,
                     point_diag) -> int:
    """Solve the failed sweep points again in FP64, one at a time, on one
    context per grid class (copies of the classes, so the callers' cases are
    not modified); fills lam / res / st / point_diag in place."""
    import dataclasses
    probs, done = {}, 0
    try:
        for i in failed:
            c, a = int(points[i][0]), complex(points[i][1])
            re_ov = float(points[i][2]) if len(points[i]) > 2 else 0.0
            if c not in probs:
                probs[c] = Problem(dataclasses.replace(cases[c]), device=device)
            p = probs[c]
            p.set_physics(dataclasses.replace(cases[c].physics, alpha=a,
                                              reynolds=re_ov or cases[c].physics.reynolds))
            try:
                run_pipeline(p)
                sol = EigenSolver(p).solve(nev=k, ncv=ncv, tol=tol, max_it=max_it, precision=0,
                                           start=None if starts is None else starts[i])
            except TailorError:
                continue
            n = len(sol.lam)
            lam[i] = 0.0
            lam[i, :n, 0], lam[i, :n, 1] = sol.lam.real, sol.lam.imag
            res[i] = -1.0
            res[i, :n] = sol.residual
            st[i] = 0
            point_diag[i] = dict(sol.diag, fallback=1)
            done += 1
    finally:
        for p in probs.values():
            p.close()
    return done


def symbolic_analysis(xi, eta, leaf_nodes: int = 0, ring_slack_percent: int = 0) -> dict:
    """Host-only symbolic analysis (tlr_symbolic_analyze) of the grid of the
    rules xi (bounded) and eta (periodic): the ordering and front tree the
    solver factors, with its flop and storage counts.  Returns the info
    fields plus node_rank, node_front [Ny*Nz] and front_parent [fronts]."""
    lib = L.load()
    holder = Problem.__new__(Problem)  # reuse the rule marshalling
    holder._keep = []
    rx, re_ = holder._rule(xi), holder._rule(eta)
    info = L.SymbolicInfo()
    nn = xi.n * eta.n
    rank = np.zeros(nn, dtype=np.int32)
    front = np.zeros(nn, dtype=np.int32)
    args = (ctypes.byref(rx), ctypes.byref(re_), int(leaf_nodes), int(ring_slack_percent),
            ctypes.byref(info))
    st = lib.tlr_symbolic_analyze(*args, None, None, None, 0)
    if st:
        raise TailorError(st, lib.tlr_last_error(None).decode())
    parent = np.zeros(max(info.fronts, 1), dtype=np.int32)
    st = lib.tlr_symbolic_analyze(*args, rank.ctypes.data, front.ctypes.data,
                                  parent.ctypes.data, info.fronts)
    if st:
        raise TailorError(st, lib.tlr_last_error(None).decode())
    out = {name: getattr(info, name) for name, _ in L.SymbolicInfo._fields_}
    out.update(node_rank=rank, node_front=front, front_parent=parent[:info.fronts])
    return out


def lns_points(case_or_physics, q: np.ndarray, qy: int = 10, qz: int = 6):
    """Pointwise LNS blocks on the GPU: q [np][10][5] -> [np][11][5][5]."""
    lib = L.load()
    ph = getattr(case_or_physics, "physics", case_or_physics)
    r = L.Recipe(qy, qz, ph.mach, ph.reynolds, ph.prandtl, ph.gas_constant,
                 ph.gamma, ph.reference_viscosity, ph.reference_temperature,
                 ph.sutherland_constant, 0, 0, 0, 0, 1, 1e-10, 1)
    q = np.ascontiguousarray(q, dtype=np.float64)
    npts = q.shape[0]
    out = np.zeros((npts, 11, 5, 5))
    st = np.zeros(npts, dtype=np.int32)
    rc = lib.tlr_lns_points(ctypes.byref(r), npts, _ptr(q), _ptr(out), _ptr(st))
    if rc:
        raise TailorError(rc, "tlr_lns_points failed")
    return st, out


def transform_points(alpha: np.ndarray, phys: np.ndarray, metrics: np.ndarray):
    """Fourier + curvilinear transforms on the GPU for arbitrary blocks."""
    lib = L.load()
    a = np.ascontiguousarray(np.stack([alpha.real, alpha.imag], -1), dtype=np.float64)
    phys = np.ascontiguousarray(phys, dtype=np.float64)
    met = np.ascontiguousarray(metrics, dtype=np.float64)
    npts = a.shape[0]
    four = np.zeros((npts, 7, 25, 2))
    curv = np.zeros((npts, 7, 25, 2))
    st = np.zeros(npts, dtype=np.int32)
    rc = lib.tlr_transform_points(npts, _ptr(a), _ptr(phys), _ptr(met), _ptr(four),
                                  _ptr(curv), _ptr(st))
    if rc:
        raise TailorError(rc, "tlr_transform_points failed")
    c = lambda v: (v[..., 0] + 1j * v[..., 1]).reshape(npts, 7, 5, 5)
    return st, c(four), c(curv)


def run_pipeline(problem: Problem) -> dict:
    """Process::run's stage order (Process.cpp:50-56) up to the BCs."""
    out = {}
    out["metrics"] = Metrics(problem).compute()
    out["derivatives"] = BaseFlowDerivatives(problem).compute()
    out["operator"] = GlobalOperator(problem).assemble()
    out["bc"] = BoundaryConditions(problem).apply()
    return out
