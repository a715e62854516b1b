"""Learned shift and start-vector proposal for shift-and-invert Krylov-Schur.

No reference counterpart: the reference always solves around the target
lambda_s = Im(omega) - i Re(omega) from SLEPc's random start vector
(EigenSolver.cpp:46-72).  Here an MLP, trained on eigenpairs the solver
itself produced over (alpha, log10 Re, Mach), predicts

* the nev eigenvalues nearest the target (8 complex numbers), and
* 32 complex coefficients, in a POD basis built from the training modes,
  of the start vector s = sum_k v_k / sqrt(nev) over the phase-fixed wanted
  eigenvectors v_k.

Two ways to use it:

* start (default): Krylov-Schur around the user's target from the POD
  reconstruction of s instead of a pseudo-random vector.  The problem
  solved is the plain one -- the nev eigenvalues nearest lambda_s -- and a
  start vector close to the wanted invariant subspace lets the first
  Krylov basis hold it, so fewer restarts (operator applications) are
  needed.
* shift: factor A - sigma' B at sigma' = the predicted eigenvalue nearest
  the target, ask for nev + extra eigenpairs around sigma' and keep the
  nev nearest the target.  Accepted only when it provably equals the plain
  answer: every eigenvalue within R of the target (R = distance of the
  farthest kept one) lies inside the disk around sigma' that the solve
  covered completely (|lambda_s - sigma'| + R <= r', r' = distance of the
  farthest returned eigenvalue from sigma'); otherwise the plain solve runs
  and its answer is returned.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from . import api
from .case import Physics, target_lambda

N_SHIFTS = 8
N_POD = 32


class MLP:
    """The network of tailor_gb300/csrc/tlr_mlp.cu (FP32 params on the GPU)."""

    def __init__(self, n_in=3, width=256, depth=4, n_out=2 * N_SHIFTS + 2 * N_POD, seed=1):
        self.lib = L.load()
        self.shape = (n_in, width, depth, n_out)
        h = ctypes.c_void_p()
        st = self.lib.tlr_mlp_create(n_in, width, depth, n_out, seed, ctypes.byref(h))
        if st:
            raise api.TailorError(st, "tlr_mlp_create failed")
        self.h = h
        self.n_params = int(self.lib.tlr_mlp_num_params(h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.tlr_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _f32(a):
        return np.ascontiguousarray(a, dtype=np.float32)

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        self._check(self.lib.tlr_mlp_params(self.h, p.ctypes.data, 0))
        return p

    def set_params(self, p) -> None:
        p = self._f32(p)
        self._check(self.lib.tlr_mlp_params(self.h, p.ctypes.data, 1))

    def gradients(self, X, Y):
        X, Y = self._f32(X), self._f32(Y)
        g = np.zeros(self.n_params, np.float32)
        loss = ctypes.c_float()
        self._check(self.lib.tlr_mlp_gradients(self.h, X.ctypes.data, Y.ctypes.data, X.shape[0],
                                               g.ctypes.data, ctypes.byref(loss)))
        return float(loss.value), g

    def train(self, X, Y, epochs=2000, batch=256, lr=1e-3):
        X, Y = self._f32(X), self._f32(Y)
        hist = np.zeros(epochs, np.float32)
        self._check(self.lib.tlr_mlp_train(self.h, X.ctypes.data, Y.ctypes.data, X.shape[0],
                                           epochs, batch, lr, hist.ctypes.data))
        return hist

    def forward(self, X, bf16=False):
        X = self._f32(X)
        Y = np.zeros((X.shape[0], self.shape[3]), np.float32)
        self._check(self.lib.tlr_mlp_forward(self.h, X.ctypes.data, X.shape[0], Y.ctypes.data,
                                             int(bool(bf16))))
        return Y

    @staticmethod
    def _check(st):
        if st:
            raise api.TailorError(st, "MLP call failed")


def features(alpha: float, reynolds: float, mach: float) -> np.ndarray:
    return np.array([alpha, math.log10(reynolds), mach])


def phase_fix(v: np.ndarray) -> np.ndarray:
    """Unit 2-norm, largest-magnitude entry real and positive (the phase
    convention of EigenOutput.cpp:36-82)."""
    v = v / np.linalg.norm(v)
    k = int(np.argmax(np.abs(v)))
    return v * (abs(v[k]) / v[k])


@dataclass
class Sample:
    point: tuple           # (alpha, Re, Mach)
    lam: np.ndarray        # nev eigenvalues, nearest the target first
    mode: np.ndarray       # start-vector target: sum of the phase-fixed wanted modes
    iterations: int
    solves: int


def physics_at(base: Physics, alpha, reynolds, mach, nev) -> Physics:
    return Physics(reynolds=reynolds, mach=mach, prandtl=base.prandtl, gamma=base.gamma,
                   gas_constant=base.gas_constant, reference_viscosity=base.reference_viscosity,
                   reference_temperature=base.reference_temperature,
                   sutherland_constant=base.sutherland_constant, alpha=alpha,
                   omega=base.omega, nev=nev, tol=base.tol, max_it=base.max_it)


def plain_solve(problem: api.Problem, nev: int, precision: int = 1, modes=False):
    api.run_pipeline(problem)
    return api.EigenSolver(problem).solve(nev=nev, precision=precision, modes=modes)


def generate(problem: api.Problem, points, nev=N_SHIFTS, precision=1) -> list[Sample]:
    """Plain solves at every (alpha, Re, Mach) point: the training data."""
    out = []
    base = problem.case.physics
    for (a, re, m) in points:
        problem.set_physics(physics_at(base, a, re, m, nev))
        sol = plain_solve(problem, nev, precision, modes=True)
        tgt = target_lambda(base.omega)
        order = np.argsort(np.abs(sol.lam - tgt))
        s = sum(phase_fix(sol.modes[k]) for k in order) / math.sqrt(len(order))
        out.append(Sample((a, re, m), sol.lam[order], s, sol.diag["iterations"],
                          sol.diag["solves"]))
    return out


@dataclass
class Proposal:
    mlp: MLP
    x_mean: np.ndarray
    x_std: np.ndarray
    y_mean: np.ndarray
    y_std: np.ndarray
    basis: np.ndarray              # [n][N_POD] complex, orthonormal columns
    target: complex
    n_lam: int = N_SHIFTS          # predicted eigenvalues per point
    history: np.ndarray = field(default_factory=lambda: np.zeros(0))
    grid: tuple = ()               # (Ny, Nz) of the training solves, when known

    @classmethod
    def fit(cls, samples: list[Sample], target: complex, epochs=3000, batch=256, lr=1e-3,
            width=256, depth=4, seed=1) -> "Proposal":
        X = np.array([features(*s.point) for s in samples])
        modes = np.stack([s.mode for s in samples], axis=1)
        U, sv, _ = np.linalg.svd(modes, full_matrices=False)
        k = min(N_POD, U.shape[1])
        basis = np.zeros((modes.shape[0], N_POD), complex)
        basis[:, :k] = U[:, :k]
        coef = basis.conj().T @ modes                     # [N_POD][samples]
        nl = min(N_SHIFTS, min(len(s.lam) for s in samples))
        lam = np.array([s.lam[:nl] for s in samples])
        Y = np.concatenate([lam.real, lam.imag, coef.T.real, coef.T.imag], axis=1)
        xm, xs = X.mean(0), X.std(0) + 1e-12
        ym, ys = Y.mean(0), Y.std(0) + 1e-12
        mlp = MLP(3, width, depth, Y.shape[1], seed)
        hist = mlp.train((X - xm) / xs, (Y - ym) / ys, epochs=epochs, batch=batch, lr=lr)
        return cls(mlp, xm, xs, ym, ys, basis, target, nl, hist)

    def save(self, path) -> None:
        """Weights, normalisation, POD basis and target in one .npz, with a
        SHA-256 of the parameters checked on load."""
        import hashlib
        params = self.mlp.get_params()
        np.savez_compressed(path, params=params, shape=np.array(self.mlp.shape),
                            x_mean=self.x_mean, x_std=self.x_std, y_mean=self.y_mean,
                            y_std=self.y_std, basis=self.basis,
                            target=np.array([self.target.real, self.target.imag]),
                            n_lam=np.array(self.n_lam), history=self.history,
                            grid=np.array(self.grid, dtype=np.int64),
                            sha256=np.array(hashlib.sha256(params.tobytes()).hexdigest()))

    @classmethod
    def load(cls, path) -> "Proposal":
        import hashlib
        z = np.load(path)
        params = np.asarray(z["params"], dtype=np.float32)
        if hashlib.sha256(params.tobytes()).hexdigest() != str(z["sha256"]):
            raise ValueError(f"{path}: the stored parameters do not match their digest")
        n_in, width, depth, n_out = (int(v) for v in z["shape"])
        mlp = MLP(n_in, width, depth, n_out)
        if mlp.n_params != params.size:
            raise ValueError(f"{path}: {params.size} parameters for a network of {mlp.n_params}")
        mlp.set_params(params)
        t = z["target"]
        grid = tuple(int(v) for v in z["grid"]) if "grid" in z else ()
        return cls(mlp, z["x_mean"], z["x_std"], z["y_mean"], z["y_std"], z["basis"],
                   complex(t[0], t[1]), int(z["n_lam"]), z["history"], grid)

    def predict(self, points, bf16=True):
        X = np.array([features(*p) for p in points])
        Y = self.mlp.forward((X - self.x_mean) / self.x_std, bf16=bf16) * self.y_std + self.y_mean
        nl = self.n_lam
        lam = Y[:, :nl] + 1j * Y[:, nl:2 * nl]
        c = Y[:, 2 * nl:2 * nl + N_POD] + 1j * Y[:, 2 * nl + N_POD:]
        return lam, c

    def propose(self, point, nev):
        """(sigma', start vector, predicted eigenvalues): sigma' is the
        predicted eigenvalue nearest the target."""
        lam, c = self.predict([point])
        pred = lam[0, :nev]
        sigma = complex(pred[int(np.argmin(np.abs(pred - self.target)))])
        start = self.basis @ c[0]
        return sigma, start, lam[0]

    def start_on(self, case, point) -> np.ndarray:
        """The predicted start vector at `point` on `case`'s grid.  When that
        grid differs from the training grid, the vector is carried over by
        the quintic spline operators of case preparation (tailor_gb300.
        spline): not-a-knot along the wall-normal index, periodic along the
        spanwise index, on the index coordinates that both synthetic grids
        share (y = f(j / (Ny - 1)), z = L k / Nz)."""
        _, start, _ = self.propose(point, self.n_lam)
        if not self.grid or tuple(self.grid) == (case.ny, case.nz):
            return start
        return transfer_vector(start, self.grid, (case.ny, case.nz))


def transfer_vector(v: np.ndarray, src: tuple, dst: tuple) -> np.ndarray:
    """A natural-order vector [Nz][Ny][5] on the grid src = (Ny, Nz) onto
    dst = (Ny', Nz') by quintic spline interpolation in the index
    coordinates (wall-normal j / (Ny - 1) on [0, 1], spanwise k / Nz
    periodic)."""
    from . import spline
    (ny0, nz0), (ny1, nz1) = src, dst
    w_y = spline.bounded_matrix(np.linspace(0.0, 1.0, ny0), np.linspace(0.0, 1.0, ny1))
    w_z = spline.periodic_matrix(nz0, np.arange(nz1) / nz1)
    out = spline.tensor_apply(w_z, np.asarray(v).reshape(nz0, ny0, 5), w_y)
    return np.ascontiguousarray(out.reshape(-1))


def learned_solve(problem: api.Problem, proposal: Proposal, nev: int, precision=1,
                  shift=False, extra=4):
    """Solve with the proposal.  Returns (solution, used_proposal, stats).

    start mode (shift=False) always uses the proposal: the eigenproblem is
    the plain one.  shift mode falls back to the plain solve unless the
    shifted result provably equals it."""
    (a, re, m) = (complex(problem.case.physics.alpha).real, problem.case.physics.reynolds,
                  problem.case.physics.mach)
    sigma, start, _ = proposal.propose((a, re, m), nev)
    tgt = proposal.target
    api.run_pipeline(problem)
    if not shift:
        sol = api.EigenSolver(problem).solve(nev=nev, precision=precision, start=start)
        return sol, True, {"iterations": sol.diag["iterations"], "solves": sol.diag["solves"]}
    stats = {"sigma": sigma}
    try:
        sol = api.EigenSolver(problem).solve(nev=nev + extra, precision=precision, sigma=sigma,
                                             start=start, fallback=False)
    except api.TailorError:
        sol = None
    if sol is not None and len(sol.lam) == nev + extra:
        order = np.argsort(np.abs(sol.lam - tgt))
        keep = order[:nev]
        R = float(np.max(np.abs(sol.lam[keep] - tgt)))
        rp = float(np.max(np.abs(sol.lam - sigma)))
        stats.update(R=R, r_cover=rp, iterations=sol.diag["iterations"],
                     solves=sol.diag["solves"])
        if abs(tgt - sigma) + R <= rp and np.all(sol.residual[keep] <= 1e-10):
            sol.lam = sol.lam[keep]
            sol.residual = sol.residual[keep]
            return sol, True, stats
    plain = api.EigenSolver(problem).solve(nev=nev, precision=precision)
    stats.update(fallback=True, iterations_plain=plain.diag["iterations"],
                 solves_plain=plain.diag["solves"])
    return plain, False, stats
