"""Synthetic BiGlobal cases: analytic grid and base flow on FD-q nodes.

The workload family is a spanwise-periodic wavy-wall boundary layer:

* wall-normal index i = 0..Ny-1 on a bounded FD-q rule, spanwise index
  j = 0..Nz-1 on a half-open periodic FD-q rule;
* z_j = Lz * j / Nz with Lz = 2*pi (stored monotone; the metrics unwrap
  the periodic copy by Lz);
* y(i, j) = y_w(z_j) + 20 sinh(3 i / (Ny-1)) / sinh(3), with the wall
  y_w(z) = A cos(beta z + phi), beta = 2 pi / Lz; the seed only sets phi;
* d = y - y_w, U = tanh(1.7 d) (1 + 0.1 cos(beta z) exp(-d^2/4)), V = W = 0,
  Crocco-Busemann temperature with an adiabatic-temperature wall
  T = 1 + r (gamma-1)/2 M^2 (1 - U^2), r = sqrt(Pr), and rho = 1/T.

Arrays follow the reference's natural ``k_j_dof`` order: node
n = j * Ny + i, then the component; values are complex interleaved.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .rules import Rule, load_rule


@dataclass
class Physics:
    """Numerical part of the reference ``Recipe`` (Recipe.hpp:17-61)."""
    reynolds: float = 1000.0
    mach: float = 0.5
    prandtl: float = 0.72
    gamma: float = 1.4
    gas_constant: float = 287.0
    reference_viscosity: float = 1.716e-5
    reference_temperature: float = 288.15
    sutherland_constant: float = 110.4
    alpha: complex = 2.43 + 0.0j
    omega: complex = 0.0 + 0.0j      # search centre; lambda_s = Im w - i Re w
    nev: int = 8
    tol: float = 1e-10
    max_it: int = 1000


@dataclass
class Case:
    ny: int
    nz: int
    qy: int
    qz: int
    xi: Rule
    eta: Rule
    spanwise_period: float
    grid: np.ndarray        # [N][3][2] float64
    baseflow: np.ndarray    # [N][5][2] float64
    physics: Physics = field(default_factory=Physics)

    @property
    def nodes(self) -> int:
        return self.ny * self.nz


def make_case(ny: int, nz: int, qy: int = 10, qz: int = 6, amplitude=0.05,
              seed: int = 0, physics: Physics | None = None) -> Case:
    physics = physics or Physics()
    xi = load_rule(ny, qy, periodic=False)
    eta = load_rule(nz, qz, periodic=True)
    lz = 2.0 * math.pi
    beta = 2.0 * math.pi / lz
    phase = 0.0 if seed == 0 else float(
        np.random.default_rng(seed).uniform(0.0, 2.0 * math.pi))
    i = np.arange(ny, dtype=np.float64)
    j = np.arange(nz, dtype=np.float64)
    z = lz * j / nz
    yw = amplitude * np.cos(beta * z + phase)
    ydist = 20.0 * np.sinh(3.0 * i / (ny - 1)) / math.sinh(3.0)
    y = yw[:, None] + ydist[None, :]                       # [nz, ny]
    grid = np.zeros((nz * ny, 3, 2))
    grid[:, 1, 0] = y.reshape(-1)
    grid[:, 2, 0] = np.broadcast_to(z[:, None], (nz, ny)).reshape(-1)
    base = _baseflow(y, yw, z, beta, physics)
    return Case(ny, nz, qy, qz, xi, eta, lz, grid, base, physics)


def _baseflow(y, yw, z, beta, physics) -> np.ndarray:
    """U = tanh(1.7 d)(1 + 0.1 cos(beta z) exp(-d^2/4)), V = W = 0, Crocco-Busemann
    T with T_w = T_aw, rho = 1/T; d = y - y_w.  Arrays [nz, ny] -> [N][5][2]."""
    nz, ny = y.shape
    d = y - yw[:, None]
    u = np.tanh(1.7 * d) * (1.0 + 0.1 * np.cos(beta * z)[:, None] * np.exp(-d * d / 4.0))
    r = math.sqrt(physics.prandtl)
    t = 1.0 + r * (physics.gamma - 1.0) / 2.0 * physics.mach ** 2 * (1.0 - u * u)
    base = np.zeros((nz * ny, 5, 2))
    base[:, 0, 0] = (1.0 / t).reshape(-1)
    base[:, 1, 0] = u.reshape(-1)
    base[:, 4, 0] = t.reshape(-1)
    return base


def rebuild_baseflow(case: Case) -> np.ndarray:
    """The synthetic base flow of case's grid for case.physics (after a Mach
    change); the wall y_w(z) is the grid's first wall-normal line."""
    y = case.grid[:, 1, 0].reshape(case.nz, case.ny)
    z = case.grid[:, 2, 0].reshape(case.nz, case.ny)[:, 0]
    return _baseflow(y, y[:, 0].copy(), z, 2.0 * math.pi / case.spanwise_period, case.physics)


def target_lambda(omega: complex) -> complex:
    """lambda_s = Im(omega) - i Re(omega)  (EigenSolver.cpp:46-48)."""
    return complex(omega.imag, -omega.real)
