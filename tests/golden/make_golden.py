"""Regenerate the golden fixtures of tests/golden/.

The reference pins its pointwise physics with two Fortran fixture
generators that CMake compiles at build time
(tests/CPlusPlus/generate_lns_coefficients_gold.f90 and
generate_lns_transform_gold.f90; CMakeLists.txt:190-240).  No Fortran
compiler is available here, so this script restates those two programs in
Python -- same input points, same physics constants, the Fortran's own
expressions -- and writes the same text format (one value per line,
17 significant digits; the transform file holds real/imaginary pairs).

    lns_coefficients_gold.txt   2 points x 11 matrices x 5 x 5
    lns_transform_gold.txt      2 points x (7 Fourier + 7 curvilinear) x 5 x 5
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def lns_points() -> np.ndarray:
    """points(5,10,2) of generate_lns_coefficients_gold.f90:18-35, as
    [2][10][5] (value, dx, dy, dz, dxx, dyy, dzz, dxy, dxz, dyz)."""
    p = np.zeros((2, 10, 5))
    p[0, 0] = [1.2, 2.3, 0.14, -0.08, 1.4]
    p[0, 1] = [0.01, 0.02, -0.03, 0.04, 0.05]
    p[0, 2] = [-0.02, 0.07, 0.04, -0.05, 0.06]
    p[0, 3] = [0.03, -0.02, 0.08, 0.09, -0.04]
    p[0, 4] = [0.004, -0.006, 0.007, -0.008, 0.009]
    p[0, 5] = [-0.005, 0.011, -0.012, 0.013, -0.014]
    p[0, 6] = [0.006, -0.015, 0.016, -0.017, 0.018]
    p[0, 7] = [-0.007, 0.019, -0.020, 0.021, -0.022]
    p[0, 8] = [0.008, -0.023, 0.024, -0.025, 0.026]
    p[0, 9] = [-0.009, 0.027, -0.028, 0.029, -0.030]
    p[1, 0] = [0.95, 3.1, -0.12, 0.06, 1.15]
    p[1, 2] = [0.015, -0.045, 0.025, 0.035, -0.055]
    p[1, 3] = [-0.012, 0.038, -0.028, 0.042, 0.048]
    p[1, 5] = [0.003, -0.009, 0.008, -0.007, 0.011]
    p[1, 6] = [-0.004, 0.010, -0.012, 0.014, -0.013]
    p[1, 9] = [0.005, -0.016, 0.017, -0.018, 0.019]
    return p


# canonical physics of the fixture (generate_lns_coefficients_gold.f90:58-59)
RE, MA, PR, GAMMA, TE, C1 = 32500.0, 6.0, 0.72, 1.4, 63.334, 110.4


def get_unadorned(q: np.ndarray) -> np.ndarray:
    """The 11 matrices G, A, B, C, D, Vxx, Vxy, Vxz, Vyy, Vyz, Vzz with the
    Fortran's 1-based (row, column) entries written 0-based."""
    d1d3, d2d3, d4d3 = 1.0 / 3.0, 2.0 / 3.0, 4.0 / 3.0
    rho, U, V, W, T = q[0]
    rhox, Ux, Vx, Wx, Tx = q[1]
    rhoy, Uy, Vy, Wy, Ty = q[2]
    rhoz, Uz, Vz, Wz, Tz = q[3]
    _, Uxx, nVxx, Wxx, Txx = q[4]
    _, Uyy, nVyy, Wyy, Tyy = q[5]
    _, Uzz, nVzz, Wzz, Tzz = q[6]
    _, Uxy, nVxy, Wxy, _ = q[7]
    _, Uxz, nVxz, Wxz, _ = q[8]
    _, Uyz, nVyz, Wyz, _ = q[9]
    Re, Pr = RE, PR
    Pe = 1.0 / (GAMMA * MA * MA)
    g2 = 1.0 / ((GAMMA - 1.0) * MA * MA)
    cm = C1 / TE
    mu = T * np.sqrt(T) * (1.0 + cm) / (T + cm)
    muT = mu * (1.5 / T - 1.0 / (T + cm))
    muTT = muT * (1.5 / T - 1.0 / (T + cm)) - mu * (1.5 / T ** 2 - 1.0 / (T + cm) ** 2)
    mux, muy, muz = muT * Tx, muT * Ty, muT * Tz
    M = np.zeros((11, 5, 5))
    G, A, B, C, D, Vxxm, Vxym, Vxzm, Vyym, Vyzm, Vzzm = M
    G[0, 0] = 1; G[1, 1] = rho; G[2, 2] = rho; G[3, 3] = rho
    G[4, 0] = -Pe * T; G[4, 4] = rho * g2 - Pe * rho
    A[0, 0] = U; A[0, 1] = rho; A[1, 0] = Pe * T
    A[1, 1] = rho * U - d4d3 * mux / Re
    A[1, 2] = -muy / Re; A[1, 3] = -muz / Re
    A[1, 4] = Pe * rho - muT / Re * (d4d3 * Ux - d2d3 * Vy - d2d3 * Wz)
    A[2, 1] = d2d3 * muy / Re; A[2, 2] = rho * U - mux / Re
    A[2, 4] = -muT * (Uy + Vx) / Re
    A[3, 1] = d2d3 * muz / Re; A[3, 3] = rho * U - mux / Re
    A[3, 4] = -muT * (Wx + Uz) / Re
    A[4, 0] = -Pe * U * T
    A[4, 1] = -2.0 * mu * (d4d3 * Ux - d2d3 * Vy - d2d3 * Wz) / Re
    A[4, 2] = -2.0 * mu * (Uy + Vx) / Re
    A[4, 3] = -2.0 * mu * (Wx + Uz) / Re
    A[4, 4] = rho * U * g2 - rho * U * Pe - 2.0 * Tx * muT / Re / Pr * g2
    B[0, 0] = V; B[0, 2] = rho
    B[1, 1] = rho * V - muy / Re; B[1, 2] = d2d3 * mux / Re
    B[1, 4] = -muT * (Uy + Vx) / Re
    B[2, 0] = Pe * T; B[2, 1] = -mux / Re
    B[2, 2] = rho * V - d4d3 * muy / Re; B[2, 3] = -muz / Re
    B[2, 4] = Pe * rho - muT * (-d2d3 * Ux + d4d3 * Vy - d2d3 * Wz) / Re
    B[3, 2] = d2d3 * muz / Re; B[3, 3] = rho * V - muy / Re
    B[3, 4] = -muT * (Vz + Wy) / Re
    B[4, 0] = -Pe * V * T; B[4, 1] = -2.0 * mu * (Uy + Vx) / Re
    B[4, 2] = -2.0 * mu * (-d2d3 * Ux + d4d3 * Vy - d2d3 * Wz) / Re
    B[4, 3] = -2.0 * mu * (Vz + Wy) / Re
    B[4, 4] = rho * V * g2 - rho * V * Pe - 2.0 * Ty * muT * g2 / Re / Pr
    C[0, 0] = W; C[0, 3] = rho
    C[1, 1] = rho * W - muz / Re; C[1, 3] = d2d3 * mux / Re
    C[1, 4] = -muT * (Wx + Uz) / Re
    C[2, 2] = rho * W - muz / Re; C[2, 3] = d2d3 * muy / Re
    C[2, 4] = -muT * (Vz + Wy) / Re
    C[3, 0] = Pe * T; C[3, 1] = -mux / Re; C[3, 2] = -muy / Re
    C[3, 3] = rho * W - d4d3 * muz / Re
    C[3, 4] = Pe * rho - muT * (-d2d3 * Ux - d2d3 * Vy + d4d3 * Wz) / Re
    C[4, 0] = -Pe * W * T; C[4, 1] = -2.0 * mu * (Wx + Uz) / Re
    C[4, 2] = -2.0 * mu * (Vz + Wy) / Re
    C[4, 3] = -2.0 * mu * (-d2d3 * Ux - d2d3 * Vy + d4d3 * Wz) / Re
    C[4, 4] = rho * W * g2 - rho * W * Pe - 2.0 * Tz * muT * g2 / Re / Pr
    D[0, 0] = Ux + Vy + Wz; D[0, 1] = rhox; D[0, 2] = rhoy; D[0, 3] = rhoz
    D[1, 0] = U * Ux + V * Uy + W * Uz + Pe * Tx
    D[1, 1] = rho * Ux; D[1, 2] = rho * Uy; D[1, 3] = rho * Uz
    D[1, 4] = Pe * rhox - (muTT * Tx * d2d3 * (2.0 * Ux - Vy - Wz) +
                           muTT * Ty * (Uy + Vx) + muTT * Tz * (Wx + Uz) +
                           muT * (d4d3 * Uxx + Uyy + Uzz + d1d3 * nVxy + d1d3 * Wxz)) / Re
    D[2, 0] = U * Vx + V * Vy + W * Vz + Pe * Ty
    D[2, 1] = rho * Vx; D[2, 2] = rho * Vy; D[2, 3] = rho * Vz
    D[2, 4] = Pe * rhoy - (muTT * Tx * (Uy + Vx) +
                           muTT * Ty * d2d3 * (-Ux + 2.0 * Vy - Wz) + muTT * Tz * (Vz + Wy) +
                           muT * (nVxx + d4d3 * nVyy + nVzz + d1d3 * Uxy + d1d3 * Wyz)) / Re
    D[3, 0] = U * Wx + V * Wy + W * Wz + Pe * Tz
    D[3, 1] = rho * Wx; D[3, 2] = rho * Wy; D[3, 3] = rho * Wz
    D[3, 4] = Pe * rhoz - (muTT * Tx * (Wx + Uz) + muTT * Ty * (Vz + Wy) +
                           muTT * Tz * d2d3 * (-Ux - Vy + 2.0 * Wz) +
                           muT * (Wxx + Wyy + d4d3 * Wzz + d1d3 * Uxz + d1d3 * nVyz)) / Re
    D[4, 0] = (g2 - Pe) * (U * Tx + V * Ty + W * Tz)
    D[4, 1] = rho * Tx * g2 - Pe * (rho * Tx + T * rhox)
    D[4, 2] = rho * Ty * g2 - Pe * (rho * Ty + T * rhoy)
    D[4, 3] = rho * Tz * g2 - Pe * (rho * Tz + T * rhoz)
    D[4, 4] = (-Pe * (U * rhox + V * rhoy + W * rhoz)
               - (Txx + Tyy + Tzz) * muT * g2 / Re / Pr
               - (Tx * Tx + Ty * Ty + Tz * Tz) * muTT * g2 / Re / Pr
               - muT * (Uy * Uy + Vx * Vx + 2.0 * Uy * Vx + Uz * Uz + Wx * Wx +
                        2.0 * Uz * Wx + Vz * Vz + Wy * Wy + 2.0 * Vz * Wy) / Re
               - muT * d4d3 * (Ux * Ux + Vy * Vy + Wz * Wz - Ux * Wz - Ux * Vy - Vy * Wz) / Re)
    Vxxm[1, 1] = d4d3 * mu / Re; Vxxm[2, 2] = mu / Re
    Vxxm[3, 3] = mu / Re; Vxxm[4, 4] = mu * g2 / Re / Pr
    Vyym[1, 1] = mu / Re; Vyym[2, 2] = d4d3 * mu / Re
    Vyym[3, 3] = mu / Re; Vyym[4, 4] = mu * g2 / Re / Pr
    Vzzm[1, 1] = mu / Re; Vzzm[2, 2] = mu / Re
    Vzzm[3, 3] = d4d3 * mu / Re; Vzzm[4, 4] = mu * g2 / Re / Pr
    Vxym[1, 2] = d1d3 * mu / Re; Vxym[2, 1] = d1d3 * mu / Re
    Vxzm[1, 3] = d1d3 * mu / Re; Vxzm[3, 1] = d1d3 * mu / Re
    Vyzm[2, 3] = d1d3 * mu / Re; Vyzm[3, 2] = d1d3 * mu / Re
    return M


def transform_physical(point: int) -> np.ndarray:
    """make_physical (generate_lns_transform_gold.f90): 1-based point."""
    out = np.zeros((11, 5, 5))
    for m in range(1, 12):
        for r in range(1, 6):
            for c in range(1, 6):
                v = 0.13 * m + 0.017 * r + 0.003 * c + 0.0007 * point
                if (m + r + c + point) % 2 == 0:
                    v = -v
                out[m - 1, r - 1, c - 1] = v
    return out


def transform_parameters(point: int):
    if point == 1:
        return complex(2.43, 0.17), np.array(
            [0.81, -0.23, 0.19, 1.07, -0.031, 0.024, -0.017, 0.028, -0.022, 0.013])
    return complex(-0.64, 0.29), np.array(
        [1.14, 0.37, -0.26, 0.72, 0.041, -0.036, 0.025, -0.033, 0.019, -0.027])


def streamwise_fourier(phys: np.ndarray, alpha: complex) -> np.ndarray:
    ph = phys.astype(np.complex128)
    ci = 1j
    f = np.zeros((7, 5, 5), dtype=np.complex128)
    f[0] = ph[0]
    f[1] = ph[4] + ci * alpha * ph[1] + alpha * alpha * ph[5]
    f[2] = ph[2] - ci * alpha * ph[6]
    f[3] = ph[3] - ci * alpha * ph[7]
    f[4] = ph[8]
    f[5] = ph[9]
    f[6] = ph[10]
    return f


def curvilinear_transform(f: np.ndarray, m: np.ndarray) -> np.ndarray:
    xy, xz, ey, ez, xyy, xzz, xyz, eyy, ezz, eyz = m
    c = np.zeros((7, 5, 5), dtype=np.complex128)
    c[0] = f[0]
    c[1] = f[1]
    c[2] = xy * f[2] + xz * f[3] - xyy * f[4] - xzz * f[6] - xyz * f[5]
    c[3] = ey * f[2] + ez * f[3] - eyy * f[4] - ezz * f[6] - eyz * f[5]
    c[4] = xy * xy * f[4] + xz * xz * f[6] + xy * xz * f[5]
    c[5] = 2.0 * xy * ey * f[4] + 2.0 * xz * ez * f[6] + (xy * ez + ey * xz) * f[5]
    c[6] = ey * ey * f[4] + ez * ez * f[6] + ey * ez * f[5]
    return c


def main() -> None:
    lines = []
    for q in lns_points():
        for mat in get_unadorned(q):
            lines += [f"{v: .17E}" for v in mat.reshape(-1)]
    (HERE / "lns_coefficients_gold.txt").write_text("\n".join(lines) + "\n")
    lines = []
    for point in (1, 2):
        alpha, metric = transform_parameters(point)
        f = streamwise_fourier(transform_physical(point), alpha)
        c = curvilinear_transform(f, metric)
        for mat in list(f) + list(c):
            lines += [f"{v.real: .17E} {v.imag: .17E}" for v in mat.reshape(-1)]
    (HERE / "lns_transform_gold.txt").write_text("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
