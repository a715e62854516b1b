// tlr_dense.h -- small dense complex kernels on the host for the projected
// Krylov-Schur problem (ncv <= a few dozen): Householder reduction to upper
// Hessenberg form, the single-shift QR iteration to complex Schur form,
// reordering of the Schur form by adjacent swaps, and eigenvectors of an
// upper-triangular matrix.  Column-major storage, leading dimension ld.
//
// The algorithms are the textbook ones (Golub & Van Loan, "Matrix
// Computations", 4th ed., sections 7.4-7.6 and 7.6.2 for the swap of two
// adjacent 1x1 blocks of a complex Schur form).
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace tlr {
namespace dense {

using cd = std::complex<double>;

struct Mat {
  int n = 0, ld = 0;
  std::vector<cd> a;
  Mat() = default;
  Mat(int n_, int m_) : n(n_), ld(n_), a((size_t)n_ * m_) {}
  cd &operator()(int i, int j) { return a[(size_t)j * ld + i]; }
  cd operator()(int i, int j) const { return a[(size_t)j * ld + i]; }
};

// Givens rotation [c s; -conj(s) c] [f; g] = [r; 0], c real.
inline void givens(cd f, cd g, double &c, cd &s, cd &r) {
  const double af = std::abs(f), ag = std::abs(g);
  if (ag == 0.0) { c = 1.0; s = 0.0; r = f; return; }
  if (af == 0.0) { c = 0.0; s = std::conj(g) / ag; r = ag; return; }
  const double nrm = std::hypot(af, ag);
  const cd ph = f / af;
  c = af / nrm;
  s = ph * std::conj(g) / nrm;
  r = ph * nrm;
}

// rows k, k+1 of columns [c0, c1): x <- c x + s y ; y <- -conj(s) x + c y
inline void rot_rows(Mat &A, int k, int c0, int c1, double c, cd s) {
  for (int j = c0; j < c1; ++j) {
    const cd x = A(k, j), y = A(k + 1, j);
    A(k, j) = c * x + s * y;
    A(k + 1, j) = -std::conj(s) * x + c * y;
  }
}
// columns k, k+1 of rows [r0, r1) times G^H
inline void rot_cols(Mat &A, int k, int r0, int r1, double c, cd s) {
  for (int i = r0; i < r1; ++i) {
    const cd x = A(i, k), y = A(i, k + 1);
    A(i, k) = c * x + std::conj(s) * y;
    A(i, k + 1) = -s * x + c * y;
  }
}

// A <- Q^H A Q upper Hessenberg, Z <- Z Q.
inline void hessenberg(Mat &A, Mat &Z) {
  const int n = A.n;
  std::vector<cd> v(n);
  for (int k = 0; k + 2 < n; ++k) {
    double alpha_n = 0.0;
    for (int i = k + 1; i < n; ++i) alpha_n += std::norm(A(i, k));
    alpha_n = std::sqrt(alpha_n);
    if (alpha_n == 0.0) continue;
    const cd x0 = A(k + 1, k);
    const cd ph = std::abs(x0) > 0 ? x0 / std::abs(x0) : cd(1.0);
    for (int i = 0; i < n; ++i) v[i] = 0.0;
    for (int i = k + 1; i < n; ++i) v[i] = A(i, k);
    v[k + 1] += ph * alpha_n;
    double vn = 0.0;
    for (int i = k + 1; i < n; ++i) vn += std::norm(v[i]);
    if (vn == 0.0) continue;
    // A <- (I - 2 v v^H / vn) A (I - 2 v v^H / vn)
    for (int j = 0; j < n; ++j) {
      cd d = 0.0;
      for (int i = k + 1; i < n; ++i) d += std::conj(v[i]) * A(i, j);
      d *= 2.0 / vn;
      for (int i = k + 1; i < n; ++i) A(i, j) -= v[i] * d;
    }
    for (int i = 0; i < n; ++i) {
      cd d = 0.0;
      for (int j = k + 1; j < n; ++j) d += A(i, j) * v[j];
      d *= 2.0 / vn;
      for (int j = k + 1; j < n; ++j) A(i, j) -= d * std::conj(v[j]);
    }
    for (int i = 0; i < Z.n; ++i) {
      cd d = 0.0;
      for (int j = k + 1; j < n; ++j) d += Z(i, j) * v[j];
      d *= 2.0 / vn;
      for (int j = k + 1; j < n; ++j) Z(i, j) -= d * std::conj(v[j]);
    }
    for (int i = k + 2; i < n; ++i) A(i, k) = 0.0;
  }
}

// Hessenberg A -> upper triangular Schur form, Z <- Z Q.  Returns false
// when the iteration does not converge (30 max(10, n) sweeps for one
// deflation).  A subdiagonal entry is neglected by the conservative test
// of Ahues and Tisseur (LAPACK Working Note 122, 1997), which keeps small
// eigenvalues accurate next to large ones; projected matrices of shift-and-
// invert hold both (theta of infinite eigenvalues is 0).
inline bool schur(Mat &A, Mat &Z) {
  const int n = A.n;
  const double ulp = 2.220446049250313e-16;
  const double smlnum = 2.2250738585072014e-308 * ((double)n / ulp);
  auto c1 = [](cd z) { return std::abs(z.real()) + std::abs(z.imag()); };
  const int itmax = 30 * std::max(10, n);
  int hi = n - 1, iter = 0;
  while (hi > 0) {
    int l = hi;
    for (; l > 0; --l) {
      const double h21 = c1(A(l, l - 1));
      if (h21 <= smlnum) {
        A(l, l - 1) = 0.0;
        break;
      }
      double tst = c1(A(l - 1, l - 1)) + c1(A(l, l));
      if (tst == 0.0) {
        if (l - 2 >= 0) tst += std::abs(A(l - 1, l - 2).real());
        if (l + 1 <= hi) tst += std::abs(A(l + 1, l).real());
      }
      if (h21 <= ulp * tst) {
        const double h12 = c1(A(l - 1, l));
        const double ab = std::max(h21, h12), ba = std::min(h21, h12);
        const double d1 = c1(A(l, l)), d2 = c1(A(l - 1, l - 1) - A(l, l));
        const double aa = std::max(d1, d2), bb = std::min(d1, d2);
        const double sum = aa + ab;
        if (ba * (ab / sum) <= std::max(smlnum, ulp * (bb * (aa / sum)))) {
          A(l, l - 1) = 0.0;
          break;
        }
      }
    }
    if (l == hi) {
      --hi;
      iter = 0;
      continue;
    }
    if (++iter > itmax) return false;
    cd shift;
    if (iter % 10 == 0) {
      shift = A(hi, hi) + std::abs(A(hi, hi - 1));
    } else {
      const cd a = A(hi - 1, hi - 1), b = A(hi - 1, hi), c = A(hi, hi - 1), d = A(hi, hi);
      const cd tr = a + d, det = a * d - b * c;
      const cd disc = std::sqrt(tr * tr / 4.0 - det);
      const cd m1 = tr / 2.0 + disc, m2 = tr / 2.0 - disc;
      shift = std::abs(m1 - d) < std::abs(m2 - d) ? m1 : m2;
    }
    cd x = A(l, l) - shift, y = A(l + 1, l);
    for (int k = l; k < hi; ++k) {
      if (k > l) {
        x = A(k, k - 1);
        y = A(k + 1, k - 1);
      }
      double c;
      cd s, r;
      givens(x, y, c, s, r);
      rot_rows(A, k, k > l ? k - 1 : l, n, c, s);
      if (k > l) A(k + 1, k - 1) = 0.0;
      rot_cols(A, k, 0, std::min(k + 3, hi + 1), c, s);
      rot_cols(Z, k, 0, Z.n, c, s);
    }
  }
  for (int j = 0; j < n; ++j)
    for (int i = j + 1; i < n; ++i) A(i, j) = 0.0;
  return true;
}

// Swap diagonal entries k and k+1 of the Schur form T (and update Z).
inline void swap_adjacent(Mat &T, Mat &Z, int k) {
  const int n = T.n;
  const cd t11 = T(k, k), t22 = T(k + 1, k + 1);
  double c;
  cd s, r;
  givens(T(k, k + 1), t22 - t11, c, s, r);
  rot_rows(T, k, k + 2, n, c, s);
  rot_cols(T, k, 0, k, c, s);
  T(k, k) = t22;
  T(k + 1, k + 1) = t11;
  rot_cols(Z, k, 0, Z.n, c, s);
}

// Eigenvector of upper-triangular T for eigenvalue T(k, k).
inline std::vector<cd> tri_eigvec(const Mat &T, int k) {
  std::vector<cd> y(T.n, 0.0);
  y[k] = 1.0;
  const cd lam = T(k, k);
  double smin = 0.0;
  for (int i = 0; i <= k; ++i) smin = std::max(smin, std::abs(T(i, i)));
  smin = std::max(smin * 1e-15, 1e-300);
  for (int i = k - 1; i >= 0; --i) {
    cd acc = 0.0;
    for (int j = i + 1; j <= k; ++j) acc += T(i, j) * y[j];
    cd d = T(i, i) - lam;
    if (std::abs(d) < smin) d = smin;
    y[i] = -acc / d;
  }
  return y;
}

}  // namespace dense
}  // namespace tlr
