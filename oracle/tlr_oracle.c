/*
 * tlr_oracle.c -- CPU restatement of the Tailor hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA product:
 * only tests/, the smoke check and the CPU-baseline leg of bench.py load it.
 * The product library never links or calls it.
 *
 * It restates, in plain C with scalar loops and no fused multiply-add
 * (built with -ffp-contract=off), the reference algorithm of
 *   - Metrics.cpp:57-225 (first-order metrics, Jacobian checks)
 *   - Metrics.cpp:227-352 (second-order metrics by the chain rule)
 *   - BaseFlowDerivatives.cpp:51-251 (25 physical base-flow derivatives)
 *   - LNSCoefficients.cpp:75-110, 173-404 (point validation, 11 physical blocks)
 *   - StreamwiseFourier.cpp:16-44 (d/dx = i alpha substitution)
 *   - CurvilinearTransform.cpp:35-101 (chain rule to xi/eta blocks)
 *   - GlobalOperator.cpp:162-378 (validation, exact pattern, insertion in
 *     the reference's ADD order: centre K0, xi line, eta line, eta-major
 *     cross product)
 * Complex arithmetic is written out in real parts.  With the imaginary
 * parts of every physical and curvilinear viscous block identically zero,
 * the reference's complex products reduce to these real products exactly
 * (up to the sign of zero).
 *
 * Layout conventions (shared with the product's C ABI):
 *   node index  n = j * ny + i   (j: periodic eta/z, i: bounded xi/y),
 *                                (the reference's natural k_j_dof order)
 *   grid        [n][3] complex interleaved (x, y, z), only y and z used
 *   baseflow    [n][5] complex interleaved (rho, U, V, W, T)
 *   metrics     [n][10] real (xi_y, xi_z, eta_y, eta_z, xi_yy, xi_zz,
 *                xi_yz, eta_yy, eta_zz, eta_yz)          Metrics.hpp:15-26
 *   derivs      [n][25] real, derivative-major [dy,dz,dyy,dzz,dyz]x[5]
 *                                               BaseFlowDerivatives.hpp:60
 *   BSR         row_ptr[n+1], col_idx[nnzb] (sorted), values
 *               [nnzb][5][5] complex interleaved, row-major blocks.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_EPS DBL_EPSILON

typedef struct {
  int n;             /* unique nodes */
  int q;             /* degree, stencil has q+1 entries */
  int periodic;      /* 0 bounded, 1 periodic */
  const int *idx;    /* [n][q+1] wrapped node index */
  const int *off;    /* [n][q+1] unwrapped displacement */
  const double *w0;  /* [n][q+1] */
  const double *w1;
  const double *w2;
} orc_rule;

typedef struct {
  double reynolds, mach, prandtl, gamma, sutherland_ratio;
  double alpha_re, alpha_im;
} orc_physics;

/* Status codes; they follow the order in which the reference checks its
 * collective failure flags. */
enum {
  ORC_OK = 0,
  ORC_STENCIL = 1,
  ORC_NONFINITE = 2,
  ORC_JACOBIAN = 3,
  ORC_COMPLEX = 4,
  ORC_SECOND_NONFINITE = 5,
  ORC_NONPOSITIVE = 6,
  ORC_DERIV_NONFINITE = 7,
  ORC_COEFFICIENTS = 8,
};

static int finite_d(double v) { return isfinite(v); }

static int wrap_count(int index, int count) {
  /* periodicWrap, Metrics.cpp:28-32 */
  if (index >= 0) return index / count;
  return -((-index + count - 1) / count);
}

static int mod_index(int index, int count) {
  int r = index % count;
  return r < 0 ? r + count : r;
}

/* ---------------------------------------------------------------- metrics */

int orc_metrics(int ny, int nz, double spanwise_period, const orc_rule *xi,
                const orc_rule *eta, const double *grid, double *metrics,
                double *diag /* [3 + 10]: minJ, maxJ, maxIm, norms */) {
  const int sx = xi->q + 1, se = eta->q + 1;
  const int nn = ny * nz;
  int fail[4] = {0, 0, 0, 0};
  double min_j = DBL_MAX, max_j = -DBL_MAX, max_im = 0.0;
  memset(metrics, 0, sizeof(double) * (size_t)nn * 10);

  /* first order: Metrics.cpp:91-186 */
  for (int j = 0; j < nz; ++j) {
    for (int i = 0; i < ny; ++i) {
      double y_xi = 0.0, y_eta = 0.0, z_xi = 0.0, z_eta = 0.0;
      int avail = 1;
      for (int s = 0; s < sx; ++s) {
        const int col = i + xi->off[i * sx + s];
        if (col < 0 || col >= ny) { avail = 0; continue; }
        const double *g = grid + ((size_t)(j * ny + col) * 3) * 2;
        const double yr = g[2], yi = g[3], zr = g[4], zi = g[5];
        if (!finite_d(yr) || !finite_d(yi) || !finite_d(zr) || !finite_d(zi))
          fail[1] = 1;
        if (fabs(yi) > max_im) max_im = fabs(yi);
        if (fabs(zi) > max_im) max_im = fabs(zi);
        const double w = xi->w1[i * sx + s];
        y_xi += w * yr;
        z_xi += w * zr;
      }
      for (int s = 0; s < se; ++s) {
        const int row = j + eta->off[j * se + s];
        const int jr = mod_index(row, nz);
        const double *g = grid + ((size_t)(jr * ny + i) * 3) * 2;
        const double yr = g[2], yi = g[3];
        const double zr = g[4] + (double)wrap_count(row, nz) * spanwise_period;
        const double zi = g[5];
        if (!finite_d(yr) || !finite_d(yi) || !finite_d(zr) || !finite_d(zi))
          fail[1] = 1;
        if (fabs(yi) > max_im) max_im = fabs(yi);
        if (fabs(zi) > max_im) max_im = fabs(zi);
        const double w = eta->w1[j * se + s];
        y_eta += w * yr;
        z_eta += w * zr;
      }
      if (!avail) { fail[0] = 1; continue; }
      if (!finite_d(y_xi) || !finite_d(y_eta) || !finite_d(z_xi) ||
          !finite_d(z_eta)) {
        fail[1] = 1;
        continue;
      }
      const double p1 = y_xi * z_eta;
      const double p2 = y_eta * z_xi;
      const double jac = p1 - p2;
      double scale = 1.0;
      if (fabs(p1) > scale) scale = fabs(p1);
      if (fabs(p2) > scale) scale = fabs(p2);
      const double tol = 100.0 * ORC_EPS * scale;
      if (!finite_d(jac)) { fail[1] = 1; continue; }
      if (jac < min_j) min_j = jac;
      if (jac > max_j) max_j = jac;
      if (jac <= tol) { fail[2] = 1; continue; }
      const double m0 = z_eta / jac, m1 = -y_eta / jac, m2 = -z_xi / jac,
                   m3 = y_xi / jac;
      if (!finite_d(m0) || !finite_d(m1) || !finite_d(m2) || !finite_d(m3)) {
        fail[1] = 1;
        continue;
      }
      double *m = metrics + (size_t)(j * ny + i) * 10;
      m[0] = m0; m[1] = m1; m[2] = m2; m[3] = m3;
    }
  }
  if (max_im > 100.0 * ORC_EPS) fail[3] = 1;
  diag[0] = min_j;
  diag[1] = max_j;
  diag[2] = max_im;
  if (fail[0]) return ORC_STENCIL;
  if (fail[1]) return ORC_NONFINITE;
  if (fail[2]) return ORC_JACOBIAN;
  if (fail[3]) return ORC_COMPLEX;

  /* second order: Metrics.cpp:255-336.  Reads the first-order values of
   * all nodes (the reference's ghosted copy), writes components 4..9. */
  double *first = (double *)malloc(sizeof(double) * (size_t)nn * 4);
  for (int n = 0; n < nn; ++n)
    for (int c = 0; c < 4; ++c) first[n * 4 + c] = metrics[(size_t)n * 10 + c];
  int fail2 = 0;
  for (int j = 0; j < nz; ++j) {
    for (int i = 0; i < ny; ++i) {
      double dxi[4] = {0, 0, 0, 0}, deta[4] = {0, 0, 0, 0};
      for (int s = 0; s < sx; ++s) {
        const int col = i + xi->off[i * sx + s];
        const double w = xi->w1[i * sx + s];
        for (int c = 0; c < 4; ++c) dxi[c] += w * first[(j * ny + col) * 4 + c];
      }
      for (int s = 0; s < se; ++s) {
        const int jr = mod_index(j + eta->off[j * se + s], nz);
        const double w = eta->w1[j * se + s];
        for (int c = 0; c < 4; ++c) deta[c] += w * first[(jr * ny + i) * 4 + c];
      }
      const double *f = first + (j * ny + i) * 4;
      const double xy = f[0], xz = f[1], ey = f[2], ez = f[3];
      double sm[6];
      sm[0] = xy * dxi[0] + ey * deta[0]; /* xi_yy */
      sm[1] = xz * dxi[1] + ez * deta[1]; /* xi_zz */
      sm[2] = xz * dxi[0] + ez * deta[0]; /* xi_yz */
      sm[3] = xy * dxi[2] + ey * deta[2]; /* eta_yy */
      sm[4] = xz * dxi[3] + ez * deta[3]; /* eta_zz */
      sm[5] = xz * dxi[2] + ez * deta[2]; /* eta_yz */
      int ok = 1;
      for (int c = 0; c < 6; ++c) ok &= finite_d(sm[c]);
      if (!ok) { fail2 = 1; continue; }
      double *m = metrics + (size_t)(j * ny + i) * 10;
      for (int c = 0; c < 6; ++c) m[4 + c] = sm[c];
    }
  }
  free(first);
  for (int c = 0; c < 10; ++c) {
    double s = 0.0;
    for (int n = 0; n < nn; ++n) s += metrics[(size_t)n * 10 + c] * metrics[(size_t)n * 10 + c];
    diag[3 + c] = sqrt(s);
  }
  return fail2 ? ORC_SECOND_NONFINITE : ORC_OK;
}

/* ---------------------------------------------------- base-flow derivatives */

int orc_baseflow_derivatives(int ny, int nz, const orc_rule *xi,
                             const orc_rule *eta, const double *baseflow,
                             const double *metrics, double *derivs,
                             double *diag /* [1 + 25] */) {
  const int sx = xi->q + 1, se = eta->q + 1;
  const int nn = ny * nz;
  int fail[5] = {0, 0, 0, 0, 0};
  double max_im = 0.0;
  memset(derivs, 0, sizeof(double) * (size_t)nn * 25);
#define BF(n, f) (baseflow + ((size_t)(n) * 5 + (f)) * 2)
  for (int j = 0; j < nz; ++j) {
    for (int i = 0; i < ny; ++i) {
      const int node = j * ny + i;
      const double *rho = BF(node, 0), *tem = BF(node, 4);
      if (!finite_d(rho[0]) || !finite_d(rho[1]) || !finite_d(tem[0]) ||
          !finite_d(tem[1]))
        fail[1] = 1;
      else if (rho[0] <= 0.0 || tem[0] <= 0.0)
        fail[2] = 1;
      for (int f = 0; f < 5; ++f) {
        double vx = 0.0, ve = 0.0, vxx = 0.0, vee = 0.0, vxe = 0.0;
        for (int s = 0; s < sx; ++s) {
          const int col = i + xi->off[i * sx + s];
          const double *v = BF(j * ny + col, f);
          if (!finite_d(v[0]) || !finite_d(v[1])) fail[1] = 1;
          if (fabs(v[1]) > max_im) max_im = fabs(v[1]);
          vx += xi->w1[i * sx + s] * v[0];
          vxx += xi->w2[i * sx + s] * v[0];
        }
        for (int s = 0; s < se; ++s) {
          const int jr = mod_index(j + eta->off[j * se + s], nz);
          const double *v = BF(jr * ny + i, f);
          if (!finite_d(v[0]) || !finite_d(v[1])) fail[1] = 1;
          if (fabs(v[1]) > max_im) max_im = fabs(v[1]);
          ve += eta->w1[j * se + s] * v[0];
          vee += eta->w2[j * se + s] * v[0];
        }
        for (int se_ = 0; se_ < se; ++se_) {
          const int jr = mod_index(j + eta->off[j * se + se_], nz);
          const double we = eta->w1[j * se + se_];
          for (int s = 0; s < sx; ++s) {
            const int col = i + xi->off[i * sx + s];
            const double *v = BF(jr * ny + col, f);
            if (!finite_d(v[0]) || !finite_d(v[1])) fail[1] = 1;
            if (fabs(v[1]) > max_im) max_im = fabs(v[1]);
            vxe += we * xi->w1[i * sx + s] * v[0];
          }
        }
        const double *m = metrics + (size_t)node * 10;
        const double xy = m[0], xz = m[1], ey = m[2], ez = m[3];
        const double xyy = m[4], xzz = m[5], xyz = m[6];
        const double eyy = m[7], ezz = m[8], eyz = m[9];
        double out[5];
        out[0] = xy * vx + ey * ve;
        out[1] = xz * vx + ez * ve;
        out[2] = xy * xy * vxx + 2.0 * xy * ey * vxe + ey * ey * vee +
                 xyy * vx + eyy * ve;
        out[3] = xz * xz * vxx + 2.0 * xz * ez * vxe + ez * ez * vee +
                 xzz * vx + ezz * ve;
        out[4] = xy * xz * vxx + (xy * ez + ey * xz) * vxe + ey * ez * vee +
                 xyz * vx + eyz * ve;
        int ok = 1;
        for (int d = 0; d < 5; ++d) ok &= finite_d(out[d]);
        if (!ok) { fail[3] = 1; continue; }
        for (int d = 0; d < 5; ++d) derivs[(size_t)node * 25 + d * 5 + f] = out[d];
      }
    }
  }
#undef BF
  if (max_im > 100.0 * ORC_EPS) fail[4] = 1;
  diag[0] = max_im;
  for (int c = 0; c < 25; ++c) {
    double s = 0.0;
    for (int n = 0; n < nn; ++n) s += derivs[(size_t)n * 25 + c] * derivs[(size_t)n * 25 + c];
    diag[1 + c] = sqrt(s);
  }
  if (fail[0]) return ORC_STENCIL;
  if (fail[1]) return ORC_NONFINITE;
  if (fail[2]) return ORC_NONPOSITIVE;
  if (fail[3]) return ORC_DERIV_NONFINITE;
  if (fail[4]) return ORC_COMPLEX;
  return ORC_OK;
}

/* ------------------------------------------------- pointwise LNS blocks */

/* Physical blocks, order Gamma, A, B, C, D, Vxx, Vxy, Vxz, Vyy, Vyz, Vzz;
 * each real 5x5 row-major.  q[10][5]: value, dx, dy, dz, dxx, dyy, dzz,
 * dxy, dxz, dyz (LNSCoefficients.hpp:21-42).  Returns 0 or the
 * CoefficientStatus of LNSCoefficients.hpp:125-131. */
int orc_lns_physical(const orc_physics *ph, const double *q, double *blk) {
  for (int k = 0; k < 50; ++k)
    if (!finite_d(q[k])) return 1;
  const double rho = q[0], U = q[1], V = q[2], W = q[3], T = q[4];
  if (rho <= 0.0) return 2;
  if (T <= 0.0) return 3;
  const double rhox = q[5], Ux = q[6], Vx = q[7], Wx = q[8], Tx = q[9];
  const double rhoy = q[10], Uy = q[11], Vy = q[12], Wy = q[13], Ty = q[14];
  const double rhoz = q[15], Uz = q[16], Vz = q[17], Wz = q[18], Tz = q[19];
  const double Uxx = q[21], Vxx = q[22], Wxx = q[23], Txx = q[24];
  const double Uyy = q[26], Vyy = q[27], Wyy = q[28], Tyy = q[29];
  const double Uzz = q[31], Vzz = q[32], Wzz = q[33], Tzz = q[34];
  const double Uxy = q[36], Wxy = q[38];
  const double Uxz = q[41], Vxz = q[42], Wxz = q[43];
  const double Vxy = q[37];
  const double Uyz = q[46], Vyz = q[47], Wyz = q[48];
  (void)Uyz; (void)Wxy; (void)Vxz; (void)Vxy;
  const double Re = ph->reynolds, Pr = ph->prandtl, M = ph->mach;
  const double ga = ph->gamma, s = ph->sutherland_ratio;
  const double t1 = 1.0 / 3.0, t2 = 2.0 / 3.0, t4 = 4.0 / 3.0;

  const double Pe = 1.0 / (ga * M * M);
  const double g2 = 1.0 / ((ga - 1.0) * M * M);
  const double mu = T * sqrt(T) * (1.0 + s) / (T + s);
  const double muT = mu * (1.5 / T - 1.0 / (T + s));
  const double muTT = muT * (1.5 / T - 1.0 / (T + s)) -
                      mu * (1.5 / (T * T) - 1.0 / ((T + s) * (T + s)));
  const double mux = muT * Tx, muy = muT * Ty, muz = muT * Tz;

  memset(blk, 0, sizeof(double) * 11 * 25);
  double *G = blk, *A = blk + 25, *B = blk + 50, *C = blk + 75, *D = blk + 100;
  double *Mxx = blk + 125, *Mxy = blk + 150, *Mxz = blk + 175;
  double *Myy = blk + 200, *Myz = blk + 225, *Mzz = blk + 250;
#define E(X, r, c) X[(r) * 5 + (c)]
  E(G, 0, 0) = 1.0;
  E(G, 1, 1) = rho;
  E(G, 2, 2) = rho;
  E(G, 3, 3) = rho;
  E(G, 4, 0) = -Pe * T;
  E(G, 4, 4) = rho * g2 - Pe * rho;

  E(A, 0, 0) = U;
  E(A, 0, 1) = rho;
  E(A, 1, 0) = Pe * T;
  E(A, 1, 1) = rho * U - t4 * mux / Re;
  E(A, 1, 2) = -muy / Re;
  E(A, 1, 3) = -muz / Re;
  E(A, 1, 4) = Pe * rho - muT / Re * (t4 * Ux - t2 * Vy - t2 * Wz);
  E(A, 2, 1) = t2 * muy / Re;
  E(A, 2, 2) = rho * U - mux / Re;
  E(A, 2, 4) = -muT * (Uy + Vx) / Re;
  E(A, 3, 1) = t2 * muz / Re;
  E(A, 3, 3) = rho * U - mux / Re;
  E(A, 3, 4) = -muT * (Wx + Uz) / Re;
  E(A, 4, 0) = -Pe * U * T;
  E(A, 4, 1) = -2.0 * mu * (t4 * Ux - t2 * Vy - t2 * Wz) / Re;
  E(A, 4, 2) = -2.0 * mu * (Uy + Vx) / Re;
  E(A, 4, 3) = -2.0 * mu * (Wx + Uz) / Re;
  E(A, 4, 4) = rho * U * g2 - rho * U * Pe - 2.0 * Tx * muT * g2 / (Re * Pr);

  E(B, 0, 0) = V;
  E(B, 0, 2) = rho;
  E(B, 1, 1) = rho * V - muy / Re;
  E(B, 1, 2) = t2 * mux / Re;
  E(B, 1, 4) = -muT * (Uy + Vx) / Re;
  E(B, 2, 0) = Pe * T;
  E(B, 2, 1) = -mux / Re;
  E(B, 2, 2) = rho * V - t4 * muy / Re;
  E(B, 2, 3) = -muz / Re;
  E(B, 2, 4) = Pe * rho - muT / Re * (-t2 * Ux + t4 * Vy - t2 * Wz);
  E(B, 3, 2) = t2 * muz / Re;
  E(B, 3, 3) = rho * V - muy / Re;
  E(B, 3, 4) = -muT * (Vz + Wy) / Re;
  E(B, 4, 0) = -Pe * V * T;
  E(B, 4, 1) = -2.0 * mu * (Uy + Vx) / Re;
  E(B, 4, 2) = -2.0 * mu * (-t2 * Ux + t4 * Vy - t2 * Wz) / Re;
  E(B, 4, 3) = -2.0 * mu * (Vz + Wy) / Re;
  E(B, 4, 4) = rho * V * g2 - rho * V * Pe - 2.0 * Ty * muT * g2 / (Re * Pr);

  E(C, 0, 0) = W;
  E(C, 0, 3) = rho;
  E(C, 1, 1) = rho * W - muz / Re;
  E(C, 1, 3) = t2 * mux / Re;
  E(C, 1, 4) = -muT * (Wx + Uz) / Re;
  E(C, 2, 2) = rho * W - muz / Re;
  E(C, 2, 3) = t2 * muy / Re;
  E(C, 2, 4) = -muT * (Vz + Wy) / Re;
  E(C, 3, 0) = Pe * T;
  E(C, 3, 1) = -mux / Re;
  E(C, 3, 2) = -muy / Re;
  E(C, 3, 3) = rho * W - t4 * muz / Re;
  E(C, 3, 4) = Pe * rho - muT / Re * (-t2 * Ux - t2 * Vy + t4 * Wz);
  E(C, 4, 0) = -Pe * W * T;
  E(C, 4, 1) = -2.0 * mu * (Wx + Uz) / Re;
  E(C, 4, 2) = -2.0 * mu * (Vz + Wy) / Re;
  E(C, 4, 3) = -2.0 * mu * (-t2 * Ux - t2 * Vy + t4 * Wz) / Re;
  E(C, 4, 4) = rho * W * g2 - rho * W * Pe - 2.0 * Tz * muT * g2 / (Re * Pr);

  E(D, 0, 0) = Ux + Vy + Wz;
  E(D, 0, 1) = rhox;
  E(D, 0, 2) = rhoy;
  E(D, 0, 3) = rhoz;
  E(D, 1, 0) = U * Ux + V * Uy + W * Uz + Pe * Tx;
  E(D, 1, 1) = rho * Ux;
  E(D, 1, 2) = rho * Uy;
  E(D, 1, 3) = rho * Uz;
  E(D, 1, 4) = Pe * rhox -
               (muTT * Tx * t2 * (2.0 * Ux - Vy - Wz) + muTT * Ty * (Uy + Vx) +
                muTT * Tz * (Wx + Uz) +
                muT * (t4 * Uxx + Uyy + Uzz + t1 * Vxy + t1 * Wxz)) / Re;
  E(D, 2, 0) = U * Vx + V * Vy + W * Vz + Pe * Ty;
  E(D, 2, 1) = rho * Vx;
  E(D, 2, 2) = rho * Vy;
  E(D, 2, 3) = rho * Vz;
  E(D, 2, 4) = Pe * rhoy -
               (muTT * Tx * (Uy + Vx) + muTT * Ty * t2 * (-Ux + 2.0 * Vy - Wz) +
                muTT * Tz * (Vz + Wy) +
                muT * (Vxx + t4 * Vyy + Vzz + t1 * Uxy + t1 * Wyz)) / Re;
  E(D, 3, 0) = U * Wx + V * Wy + W * Wz + Pe * Tz;
  E(D, 3, 1) = rho * Wx;
  E(D, 3, 2) = rho * Wy;
  E(D, 3, 3) = rho * Wz;
  E(D, 3, 4) = Pe * rhoz -
               (muTT * Tx * (Wx + Uz) + muTT * Ty * (Vz + Wy) +
                muTT * Tz * t2 * (-Ux - Vy + 2.0 * Wz) +
                muT * (Wxx + Wyy + t4 * Wzz + t1 * Uxz + t1 * Vyz)) / Re;
  E(D, 4, 0) = (g2 - Pe) * (U * Tx + V * Ty + W * Tz);
  E(D, 4, 1) = rho * Tx * g2 - Pe * (rho * Tx + T * rhox);
  E(D, 4, 2) = rho * Ty * g2 - Pe * (rho * Ty + T * rhoy);
  E(D, 4, 3) = rho * Tz * g2 - Pe * (rho * Tz + T * rhoz);
  E(D, 4, 4) = -Pe * (U * rhox + V * rhoy + W * rhoz) -
               (Txx + Tyy + Tzz) * muT * g2 / (Re * Pr) -
               (Tx * Tx + Ty * Ty + Tz * Tz) * muTT * g2 / (Re * Pr) -
               muT * (Uy * Uy + Vx * Vx + 2.0 * Uy * Vx + Uz * Uz + Wx * Wx +
                      2.0 * Uz * Wx + Vz * Vz + Wy * Wy + 2.0 * Vz * Wy) / Re -
               muT * t4 * (Ux * Ux + Vy * Vy + Wz * Wz - Ux * Wz - Ux * Vy -
                           Vy * Wz) / Re;

  E(Mxx, 1, 1) = t4 * mu / Re;
  E(Mxx, 2, 2) = mu / Re;
  E(Mxx, 3, 3) = mu / Re;
  E(Mxx, 4, 4) = mu * g2 / (Re * Pr);
  E(Myy, 1, 1) = mu / Re;
  E(Myy, 2, 2) = t4 * mu / Re;
  E(Myy, 3, 3) = mu / Re;
  E(Myy, 4, 4) = mu * g2 / (Re * Pr);
  E(Mzz, 1, 1) = mu / Re;
  E(Mzz, 2, 2) = mu / Re;
  E(Mzz, 3, 3) = t4 * mu / Re;
  E(Mzz, 4, 4) = mu * g2 / (Re * Pr);
  E(Mxy, 1, 2) = t1 * mu / Re;
  E(Mxy, 2, 1) = t1 * mu / Re;
  E(Mxz, 1, 3) = t1 * mu / Re;
  E(Mxz, 3, 1) = t1 * mu / Re;
  E(Myz, 2, 3) = t1 * mu / Re;
  E(Myz, 3, 2) = t1 * mu / Re;
#undef E
  for (int k = 0; k < 275; ++k)
    if (!finite_d(blk[k])) return 4;
  return 0;
}

/* Inviscid Gamma, Bc, Cc (LNSCoefficients.cpp:118-171). */
int orc_lns_inviscid(const orc_physics *ph, const double *state, double *blk) {
  for (int k = 0; k < 5; ++k)
    if (!finite_d(state[k])) return 1;
  const double rho = state[0], V = state[2], W = state[3], T = state[4];
  if (rho <= 0.0) return 2;
  if (T <= 0.0) return 3;
  const double M = ph->mach, ga = ph->gamma;
  const double Pe = 1.0 / (ga * M * M);
  const double g2 = 1.0 / ((ga - 1.0) * M * M);
  memset(blk, 0, sizeof(double) * 75);
  double *G = blk, *Bc = blk + 25, *Cc = blk + 50;
  G[0] = 1.0; G[6] = rho; G[12] = rho; G[18] = rho;
  G[20] = -Pe * T; G[24] = rho * g2 - Pe * rho;
  Bc[0] = V; Bc[2] = rho; Bc[6] = rho * V; Bc[10] = Pe * T; Bc[12] = rho * V;
  Bc[14] = Pe * rho; Bc[18] = rho * V; Bc[20] = -Pe * V * T;
  Bc[24] = rho * V * g2 - rho * V * Pe;
  Cc[0] = W; Cc[3] = rho; Cc[6] = rho * W; Cc[12] = rho * W; Cc[15] = Pe * T;
  Cc[18] = rho * W; Cc[19] = Pe * rho; Cc[20] = -Pe * W * T;
  Cc[24] = rho * W * g2 - rho * W * Pe;
  for (int k = 0; k < 75; ++k)
    if (!finite_d(blk[k])) return 4;
  return 0;
}

/* Fourier + curvilinear transforms (StreamwiseFourier.cpp:16-44,
 * CurvilinearTransform.cpp:62-101).  phys: 11 real blocks; m: 10 metrics.
 * out: 7 complex blocks Gamma, K0, Kxi, Keta, Vxixi, Vxieta, Vetaeta,
 * each [25][2].  Also writes the Fourier blocks (Gamma, K0, Ky, Kz, Vyy,
 * Vyz, Vzz) into four if non-null. */
int orc_transform(double ar, double ai, const double *phys, const double *m,
                  double *out, double *four) {
  if (!finite_d(ar) || !finite_d(ai)) return 1;
  for (int k = 0; k < 275; ++k)
    if (!finite_d(phys[k])) return 1;
  for (int k = 0; k < 10; ++k)
    if (!finite_d(m[k])) return 1;
  const double *G = phys, *A = phys + 25, *B = phys + 50, *C = phys + 75;
  const double *D = phys + 100, *Vxx = phys + 125, *Vxy = phys + 150;
  const double *Vxz = phys + 175, *Vyy = phys + 200, *Vyz = phys + 225;
  const double *Vzz = phys + 250;
  /* i*alpha = (-ai, ar); alpha^2 = (ar*ar - ai*ai, ar*ai + ai*ar) */
  const double ia_re = 0.0 * ar - 1.0 * ai, ia_im = 0.0 * ai + 1.0 * ar;
  const double a2_re = ar * ar - ai * ai, a2_im = ar * ai + ai * ar;
  double K0[50], Ky[50], Kz[50];
  for (int e = 0; e < 25; ++e) {
    /* K0 = D + (i alpha) A + alpha^2 Vxx */
    K0[2 * e] = (D[e] + (ia_re * A[e] - ia_im * 0.0)) + (a2_re * Vxx[e] - a2_im * 0.0);
    K0[2 * e + 1] = (0.0 + (ia_re * 0.0 + ia_im * A[e])) + (a2_re * 0.0 + a2_im * Vxx[e]);
    /* Ky = B - (i alpha) Vxy ; Kz = C - (i alpha) Vxz */
    Ky[2 * e] = B[e] - (ia_re * Vxy[e] - ia_im * 0.0);
    Ky[2 * e + 1] = 0.0 - (ia_re * 0.0 + ia_im * Vxy[e]);
    Kz[2 * e] = C[e] - (ia_re * Vxz[e] - ia_im * 0.0);
    Kz[2 * e + 1] = 0.0 - (ia_re * 0.0 + ia_im * Vxz[e]);
  }
  if (four) {
    for (int e = 0; e < 25; ++e) {
      four[2 * e] = G[e]; four[2 * e + 1] = 0.0;
      four[50 + 2 * e] = K0[2 * e]; four[50 + 2 * e + 1] = K0[2 * e + 1];
      four[100 + 2 * e] = Ky[2 * e]; four[100 + 2 * e + 1] = Ky[2 * e + 1];
      four[150 + 2 * e] = Kz[2 * e]; four[150 + 2 * e + 1] = Kz[2 * e + 1];
      four[200 + 2 * e] = Vyy[e]; four[200 + 2 * e + 1] = 0.0;
      four[250 + 2 * e] = Vyz[e]; four[250 + 2 * e + 1] = 0.0;
      four[300 + 2 * e] = Vzz[e]; four[300 + 2 * e + 1] = 0.0;
    }
  }
  const double xy = m[0], xz = m[1], ey = m[2], ez = m[3];
  const double xyy = m[4], xzz = m[5], xyz = m[6];
  const double eyy = m[7], ezz = m[8], eyz = m[9];
  for (int e = 0; e < 25; ++e) {
    double *o = out;
    o[2 * e] = G[e]; o[2 * e + 1] = 0.0;
    o[50 + 2 * e] = K0[2 * e]; o[50 + 2 * e + 1] = K0[2 * e + 1];
    for (int p = 0; p < 2; ++p) {
      const double vyy = p ? 0.0 : Vyy[e], vzz = p ? 0.0 : Vzz[e],
                   vyz = p ? 0.0 : Vyz[e];
      o[100 + 2 * e + p] = xy * Ky[2 * e + p] + xz * Kz[2 * e + p] -
                           xyy * vyy - xzz * vzz - xyz * vyz;
      o[150 + 2 * e + p] = ey * Ky[2 * e + p] + ez * Kz[2 * e + p] -
                           eyy * vyy - ezz * vzz - eyz * vyz;
      o[200 + 2 * e + p] = xy * xy * vyy + xz * xz * vzz + xy * xz * vyz;
      o[250 + 2 * e + p] = 2.0 * xy * ey * vyy + 2.0 * xz * ez * vzz +
                           (xy * ez + ey * xz) * vyz;
      o[300 + 2 * e + p] = ey * ey * vyy + ez * ez * vzz + ey * ez * vyz;
    }
  }
  for (int k = 0; k < 350; ++k)
    if (!finite_d(out[k])) return 4;
  return 0;
}

/* One node through GlobalOperator.cpp:124-145 (evaluateNode) with the
 * BiGlobal point of LNSCoefficients.cpp:75-110 (x derivatives zero). */
static int evaluate_node(const orc_physics *ph, const double *bf /*[5][2]*/,
                         const double *dv /*[25]*/, const double *m,
                         double *curv /*[7][25][2]*/) {
  double q[50];
  memset(q, 0, sizeof(q));
  for (int f = 0; f < 5; ++f) {
    if (!finite_d(bf[2 * f]) || !finite_d(bf[2 * f + 1]) || bf[2 * f + 1] != 0.0)
      return 1;
    q[f] = bf[2 * f];
    /* dy, dz, dyy, dzz, dyz into slots 2, 3, 5, 6, 9 */
    q[10 + f] = dv[0 * 5 + f];
    q[15 + f] = dv[1 * 5 + f];
    q[25 + f] = dv[2 * 5 + f];
    q[30 + f] = dv[3 * 5 + f];
    q[45 + f] = dv[4 * 5 + f];
  }
  for (int k = 0; k < 25; ++k)
    if (!finite_d(dv[k])) return 1;
  if (q[0] <= 0.0) return 2;
  if (q[4] <= 0.0) return 3;
  double phys[275];
  int st = orc_lns_physical(ph, q, phys);
  if (st) return st;
  return orc_transform(ph->alpha_re, ph->alpha_im, phys, m, curv, NULL);
}

/* ------------------------------------------------------- BSR structure */

/* Sorted eta slot order for row j: slots ordered by wrapped index. */
static void eta_order(const orc_rule *eta, int j, int *order) {
  const int se = eta->q + 1;
  for (int s = 0; s < se; ++s) order[s] = s;
  for (int a = 1; a < se; ++a) {
    int v = order[a], b = a - 1;
    while (b >= 0 && eta->idx[j * se + order[b]] > eta->idx[j * se + v]) {
      order[b + 1] = order[b];
      --b;
    }
    order[b + 1] = v;
  }
}

/* Column pattern of L (GlobalOperator.cpp:209-283); M is block diagonal. */
int orc_pattern(int ny, int nz, const orc_rule *xi, const orc_rule *eta,
                int *row_ptr, int *col_idx) {
  const int sx = xi->q + 1, se = eta->q + 1, S = sx * se;
  int order[64];
  for (int j = 0; j < nz; ++j) {
    eta_order(eta, j, order);
    for (int i = 0; i < ny; ++i) {
      const int node = j * ny + i;
      row_ptr[node] = node * S;
      int k = 0;
      for (int r = 0; r < se; ++r) {
        const int jj = eta->idx[j * se + order[r]];
        for (int s = 0; s < sx; ++s) col_idx[node * S + k++] = jj * ny + xi->idx[i * sx + s];
      }
    }
  }
  row_ptr[ny * nz] = ny * nz * S;
  return 0;
}

/* Numeric assembly (GlobalOperator.cpp:285-378).  mass: [nn][25][2];
 * spatial: [nn*S][25][2] in the pattern order of orc_pattern. */
int orc_assemble(int ny, int nz, const orc_rule *xi, const orc_rule *eta,
                 const orc_physics *ph, const double *baseflow,
                 const double *derivs, const double *metrics, double *mass,
                 double *spatial) {
  const int sx = xi->q + 1, se = eta->q + 1, S = sx * se;
  const int nn = ny * nz;
  int order[64], rank[64];
  double curv[350];
  /* validation pass (GlobalOperator.cpp:162-207) */
  for (int n = 0; n < nn; ++n) {
    if (evaluate_node(ph, baseflow + (size_t)n * 10, derivs + (size_t)n * 25,
                      metrics + (size_t)n * 10, curv))
      return ORC_COEFFICIENTS;
  }
  memset(mass, 0, sizeof(double) * (size_t)nn * 50);
  memset(spatial, 0, sizeof(double) * (size_t)nn * S * 50);
  for (int j = 0; j < nz; ++j) {
    eta_order(eta, j, order);
    for (int r = 0; r < se; ++r) rank[order[r]] = r;
    for (int i = 0; i < ny; ++i) {
      const int node = j * ny + i;
      evaluate_node(ph, baseflow + (size_t)node * 10, derivs + (size_t)node * 25,
                    metrics + (size_t)node * 10, curv);
      const double *Gm = curv, *K0 = curv + 50, *Kxi = curv + 100,
                   *Keta = curv + 150, *Vxx = curv + 200, *Vxe = curv + 250,
                   *Vee = curv + 300;
      double *row = spatial + (size_t)node * S * 50;
      /* mass block: INSERT */
      for (int e = 0; e < 50; ++e) mass[(size_t)node * 50 + e] = Gm[e];
      /* slot of the centre in each direction */
      int cx = -1, ce = -1;
      for (int s = 0; s < sx; ++s)
        if (xi->off[i * sx + s] == 0) cx = s;
      for (int s = 0; s < se; ++s)
        if (eta->off[j * se + s] == 0) ce = s;
      /* K0 at the centre */
      {
        double *b = row + (size_t)(rank[ce] * sx + cx) * 50;
        for (int e = 0; e < 50; ++e) b[e] += K0[e];
      }
      /* xi line: Kxi*w1 - Vxixi*w2 (two-term combination first) */
      for (int s = 0; s < sx; ++s) {
        const double w1 = xi->w1[i * sx + s], w2 = -xi->w2[i * sx + s];
        double *b = row + (size_t)(rank[ce] * sx + s) * 50;
        for (int e = 0; e < 25; ++e) {
          const double re = (0.0 + w1 * Kxi[2 * e]) + w2 * Vxx[2 * e];
          const double im = (0.0 + w1 * Kxi[2 * e + 1]) + w2 * Vxx[2 * e + 1];
          b[2 * e] += re;
          b[2 * e + 1] += im;
        }
      }
      /* eta line: Keta*w1 - Vetaeta*w2 */
      for (int s = 0; s < se; ++s) {
        const double w1 = eta->w1[j * se + s], w2 = -eta->w2[j * se + s];
        double *b = row + (size_t)(rank[s] * sx + cx) * 50;
        for (int e = 0; e < 25; ++e) {
          const double re = (0.0 + w1 * Keta[2 * e]) + w2 * Vee[2 * e];
          const double im = (0.0 + w1 * Keta[2 * e + 1]) + w2 * Vee[2 * e + 1];
          b[2 * e] += re;
          b[2 * e + 1] += im;
        }
      }
      /* cross: -(w1_eta * w1_xi) * Vxieta, eta-major */
      for (int s = 0; s < se; ++s) {
        const double we = eta->w1[j * se + s];
        for (int t = 0; t < sx; ++t) {
          const double scale = -we * xi->w1[i * sx + t];
          double *b = row + (size_t)(rank[s] * sx + t) * 50;
          for (int e = 0; e < 25; ++e) {
            b[2 * e] += scale * Vxe[2 * e];
            b[2 * e + 1] += scale * Vxe[2 * e + 1];
          }
        }
      }
    }
  }
  return ORC_OK;
}

/* y = A x for a BSR matrix with 5x5 complex row-major blocks. */
void orc_bsr_spmv(int nrows, const int *row_ptr, const int *col_idx,
                  const double *val, const double *x, double *y) {
  for (int r = 0; r < nrows; ++r) {
    double acc[10] = {0};
    for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
      const double *b = val + (size_t)k * 50;
      const double *xv = x + (size_t)col_idx[k] * 10;
      for (int a = 0; a < 5; ++a)
        for (int c = 0; c < 5; ++c) {
          const double br = b[(a * 5 + c) * 2], bi = b[(a * 5 + c) * 2 + 1];
          acc[2 * a] += br * xv[2 * c] - bi * xv[2 * c + 1];
          acc[2 * a + 1] += br * xv[2 * c + 1] + bi * xv[2 * c];
        }
    }
    for (int k = 0; k < 10; ++k) y[(size_t)r * 10 + k] = acc[k];
  }
}
