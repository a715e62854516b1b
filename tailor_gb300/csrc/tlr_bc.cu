// tlr_bc.cu -- wall and characteristic far-field rows (K4).
//
// Reference: BoundaryConditions.cpp:353-548.  A_bc = -L and B_bc = M_Gamma
// are copied on the device; the wall (xi plane i = 0) keeps its continuity
// row and gets Dirichlet rows for u, v, w, T; each far-field node (i = Ny-1)
// gets rows R^-1[m,:] on its own columns for incoming modes and
// P[m,:] (-L rows), P[m,:] M rows otherwise, with P = R^-1 Gamma^-1.
//
// The reference obtains the normal eigensystem (n_y B_c + n_z C_c) r =
// s Gamma r from LAPACK zggev, whose eigenvector scaling and order are
// implementation details.  The inviscid blocks of LNSCoefficients.cpp:
// 303-356 give it in closed form -- speeds u_n (three times) and u_n +- c
// with c = sqrt(T)/M -- so each far-field node builds R analytically
// (acoustic, entropy, streamwise and tangential waves) and inverts it with
// the same pivoted Gauss-Jordan step as the reference (92-140).  The
// replaced rows span the reference's rows node by node (they differ by an
// invertible 5x5 left factor), which leaves the pencil's spectrum unchanged.
#include <cfloat>

#include "tlr_internal.h"

namespace tlr {
namespace {

constexpr double kEps = DBL_EPSILON;

__global__ void k_negate_copy(long long count, const double2 *__restrict__ L,
                              double2 *__restrict__ A) {
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < count;
       x += (long long)gridDim.x * blockDim.x) {
    const double2 v = __ldcs(L + x);
    __stcs(A + x, make_double2(-v.x, -v.y));
  }
}

// Wall: rows 1..4 of block row j*ny become e_row (A) and zero (B).
__global__ void k_wall(int ny, int nz, int S, const int *__restrict__ col,
                       double2 *__restrict__ A, double2 *__restrict__ B) {
  const long long total = (long long)nz * S * 20;
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < (long long)nz * 20) {
    const int j = (int)(x / 20), e = 5 + (int)(x % 20);
    B[(long long)(j * ny) * 25 + e] = make_double2(0.0, 0.0);
  }
  if (x >= total) return;
  const int j = (int)(x / (S * 20));
  const int rem = (int)(x % (S * 20));
  const int k = rem / 20, e = 5 + rem % 20;
  const int node = j * ny;
  const long long blk = (long long)node * S + k;
  const int r = e / 5, c = e % 5;
  const bool diag = col[blk] == node && r == c;
  A[blk * 25 + e] = make_double2(diag ? 1.0 : 0.0, 0.0);
}

struct Char {
  double Rinv[25];
  double P[25];
  int incoming[5];
  int ok;  // 0 success, else characteristic status
  int n_in, n_neutral;
  double cond;
};

__device__ bool invert5(const double *a, double *inv) {
  double m[25];
  for (int k = 0; k < 25; ++k) {
    m[k] = a[k];
    inv[k] = (k % 6 == 0) ? 1.0 : 0.0;
  }
  for (int pc = 0; pc < 5; ++pc) {
    int pr = pc;
    double mag = fabs(m[pr * 5 + pc]);
    for (int r = pc + 1; r < 5; ++r)
      if (fabs(m[r * 5 + pc]) > mag) { mag = fabs(m[r * 5 + pc]); pr = r; }
    if (!isfinite(mag) || mag <= 100.0 * kEps) return false;
    if (pr != pc)
      for (int c = 0; c < 5; ++c) {
        double t = m[pr * 5 + c]; m[pr * 5 + c] = m[pc * 5 + c]; m[pc * 5 + c] = t;
        t = inv[pr * 5 + c]; inv[pr * 5 + c] = inv[pc * 5 + c]; inv[pc * 5 + c] = t;
      }
    const double piv = m[pc * 5 + pc];
    for (int c = 0; c < 5; ++c) { m[pc * 5 + c] /= piv; inv[pc * 5 + c] /= piv; }
    for (int r = 0; r < 5; ++r) {
      if (r == pc) continue;
      const double f = m[r * 5 + pc];
      for (int c = 0; c < 5; ++c) {
        m[r * 5 + c] -= f * m[pc * 5 + c];
        inv[r * 5 + c] -= f * inv[pc * 5 + c];
      }
    }
  }
  return true;
}

__device__ double inf_norm5(const double *a) {
  double best = 0.0;
  for (int r = 0; r < 5; ++r) {
    double s = 0.0;
    for (int c = 0; c < 5; ++c) s += fabs(a[r * 5 + c]);
    best = fmax(best, s);
  }
  return best;
}

// computeCharacteristics (BoundaryConditions.cpp:152-280), closed form.
__device__ void characteristics(const double *state, const double *m10,
                                double M, double gamma, Char &ch) {
  ch.ok = 0;
  const double rho = state[0], V = state[2], W = state[3], T = state[4];
  if (!isfinite(rho) || !isfinite(V) || !isfinite(W) || !isfinite(T) ||
      !(rho > 0.0) || !(T > 0.0)) {
    ch.ok = 1;  // InvalidInput
    return;
  }
  const double mag = sqrt(m10[0] * m10[0] + m10[1] * m10[1]);
  if (!isfinite(mag) || mag <= 100.0 * kEps) {
    ch.ok = 2;  // SingularMetric
    return;
  }
  const double ny = m10[0] / mag, nz = m10[1] / mag;
  const double Pe = 1.0 / (gamma * M * M);
  const double g2 = 1.0 / ((gamma - 1.0) * M * M);
  const double c = sqrt(T) / M;
  const double un = ny * V + nz * W;
  const double speed[5] = {un - c, un, un, un, un + c};
  double R[25];  // columns: -acoustic, entropy, streamwise, tangential, +acoustic
  const double th = (gamma - 1.0) * T / rho;
  const double cols[5][5] = {{1.0, 0.0, -c * ny / rho, -c * nz / rho, th},
                             {1.0, 0.0, 0.0, 0.0, -T / rho},
                             {0.0, 1.0, 0.0, 0.0, 0.0},
                             {0.0, 0.0, -nz, ny, 0.0},
                             {1.0, 0.0, c * ny / rho, c * nz / rho, th}};
  for (int r = 0; r < 5; ++r)
    for (int mm = 0; mm < 5; ++mm) R[r * 5 + mm] = cols[mm][r];
  if (!invert5(R, ch.Rinv)) {
    ch.ok = 6;  // SingularEigenvectors
    return;
  }
  // Gamma (LNSCoefficients.cpp:141-146) is diag(1, rho, rho, rho, g44)
  // plus Gamma[4][0] = -Pe T; its inverse in closed form.
  const double g44 = rho * g2 - Pe * rho;
  if (!isfinite(g44) || fabs(g44) <= 100.0 * kEps) {
    ch.ok = 6;
    return;
  }
  double Ginv[25] = {0};
  Ginv[0] = 1.0;
  Ginv[6] = 1.0 / rho;
  Ginv[12] = 1.0 / rho;
  Ginv[18] = 1.0 / rho;
  Ginv[24] = 1.0 / g44;
  Ginv[20] = Pe * T / g44;
  for (int r = 0; r < 5; ++r)
    for (int q = 0; q < 5; ++q) {
      double s = 0.0;
      for (int k = 0; k < 5; ++k) s += ch.Rinv[r * 5 + k] * Ginv[k * 5 + q];
      ch.P[r * 5 + q] = s;
    }
  // self-check: R R^-1 = I to rounding
  double worst = 0.0;
  for (int r = 0; r < 5; ++r)
    for (int q = 0; q < 5; ++q) {
      double s = 0.0;
      for (int k = 0; k < 5; ++k) s += R[r * 5 + k] * ch.Rinv[k * 5 + q];
      worst = fmax(worst, fabs(s - (r == q ? 1.0 : 0.0)));
    }
  if (!(worst <= 1e-10)) {
    ch.ok = 6;
    return;
  }
  ch.cond = inf_norm5(R) * inf_norm5(ch.Rinv);
  if (!isfinite(ch.cond) || ch.cond > 1.0e12) {
    ch.ok = 7;  // IllConditionedEigenvectors
    return;
  }
  double smax = 1.0;
  for (int mm = 0; mm < 5; ++mm) smax = fmax(smax, fabs(speed[mm]));
  const double tol = 1000.0 * kEps * smax;
  ch.n_in = 0;
  ch.n_neutral = 0;
  for (int mm = 0; mm < 5; ++mm) {
    ch.incoming[mm] = speed[mm] < -tol;
    ch.n_in += ch.incoming[mm];
    ch.n_neutral += fabs(speed[mm]) <= tol;
  }
}

// One CTA (one warp) per far-field node j.
__global__ void k_farfield(int ny, int nz, int S, double M, double gamma,
                           const double *__restrict__ base,
                           const double *__restrict__ met,
                           const int *__restrict__ col, double2 *__restrict__ A,
                           double2 *__restrict__ B, int *modes, double *cond,
                           int *status) {
  __shared__ Char ch;
  const int j = blockIdx.x;
  const int nn = ny * nz;
  const int node = j * ny + ny - 1;
  if (threadIdx.x == 0) {
    double state[5], m10[10];
    for (int f = 0; f < 5; ++f) state[f] = base[f * (size_t)nn + node];
    for (int k = 0; k < 10; ++k) m10[k] = met[k * (size_t)nn + node];
    characteristics(state, m10, M, gamma, ch);
    if (ch.ok) atomicMax(status + ST_CHAR, ch.ok);
    modes[j * 2 + 0] = ch.ok ? 0 : ch.n_in;
    modes[j * 2 + 1] = ch.ok ? 0 : ch.n_neutral;
    cond[j] = ch.ok ? 0.0 : ch.cond;
  }
  __syncthreads();
  if (ch.ok) return;
  // A rows of the node: blocks k, columns c.
  for (int x = threadIdx.x; x < S * 5; x += blockDim.x) {
    const int k = x / 5, c = x % 5;
    const long long blk = (long long)node * S + k;
    double2 old[5];
    for (int s = 0; s < 5; ++s) old[s] = A[blk * 25 + s * 5 + c];
    const bool own = col[blk] == node;
    for (int mm = 0; mm < 5; ++mm) {
      double2 v = make_double2(0.0, 0.0);
      if (ch.incoming[mm]) {
        if (own) v.x = ch.Rinv[mm * 5 + c];
      } else {
        for (int s = 0; s < 5; ++s) {
          const double p = ch.P[mm * 5 + s];
          if (p == 0.0) continue;
          v.x += p * old[s].x;
          v.y += p * old[s].y;
        }
      }
      A[blk * 25 + mm * 5 + c] = v;
    }
  }
  if (threadIdx.x < 5) {
    const int c = threadIdx.x;
    double2 old[5];
    for (int s = 0; s < 5; ++s) old[s] = B[(long long)node * 25 + s * 5 + c];
    for (int mm = 0; mm < 5; ++mm) {
      double2 v = make_double2(0.0, 0.0);
      if (!ch.incoming[mm])
        for (int s = 0; s < 5; ++s) {
          const double p = ch.P[mm * 5 + s];
          if (p == 0.0) continue;
          v.x += p * old[s].x;
          v.y += p * old[s].y;
        }
      B[(long long)node * 25 + mm * 5 + c] = v;
    }
  }
}

}  // namespace

int run_bc(tlr_ctx *ctx, tlr_bc_diag *diag) {
  const long long nA = ctx->nnzb * 25, nB = (long long)ctx->nn * 25;
  TLR_CUDA(ctx, cudaMemsetAsync(ctx->status, 0, sizeof(int) * ST_COUNT, ctx->stream));
  { k_negate_copy<<<std::min<long long>(blocks_for(nA, 256), 152 * 16), 256, 0,
                  ctx->stream>>>(nA, ctx->L, ctx->A); count_launches(); }
  TLR_CUDA(ctx, cudaMemcpyAsync(ctx->B, ctx->M, sizeof(double2) * nB,
                                cudaMemcpyDeviceToDevice, ctx->stream));
  const long long wall = (long long)ctx->nz * ctx->S * 20;
  { k_wall<<<blocks_for(wall, 256), 256, 0, ctx->stream>>>(ctx->ny, ctx->nz, ctx->S,
                                                         ctx->col, ctx->A, ctx->B); count_launches(); }
  { k_farfield<<<ctx->nz, 64, 0, ctx->stream>>>(
      ctx->ny, ctx->nz, ctx->S, ctx->recipe.mach, ctx->recipe.gamma, ctx->base,
      ctx->metrics, ctx->col, ctx->A, ctx->B, ctx->bc_modes, ctx->bc_cond,
      ctx->status); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  int st[ST_COUNT];
  std::vector<int> modes(ctx->nz * 2);
  std::vector<double> cond(ctx->nz);
  TLR_CUDA(ctx, cudaMemcpyAsync(st, ctx->status, sizeof(st), cudaMemcpyDeviceToHost,
                                ctx->stream));
  TLR_CUDA(ctx, cudaMemcpyAsync(modes.data(), ctx->bc_modes, sizeof(int) * ctx->nz * 2,
                                cudaMemcpyDeviceToHost, ctx->stream));
  TLR_CUDA(ctx, cudaMemcpyAsync(cond.data(), ctx->bc_cond, sizeof(double) * ctx->nz,
                                cudaMemcpyDeviceToHost, ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (st[ST_CHAR]) {
    char buf[128];
    snprintf(buf, sizeof(buf),
             "Far-field characteristic decomposition failed (status %d)", st[ST_CHAR]);
    return fail(ctx, TLR_ERR_CHARACTERISTIC, buf);
  }
  tlr_bc_diag d{};
  d.wall_nodes = ctx->nz;
  d.farfield_nodes = ctx->nz;
  d.min_incoming_per_node = 5;
  for (int j = 0; j < ctx->nz; ++j) {
    d.incoming_modes += modes[j * 2];
    d.neutral_modes += modes[j * 2 + 1];
    d.min_incoming_per_node = std::min(d.min_incoming_per_node, modes[j * 2]);
    d.max_incoming_per_node = std::max(d.max_incoming_per_node, modes[j * 2]);
    d.max_eigenvector_condition = std::max(d.max_eigenvector_condition, cond[j]);
  }
  d.max_characteristic_imaginary = 0.0;
  int rc = frobenius(ctx, ctx->A, nA, &d.eigen_frobenius_norm);
  if (rc) return rc;
  rc = frobenius(ctx, ctx->B, nB, &d.eigen_mass_frobenius_norm);
  if (rc) return rc;
  if (diag) *diag = d;
  return TLR_OK;
}

}  // namespace tlr
