// tlr_fields.cu -- curvilinear metrics and base-flow derivatives (K1, K2).
//
// Thread-per-node stencil kernels.  Every node's sums run over the same
// slots in the same order as the reference (Metrics.cpp:91-186 and
// 255-336, BaseFlowDerivatives.cpp:85-218), and this file is compiled with
// --fmad=false, so each product and sum is rounded separately: the device
// values equal a scalar CPU evaluation of the same expressions bit for bit.
// Failure flags follow the reference's collective checks; diagnostics use
// deterministic two-pass reductions (block partials, then one ordered sum).
#include <cfloat>

#include "tlr_internal.h"

namespace tlr {
namespace {

// one warp per CTA: node counts of a few thousand still spread over every SM
constexpr int kNodeThreads = 32;

constexpr double kEps = DBL_EPSILON;

__device__ inline bool finite(double v) { return isfinite(v); }

__device__ void atomic_max_d(double *addr, double v) {
  unsigned long long *p = reinterpret_cast<unsigned long long *>(addr);
  unsigned long long old = *p, assumed;
  while (__longlong_as_double(old) < v) {
    assumed = old;
    old = atomicCAS(p, assumed, __double_as_longlong(v));
    if (old == assumed) break;
  }
}

__device__ void atomic_min_d(double *addr, double v) {
  unsigned long long *p = reinterpret_cast<unsigned long long *>(addr);
  unsigned long long old = *p, assumed;
  while (__longlong_as_double(old) > v) {
    assumed = old;
    old = atomicCAS(p, assumed, __double_as_longlong(v));
    if (old == assumed) break;
  }
}

__device__ inline double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ inline double warp_min(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ inline int wrap_count(int index, int count) {
  return index >= 0 ? index / count : -((-index + count - 1) / count);
}
__device__ inline int wrap_index(int index, int count) {
  int r = index % count;
  return r < 0 ? r + count : r;
}

// First-order metrics, Jacobian checks (Metrics.cpp:91-224).
__global__ void k_metrics_first(int ny, int nz, double span, DevRule xi,
                                DevRule eta, const double *__restrict__ grid,
                                double *__restrict__ met, int *status,
                                double *red) {
  const int nn = ny * nz;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double jmin = DBL_MAX, jmax = -DBL_MAX, imax = 0.0;
  if (n < nn) {
    const int i = n % ny, j = n / ny;
    double yxi = 0.0, yeta = 0.0, zxi = 0.0, zeta = 0.0;
    bool avail = true, nonfinite = false;
    for (int s = 0; s < xi.s; ++s) {
      const int col = i + xi.off[i * xi.s + s];
      if (col < 0 || col >= ny) { avail = false; continue; }
      const double *g = grid + (size_t)(j * ny + col) * 6;
      const double yr = g[2], yi = g[3], zr = g[4], zi = g[5];
      if (!finite(yr) || !finite(yi) || !finite(zr) || !finite(zi)) nonfinite = true;
      imax = fmax(imax, fmax(fabs(yi), fabs(zi)));
      const double w = xi.w1[i * xi.s + s];
      yxi += w * yr;
      zxi += w * zr;
    }
    for (int s = 0; s < eta.s; ++s) {
      const int row = j + eta.off[j * eta.s + s];
      const int jr = wrap_index(row, nz);
      const double *g = grid + (size_t)(jr * ny + i) * 6;
      const double yr = g[2], yi = g[3], zi = g[5];
      const double zr = g[4] + (double)wrap_count(row, nz) * span;
      if (!finite(yr) || !finite(yi) || !finite(zr) || !finite(zi)) nonfinite = true;
      imax = fmax(imax, fmax(fabs(yi), fabs(zi)));
      const double w = eta.w1[j * eta.s + s];
      yeta += w * yr;
      zeta += w * zr;
    }
    if (nonfinite) atomicMax(status + ST_NONFINITE, 1);
    if (!avail) {
      atomicMax(status + ST_STENCIL, 1);
    } else if (!finite(yxi) || !finite(yeta) || !finite(zxi) || !finite(zeta)) {
      atomicMax(status + ST_NONFINITE, 1);
    } else {
      const double p1 = yxi * zeta, p2 = yeta * zxi;
      const double jac = p1 - p2;
      const double scale = fmax(1.0, fmax(fabs(p1), fabs(p2)));
      const double tol = 100.0 * kEps * scale;
      if (!finite(jac)) {
        atomicMax(status + ST_NONFINITE, 1);
      } else {
        jmin = jac;
        jmax = jac;
        if (jac <= tol) {
          atomicMax(status + ST_JACOBIAN, 1);
        } else {
          const double m0 = zeta / jac, m1 = -yeta / jac, m2 = -zxi / jac,
                       m3 = yxi / jac;
          if (!finite(m0) || !finite(m1) || !finite(m2) || !finite(m3)) {
            atomicMax(status + ST_NONFINITE, 1);
          } else {
            met[0 * (size_t)nn + n] = m0;
            met[1 * (size_t)nn + n] = m1;
            met[2 * (size_t)nn + n] = m2;
            met[3 * (size_t)nn + n] = m3;
          }
        }
      }
    }
  }
  jmin = warp_min(jmin);
  jmax = warp_max(jmax);
  imax = warp_max(imax);
  if ((threadIdx.x & 31) == 0) {
    atomic_min_d(red + RD_MINJ, jmin);
    atomic_max_d(red + RD_MAXJ, jmax);
    atomic_max_d(red + RD_MAXIM, imax);
  }
}

// Second-order metrics by the chain rule (Metrics.cpp:255-336).
__global__ void k_metrics_second(int ny, int nz, DevRule xi, DevRule eta,
                                 double *__restrict__ met, int *status) {
  const int nn = ny * nz;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const int i = n % ny, j = n / ny;
  double dxi[4] = {0.0, 0.0, 0.0, 0.0}, deta[4] = {0.0, 0.0, 0.0, 0.0};
  for (int s = 0; s < xi.s; ++s) {
    const int col = i + xi.off[i * xi.s + s];
    const double w = xi.w1[i * xi.s + s];
#pragma unroll
    for (int c = 0; c < 4; ++c) dxi[c] += w * met[c * (size_t)nn + j * ny + col];
  }
  for (int s = 0; s < eta.s; ++s) {
    const int jr = wrap_index(j + eta.off[j * eta.s + s], nz);
    const double w = eta.w1[j * eta.s + s];
#pragma unroll
    for (int c = 0; c < 4; ++c) deta[c] += w * met[c * (size_t)nn + jr * ny + i];
  }
  const double xy = met[n], xz = met[(size_t)nn + n];
  const double ey = met[2 * (size_t)nn + n], ez = met[3 * (size_t)nn + n];
  double sm[6];
  sm[0] = xy * dxi[0] + ey * deta[0];
  sm[1] = xz * dxi[1] + ez * deta[1];
  sm[2] = xz * dxi[0] + ez * deta[0];
  sm[3] = xy * dxi[2] + ey * deta[2];
  sm[4] = xz * dxi[3] + ez * deta[3];
  sm[5] = xz * dxi[2] + ez * deta[2];
  bool ok = true;
#pragma unroll
  for (int c = 0; c < 6; ++c) ok = ok && finite(sm[c]);
  if (!ok) {
    atomicMax(status + ST_SECOND, 1);
    return;
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) met[(4 + c) * (size_t)nn + n] = sm[c];
}

// Complex base flow -> real SoA, with the node checks of
// BaseFlowDerivatives.cpp:89-98 and the realness test (228-229).
__global__ void k_baseflow_prep(int nn, const double *__restrict__ base_c,
                                double *__restrict__ base, int *status,
                                double *red) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double imax = 0.0;
  if (n < nn) {
    const double *b = base_c + (size_t)n * 10;
    bool nonfinite = false;
#pragma unroll
    for (int f = 0; f < 5; ++f) {
      const double re = b[2 * f], im = b[2 * f + 1];
      if (!finite(re) || !finite(im)) nonfinite = true;
      imax = fmax(imax, fabs(im));
      base[f * (size_t)nn + n] = re;
    }
    if (nonfinite) atomicMax(status + ST_NONFINITE, 1);
    else if (b[0] <= 0.0 || b[8] <= 0.0) atomicMax(status + ST_NONPOSITIVE, 1);
  }
  imax = warp_max(imax);
  if ((threadIdx.x & 31) == 0) atomic_max_d(red + RD_BFIM, imax);
}

// 25 physical derivatives per node (BaseFlowDerivatives.cpp:100-213).
__global__ void k_derivatives(int ny, int nz, DevRule xi, DevRule eta,
                              const double *__restrict__ base,
                              const double *__restrict__ met,
                              double *__restrict__ der, int *status) {
  const int nn = ny * nz;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const int i = n % ny, j = n / ny;
  const double xy = met[n], xz = met[(size_t)nn + n];
  const double ey = met[2 * (size_t)nn + n], ez = met[3 * (size_t)nn + n];
  const double xyy = met[4 * (size_t)nn + n], xzz = met[5 * (size_t)nn + n];
  const double xyz = met[6 * (size_t)nn + n], eyy = met[7 * (size_t)nn + n];
  const double ezz = met[8 * (size_t)nn + n], eyz = met[9 * (size_t)nn + n];
  const int *xoff = xi.off + i * xi.s;
  const double *xw1 = xi.w1 + i * xi.s, *xw2 = xi.w2 + i * xi.s;
  const int *eoff = eta.off + j * eta.s;
  const double *ew1 = eta.w1 + j * eta.s, *ew2 = eta.w2 + j * eta.s;
  for (int f = 0; f < 5; ++f) {
    const double *v = base + f * (size_t)nn;
    double vx = 0.0, ve = 0.0, vxx = 0.0, vee = 0.0, vxe = 0.0;
    for (int s = 0; s < xi.s; ++s) {
      const double val = v[j * ny + i + xoff[s]];
      vx += xw1[s] * val;
      vxx += xw2[s] * val;
    }
    for (int s = 0; s < eta.s; ++s) {
      const double val = v[wrap_index(j + eoff[s], nz) * ny + i];
      ve += ew1[s] * val;
      vee += ew2[s] * val;
    }
    for (int se = 0; se < eta.s; ++se) {
      const double we = ew1[se];
      const double *rowp = v + wrap_index(j + eoff[se], nz) * ny + i;
      for (int s = 0; s < xi.s; ++s) vxe += we * xw1[s] * rowp[xoff[s]];
    }
    double out[5];
    out[0] = xy * vx + ey * ve;
    out[1] = xz * vx + ez * ve;
    out[2] = xy * xy * vxx + 2.0 * xy * ey * vxe + ey * ey * vee + xyy * vx +
             eyy * ve;
    out[3] = xz * xz * vxx + 2.0 * xz * ez * vxe + ez * ez * vee + xzz * vx +
             ezz * ve;
    out[4] = xy * xz * vxx + (xy * ez + ey * xz) * vxe + ey * ez * vee +
             xyz * vx + eyz * ve;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 5; ++d) ok = ok && finite(out[d]);
    if (!ok) {
      atomicMax(status + ST_DERIV, 1);
      continue;
    }
#pragma unroll
    for (int d = 0; d < 5; ++d) der[(d * 5 + f) * (size_t)nn + n] = out[d];
  }
}

// Sum of squares of ncomp SoA planes: block partials, then ordered sums.
__global__ void k_sq_partial(int nn, int ncomp, const double *__restrict__ v,
                             double *__restrict__ partial) {
  __shared__ double sh[32];
  for (int c = 0; c < ncomp; ++c) {
    double s = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nn;
         n += gridDim.x * blockDim.x) {
      const double x = v[c * (size_t)nn + n];
      s += x * x;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
      partial[blockIdx.x * ncomp + c] = t;
    }
    __syncthreads();
  }
}

__global__ void k_sq_final(int nblocks, int ncomp, const double *partial,
                           double *out) {
  const int c = threadIdx.x;
  if (c >= ncomp) return;
  double t = 0.0;
  for (int b = 0; b < nblocks; ++b) t += partial[b * ncomp + c];
  out[c] = sqrt(t);
}

int norms(tlr_ctx *ctx, const double *planes, int ncomp, double *host_out) {
  const int blocks = ctx->partial_blocks;
  { k_sq_partial<<<blocks, 256, 0, ctx->stream>>>(ctx->nn, ncomp, planes,
                                                ctx->partial); count_launches(); }
  { k_sq_final<<<1, 32, 0, ctx->stream>>>(blocks, ncomp, ctx->partial,
                                        ctx->partial + blocks * 32); count_launches(); }
  TLR_CUDA(ctx, cudaMemcpyAsync(host_out, ctx->partial + blocks * 32,
                                sizeof(double) * ncomp, cudaMemcpyDeviceToHost,
                                ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TLR_OK;
}

int read_status(tlr_ctx *ctx, int *st, double *red) {
  TLR_CUDA(ctx, cudaMemcpyAsync(st, ctx->status, sizeof(int) * ST_COUNT,
                                cudaMemcpyDeviceToHost, ctx->stream));
  TLR_CUDA(ctx, cudaMemcpyAsync(red, ctx->red, sizeof(double) * RD_COUNT,
                                cudaMemcpyDeviceToHost, ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TLR_OK;
}

int reset_status(tlr_ctx *ctx) {
  double init[RD_COUNT] = {DBL_MAX, -DBL_MAX, 0, 0, 0, 0, 0, 0};
  TLR_CUDA(ctx, cudaMemsetAsync(ctx->status, 0, sizeof(int) * ST_COUNT,
                                ctx->stream));
  TLR_CUDA(ctx, cudaMemcpyAsync(ctx->red, init, sizeof(init),
                                cudaMemcpyHostToDevice, ctx->stream));
  return TLR_OK;
}

}  // namespace

int run_metrics(tlr_ctx *ctx, tlr_metric_diag *diag) {
  const int nn = ctx->nn;
  int rc = reset_status(ctx);
  if (rc) return rc;
  TLR_CUDA(ctx, cudaMemsetAsync(ctx->metrics, 0, sizeof(double) * 10 * nn,
                                ctx->stream));
  { k_metrics_first<<<blocks_for(nn, kNodeThreads), kNodeThreads, 0, ctx->stream>>>(
      ctx->ny, ctx->nz, ctx->span, ctx->xi, ctx->eta, ctx->grid_c,
      ctx->metrics, ctx->status, ctx->red); count_launches(); }
  int st[ST_COUNT];
  double red[RD_COUNT];
  if ((rc = read_status(ctx, st, red))) return rc;
  tlr_metric_diag d{};
  d.min_jacobian = red[RD_MINJ];
  d.max_jacobian = red[RD_MAXJ];
  d.max_grid_imaginary = red[RD_MAXIM];
  const bool complex_grid = red[RD_MAXIM] > 100.0 * kEps;
  if (diag) *diag = d;
  char buf[256];
  if (st[ST_STENCIL])
    return fail(ctx, TLR_ERR_STENCIL,
                "An FD-q stencil extends outside the local DMDA ghost region");
  if (st[ST_NONFINITE])
    return fail(ctx, TLR_ERR_NONFINITE,
                "Grid coordinates or computed first-order metrics are not finite");
  if (st[ST_JACOBIAN]) {
    snprintf(buf, sizeof(buf),
             "Grid Jacobian must be positive and nonsingular; global range is "
             "[%.16g, %.16g]", d.min_jacobian, d.max_jacobian);
    return fail(ctx, TLR_ERR_JACOBIAN, buf);
  }
  if (complex_grid) {
    snprintf(buf, sizeof(buf),
             "Grid y/z coordinates must be real; maximum imaginary magnitude "
             "is %.16g", d.max_grid_imaginary);
    return fail(ctx, TLR_ERR_COMPLEX, buf);
  }
  { k_metrics_second<<<blocks_for(nn, kNodeThreads), kNodeThreads, 0, ctx->stream>>>(
      ctx->ny, ctx->nz, ctx->xi, ctx->eta, ctx->metrics, ctx->status); count_launches(); }
  if ((rc = read_status(ctx, st, red))) return rc;
  if (st[ST_SECOND])
    return fail(ctx, TLR_ERR_NONFINITE,
                "Computed second-order metrics are not finite");
  if ((rc = norms(ctx, ctx->metrics, 10, d.norms))) return rc;
  if (diag) *diag = d;
  return TLR_OK;
}

int run_derivatives(tlr_ctx *ctx, tlr_deriv_diag *diag) {
  const int nn = ctx->nn;
  int rc = reset_status(ctx);
  if (rc) return rc;
  TLR_CUDA(ctx, cudaMemsetAsync(ctx->derivs, 0, sizeof(double) * 25 * nn,
                                ctx->stream));
  { k_baseflow_prep<<<blocks_for(nn, kNodeThreads), kNodeThreads, 0, ctx->stream>>>(
      nn, ctx->base_c, ctx->base, ctx->status, ctx->red); count_launches(); }
  { k_derivatives<<<blocks_for(nn, kNodeThreads), kNodeThreads, 0, ctx->stream>>>(
      ctx->ny, ctx->nz, ctx->xi, ctx->eta, ctx->base, ctx->metrics,
      ctx->derivs, ctx->status); count_launches(); }
  int st[ST_COUNT];
  double red[RD_COUNT];
  if ((rc = read_status(ctx, st, red))) return rc;
  tlr_deriv_diag d{};
  d.max_baseflow_imaginary = red[RD_BFIM];
  if ((rc = norms(ctx, ctx->derivs, 25, d.norms))) return rc;
  if (diag) *diag = d;
  if (st[ST_STENCIL])
    return fail(ctx, TLR_ERR_STENCIL,
                "An FD-q stencil extends outside the base-flow DMDA ghost region");
  if (st[ST_NONFINITE])
    return fail(ctx, TLR_ERR_NONFINITE, "Base-flow values are not finite");
  if (st[ST_NONPOSITIVE])
    return fail(ctx, TLR_ERR_NONPOSITIVE,
                "Base-flow density and temperature must both be positive");
  if (st[ST_DERIV])
    return fail(ctx, TLR_ERR_NONFINITE,
                "Computed base-flow derivatives are not finite");
  if (red[RD_BFIM] > 100.0 * kEps) {
    char buf[200];
    snprintf(buf, sizeof(buf),
             "Base-flow values must be real; maximum imaginary magnitude is "
             "%.16g", red[RD_BFIM]);
    return fail(ctx, TLR_ERR_COMPLEX, buf);
  }
  return TLR_OK;
}

}  // namespace tlr
