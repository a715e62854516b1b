// tlr_kvec.cu -- Krylov basis primitives: block inner products, basis
// updates, basis combinations, scaling and axpy on complex128 vectors.
//
// These replace what SLEPc does inside EPSSolve with BLAS (EigenSolver.cpp:72:
// classical Gram-Schmidt against the basis, Ritz vectors V Y, thick-restart
// bases V Q).  Everything runs on the context stream and leaves its results in
// device memory, so an Arnoldi step needs no host round trip: the Gram-Schmidt
// coefficients, ||w|| and the next basis vector w / ||w|| are all formed on the
// device, and the host reads the projected matrix once per restart.
//
// The basis V is column-major (vector q at V + q * ldv).  Every kernel is bound
// by HBM: each reads each basis vector it touches once.  Inner products are
// reduced in a fixed order (per-CTA partials, then one warp per coefficient
// summing the partials in CTA order), so results are bitwise reproducible.
#include <algorithm>

#include "tlr_complex.cuh"
#include "tlr_internal.h"

namespace tlr {
namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 16;  // basis vectors per CTA column chunk

// conj(v) * w
__device__ __forceinline__ double2 cdotc(double2 acc, double2 v, double2 w) {
  acc.x = fma(v.x, w.x, acc.x);
  acc.x = fma(v.y, w.y, acc.x);
  acc.y = fma(v.x, w.y, acc.y);
  acc.y = fma(-v.y, w.x, acc.y);
  return acc;
}

// part[blockIdx.x * ldp + k] = sum over this CTA's rows of conj(V_k[i]) w[i],
// k = blockIdx.y * kChunk + (0 .. kChunk-1) < nk.
__global__ void __launch_bounds__(kThreads)
    k_dot_partial(long long n, const double2 *__restrict__ V, long long ldv, int nk,
                  const double2 *__restrict__ w, double2 *__restrict__ part, int ldp) {
  __shared__ double2 red[kThreads / 32][kChunk];
  const int k0 = blockIdx.y * kChunk;
  const int kc = min(kChunk, nk - k0);
  double2 acc[kChunk];
#pragma unroll
  for (int q = 0; q < kChunk; ++q) acc[q] = make_double2(0.0, 0.0);
  const double2 *Vb = V + (long long)k0 * ldv;
  for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kThreads) {
    const double2 wi = w[i];
    if (kc == kChunk) {
#pragma unroll
      for (int q = 0; q < kChunk; ++q) acc[q] = cdotc(acc[q], Vb[q * ldv + i], wi);
    } else {
#pragma unroll
      for (int q = 0; q < kChunk; ++q)
        if (q < kc) acc[q] = cdotc(acc[q], Vb[q * ldv + i], wi);
    }
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kChunk; ++q) {
    double x = acc[q].x, y = acc[q].y;
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_xor_sync(0xffffffffu, x, o);
      y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    if (lane == 0) red[wp][q] = make_double2(x, y);
  }
  __syncthreads();
  if (threadIdx.x < kc) {
    double2 s = make_double2(0.0, 0.0);
#pragma unroll
    for (int p = 0; p < kThreads / 32; ++p) {
      s.x += red[p][threadIdx.x].x;
      s.y += red[p][threadIdx.x].y;
    }
    part[(long long)blockIdx.x * ldp + k0 + threadIdx.x] = s;
  }
}

// h[k] = sum over CTAs b (in order) of part[b * ldp + k]; one warp per k.
__global__ void k_dot_reduce(int nb, int nk, const double2 *__restrict__ part, int ldp,
                             double2 *__restrict__ h) {
  const int k = blockIdx.x;
  if (k >= nk) return;
  const int lane = threadIdx.x;
  double x = 0.0, y = 0.0;
  for (int b = lane; b < nb; b += 32) {
    const double2 p = part[(long long)b * ldp + k];
    x += p.x;
    y += p.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    x += __shfl_xor_sync(0xffffffffu, x, o);
    y += __shfl_xor_sync(0xffffffffu, y, o);
  }
  if (lane == 0) h[k] = make_double2(x, y);
}

// w[i] -= sum_k V_k[i] h[k]; with npart, also the per-CTA partial sums of
// |w[i]|^2 of the updated vector (for ||w||).
__global__ void __launch_bounds__(kThreads)
    k_update(long long n, const double2 *__restrict__ V, long long ldv, int nk,
             const double2 *__restrict__ h, double2 *__restrict__ w, double *__restrict__ npart) {
  extern __shared__ double2 hs[];
  __shared__ double red[kThreads / 32];
  for (int k = threadIdx.x; k < nk; k += kThreads) hs[k] = h[k];
  __syncthreads();
  double s2 = 0.0;
  for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kThreads) {
    double2 acc = w[i];
    const double2 *Vi = V + i;
    int k = 0;
    for (; k + 4 <= nk; k += 4) {  // four independent loads in flight
      const double2 v0 = Vi[(long long)k * ldv], v1 = Vi[(long long)(k + 1) * ldv];
      const double2 v2 = Vi[(long long)(k + 2) * ldv], v3 = Vi[(long long)(k + 3) * ldv];
      acc = cfms(acc, v0, hs[k]);
      acc = cfms(acc, v1, hs[k + 1]);
      acc = cfms(acc, v2, hs[k + 2]);
      acc = cfms(acc, v3, hs[k + 3]);
    }
    for (; k < nk; ++k) acc = cfms(acc, Vi[(long long)k * ldv], hs[k]);
    w[i] = acc;
    s2 = fma(acc.x, acc.x, s2);
    s2 = fma(acc.y, acc.y, s2);
  }
  if (!npart) return;
  for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int p = 0; p < kThreads / 32; ++p) t += red[p];
    npart[blockIdx.x] = t;
  }
}

__global__ void k_norm_reduce(int nb, const double *__restrict__ part, double *__restrict__ out) {
  const int lane = threadIdx.x;
  double s = 0.0;
  for (int b = lane; b < nb; b += 32) s += part[b];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) *out = sqrt(s);
}

// out[:, j] = sum_q V[:, q] Y(q, j) for j in this CTA's chunk of kChunk
// columns; Y column-major with leading dimension ldy.
__global__ void __launch_bounds__(kThreads)
    k_combine(long long n, const double2 *__restrict__ V, long long ldv, int nq,
              const double2 *__restrict__ Y, int ldy, int nl, double2 *__restrict__ out,
              long long ldo) {
  extern __shared__ double2 ys[];  // [nq][kChunk]
  const int j0 = blockIdx.y * kChunk;
  const int jc = min(kChunk, nl - j0);
  for (int x = threadIdx.x; x < nq * kChunk; x += kThreads) {
    const int q = x / kChunk, jj = x % kChunk;
    ys[x] = jj < jc ? Y[(long long)(j0 + jj) * ldy + q] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kThreads) {
    double2 acc[kChunk];
#pragma unroll
    for (int jj = 0; jj < kChunk; ++jj) acc[jj] = make_double2(0.0, 0.0);
    for (int q = 0; q < nq; ++q) {
      const double2 v = V[(long long)q * ldv + i];
#pragma unroll
      for (int jj = 0; jj < kChunk; ++jj) acc[jj] = cfma(acc[jj], v, ys[q * kChunk + jj]);
    }
#pragma unroll
    for (int jj = 0; jj < kChunk; ++jj)
      if (jj < jc) out[(long long)(j0 + jj) * ldo + i] = acc[jj];
  }
}

// dst = src * s / *dnorm (dnorm may be null: dst = src * s).  A zero or
// non-finite norm writes zeros; the host sees that norm and reports the
// breakdown.
__global__ void k_scale(long long n, const double2 *src, const double *dnorm, double s,
                        double2 *dst) {  // src and dst may be the same vector
  double f = s;
  if (dnorm) {
    const double d = *dnorm;
    f = (d > 0.0 && d < INFINITY) ? s / d : 0.0;
  }
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 v = src[i];
    dst[i] = make_double2(v.x * f, v.y * f);
  }
}

__global__ void k_axpy(long long n, double2 a, const double2 *__restrict__ x,
                       double2 *__restrict__ y) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = cfma(y[i], a, x[i]);
}

int row_blocks(tlr_ctx *ctx, long long n) {
  return (int)std::max<long long>(1, std::min<long long>(ctx->partial_blocks,
                                                         (n + kThreads - 1) / kThreads));
}

}  // namespace

int kv_dot(tlr_ctx *ctx, long long n, const double2 *V, long long ldv, int nk,
           const double2 *w, double2 *part, double2 *h) {
  if (nk <= 0) return TLR_OK;
  const int nb = row_blocks(ctx, n);
  const dim3 grid(nb, (nk + kChunk - 1) / kChunk);
  { k_dot_partial<<<grid, kThreads, 0, ctx->stream>>>(n, V, ldv, nk, w, part, nk); count_launches(); }
  { k_dot_reduce<<<nk, 32, 0, ctx->stream>>>(nb, nk, part, nk, h); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int kv_update(tlr_ctx *ctx, long long n, const double2 *V, long long ldv, int nk,
              const double2 *h, double2 *w, double *npart, double *norm) {
  const int nb = row_blocks(ctx, n);
  { k_update<<<nb, kThreads, (size_t)std::max(nk, 1) * sizeof(double2), ctx->stream>>>(
      n, V, ldv, nk, h, w, norm ? npart : nullptr); count_launches(); }
  if (norm) { k_norm_reduce<<<1, 32, 0, ctx->stream>>>(nb, npart, norm); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int kv_combine(tlr_ctx *ctx, long long n, const double2 *V, long long ldv, int nq,
               const double2 *Y, int ldy, int nl, double2 *out, long long ldo) {
  if (nl <= 0) return TLR_OK;
  const int nb = row_blocks(ctx, n);
  const dim3 grid(nb, (nl + kChunk - 1) / kChunk);
  const size_t sm = (size_t)nq * kChunk * sizeof(double2);
  if (sm > 48 * 1024) {
    // more than 192 basis vectors: the shared-memory stage needs opting in
    TLR_CUDA(ctx, cudaFuncSetAttribute(k_combine, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sm));
  }
  { k_combine<<<grid, kThreads, sm, ctx->stream>>>(n, V, ldv, nq, Y, ldy, nl, out, ldo); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int kv_scale(tlr_ctx *ctx, long long n, const double2 *src, const double *dnorm, double s,
             double2 *dst) {
  const int nb = row_blocks(ctx, n);
  { k_scale<<<nb, kThreads, 0, ctx->stream>>>(n, src, dnorm, s, dst); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int kv_axpy(tlr_ctx *ctx, long long n, double2 a, const double2 *x, double2 *y) {
  const int nb = row_blocks(ctx, n);
  { k_axpy<<<nb, kThreads, 0, ctx->stream>>>(n, a, x, y); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

}  // namespace tlr
