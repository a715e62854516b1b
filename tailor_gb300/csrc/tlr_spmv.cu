// tlr_spmv.cu -- BSR SpMV with 5x5 complex128 blocks (K5) and the
// Frobenius norm reductions of the assembled operators.
//
// PETSc's MatMult on the BAIJ operators has no call site in the reference;
// it runs inside SLEPc (shift-invert applications, EPSComputeError) and in
// test_global_operator.cpp:233.  One warp owns one block row; lane r*5+c
// holds entry (r, c) of each block, so a block is one coalesced 400-byte
// load, and each lane accumulates its own complex partial sum over the row
// before a five-lane reduction.  The blocks are streamed with evict-first
// loads; x stays L2-resident.
#include <atomic>

#include "tlr_internal.h"

namespace tlr {
namespace {

constexpr int kRowsPerCta = 8;

__global__ void __launch_bounds__(32 * kRowsPerCta)
    k_bsr_spmv(int nrows, const int *__restrict__ row_ptr,
               const int *__restrict__ col, const double2 *__restrict__ val,
               const double2 *__restrict__ x, double2 *__restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * kRowsPerCta + (threadIdx.x >> 5);
  if (row >= nrows) return;
  const int c = lane % 5;
  const bool active = lane < 25;
  double ar = 0.0, ai = 0.0;
  const int k0 = row_ptr[row], k1 = row_ptr[row + 1];
  int k = k0;
  for (; k + 4 <= k1; k += 4) {
    double2 a[4], xv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int cc = col[k + u];
      a[u] = active ? __ldcs(val + (size_t)(k + u) * 25 + lane) : make_double2(0, 0);
      xv[u] = active ? x[(size_t)cc * 5 + c] : make_double2(0, 0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      ar = fma(a[u].x, xv[u].x, ar);
      ar = fma(-a[u].y, xv[u].y, ar);
      ai = fma(a[u].x, xv[u].y, ai);
      ai = fma(a[u].y, xv[u].x, ai);
    }
  }
  for (; k < k1; ++k) {
    const int cc = col[k];
    const double2 a = active ? __ldcs(val + (size_t)k * 25 + lane) : make_double2(0, 0);
    const double2 xv = active ? x[(size_t)cc * 5 + c] : make_double2(0, 0);
    ar = fma(a.x, xv.x, ar);
    ar = fma(-a.y, xv.y, ar);
    ai = fma(a.x, xv.y, ai);
    ai = fma(a.y, xv.x, ai);
  }
  // sum the five columns of each block row r held by lanes 5r .. 5r+4
  double sr = ar, si = ai;
#pragma unroll
  for (int d = 1; d < 5; ++d) {
    sr += __shfl_down_sync(0xffffffffu, ar, d);
    si += __shfl_down_sync(0xffffffffu, ai, d);
  }
  if (active && c == 0) y[(size_t)row * 5 + lane / 5] = make_double2(sr, si);
}

__global__ void k_sq2_partial(long long n, const double2 *__restrict__ v,
                              double *__restrict__ partial) {
  __shared__ double sh[32];
  double s = 0.0;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n;
       x += (long long)gridDim.x * blockDim.x) {
    const double2 a = v[x];
    s += a.x * a.x + a.y * a.y;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    partial[blockIdx.x] = t;
  }
}

__global__ void k_sum_sqrt(int n, const double *partial, double *out) {
  if (threadIdx.x != 0) return;
  double t = 0.0;
  for (int b = 0; b < n; ++b) t += partial[b];
  *out = sqrt(t);
}

}  // namespace

int run_spmv(tlr_ctx *ctx, int which, const double2 *x, double2 *y) {
  const int nrows = ctx->nn;
  const double2 *val;
  const int *rp = ctx->row_ptr, *cl = ctx->col;
  switch (which) {
    case TLR_MAT_L: val = ctx->L; break;
    case TLR_MAT_A: val = ctx->A; break;
    case TLR_MAT_M: val = ctx->M; rp = ctx->row_ptr + 0; cl = nullptr; break;
    case TLR_MAT_B: val = ctx->B; cl = nullptr; break;
    default: return fail(ctx, TLR_ERR_ARG, "unknown matrix selector");
  }
  if (cl == nullptr) {
    // block-diagonal operators use the identity pattern stored after the
    // row pointers (row_ptr_id / col_id, set up at context creation)
    rp = ctx->row_ptr + (ctx->nn + 1);
    cl = rp + (ctx->nn + 1);
  }
  { k_bsr_spmv<<<blocks_for(nrows, kRowsPerCta), 32 * kRowsPerCta, 0, ctx->stream>>>(
      nrows, rp, cl, val, x, y); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

namespace {

// float-float helpers (Dekker/Knuth error-free transformations on FP32):
// (hi, lo) += a * x with a = ah + al, x = xh + xl
__device__ __forceinline__ void ff_mac(float &hi, float &lo, float ah, float al, float xh,
                                       float xl) {
  const float p = ah * xh;
  const float e = fmaf(ah, xh, -p) + fmaf(ah, xl, al * xh);
  const float s = hi + p;
  const float bb = s - hi;
  lo += ((hi - (s - bb)) + (p - bb)) + e;
  hi = s;
}

__device__ __forceinline__ void ff_add(float &hi, float &lo, float h2, float l2) {
  const float s = hi + h2;
  const float bb = s - hi;
  lo = lo + l2 + ((hi - (s - bb)) + (h2 - bb));
  hi = s;
}

__global__ void k_split_ff(long long n, const double2 *__restrict__ a, float4 *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 v = a[i];
  const float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
  out[i] = make_float4(rh, __double2float_rn(v.x - (double)rh), ih,
                       __double2float_rn(v.y - (double)ih));
}

// r = y - (A w - sigma B w): warp per block row, lane (r, c) = 5 r + c
// accumulates the row's blocks in float-float; B (block diagonal) in FP64.
__global__ void __launch_bounds__(32 * kRowsPerCta)
    k_residual_ff(int nrows, const int *__restrict__ row_ptr, const int *__restrict__ col,
                  const float4 *__restrict__ aff, const double2 *__restrict__ B,
                  const float4 *__restrict__ wff, const double2 *__restrict__ w,
                  const double2 *__restrict__ y, double sr, double si, double2 *__restrict__ r) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * kRowsPerCta + (threadIdx.x >> 5);
  if (row >= nrows) return;
  const int c = lane % 5;
  const bool active = lane < 25;
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  const int k0 = row_ptr[row], k1 = row_ptr[row + 1];
  // eight blocks in flight per lane: the kernel is load-latency bound
  constexpr int kU = 8;
  for (int k = k0; k < k1; k += kU) {
    float4 a[kU], xv[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const bool ok = active && k + u < k1;
      a[u] = ok ? __ldcs(aff + (size_t)(k + u) * 25 + lane) : make_float4(0.f, 0.f, 0.f, 0.f);
      xv[u] = ok ? wff[(size_t)col[k + u] * 5 + c] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      // (ar + i ai)(xr + i xi), every part a float-float pair
      ff_mac(rh, rl, a[u].x, a[u].y, xv[u].x, xv[u].y);
      ff_mac(rh, rl, -a[u].z, -a[u].w, xv[u].z, xv[u].w);
      ff_mac(ih, il, a[u].x, a[u].y, xv[u].z, xv[u].w);
      ff_mac(ih, il, a[u].z, a[u].w, xv[u].x, xv[u].y);
    }
  }
  // the five column lanes of block row rr = lane / 5
#pragma unroll
  for (int d = 1; d < 5; ++d) {
    const float h1 = __shfl_down_sync(0xffffffffu, rh, d), l1 = __shfl_down_sync(0xffffffffu, rl, d);
    const float h2 = __shfl_down_sync(0xffffffffu, ih, d), l2 = __shfl_down_sync(0xffffffffu, il, d);
    if (c == 0 && d < 5) {
      ff_add(rh, rl, h1, l1);
      ff_add(ih, il, h2, l2);
    }
  }
  // lanes 5 rr carry row rr's sums (shuffles above read lanes 5 rr + d, all in the same row)
  if (active && c == 0) {
    const int rr = lane / 5;
    const size_t i = (size_t)row * 5 + rr;
    double bx = 0.0, by = 0.0;
    const double2 *Bb = B + (size_t)row * 25 + rr * 5;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const double2 b = Bb[q], v = w[(size_t)row * 5 + q];
      bx = fma(b.x, v.x, bx);
      bx = fma(-b.y, v.y, bx);
      by = fma(b.x, v.y, by);
      by = fma(b.y, v.x, by);
    }
    const double ax = (double)rh + (double)rl, ay = (double)ih + (double)il;
    const double2 yy = y[i];
    r[i] = make_double2(yy.x - (ax - (sr * bx - si * by)), yy.y - (ay - (sr * by + si * bx)));
  }
}

// The two products above on NR vectors at once (vector v at + v * n, n the
// operator's scalar rows): each block of the operator is loaded once and
// applied to all NR vectors.  Per vector, arithmetic and order are those of
// the single-vector kernels.
template <int NR>
__global__ void __launch_bounds__(32 * kRowsPerCta)
    k_bsr_spmv_m(int nrows, const int *__restrict__ row_ptr, const int *__restrict__ col,
                 const double2 *__restrict__ val, const double2 *__restrict__ x,
                 double2 *__restrict__ y, long long n) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * kRowsPerCta + (threadIdx.x >> 5);
  if (row >= nrows) return;
  const int c = lane % 5;
  const bool active = lane < 25;
  double ar[NR], ai[NR];
#pragma unroll
  for (int v = 0; v < NR; ++v) ar[v] = ai[v] = 0.0;
  const int k0 = row_ptr[row], k1 = row_ptr[row + 1];
  int k = k0;
  for (; k + 4 <= k1; k += 4) {
    double2 a[4];
    int cc[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      cc[u] = col[k + u];
      a[u] = active ? __ldcs(val + (size_t)(k + u) * 25 + lane) : make_double2(0, 0);
    }
#pragma unroll
    for (int v = 0; v < NR; ++v) {
      double2 xv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        xv[u] = active ? x[v * n + (size_t)cc[u] * 5 + c] : make_double2(0, 0);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        ar[v] = fma(a[u].x, xv[u].x, ar[v]);
        ar[v] = fma(-a[u].y, xv[u].y, ar[v]);
        ai[v] = fma(a[u].x, xv[u].y, ai[v]);
        ai[v] = fma(a[u].y, xv[u].x, ai[v]);
      }
    }
  }
  for (; k < k1; ++k) {
    const int cc = col[k];
    const double2 a = active ? __ldcs(val + (size_t)k * 25 + lane) : make_double2(0, 0);
#pragma unroll
    for (int v = 0; v < NR; ++v) {
      const double2 xv = active ? x[v * n + (size_t)cc * 5 + c] : make_double2(0, 0);
      ar[v] = fma(a.x, xv.x, ar[v]);
      ar[v] = fma(-a.y, xv.y, ar[v]);
      ai[v] = fma(a.x, xv.y, ai[v]);
      ai[v] = fma(a.y, xv.x, ai[v]);
    }
  }
#pragma unroll
  for (int v = 0; v < NR; ++v) {
    double sr = ar[v], si = ai[v];
#pragma unroll
    for (int d = 1; d < 5; ++d) {
      sr += __shfl_down_sync(0xffffffffu, ar[v], d);
      si += __shfl_down_sync(0xffffffffu, ai[v], d);
    }
    if (active && c == 0) y[v * n + (size_t)row * 5 + lane / 5] = make_double2(sr, si);
  }
}

template <int NR>
__global__ void __launch_bounds__(32 * kRowsPerCta)
    k_residual_ff_m(int nrows, const int *__restrict__ row_ptr, const int *__restrict__ col,
                    const float4 *__restrict__ aff, const double2 *__restrict__ B,
                    const float4 *__restrict__ wff, const double2 *__restrict__ w,
                    const double2 *__restrict__ y, double sr, double si, double2 *__restrict__ r,
                    long long n) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * kRowsPerCta + (threadIdx.x >> 5);
  if (row >= nrows) return;
  const int c = lane % 5;
  const bool active = lane < 25;
  float rh[NR], rl[NR], ih[NR], il[NR];
#pragma unroll
  for (int v = 0; v < NR; ++v) rh[v] = rl[v] = ih[v] = il[v] = 0.f;
  const int k0 = row_ptr[row], k1 = row_ptr[row + 1];
  constexpr int kU = NR >= 4 ? 2 : 4;
  for (int k = k0; k < k1; k += kU) {
    float4 a[kU];
    int cc[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const bool ok = active && k + u < k1;
      cc[u] = ok ? col[k + u] : 0;
      a[u] = ok ? __ldcs(aff + (size_t)(k + u) * 25 + lane) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int v = 0; v < NR; ++v) {
      float4 xv[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u)
        xv[u] = (active && k + u < k1) ? wff[v * n + (size_t)cc[u] * 5 + c]
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        ff_mac(rh[v], rl[v], a[u].x, a[u].y, xv[u].x, xv[u].y);
        ff_mac(rh[v], rl[v], -a[u].z, -a[u].w, xv[u].z, xv[u].w);
        ff_mac(ih[v], il[v], a[u].x, a[u].y, xv[u].z, xv[u].w);
        ff_mac(ih[v], il[v], a[u].z, a[u].w, xv[u].x, xv[u].y);
      }
    }
  }
#pragma unroll
  for (int v = 0; v < NR; ++v) {
#pragma unroll
    for (int d = 1; d < 5; ++d) {
      const float h1 = __shfl_down_sync(0xffffffffu, rh[v], d);
      const float l1 = __shfl_down_sync(0xffffffffu, rl[v], d);
      const float h2 = __shfl_down_sync(0xffffffffu, ih[v], d);
      const float l2 = __shfl_down_sync(0xffffffffu, il[v], d);
      if (c == 0) {
        ff_add(rh[v], rl[v], h1, l1);
        ff_add(ih[v], il[v], h2, l2);
      }
    }
  }
  if (active && c == 0) {
    const int rr = lane / 5;
    const size_t i = (size_t)row * 5 + rr;
    const double2 *Bb = B + (size_t)row * 25 + rr * 5;
#pragma unroll
    for (int v = 0; v < NR; ++v) {
      double bx = 0.0, by = 0.0;
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        const double2 b = Bb[q], wv = w[v * n + (size_t)row * 5 + q];
        bx = fma(b.x, wv.x, bx);
        bx = fma(-b.y, wv.y, bx);
        by = fma(b.x, wv.y, by);
        by = fma(b.y, wv.x, by);
      }
      const double ax = (double)rh[v] + (double)rl[v], ay = (double)ih[v] + (double)il[v];
      const double2 yy = y[v * n + i];
      r[v * n + i] =
          make_double2(yy.x - (ax - (sr * bx - si * by)), yy.y - (ay - (sr * by + si * bx)));
    }
  }
}

}  // namespace

int prepare_ff(tlr_ctx *ctx) {
  const long long nv = ctx->nnzb * 25;
  if (!ctx->aff) TLR_CUDA(ctx, cudaMalloc(&ctx->aff, (size_t)nv * sizeof(float4)));
  const long long n = 5LL * ctx->nn;
  if (!ctx->wff) TLR_CUDA(ctx, cudaMalloc(&ctx->wff, (size_t)n * sizeof(float4)));
  if (!ctx->aff_valid) {
    { k_split_ff<<<blocks_for(nv, 256), 256, 0, ctx->stream>>>(nv, ctx->A, ctx->aff); count_launches(); }
    ctx->aff_valid = true;
  }
  return TLR_OK;
}

int residual_ff(tlr_ctx *ctx, const double2 *y, const double2 *w, double sr, double si,
                double2 *r) {
  int rc = prepare_ff(ctx);
  if (rc) return rc;
  const long long n = 5LL * ctx->nn;
  { k_split_ff<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(n, w, ctx->wff); count_launches(); }
  { k_residual_ff<<<blocks_for(ctx->nn, kRowsPerCta), 32 * kRowsPerCta, 0, ctx->stream>>>(
      ctx->nn, ctx->row_ptr, ctx->col, ctx->aff, ctx->B, ctx->wff, w, y, sr, si, r); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int vec_norm_async(tlr_ctx *ctx, const double2 *v, long long count, double *scratch,
                   double *out) {
  const int blocks = ctx->partial_blocks;
  { k_sq2_partial<<<blocks, 256, 0, ctx->stream>>>(count, v, scratch); count_launches(); }
  { k_sum_sqrt<<<1, 32, 0, ctx->stream>>>(blocks, scratch, out); count_launches(); }
  return TLR_OK;
}

int frobenius(tlr_ctx *ctx, const double2 *v, long long count, double *out) {
  const int blocks = ctx->partial_blocks;
  { k_sq2_partial<<<blocks, 256, 0, ctx->stream>>>(count, v, ctx->partial); count_launches(); }
  { k_sum_sqrt<<<1, 32, 0, ctx->stream>>>(blocks, ctx->partial, ctx->partial + blocks); count_launches(); }
  TLR_CUDA(ctx, cudaMemcpyAsync(out, ctx->partial + blocks, sizeof(double),
                                cudaMemcpyDeviceToHost, ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TLR_OK;
}

int run_spmv_multi(tlr_ctx *ctx, int which, const double2 *x, double2 *y, int nr) {
  const int nrows = ctx->nn;
  const long long n = 5LL * ctx->nn;
  const double2 *val;
  const int *rp = ctx->row_ptr, *cl = ctx->col;
  switch (which) {
    case TLR_MAT_L: val = ctx->L; break;
    case TLR_MAT_A: val = ctx->A; break;
    case TLR_MAT_M: val = ctx->M; cl = nullptr; break;
    case TLR_MAT_B: val = ctx->B; cl = nullptr; break;
    default: return fail(ctx, TLR_ERR_ARG, "unknown matrix selector");
  }
  if (cl == nullptr) {
    rp = ctx->row_ptr + (ctx->nn + 1);
    cl = rp + (ctx->nn + 1);
  }
  const dim3 g(blocks_for(nrows, kRowsPerCta)), b(32 * kRowsPerCta);
  switch (nr) {
    case 1: k_bsr_spmv<<<g, b, 0, ctx->stream>>>(nrows, rp, cl, val, x, y); break;
    case 2: k_bsr_spmv_m<2><<<g, b, 0, ctx->stream>>>(nrows, rp, cl, val, x, y, n); break;
    case 4: k_bsr_spmv_m<4><<<g, b, 0, ctx->stream>>>(nrows, rp, cl, val, x, y, n); break;
    case 8: k_bsr_spmv_m<8><<<g, b, 0, ctx->stream>>>(nrows, rp, cl, val, x, y, n); break;
    default: return fail(ctx, TLR_ERR_ARG, "multi-vector products take 1, 2, 4 or 8 vectors");
  }
  count_launches();
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int residual_ff_multi_prepare(tlr_ctx *ctx) {
  int rc = prepare_ff(ctx);
  if (rc) return rc;
  if (!ctx->wff_m)
    TLR_CUDA(ctx, cudaMalloc(&ctx->wff_m, (size_t)8 * 5 * ctx->nn * sizeof(float4)));
  return TLR_OK;
}

int residual_ff_multi(tlr_ctx *ctx, const double2 *y, const double2 *w, double sr, double si,
                      double2 *r, int nr) {
  if (nr == 1) return residual_ff(ctx, y, w, sr, si, r);
  if (!ctx->aff || !ctx->wff_m || !ctx->aff_valid)
    return fail(ctx, TLR_ERR_ARG, "float-float residual buffers not prepared");
  const long long n = 5LL * ctx->nn;
  { k_split_ff<<<blocks_for(nr * n, 256), 256, 0, ctx->stream>>>(nr * n, w, ctx->wff_m); count_launches(); }
  const dim3 g(blocks_for(ctx->nn, kRowsPerCta)), b(32 * kRowsPerCta);
  switch (nr) {
    case 2: k_residual_ff_m<2><<<g, b, 0, ctx->stream>>>(ctx->nn, ctx->row_ptr, ctx->col, ctx->aff, ctx->B, ctx->wff_m, w, y, sr, si, r, n); break;
    case 4: k_residual_ff_m<4><<<g, b, 0, ctx->stream>>>(ctx->nn, ctx->row_ptr, ctx->col, ctx->aff, ctx->B, ctx->wff_m, w, y, sr, si, r, n); break;
    case 8: k_residual_ff_m<8><<<g, b, 0, ctx->stream>>>(ctx->nn, ctx->row_ptr, ctx->col, ctx->aff, ctx->B, ctx->wff_m, w, y, sr, si, r, n); break;
    default: return fail(ctx, TLR_ERR_ARG, "multi-vector residuals take 1, 2, 4 or 8 vectors");
  }
  count_launches();
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

// ---------------------------------------------------------- launch count
namespace {
std::atomic<long long> g_launches{0};
thread_local int t_capturing = 0;
}  // namespace

void count_launches(long long n) {
  if (!t_capturing) g_launches.fetch_add(n, std::memory_order_relaxed);
}
long long launch_total() { return g_launches.load(std::memory_order_relaxed); }
CaptureScope::CaptureScope() { ++t_capturing; }
CaptureScope::~CaptureScope() { --t_capturing; }

}  // namespace tlr
