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

int frobenius(tlr_ctx *ctx, const double2 *v, long long count, double *out) {
  const int blocks = ctx->partial_blocks;
  { k_sq2_partial<<<blocks, 256, 0, ctx->stream>>>(count, v, ctx->partial); count_launches(); }
  { k_sum_sqrt<<<1, 32, 0, ctx->stream>>>(blocks, ctx->partial, ctx->partial + blocks); count_launches(); }
  TLR_CUDA(ctx, cudaMemcpyAsync(out, ctx->partial + blocks, sizeof(double),
                                cudaMemcpyDeviceToHost, ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
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
