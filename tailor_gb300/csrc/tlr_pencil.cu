// tlr_pencil.cu -- an explicit generalized pencil as a solver context.
//
// The reference's EigenSolver has a second overload that solves an explicit
// matrix pair, used for small independently known regression problems
// (EigenSolver.hpp:60-67, EigenSolver.cpp:31-89; test_eigen_solver.cpp
// drives it with a 10 x 10 pencil).  tlr_pencil_create turns a dense pair
// (A, B) into a context that tlr_solve accepts: A becomes a dense 5 x 5 block
// operator (every block column present), B must be block diagonal in the
// same 5 x 5 blocks (the shift-and-invert assembly subtracts sigma B block by
// block), and the symbolic analysis is one dense front holding every
// unknown.  An order that is not a multiple of 5 is padded with rows and
// columns of the identity in A and zero in B; their eigenvalues are
// infinite, so a finite target never selects them, and the padded entries
// of the returned modes are zero.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "tlr_internal.h"
#include "tlr_symbolic.h"

namespace {

void free_symbolic(void *p) { delete static_cast<tlr::Symbolic *>(p); }

template <class T>
int alloc(tlr_ctx *ctx, T **p, size_t count) {
  const cudaError_t e = cudaMalloc(p, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    ctx->last_error = std::string("device allocation failed: ") + cudaGetErrorString(e);
    return TLR_ERR_NOMEM;
  }
  return TLR_OK;
}

}  // namespace

extern "C" int tlr_pencil_create(const tlr_recipe *recipe, int n, const double *A,
                                 const double *B, int device, tlr_ctx **out) {
  using tlr::set_global_error;
  if (!out || !recipe || !A || !B) {
    set_global_error("null argument");
    return TLR_ERR_ARG;
  }
  *out = nullptr;
  if (n < 1 || n > 5000) {
    set_global_error("the pencil order must be between 1 and 5000");
    return TLR_ERR_SIZE;
  }
  const int nb = (n + 4) / 5, N = 5 * nb;
  auto a = [&](int i, int j, int part) { return A[2 * ((size_t)j * n + i) + part]; };
  auto b = [&](int i, int j, int part) { return B[2 * ((size_t)j * n + i) + part]; };
  for (size_t k = 0; k < 2 * (size_t)n * n; ++k)
    if (!std::isfinite(A[k]) || !std::isfinite(B[k])) {
      set_global_error("the pencil contains non-finite entries");
      return TLR_ERR_NONFINITE;
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i)
      if (i / 5 != j / 5 && (b(i, j, 0) != 0.0 || b(i, j, 1) != 0.0)) {
        set_global_error("the mass matrix must be block diagonal in 5 x 5 blocks");
        return TLR_ERR_ARG;
      }

  tlr_ctx *ctx = new tlr_ctx();
  auto bail = [&](int code) {
    set_global_error(ctx->last_error);
    tlr_ctx_destroy(ctx);
    return code;
  };
  ctx->recipe = *recipe;
  ctx->ny = nb;
  ctx->nz = 1;
  ctx->nn = nb;
  ctx->S = nb;
  ctx->nnzb = (long long)nb * nb;
  if (device >= 0 && cudaSetDevice(device) != cudaSuccess) {
    ctx->last_error = "cannot select CUDA device";
    return bail(TLR_ERR_CUDA);
  }
  cudaGetDevice(&ctx->device);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess) {
    ctx->last_error = "cannot create stream/events";
    return bail(TLR_ERR_CUDA);
  }
  ctx->partial_blocks = 304;
  int rc;
  if ((rc = alloc(ctx, &ctx->row_ptr, 3 * (size_t)nb + 2)) ||
      (rc = alloc(ctx, &ctx->col, (size_t)ctx->nnzb)) ||
      (rc = alloc(ctx, &ctx->A, (size_t)ctx->nnzb * 25)) ||
      (rc = alloc(ctx, &ctx->B, (size_t)nb * 25)) ||
      (rc = alloc(ctx, &ctx->status, (size_t)tlr::ST_COUNT)) ||
      (rc = alloc(ctx, &ctx->red, (size_t)tlr::RD_COUNT)) ||
      (rc = alloc(ctx, &ctx->partial, (size_t)ctx->partial_blocks * 64)))
    return bail(rc);

  // dense block pattern, then the identity pattern of the block-diagonal B
  std::vector<int> rp(3 * (size_t)nb + 2), col((size_t)ctx->nnzb);
  for (int i = 0; i <= nb; ++i) rp[i] = i * nb;
  for (int i = 0; i <= nb; ++i) rp[nb + 1 + i] = i;
  for (int i = 0; i < nb; ++i) rp[2 * nb + 2 + i] = i;
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j < nb; ++j) col[(size_t)i * nb + j] = j;
  auto entry = [&](bool mass, int r, int c) -> double2 {
    if (r >= n || c >= n) return make_double2(!mass && r == c ? 1.0 : 0.0, 0.0);
    return mass ? make_double2(b(r, c, 0), b(r, c, 1)) : make_double2(a(r, c, 0), a(r, c, 1));
  };
  std::vector<double2> hA((size_t)ctx->nnzb * 25), hB((size_t)nb * 25);
  for (int I = 0; I < nb; ++I)
    for (int J = 0; J < nb; ++J)
      for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c)
          hA[((size_t)I * nb + J) * 25 + r * 5 + c] = entry(false, 5 * I + r, 5 * J + c);
  for (int I = 0; I < nb; ++I)
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c) hB[(size_t)I * 25 + r * 5 + c] = entry(true, 5 * I + r, 5 * I + c);
  if (cudaMemcpy(ctx->row_ptr, rp.data(), rp.size() * sizeof(int), cudaMemcpyHostToDevice) ||
      cudaMemcpy(ctx->col, col.data(), col.size() * sizeof(int), cudaMemcpyHostToDevice) ||
      cudaMemcpy(ctx->A, hA.data(), hA.size() * sizeof(double2), cudaMemcpyHostToDevice) ||
      cudaMemcpy(ctx->B, hB.data(), hB.size() * sizeof(double2), cudaMemcpyHostToDevice)) {
    ctx->last_error = "cannot upload the pencil";
    return bail(TLR_ERR_CUDA);
  }

  // one dense front over every node, assembled block by block
  auto *s = new tlr::Symbolic();
  s->ny = nb;
  s->nz = 1;
  s->nn = nb;
  tlr::FrontInfo f;
  for (int i = 0; i < nb; ++i) f.piv.push_back(i);
  f.p = f.m = N;
  s->fronts.push_back(f);
  s->rank.resize(nb);
  for (int i = 0; i < nb; ++i) s->rank[i] = i;
  s->levels.push_back({0});
  for (int I = 0; I < nb; ++I)
    for (int J = 0; J < nb; ++J)
      s->entries.push_back({I * nb + J, I, J, 0, I == J ? I : -1});
  s->level_entry_begin = {0, (long long)s->entries.size()};
  s->cmap_off = {-1};
  s->pool_elems = (long long)N * N;
  s->work_elems = N;
  s->flops = 8.0 * (double)N * N * N / 3.0;
  s->factor_elems = (long long)N * N;
  ctx->own_sym = s;
  ctx->own_sym_free = free_symbolic;
  ctx->shared_sym = s;
  ctx->pencil = true;
  ctx->assembled = ctx->have_bc = true;
  *out = ctx;
  return TLR_OK;
}
