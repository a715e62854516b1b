// tlr_capi.cu -- the extern "C" entry points declared in tailor_gb300.h:
// context lifetime, rule validation, host<->device transfers and the stage
// preconditions of the reference's operator objects.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>

#include "tlr_internal.h"
#include "tlr_lu.h"

namespace tlr {

int fail(tlr_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

int cuda_fail(tlr_ctx *ctx, cudaError_t err, const char *what) {
  std::string m = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(err);
  return fail(ctx, TLR_ERR_CUDA, m);
}

namespace {

thread_local std::string g_error;

int upload_rule(tlr_ctx *ctx, const tlr_rule *r, int expected_nodes,
                int periodic, DevRule &d, std::vector<int> &h_off,
                std::vector<int> &h_idx, std::vector<double> &h_w1,
                std::vector<double> &h_w2) {
  // Prepare.cpp:194-248, 328-437: shape, topology and stencil consistency.
  if (!r || !r->stencil_indices || !r->stencil_offsets || !r->weights)
    return fail(ctx, TLR_ERR_ARG, "FD-q rule arrays are missing");
  if (r->node_count != expected_nodes)
    return fail(ctx, TLR_ERR_SIZE, periodic ? "eta rule node count does not match Nz"
                                            : "xi rule node count does not match Ny");
  if (r->periodic != periodic)
    return fail(ctx, TLR_ERR_ARG, periodic ? "eta rule must be periodic"
                                           : "xi rule must be bounded");
  if (r->q < 1 || r->q + 1 > r->node_count + (periodic ? 0 : 0))
    return fail(ctx, TLR_ERR_ARG, "FD-q degree out of range");
  const int n = r->node_count, s = r->q + 1;
  h_off.assign(r->stencil_offsets, r->stencil_offsets + (size_t)n * s);
  h_idx.assign(r->stencil_indices, r->stencil_indices + (size_t)n * s);
  h_w1.assign(r->weights + (size_t)n * s, r->weights + (size_t)2 * n * s);
  h_w2.assign(r->weights + (size_t)2 * n * s, r->weights + (size_t)3 * n * s);
  std::vector<int> centre(n, -1), order((size_t)n * s);
  // messages of Prepare.cpp:374-407 (validateRule)
  const char *name = periodic ? "eta" : "xi";
  char msg[160];
  for (int row = 0; row < n; ++row) {
    for (int k = 0; k < s; ++k) {
      const int off = h_off[(size_t)row * s + k], idx = h_idx[(size_t)row * s + k];
      const int un = row + off;
      const int wrapped = periodic ? ((un % n) + n) % n : un;
      if (idx < 0 || idx >= n) {
        snprintf(msg, sizeof msg, "%s FD-q row %d contains out-of-range index %d", name, row, idx);
        return fail(ctx, TLR_ERR_STENCIL, msg);
      }
      if (wrapped != idx) {
        snprintf(msg, sizeof msg, "%s %s row %d has inconsistent stencil index/offset", name,
                 periodic ? "periodic" : "bounded", row);
        return fail(ctx, TLR_ERR_STENCIL, msg);
      }
      if (off == 0) centre[row] = k;
      for (int d = 0; d < 3; ++d)
        if (!std::isfinite(r->weights[(size_t)d * n * s + (size_t)row * s + k])) {
          snprintf(msg, sizeof msg, "%s FD-q weight is not finite at row %d", name, row);
          return fail(ctx, TLR_ERR_NONFINITE, msg);
        }
    }
    if (centre[row] < 0) {
      snprintf(msg, sizeof msg, "%s FD-q stencil row %d does not contain its evaluation node",
               name, row);
      return fail(ctx, TLR_ERR_STENCIL, msg);
    }
    std::vector<int> o(s);
    std::iota(o.begin(), o.end(), 0);
    std::stable_sort(o.begin(), o.end(), [&](int a, int b) {
      return h_idx[(size_t)row * s + a] < h_idx[(size_t)row * s + b];
    });
    for (int k = 0; k < s; ++k) {
      if (k > 0 && h_idx[(size_t)row * s + o[k]] == h_idx[(size_t)row * s + o[k - 1]])
        return fail(ctx, TLR_ERR_STENCIL, "FD-q stencil repeats a node");
      order[(size_t)row * s + k] = o[k];
    }
  }
  d.n = n;
  d.q = r->q;
  d.s = s;
  const size_t ni = (size_t)n * s;
  TLR_CUDA(ctx, cudaMalloc(&d.off, ni * sizeof(int)));
  TLR_CUDA(ctx, cudaMalloc(&d.idx, ni * sizeof(int)));
  TLR_CUDA(ctx, cudaMalloc(&d.order, ni * sizeof(int)));
  TLR_CUDA(ctx, cudaMalloc(&d.centre, n * sizeof(int)));
  TLR_CUDA(ctx, cudaMalloc(&d.w1, ni * sizeof(double)));
  TLR_CUDA(ctx, cudaMalloc(&d.w2, ni * sizeof(double)));
  TLR_CUDA(ctx, cudaMemcpy(d.off, h_off.data(), ni * sizeof(int), cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d.idx, h_idx.data(), ni * sizeof(int), cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d.order, order.data(), ni * sizeof(int), cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d.centre, centre.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d.w1, h_w1.data(), ni * sizeof(double), cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d.w2, h_w2.data(), ni * sizeof(double), cudaMemcpyHostToDevice));
  return TLR_OK;
}

void free_rule(DevRule &d) {
  cudaFree(d.off); cudaFree(d.idx); cudaFree(d.order); cudaFree(d.centre);
  cudaFree(d.w1); cudaFree(d.w2);
  d = DevRule{};
}

template <typename T>
int dalloc(tlr_ctx *ctx, T **p, size_t count) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(ctx, TLR_ERR_NOMEM, std::string("device allocation failed: ") +
                                        cudaGetErrorString(e));
  }
  return TLR_OK;
}

// Transpose a [comp][N] SoA device array into [N][comp] host memory.
int copy_soa(tlr_ctx *ctx, const double *src, int comp, double *dst) {
  std::vector<double> tmp((size_t)comp * ctx->nn);
  TLR_CUDA(ctx, cudaMemcpyAsync(tmp.data(), src, tmp.size() * sizeof(double),
                                cudaMemcpyDeviceToHost, ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int n = 0; n < ctx->nn; ++n)
    for (int c = 0; c < comp; ++c) dst[(size_t)n * comp + c] = tmp[(size_t)c * ctx->nn + n];
  return TLR_OK;
}

}  // namespace

void set_global_error(const std::string &msg) { g_error = msg; }

}  // namespace tlr

using namespace tlr;

extern "C" {

const char *tlr_status_string(int status) {
  switch (status) {
    case TLR_OK: return "success";
    case TLR_ERR_ARG: return "invalid argument";
    case TLR_ERR_WRONGSTATE: return "stage called out of order";
    case TLR_ERR_SIZE: return "size mismatch";
    case TLR_ERR_STENCIL: return "stencil outside the grid";
    case TLR_ERR_NONFINITE: return "non-finite value";
    case TLR_ERR_JACOBIAN: return "non-positive Jacobian";
    case TLR_ERR_COMPLEX: return "non-real input";
    case TLR_ERR_NONPOSITIVE: return "non-positive density or temperature";
    case TLR_ERR_COEFFICIENTS: return "invalid LNS coefficients";
    case TLR_ERR_CHARACTERISTIC: return "far-field characteristic failure";
    case TLR_ERR_CUDA: return "CUDA error";
    case TLR_ERR_NOMEM: return "out of device memory";
    case TLR_ERR_NOT_CONVERGED: return "eigensolver did not converge";
    case TLR_ERR_TIMEOUT: return "device wait timed out";
    case TLR_ERR_SINGULAR: return "singular factorisation";
    case TLR_ERR_RULE: return "FD-q rule generation failed";
  }
  return "unknown status";
}

void *tlr_stream(tlr_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

long long tlr_kernel_launches(void) { return tlr::launch_total(); }

const char *tlr_last_error(const tlr_ctx *ctx) {
  return ctx ? ctx->last_error.c_str() : g_error.c_str();
}

int tlr_ctx_create(const tlr_recipe *recipe, const tlr_rule *xi, const tlr_rule *eta,
                   int ny, int nz, double spanwise_period, int device, tlr_ctx **out) {
  if (!out || !recipe) {
    g_error = "null argument";
    return TLR_ERR_ARG;
  }
  *out = nullptr;
  if (ny < 2 || nz < 3) {
    g_error = "At least two xi planes and three eta planes are required";
    return TLR_ERR_SIZE;
  }
  tlr_ctx *ctx = new tlr_ctx();
  ctx->recipe = *recipe;
  ctx->ny = ny;
  ctx->nz = nz;
  ctx->nn = ny * nz;
  ctx->span = spanwise_period;
  int rc = TLR_OK;
  auto bail = [&](int code) {
    g_error = ctx->last_error;
    tlr_ctx_destroy(ctx);
    return code;
  };
  if (device >= 0) {
    if (cudaSetDevice(device) != cudaSuccess) {
      ctx->last_error = "cannot select CUDA device";
      return bail(TLR_ERR_CUDA);
    }
  }
  cudaGetDevice(&ctx->device);
  if (xi && recipe->q_y != xi->q) {
    ctx->last_error = "xi rule degree does not match Q-Value.y";
    return bail(TLR_ERR_SIZE);
  }
  if (eta && recipe->q_z != eta->q) {
    ctx->last_error = "eta rule degree does not match Q-Value.z";
    return bail(TLR_ERR_SIZE);
  }
  if ((rc = upload_rule(ctx, xi, ny, 0, ctx->xi, ctx->h_xi_off, ctx->h_xi_idx,
                        ctx->h_xi_w1, ctx->h_xi_w2)))
    return bail(rc);
  if ((rc = upload_rule(ctx, eta, nz, 1, ctx->eta, ctx->h_eta_off, ctx->h_eta_idx,
                        ctx->h_eta_w1, ctx->h_eta_w2)))
    return bail(rc);
  ctx->sx = ctx->xi.s;
  ctx->se = ctx->eta.s;
  ctx->S = ctx->sx * ctx->se;
  ctx->nnzb = (long long)ctx->nn * ctx->S;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess) {
    ctx->last_error = "cannot create stream/events";
    return bail(TLR_ERR_CUDA);
  }
  const size_t nn = ctx->nn;
  ctx->partial_blocks = 304;
  if ((rc = dalloc(ctx, &ctx->grid_c, nn * 6)) || (rc = dalloc(ctx, &ctx->base_c, nn * 10)) ||
      (rc = dalloc(ctx, &ctx->base, nn * 5)) || (rc = dalloc(ctx, &ctx->metrics, nn * 10)) ||
      (rc = dalloc(ctx, &ctx->derivs, nn * 25)) ||
      (rc = dalloc(ctx, &ctx->coef, nn * CF_COUNT)) ||
      (rc = dalloc(ctx, &ctx->row_ptr, 3 * nn + 2)) ||
      (rc = dalloc(ctx, &ctx->col, (size_t)ctx->nnzb)) ||
      (rc = dalloc(ctx, &ctx->L, (size_t)ctx->nnzb * 25)) ||
      (rc = dalloc(ctx, &ctx->A, (size_t)ctx->nnzb * 25)) ||
      (rc = dalloc(ctx, &ctx->M, nn * 25)) || (rc = dalloc(ctx, &ctx->B, nn * 25)) ||
      (rc = dalloc(ctx, &ctx->status, ST_COUNT)) || (rc = dalloc(ctx, &ctx->red, RD_COUNT)) ||
      (rc = dalloc(ctx, &ctx->partial, (size_t)ctx->partial_blocks * 64)) ||
      (rc = dalloc(ctx, &ctx->bc_modes, (size_t)nz * 2)) ||
      (rc = dalloc(ctx, &ctx->bc_cond, (size_t)nz)))
    return bail(rc);
  // identity pattern of the block-diagonal operators after L's row_ptr
  std::vector<int> ident(2 * nn + 1);
  for (size_t k = 0; k <= nn; ++k) ident[k] = (int)k;
  for (size_t k = 0; k < nn; ++k) ident[nn + 1 + k] = (int)k;
  if (cudaMemcpy(ctx->row_ptr + nn + 1, ident.data(), ident.size() * sizeof(int),
                 cudaMemcpyHostToDevice) != cudaSuccess) {
    ctx->last_error = "cannot upload identity pattern";
    return bail(TLR_ERR_CUDA);
  }
  if ((rc = run_pattern(ctx))) return bail(rc);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    ctx->last_error = "pattern kernel failed";
    return bail(TLR_ERR_CUDA);
  }
  *out = ctx;
  return TLR_OK;
}

void tlr_ctx_destroy(tlr_ctx *ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_factor(ctx);
  free_workspace(ctx);
  free_rule(ctx->xi);
  free_rule(ctx->eta);
  cudaFree(ctx->grid_c); cudaFree(ctx->base_c); cudaFree(ctx->base);
  cudaFree(ctx->metrics); cudaFree(ctx->derivs); cudaFree(ctx->coef);
  cudaFree(ctx->row_ptr); cudaFree(ctx->col); cudaFree(ctx->L); cudaFree(ctx->A);
  cudaFree(ctx->M); cudaFree(ctx->B); cudaFree(ctx->status); cudaFree(ctx->red);
  cudaFree(ctx->partial); cudaFree(ctx->bc_modes); cudaFree(ctx->bc_cond);
  cudaFree(ctx->aff); cudaFree(ctx->wff); cudaFree(ctx->wff_m);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->own_sym_free) ctx->own_sym_free(ctx->own_sym);
  delete ctx;
}

int tlr_set_alpha(tlr_ctx *ctx, double alpha_re, double alpha_im, double omega_re,
                  double omega_im) {
  if (!ctx) return TLR_ERR_ARG;
  ctx->recipe.alpha_re = alpha_re;
  ctx->recipe.alpha_im = alpha_im;
  ctx->recipe.omega_re = omega_re;
  ctx->recipe.omega_im = omega_im;
  if (ctx->pencil) {  // a new search centre; the pencil itself is unchanged
    invalidate_factor(ctx);
    return TLR_OK;
  }
  ctx->assembled = false;
  ctx->have_bc = false;
  invalidate_factor(ctx);
  return TLR_OK;
}

int tlr_set_physics(tlr_ctx *ctx, const tlr_recipe *recipe) {
  if (!ctx || !recipe) return fail(ctx, TLR_ERR_ARG, "null recipe");
  if (recipe->q_y != ctx->recipe.q_y || recipe->q_z != ctx->recipe.q_z)
    return fail(ctx, TLR_ERR_SIZE, "FD-q degrees cannot change within a context");
  ctx->recipe = *recipe;
  invalidate_factor(ctx);
  if (ctx->pencil) return TLR_OK;
  ctx->assembled = false;
  ctx->have_bc = false;
  return TLR_OK;
}

int tlr_load_fields(tlr_ctx *ctx, const double *grid, const double *baseflow) {
  if (ctx && ctx->pencil)
    return fail(ctx, TLR_ERR_WRONGSTATE, "not available for an explicit pencil");
  if (!ctx || !grid || !baseflow) return fail(ctx, TLR_ERR_ARG, "null field array");
  TLR_CUDA(ctx, cudaMemcpyAsync(ctx->grid_c, grid, sizeof(double) * 6 * ctx->nn,
                                cudaMemcpyHostToDevice, ctx->stream));
  TLR_CUDA(ctx, cudaMemcpyAsync(ctx->base_c, baseflow, sizeof(double) * 10 * ctx->nn,
                                cudaMemcpyHostToDevice, ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->fields = true;
  ctx->have_metrics = ctx->have_derivs = ctx->assembled = ctx->have_bc = false;
  invalidate_factor(ctx);
  return TLR_OK;
}

int tlr_metrics(tlr_ctx *ctx, tlr_metric_diag *diag) {
  if (ctx && ctx->pencil)
    return fail(ctx, TLR_ERR_WRONGSTATE, "not available for an explicit pencil");
  if (!ctx) return TLR_ERR_ARG;
  if (!ctx->fields)
    return fail(ctx, TLR_ERR_WRONGSTATE, "Grid data must be prepared before computing metrics");
  ctx->have_metrics = ctx->have_derivs = ctx->assembled = ctx->have_bc = false;
  const int rc = run_metrics(ctx, diag);
  if (rc == TLR_OK) ctx->have_metrics = true;
  return rc;
}

int tlr_baseflow_derivatives(tlr_ctx *ctx, tlr_deriv_diag *diag) {
  if (ctx && ctx->pencil)
    return fail(ctx, TLR_ERR_WRONGSTATE, "not available for an explicit pencil");
  if (!ctx) return TLR_ERR_ARG;
  if (!ctx->fields)
    return fail(ctx, TLR_ERR_WRONGSTATE,
                "Base-flow data must be prepared before computing derivatives");
  if (!ctx->have_metrics)
    return fail(ctx, TLR_ERR_WRONGSTATE,
                "Metrics must be computed before base-flow derivatives");
  ctx->have_derivs = ctx->assembled = ctx->have_bc = false;
  const int rc = run_derivatives(ctx, diag);
  if (rc == TLR_OK) ctx->have_derivs = true;
  return rc;
}

int tlr_assemble(tlr_ctx *ctx, tlr_operator_diag *diag) {
  if (ctx && ctx->pencil)
    return fail(ctx, TLR_ERR_WRONGSTATE, "not available for an explicit pencil");
  if (!ctx) return TLR_ERR_ARG;
  if (!ctx->have_metrics)
    return fail(ctx, TLR_ERR_WRONGSTATE, "Metrics are required before matrix assembly");
  if (!ctx->have_derivs)
    return fail(ctx, TLR_ERR_WRONGSTATE,
                "Base-flow derivatives are required before matrix assembly");
  ctx->assembled = ctx->have_bc = false;
  invalidate_factor(ctx);
  const int rc = run_assemble(ctx, diag);
  if (rc == TLR_OK) ctx->assembled = true;
  return rc;
}

int tlr_apply_bc(tlr_ctx *ctx, tlr_bc_diag *diag) {
  if (ctx && ctx->pencil)
    return fail(ctx, TLR_ERR_WRONGSTATE, "not available for an explicit pencil");
  if (!ctx) return TLR_ERR_ARG;
  if (!ctx->assembled)
    return fail(ctx, TLR_ERR_WRONGSTATE,
                "Global operators must be assembled before boundary conditions");
  ctx->have_bc = false;
  invalidate_factor(ctx);
  const int rc = run_bc(ctx, diag);
  if (rc == TLR_OK) ctx->have_bc = true;
  return rc;
}

int tlr_spmv(tlr_ctx *ctx, int which, const double *x, double *y, int device_pointers) {
  if (!ctx || !x || !y) return fail(ctx, TLR_ERR_ARG, "null vector");
  const bool need_bc = which == TLR_MAT_A || which == TLR_MAT_B;
  if (ctx->pencil && !need_bc)
    return fail(ctx, TLR_ERR_WRONGSTATE, "not available for an explicit pencil");
  if ((need_bc && !ctx->have_bc) || (!need_bc && !ctx->assembled))
    return fail(ctx, TLR_ERR_WRONGSTATE, "operator is not available yet");
  const size_t bytes = sizeof(double2) * 5 * ctx->nn;
  if (device_pointers) {
    int rc = run_spmv(ctx, which, reinterpret_cast<const double2 *>(x),
                      reinterpret_cast<double2 *>(y));
    if (rc) return rc;
    TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return TLR_OK;
  }
  double2 *dx = nullptr, *dy = nullptr;
  TLR_CUDA(ctx, cudaMallocAsync(&dx, bytes, ctx->stream));
  TLR_CUDA(ctx, cudaMallocAsync(&dy, bytes, ctx->stream));
  TLR_CUDA(ctx, cudaMemcpyAsync(dx, x, bytes, cudaMemcpyHostToDevice, ctx->stream));
  int rc = run_spmv(ctx, which, dx, dy);
  if (rc == TLR_OK) {
    TLR_CUDA(ctx, cudaMemcpyAsync(y, dy, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  }
  cudaFreeAsync(dx, ctx->stream);
  cudaFreeAsync(dy, ctx->stream);
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return rc;
}

size_t tlr_out_bytes(tlr_ctx *ctx, int what) {
  if (!ctx) return 0;
  const size_t nn = ctx->nn, nb = (size_t)ctx->nnzb;
  switch (what) {
    case TLR_OUT_METRICS: return nn * 10 * sizeof(double);
    case TLR_OUT_DERIVATIVES: return nn * 25 * sizeof(double);
    case TLR_OUT_ROW_PTR: return (nn + 1) * sizeof(int);
    case TLR_OUT_COL_IDX: return nb * sizeof(int);
    case TLR_OUT_M_VALUES:
    case TLR_OUT_B_VALUES: return nn * 25 * sizeof(double2);
    case TLR_OUT_L_VALUES:
    case TLR_OUT_A_VALUES: return nb * 25 * sizeof(double2);
  }
  return 0;
}

int tlr_copy_out(tlr_ctx *ctx, int what, void *dst, size_t bytes) {
  if (!ctx || !dst) return fail(ctx, TLR_ERR_ARG, "null destination");
  if (bytes != tlr_out_bytes(ctx, what))
    return fail(ctx, TLR_ERR_SIZE, "destination size does not match the array");
  const void *src = nullptr;
  bool ready = true;
  if (ctx->pencil && what != TLR_OUT_ROW_PTR && what != TLR_OUT_COL_IDX &&
      what != TLR_OUT_A_VALUES && what != TLR_OUT_B_VALUES)
    return fail(ctx, TLR_ERR_WRONGSTATE, "not available for an explicit pencil");
  switch (what) {
    case TLR_OUT_METRICS:
      if (!ctx->have_metrics) ready = false;
      else return copy_soa(ctx, ctx->metrics, 10, static_cast<double *>(dst));
      break;
    case TLR_OUT_DERIVATIVES:
      if (!ctx->have_derivs) ready = false;
      else return copy_soa(ctx, ctx->derivs, 25, static_cast<double *>(dst));
      break;
    case TLR_OUT_ROW_PTR: src = ctx->row_ptr; break;
    case TLR_OUT_COL_IDX: src = ctx->col; break;
    case TLR_OUT_M_VALUES: src = ctx->M; ready = ctx->assembled; break;
    case TLR_OUT_L_VALUES: src = ctx->L; ready = ctx->assembled; break;
    case TLR_OUT_A_VALUES: src = ctx->A; ready = ctx->have_bc; break;
    case TLR_OUT_B_VALUES: src = ctx->B; ready = ctx->have_bc; break;
    default: return fail(ctx, TLR_ERR_ARG, "unknown array selector");
  }
  if (!ready) return fail(ctx, TLR_ERR_WRONGSTATE, "array has not been computed yet");
  TLR_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TLR_OK;
}

int tlr_solve(tlr_ctx *ctx, const tlr_solve_opts *opts, double *lambda,
              double *residual, double *modes, tlr_eig_diag *diag) {
  if (!ctx) return TLR_ERR_ARG;
  if (!ctx->have_bc)
    return fail(ctx, TLR_ERR_WRONGSTATE,
                "Boundary-constrained matrices are required before EPSSolve");
  return run_solve(ctx, opts, lambda, residual, modes, diag);
}

int tlr_factor_solve(tlr_ctx *ctx, int nvec, const double *rhs, double *out, int multi) {
  if (!ctx || !rhs || !out || nvec < 1 || nvec > 8)
    return ctx ? fail(ctx, TLR_ERR_ARG, "tlr_factor_solve: invalid arguments") : TLR_ERR_ARG;
  Factor *F = ctx->factor;
  if (!F || !F->factored || F->prec != 1)
    return fail(ctx, TLR_ERR_WRONGSTATE,
                "tlr_factor_solve needs a complex64 factorisation (a mixed-form tlr_solve)");
  if (multi && nvec != 2 && nvec != 4 && nvec != 8)
    return fail(ctx, TLR_ERR_ARG, "multi-vector solves take 2, 4 or 8 vectors");
  cudaGetLastError();
  const long long n = 5LL * ctx->nn;
  std::vector<float2> h((size_t)nvec * n);
  for (size_t i = 0; i < h.size(); ++i)
    h[i] = make_float2((float)rhs[2 * i], (float)rhs[2 * i + 1]);
  float2 *d = nullptr;
  TLR_CUDA(ctx, cudaMalloc(&d, h.size() * sizeof(float2)));
  int rc = cudaMemcpy(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice) ==
                   cudaSuccess ? TLR_OK : TLR_ERR_CUDA;
  if (!rc && multi) rc = F->solve_multi(ctx, d, nvec);
  for (int v = 0; v < nvec && !rc && !multi; ++v) rc = F->solve(ctx, d + (size_t)v * n);
  if (!rc && cudaMemcpy(h.data(), d, h.size() * sizeof(float2), cudaMemcpyDeviceToHost) !=
                 cudaSuccess)
    rc = TLR_ERR_CUDA;
  cudaFree(d);
  if (rc) return rc == TLR_ERR_CUDA ? fail(ctx, rc, "tlr_factor_solve: CUDA error") : rc;
  for (size_t i = 0; i < h.size(); ++i) {
    out[2 * i] = h[i].x;
    out[2 * i + 1] = h[i].y;
  }
  return TLR_OK;
}

}  // extern "C"
