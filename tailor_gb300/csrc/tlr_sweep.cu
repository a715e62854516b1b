// tlr_sweep.cu -- batched alpha-sweeps: many (grid class, alpha) instances on
// one GPU.  No reference counterpart: the reference solves one recipe per
// process run (Process.cpp:34-179).
//
// Each grid class gets one symbolic analysis (computed once, copied into
// every context of the class).  Worker threads each own one context per
// class (its own CUDA stream, factor buffers, captured solve graph and
// Krylov workspace) and take points from a shared queue (or, with warm
// starts, a contiguous run of neighbouring points each), so the kernels of
// several instances overlap on the GPU while each instance's Krylov-Schur
// driver runs on its own host thread.  With autotuning on, the first
// context of a class times, on the class's first point, the factorisation
// with both Schur-update kernels (tensor cores / CUDA cores), the winning
// kernel with 128-column panels, and the triangular solves with both
// diagonal-block sizes, and keeps the fastest combination.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "tlr_internal.h"
#include "tlr_lu.h"

namespace tlr {
namespace {

constexpr int kMaxClasses = 16;

struct ClassState {
  const tlr_grid_class *gc = nullptr;
  std::unique_ptr<Symbolic> sym;
  int cuda_core_schur = 0, solve_block = 0, panel_width = 0;
  double factor_ms[2] = {0, 0}, trisolve_ms[2] = {0, 0}, wide_factor_ms = 0;
};

int make_context(const tlr_grid_class &gc, int device, tlr_ctx **out) {
  tlr_ctx *ctx = nullptr;
  int rc = tlr_ctx_create(gc.recipe, gc.xi, gc.eta, gc.ny, gc.nz, gc.spanwise_period, device,
                          &ctx);
  if (rc) return rc;
  tlr_metric_diag md;
  tlr_deriv_diag dd;
  if ((rc = tlr_load_fields(ctx, gc.grid, gc.baseflow)) || (rc = tlr_metrics(ctx, &md)) ||
      (rc = tlr_baseflow_derivatives(ctx, &dd))) {
    set_global_error(ctx->last_error);
    tlr_ctx_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return TLR_OK;
}

int stage_point(tlr_ctx *ctx, const tlr_grid_class &gc, const tlr_sweep_point &pt) {
  int rc = TLR_OK;
  const double re = pt.reynolds > 0 ? pt.reynolds : gc.recipe->reynolds;
  if (re != ctx->recipe.reynolds) {
    tlr_recipe r = ctx->recipe;
    r.reynolds = re;
    rc = tlr_set_physics(ctx, &r);
  }
  if (!rc)
    rc = tlr_set_alpha(ctx, pt.alpha_re, pt.alpha_im, ctx->recipe.omega_re, ctx->recipe.omega_im);
  tlr_operator_diag od;
  tlr_bc_diag bd;
  if (!rc) rc = tlr_assemble(ctx, &od);
  if (!rc) rc = tlr_apply_bc(ctx, &bd);
  return rc;
}

double elapsed_ms(tlr_ctx *ctx) {
  float ms = 0.f;
  cudaEventSynchronize(ctx->ev1);
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  return ms;
}

// Time factorisations and triangular solves of the mixed form on the staged
// point: Schur kernel on the 256 block, then the 128 block with the faster
// kernel, then the faster kernel with 128-column panels (the depth K of the
// Schur-update tiles) instead of 64.  Leaves ctx without a factor.
int autotune(tlr_ctx *ctx, ClassState &cs, int ring_slack) {
  double anorm = 0.0;
  int rc = frobenius(ctx, ctx->A, ctx->nnzb * 25, &anorm);
  if (rc) return rc;
  const long long n = 5LL * ctx->nn;
  const double tiny = 1e-10 * anorm / std::sqrt((double)n);
  const double sr = ctx->recipe.omega_im, si = -ctx->recipe.omega_re;
  std::vector<float2> hx(n);
  for (long long i = 0; i < n; ++i)
    hx[i] = make_float2((float)std::sin(0.37 * (double)i), (float)std::cos(0.61 * (double)i));
  float2 *dx = nullptr;
  TLR_CUDA(ctx, cudaMalloc(&dx, n * sizeof(float2)));
  free_factor(ctx);
  const int blocks[2] = {256, 128};
  double fbest = 1e300;
  for (int bi = 0; bi < 2 && !rc; ++bi) {
    Factor *F = new Factor();
    ctx->factor = F;
    if ((rc = F->setup(ctx, 1, 48, blocks[bi], 0, ring_slack))) break;
    if (!cs.sym) {  // one symbolic analysis for every factor of the class
      cs.sym.reset(new Symbolic(F->sym));
      ctx->shared_sym = cs.sym.get();
    }
    const int ntc = bi == 0 ? 2 : 1;
    for (int k = 0; k < ntc && !rc; ++k) {
      F->tensor_cores = bi == 0 ? k == 0 : !cs.cuda_core_schur;
      cudaEventRecord(ctx->ev0, ctx->stream);
      if ((rc = F->factor(ctx, sr, si, tiny))) break;
      cudaEventRecord(ctx->ev1, ctx->stream);
      const double ms = elapsed_ms(ctx);
      if (bi == 0) {
        cs.factor_ms[k] = ms;
        if (ms < fbest) {
          fbest = ms;
          cs.cuda_core_schur = k;
        }
      }
    }
    if (rc) break;
    if (bi == 0) {  // the winning kernel with 128-column panels
      Factor *W = new Factor();
      if ((rc = W->setup(ctx, 1, 48, blocks[bi], 128, ring_slack))) {
        W->release();
        delete W;
        break;
      }
      W->tensor_cores = !cs.cuda_core_schur;
      Factor *keep = ctx->factor;
      ctx->factor = W;
      cudaEventRecord(ctx->ev0, ctx->stream);
      rc = W->factor(ctx, sr, si, tiny);
      cudaEventRecord(ctx->ev1, ctx->stream);
      cs.wide_factor_ms = rc ? 1e300 : elapsed_ms(ctx);
      cs.panel_width = cs.wide_factor_ms < fbest ? 128 : 64;
      W->release();
      delete W;
      ctx->factor = keep;
      if (rc) break;
    }
    cudaMemcpyAsync(dx, hx.data(), n * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream);
    if ((rc = F->solve(ctx, dx))) break;  // first replay instantiates the graph
    F->take_solve_time(nullptr);
    for (int k = 0; k < 8 && !rc; ++k) rc = F->solve(ctx, dx);
    int cnt = 0;
    cs.trisolve_ms[bi] = F->take_solve_time(&cnt) / std::max(cnt, 1);
    free_factor(ctx);
  }
  cudaFree(dx);
  free_factor(ctx);
  if (rc) return rc;
  cs.solve_block = cs.trisolve_ms[1] < cs.trisolve_ms[0] ? 128 : 256;
  return TLR_OK;
}

}  // namespace
}  // namespace tlr

extern "C" int tlr_sweep(const tlr_grid_class *classes, int nclass, const tlr_sweep_point *points,
                         int npoints, const tlr_sweep_opts *opts, double *lambda,
                         double *residual, int *status, tlr_eig_diag *point_diag,
                         tlr_sweep_diag *diag) {
  using namespace tlr;
  using clock = std::chrono::steady_clock;
  if (!classes || !points || !opts || !lambda || !residual || !status || nclass < 1 ||
      nclass > kMaxClasses || npoints < 0) {
    set_global_error("invalid sweep arguments");
    return TLR_ERR_ARG;
  }
  for (int i = 0; i < npoints; ++i)
    if (points[i].grid_class < 0 || points[i].grid_class >= nclass) {
      set_global_error("sweep point with an invalid grid class");
      return TLR_ERR_ARG;
    }
  const int rs = opts->solve.ring_slack_percent;
  if (rs != 0 && (rs < 100 || rs > 1000)) {
    set_global_error("ring_slack_percent must lie in [100, 1000]");
    return TLR_ERR_ARG;
  }
  const auto t0 = clock::now();
  const tlr_solve_opts base = opts->solve;
  const int nev = base.nev > 0 ? base.nev : classes[0].recipe->nev;
  const int workers = std::max(1, std::min(opts->workers > 0 ? opts->workers : 8,
                                           std::max(npoints, 1)));
  std::vector<ClassState> cs(nclass);
  std::vector<std::vector<tlr_ctx *>> ctxs(workers, std::vector<tlr_ctx *>(nclass, nullptr));
  std::vector<int> first(nclass, -1);
  for (int i = 0; i < npoints; ++i)
    if (first[points[i].grid_class] < 0) first[points[i].grid_class] = i;
  cudaSetDevice(opts->device);

  // per class, serially: worker 0's context, the shared symbolic analysis,
  // and (optionally) the tuned kernel choices
  int rc = TLR_OK;
  std::string err;
  for (int c = 0; c < nclass && !rc; ++c) {
    cs[c].gc = &classes[c];
    if (first[c] < 0) continue;
    if ((rc = make_context(classes[c], opts->device, &ctxs[0][c]))) {
      err = tlr_last_error(nullptr);
      break;
    }
    tlr_ctx *ctx = ctxs[0][c];
    if ((rc = stage_point(ctx, classes[c], points[first[c]]))) {
      err = ctx->last_error;
      break;
    }
    const int prec = base.precision == 1 ? 1 : 0;
    if (prec == 1 && opts->autotune) {
      if ((rc = autotune(ctx, cs[c], base.ring_slack_percent))) {
        err = ctx->last_error;
        break;
      }
    } else {
      cs[c].cuda_core_schur = base.cuda_core_schur;
      cs[c].solve_block = base.solve_block;
    }
    Factor *F = new Factor();
    ctx->factor = F;
    if ((rc = F->setup(ctx, prec, 48, cs[c].solve_block, cs[c].panel_width,
                       base.ring_slack_percent))) {
      err = ctx->last_error;
      break;
    }
    if (!cs[c].sym) cs[c].sym.reset(new Symbolic(F->sym));
  }
  if (rc) {
    for (auto &w : ctxs)
      for (auto *x : w)
        if (x) tlr_ctx_destroy(x);
    set_global_error(err);
    return rc;
  }

  std::atomic<int> next{0};
  std::atomic<int> failed{0};
  std::vector<std::string> point_err(npoints);
  // warm starts: worker w takes the contiguous run of points
  // [w npoints / workers, (w + 1) npoints / workers) in order, so each
  // point starts from its predecessor's Ritz vectors on the same context;
  // otherwise the workers share one queue
  const bool runs = base.warm_start != 0;
  auto work = [&](int w) {
    cudaSetDevice(opts->device);
    const int run_end = (int)((long long)(w + 1) * npoints / workers);
    int run_next = (int)((long long)w * npoints / workers);
    while (true) {
      const int i = runs ? run_next++ : next.fetch_add(1);
      if (i >= (runs ? run_end : npoints)) break;
      const tlr_sweep_point &pt = points[i];
      const int c = pt.grid_class;
      tlr_ctx *&ctx = ctxs[w][c];
      int st = TLR_OK;
      if (!ctx) {
        st = make_context(classes[c], opts->device, &ctx);
        if (!st) ctx->shared_sym = cs[c].sym.get();
      }
      if (!st) st = stage_point(ctx, classes[c], pt);
      double *lam = lambda + (size_t)i * nev * 2;
      double *res = residual + (size_t)i * nev;
      std::fill(lam, lam + 2 * nev, 0.0);
      std::fill(res, res + nev, -1.0);
      tlr_eig_diag d{};
      if (!st) {
        tlr_solve_opts so = base;
        so.nev = nev;
        so.cuda_core_schur = cs[c].cuda_core_schur;
        so.solve_block = cs[c].solve_block;
        if (cs[c].panel_width) so.panel_width = cs[c].panel_width;
        so.start = pt.start;
        so.nstart = pt.start ? 1 : 0;
        // concurrent contexts replay solve graphs: a cooperative grid per
        // worker could not count on having the GPU's SMs to itself
        if (workers > 1) so.persistent_solve = 0;
        st = tlr_solve(ctx, &so, lam, res, nullptr, &d);
      }
      if (st) {
        ++failed;
        point_err[i] = ctx ? ctx->last_error : std::string(tlr_last_error(nullptr));
      }
      status[i] = st;
      if (point_diag) point_diag[i] = d;
    }
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < workers; ++w) pool.emplace_back(work, w);
  work(0);
  for (auto &t : pool) t.join();
  for (auto &w : ctxs)
    for (auto *x : w)
      if (x) tlr_ctx_destroy(x);

  if (diag) {
    tlr_sweep_diag d{};
    d.wall_ms = std::chrono::duration<double, std::milli>(clock::now() - t0).count();
    d.points = npoints;
    d.failed = failed.load();
    d.workers = workers;
    const double tol = base.tol > 0 ? base.tol : classes[0].recipe->tol;
    for (int i = 0; i < npoints; ++i)
      if (status[i] == TLR_OK)
        for (int k = 0; k < nev; ++k)
          if (residual[(size_t)i * nev + k] >= 0 && residual[(size_t)i * nev + k] <= tol)
            ++d.converged_pairs;
    for (int c = 0; c < nclass; ++c) {
      d.cuda_core_schur[c] = cs[c].cuda_core_schur;
      d.solve_block[c] = cs[c].solve_block ? cs[c].solve_block : (base.precision == 1 ? 256 : 128);
      d.tune_factor_ms[c][0] = cs[c].factor_ms[0];
      d.tune_factor_ms[c][1] = cs[c].factor_ms[1];
      d.tune_trisolve_ms[c][0] = cs[c].trisolve_ms[0];
      d.tune_trisolve_ms[c][1] = cs[c].trisolve_ms[1];
      d.panel_width[c] = cs[c].panel_width ? cs[c].panel_width : base.panel_width;
      d.tune_wide_factor_ms[c] = cs[c].wide_factor_ms;
    }
    *diag = d;
  }
  for (int i = 0; i < npoints; ++i)
    if (status[i]) {  // the first failing point's status and message
      set_global_error("sweep point " + std::to_string(i) + ": " + point_err[i]);
      return status[i];
    }
  return TLR_OK;
}
