// tlr_lu.h -- device multifrontal factorisation of K = A_bc - sigma B_bc.
#pragma once

#include <vector>

#include "tlr_internal.h"
#include "tlr_symbolic.h"

namespace tlr {

struct DevFront {
  long long off, toff, cmap_off;
  int p, m, parent, node_off;
};


// Default of Factor::cluster_rows (the automatic cluster-panel choice).
constexpr int kClusterPanelRows = 256;

struct Step {  // one panel step of one level
  int nf, max_m, max_b, max_ext, prefix_off, tiles;
  // complex64: per-front prefixes (nf + 1 each, in the schedule) of the
  // step's 128-row L21 tiles and 64-column U12 tiles, and their totals
  int pa_off = 0, pb_off = 0, atiles = 0, btiles = 0;
};

struct Level {
  int nfronts = 0, fronts_off = 0, max_m = 0;
  int pmax = 0, bmax = 0, nck_b = 1;  // backward border GEMV chunks
  int kids[2] = {0, 0}, kids_off[2] = {0, 0}, kids_maxb[2] = {0, 0};
  long long entry_begin = 0, entry_end = 0, pool_begin = 0, pool_end = 0;
  std::vector<Step> steps;
  std::vector<int> blk_nf;    // blk_nf[b]: fronts of the level with p > b sw
  std::vector<int> fwd_rows;  // rows below block b, largest over those fronts
  // dependency-driven solve of the level (levels with two or more blocks):
  // forward and backward 32-row tiles in dependency order, and their
  // counters (4 + nfronts * maxblk each)
  bool wave = false;
  int maxblk = 0;
  long long wf_off = 0, wb_off = 0;
  int wf_n = 0, wb_n = 0;
  long long wcf_off = 0, wcb_off = 0;
  int wctr_n = 0;
};

// One phase of the persistent solve: a kind of work item over a level's
// fronts (fl_off into the level schedule), block b, and an nx x ny x nz
// item grid (the CTA grid of the equivalent separate launch).
struct Phase {
  int type, fl_off, b, nx, ny, nz, nck, pmax;
};

struct Factor {
  Symbolic sym;
  int prec = 0;  // 0: complex128 fronts, 1: complex64 fronts
  // Schur updates on the tensor cores: tcgen05 (3xTF32) for complex64
  // fronts, DMMA (FP64 mma.sync) for complex128 fronts; else CUDA cores
  bool tensor_cores = true;
  // panel steps with at least this many fully summed rows left run over an
  // 8-CTA cluster (INT_MAX: never)
  int cluster_rows = kClusterPanelRows;
  int *d_tc_err = nullptr;   // set by a tensor-core kernel whose wait timed out
  // complex64 Schur updates: operand plane images of one panel step, read
  // by bulk copies (tc_bulk), else staged by every tile's own threads
  bool tc_bulk = true;
  // bulk kernel: 2 persistent warp-specialised (default), 0 one tile per CTA
  // with three stages / two CTAs per SM, 1 two stages / three CTAs per SM
  int tc_variant = 2;
  unsigned char *tc_planes = nullptr;
  int w = 32;    // panel width
  int sw = 128;  // rows of a diagonal block of the solves (128 or 256)
  int ring_slack = kRingSlackDefault;  // nested-dissection ring slack, percent
  std::vector<Level> levels;
  void *pool = nullptr, *work = nullptr, *work2 = nullptr, *vec_a = nullptr;
  DevFront *d_fronts = nullptr;
  AsmEntry *d_entries = nullptr;
  int *d_cmap = nullptr, *d_nodes = nullptr, *d_ipiv = nullptr, *d_perm = nullptr;
  int *d_sched = nullptr, *d_pert = nullptr;
  int2 *d_cinv = nullptr;  // child border rows mapped onto each front row
  // sw x sw diagonal blocks of every pivot block: inv(L_bb), inv(U_bb)
  // (scratch of the factor rewrite) and D_b = inv(U_bb) inv(L_bb)
  void *linv = nullptr, *uinv = nullptr, *dmat = nullptr;
  long long *d_inv_off = nullptr;
  int2 *d_inv_blocks = nullptr;
  int4 *d_ltiles = nullptr, *d_utiles = nullptr;
  // the same rewrite on the tensor cores (complex64, 256-row blocks, when
  // the Schur updates run there too): 128-row L tiles, 64-column U tiles
  int4 *d_ltiles_tc = nullptr, *d_utiles_tc = nullptr;
  long long n_ltiles_tc = 0, n_utiles_tc = 0;
  int n_inv_blocks = 0;
  long long inv_elems = 0, n_ltiles = 0, n_utiles = 0;
  cudaGraphExec_t graph_exec = nullptr;  // captured solve, replayed per call
  // persistent solve: one cooperative launch per solve over a phase table
  bool persistent = false;
  int persist_grid = 0;                  // CTAs (0: two per SM, capped by occupancy)
  Phase *d_phases = nullptr;
  int nphases = 0;
  unsigned *d_barrier = nullptr;
  int *d_solve_err = nullptr;
  long long graph_kernels = 0;           // kernel nodes of graph_exec
  // levels with several diagonal blocks per front solved by one dependency-
  // driven launch each way (false, the default: one launch per block step)
  bool wave = false;
  int4 *d_wave_tiles = nullptr;
  int *d_wave_ctr = nullptr;
  int wave_grid = 0;                     // CTAs of a wave launch (at most)
  double2 *d_partial = nullptr;
  int perturbed = 0;
  // CUDA events around every replayed solve graph (device time of the
  // triangular solves); collected and reset by take_solve_time()
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  double take_solve_time(int *count);
  bool factored = false;
  double sigma_re = 0.0, sigma_im = 0.0;

  // Multi-RHS solves (complex64 factors): nr vectors at once, every factor
  // tile read once for all of them.  Buffers sized for multi_cap vectors,
  // allocated on first use; one captured graph per vector count.
  static constexpr int kMaxRhs = 8;
  int multi_cap = 0;
  long long partial_stride = 0;   // border partial sums of one vector
  void *work_m = nullptr, *work2_m = nullptr, *vec_m = nullptr;
  double2 *partial_m = nullptr;
  cudaGraphExec_t graph_m[kMaxRhs + 1] = {};
  long long graph_m_kernels[kMaxRhs + 1] = {};
  // In-place x <- K^-1 x for nr vectors at x + r * 5 nn (complex64 only,
  // 2 <= nr <= kMaxRhs; events a/b, when given, bracket the triangular
  // solve and mark a capture into the caller's graph: no graph of our own).
  int solve_multi(tlr_ctx *ctx, void *x, int nr, cudaEvent_t a = nullptr,
                  cudaEvent_t b = nullptr, bool capture = false);
  // allocate the multi-vector buffers (outside any stream capture)
  int solve_multi_prepare(tlr_ctx *ctx);
  template <int SW, int NR> int solve_impl_m(tlr_ctx *ctx);
  int solve_impl_m_dispatch(tlr_ctx *ctx, int nr);

  int setup(tlr_ctx *ctx, int precision, int leaf, int solve_block = 0, int panel_width = 0,
            int ring_slack_percent = 0);
  void release();
  int factor(tlr_ctx *ctx, double sr, double si, double tiny);
  // In-place x <- K^-1 x on a device vector in the factor's precision.
  int solve(tlr_ctx *ctx, void *x);
  // Enqueue one solve's kernels on the context stream without a graph
  // (for capture into a caller's graph); events a/b, when given, bracket
  // the triangular solve.
  int enqueue_solve(tlr_ctx *ctx, void *x, cudaEvent_t a, cudaEvent_t b);

  template <class C> int factor_impl(tlr_ctx *ctx, double sr, double si, double tiny);
  template <class C, int SW> int solve_impl(tlr_ctx *ctx, void *x);
  template <class C, int SW> int rewrite_factors(tlr_ctx *ctx);
  template <class C, int SW> int solve_persistent(tlr_ctx *ctx);
  int build_phases(tlr_ctx *ctx);
  // error raised inside a persistent solve since the last call (a grid
  // barrier that gave up); resets the flag
  int take_solve_error(tlr_ctx *ctx);
};

}  // namespace tlr
