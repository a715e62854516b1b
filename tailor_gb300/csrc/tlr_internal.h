// tlr_internal.h -- context layout and helpers shared by the CUDA sources.
//
// Device layout of one problem (N = ny * nz nodes, S = (q_y+1)(q_z+1)
// stencil blocks per block row):
//   grid_c      [N][3][2]  complex grid as loaded (validated in place)
//   base_c      [N][5][2]  complex base flow as loaded
//   base        [5][N]     real base flow, structure of arrays
//   metrics     [10][N]    real metrics (Metrics.hpp:15-26 order), SoA
//   derivs      [25][N]    real derivatives, derivative-major SoA
//   coef        [CF_COUNT][N] curvilinear LNS coefficients per node, SoA
//   row_ptr/col [N+1]/[N*S] BSR pattern shared by L and A_bc
//   L, A        [N*S][25]  double2 (re, im) row-major 5x5 blocks
//   M, B        [N][25]    double2 block-diagonal mass matrices
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tailor_gb300.h"

namespace tlr {

// Coefficient record, one SoA plane per entry (CurvilinearLNSCoefficients,
// CurvilinearTransform.hpp:61-78): K0, Kxi, Keta complex (re, im planes),
// Vxixi, Vxieta, Vetaeta and Gamma real.
enum : int {
  CF_K0_RE = 0,
  CF_K0_IM = 25,
  CF_KXI_RE = 50,
  CF_KXI_IM = 75,
  CF_KETA_RE = 100,
  CF_KETA_IM = 125,
  CF_VXX = 150,
  CF_VXE = 175,
  CF_VEE = 200,
  CF_GAMMA = 225,
  CF_COUNT = 250
};

// Device status words (atomicMax targets), one per reference check.
enum : int {
  ST_STENCIL = 0,
  ST_NONFINITE = 1,
  ST_JACOBIAN = 2,
  ST_COMPLEX = 3,
  ST_SECOND = 4,
  ST_NONPOSITIVE = 5,
  ST_DERIV = 6,
  ST_COEF = 7,
  ST_CHAR = 8,
  ST_TIMEOUT = 9,
  ST_COUNT = 16
};

// Reduction scratch slots (doubles).
enum : int {
  RD_MINJ = 0,
  RD_MAXJ = 1,
  RD_MAXIM = 2,
  RD_BFIM = 3,
  RD_CHARIM = 4,
  RD_COND = 5,
  RD_COUNT = 8
};

struct DevRule {
  int n = 0, q = 0, s = 0;
  int *off = nullptr;    // [n][s]
  int *idx = nullptr;    // [n][s]
  double *w1 = nullptr;  // [n][s]
  double *w2 = nullptr;  // [n][s]
  int *centre = nullptr; // [n] slot with offset 0
  int *order = nullptr;  // [n][s] slots sorted by wrapped index
};

struct Factor;    // sparse LU state (tlr_lu.cu)
struct Symbolic;  // elimination structure (tlr_symbolic.h)

}  // namespace tlr

struct tlr_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  tlr_recipe recipe{};
  int ny = 0, nz = 0, nn = 0;
  double span = 0.0;
  int sx = 0, se = 0, S = 0;
  long long nnzb = 0;
  tlr::DevRule xi, eta;
  std::vector<int> h_xi_off, h_eta_off, h_xi_idx, h_eta_idx;
  std::vector<double> h_xi_w1, h_xi_w2, h_eta_w1, h_eta_w2;

  double *grid_c = nullptr, *base_c = nullptr, *base = nullptr;
  double *metrics = nullptr, *derivs = nullptr, *coef = nullptr;
  int *row_ptr = nullptr, *col = nullptr;
  double2 *L = nullptr, *M = nullptr, *A = nullptr, *B = nullptr;
  // A_bc split into FP32 hi/lo pairs (re_hi, re_lo, im_hi, im_lo) for the
  // float-float refinement residual; rebuilt when the operator changes
  float4 *aff = nullptr, *wff = nullptr;  // wff: the iterate split the same way
  float4 *wff_m = nullptr;                // the same for up to 8 iterates at once
  const tlr::Symbolic *shared_sym = nullptr;  // set by a sweep: reuse this analysis
  void *kws = nullptr;                          // Krylov workspace (tlr_krylov.cu)
  bool aff_valid = false;
  int *status = nullptr;     // [ST_COUNT]
  double *red = nullptr;     // [RD_COUNT]
  double *partial = nullptr; // per-block partial sums for norms
  int partial_blocks = 0;
  int *bc_modes = nullptr;   // [nz][2]: incoming and neutral counts
  double *bc_cond = nullptr; // [nz]: cond(R) per far-field node
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  bool fields = false, have_metrics = false, have_derivs = false;
  bool assembled = false, have_bc = false;
  // an explicit pencil (tlr_pencil_create): only A, B and the solve exist
  bool pencil = false;
  void *own_sym = nullptr;                 // symbolic analysis owned by the context
  void (*own_sym_free)(void *) = nullptr;
  std::string last_error;
  tlr::Factor *factor = nullptr;
};

namespace tlr {

int fail(tlr_ctx *ctx, int code, const std::string &msg);
int cuda_fail(tlr_ctx *ctx, cudaError_t err, const char *what);

#define TLR_CUDA(ctx, call)                                   \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return tlr::cuda_fail(ctx, e_, #call); \
  } while (0)

// Stage launchers (one .cu file each).
int run_metrics(tlr_ctx *ctx, tlr_metric_diag *diag);
int run_derivatives(tlr_ctx *ctx, tlr_deriv_diag *diag);
int run_pattern(tlr_ctx *ctx);
int run_assemble(tlr_ctx *ctx, tlr_operator_diag *diag);
int run_bc(tlr_ctx *ctx, tlr_bc_diag *diag);
int run_spmv(tlr_ctx *ctx, int which, const double2 *x, double2 *y);
int frobenius(tlr_ctx *ctx, const double2 *v, long long count, double *out);
// r = y - (A_bc - sigma B_bc) w with A_bc w in float-float arithmetic on the
// FP32 pipe (about 48-bit significands); builds ctx->aff on first use.
int residual_ff(tlr_ctx *ctx, const double2 *y, const double2 *w, double sr, double si,
                double2 *r);
// The same products on nr vectors at once (nr 1, 2, 4 or 8; vector v at
// + v * 5 nn): each operator block is read once for all of them.
int run_spmv_multi(tlr_ctx *ctx, int which, const double2 *x, double2 *y, int nr);
int residual_ff_multi(tlr_ctx *ctx, const double2 *y, const double2 *w, double sr, double si,
                      double2 *r, int nr);
// allocate the buffers residual_ff_multi uses (outside any stream capture)
int residual_ff_multi_prepare(tlr_ctx *ctx);
// ||v||_2 into device memory out (scratch: ctx->partial_blocks doubles),
// stream-ordered, no host synchronisation (capturable).
int vec_norm_async(tlr_ctx *ctx, const double2 *v, long long count, double *scratch,
                   double *out);
// Krylov basis primitives (tlr_kvec.cu), stream-ordered, results in device
// memory.  V is column-major with leading dimension ldv; part holds
// partial_blocks x nk complex partial sums, npart partial_blocks doubles.
// h = V(:, 0:nk)^H w
int kv_dot(tlr_ctx *ctx, long long n, const double2 *V, long long ldv, int nk,
           const double2 *w, double2 *part, double2 *h);
// w -= V(:, 0:nk) h; with norm, also *norm = ||w|| of the result
int kv_update(tlr_ctx *ctx, long long n, const double2 *V, long long ldv, int nk,
              const double2 *h, double2 *w, double *npart, double *norm);
// out(:, 0:nl) = V(:, 0:nq) Y(0:nq, 0:nl); out must not overlap V
int kv_combine(tlr_ctx *ctx, long long n, const double2 *V, long long ldv, int nq,
               const double2 *Y, int ldy, int nl, double2 *out, long long ldo);
// dst = src * s / *dnorm (dnorm null: dst = src * s; a zero norm gives zeros)
int kv_scale(tlr_ctx *ctx, long long n, const double2 *src, const double *dnorm, double s,
             double2 *dst);
// y += a x
int kv_axpy(tlr_ctx *ctx, long long n, double2 a, const double2 *x, double2 *y);
// Launch the persistent solve's grid barrier on one CTA with a target it
// cannot reach (bounded-wait self test).
int grid_barrier_probe(unsigned *count, unsigned limit, int *err);
// Allocate and fill ctx->aff / ctx->wff if needed (outside stream capture).
int prepare_ff(tlr_ctx *ctx);
int run_solve(tlr_ctx *ctx, const tlr_solve_opts *opts, double *lambda,
              double *residual, double *modes, tlr_eig_diag *diag);
void free_factor(tlr_ctx *ctx);
void free_workspace(tlr_ctx *ctx);
// Message returned by tlr_last_error(NULL) on the calling thread.
void set_global_error(const std::string &msg);
// Keep the symbolic analysis and device buffers, drop the numeric factor.
void invalidate_factor(tlr_ctx *ctx);

// Count of this library's kernel launches (tlr_kernel_launches).  Launches
// recorded while a stream is captured are not counted; a replayed graph
// adds its kernel nodes.
void count_launches(long long n = 1);
long long launch_total();
struct CaptureScope {  // suppresses counting on this thread during capture
  CaptureScope();
  ~CaptureScope();
};

struct DevFront;
// Tensor-core Schur update of one panel step (tlr_tc.cu).
// The same update with the operands converted once per panel step into
// TF32 plane images (planes: (atiles + btiles) x ceil(w / 8) x 16 KB of
// scratch) and streamed into shared memory by bulk copies; pa / pb are the
// per-front prefixes of the step's 128-row L21 tiles and 64-column U12 tiles.
int launch_gemm_tc_bulk(tlr_ctx *ctx, const int *fl, const int *prefix, const int *pa,
                        const int *pb, int nf, int s, int w, float2 *pool, const DevFront *fr,
                        int tiles, int atiles, int btiles, unsigned char *planes, int *err,
                        cudaStream_t st, int variant = 0);
size_t tc_chunk_image_bytes();
int launch_gemm_tc(tlr_ctx *ctx, const int *fl, const int *prefix, int nf, int s, int w,
                   float2 *pool, const DevFront *fr, int tiles, int *err, cudaStream_t st,
                   uint32_t lbo = 128, uint32_t sbo = 256);

// The complex64 factor rewrite of the block-scaled solves (256-row diagonal
// blocks) on the tensor cores: U' and D_b from utiles {front, block, first
// column, kind} (64 columns each), then L' from ltiles {front, block, first
// row, -} (128 rows each), in place.
int launch_rewrite_tc(tlr_ctx *ctx, const int4 *ltiles, long long nl, const int4 *utiles,
                      long long nu, float2 *pool, const DevFront *fr, const long long *inv_off,
                      const float2 *Linv, const float2 *Uinv, float2 *dmat, int *err,
                      cudaStream_t st);

inline int blocks_for(long long n, int threads) {
  return static_cast<int>((n + threads - 1) / threads);
}

}  // namespace tlr
