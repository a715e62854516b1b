/*
 * tailor_gb300.h -- C ABI of the GB300 BiGlobal hot path.
 *
 * One context (tlr_ctx) holds one stability problem on one GPU: the FD-q
 * rules, the prepared grid and base flow, and every derived device array.
 * The entry points mirror the reference's stage objects, each of which
 * takes ProblemData and fills a *Diagnostics struct:
 *
 *   tlr_metrics               Metrics::compute          (Metrics.hpp:69-70)
 *   tlr_baseflow_derivatives  BaseFlowDerivatives::compute
 *                                               (BaseFlowDerivatives.hpp:95-96)
 *   tlr_assemble              GlobalOperator::assemble  (GlobalOperator.hpp:53-54)
 *   tlr_apply_bc              BoundaryConditions::apply (BoundaryConditions.hpp:59-60)
 *   tlr_spmv                  MatMult on the BAIJ operators (PETSc, implicit)
 *   tlr_solve                 EigenSolver::solve        (EigenSolver.hpp:56-67)
 *
 * Every call returns a tlr_status (0 = success).  Failures carry the
 * reference's error category and message text (tlr_last_error); stage
 * ordering is enforced like the reference's PETSC_ERR_ARG_WRONGSTATE
 * preconditions.  All device work of a context runs on its own CUDA
 * stream; one host thread per context.
 *
 * Layout (shared by all arrays crossing this ABI):
 *   node n = j * ny + i, i = wall-normal xi index (bounded rule),
 *   j = spanwise eta index (periodic rule) -- the reference's natural
 *   k_j_dof ordering (Prepare.cpp:496-497, 537-552);
 *   complex numbers are interleaved (re, im) doubles;
 *   BSR: row_ptr[nb+1], col_idx[nnzb] sorted ascending, values
 *   [nnzb][5][5] complex, row-major 5x5 blocks (the reference inserts
 *   row-oriented blocks, GlobalOperator.cpp:117).
 */
#ifndef TAILOR_GB300_H
#define TAILOR_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TLR_OK = 0,
  TLR_ERR_ARG = 1,          /* invalid argument (PETSC_ERR_ARG_*)          */
  TLR_ERR_WRONGSTATE = 2,   /* stage called out of order                   */
  TLR_ERR_SIZE = 3,         /* rule/grid size mismatch (PETSC_ERR_ARG_SIZ) */
  TLR_ERR_STENCIL = 4,      /* stencil leaves the grid (PETSC_ERR_PLIB)    */
  TLR_ERR_NONFINITE = 5,    /* non-finite input or result (PETSC_ERR_FP)   */
  TLR_ERR_JACOBIAN = 6,     /* singular/negative Jacobian (ARG_OUTOFRANGE) */
  TLR_ERR_COMPLEX = 7,      /* imaginary part too large (PETSC_ERR_SUP)    */
  TLR_ERR_NONPOSITIVE = 8,  /* rho or T <= 0 (ARG_OUTOFRANGE)              */
  TLR_ERR_COEFFICIENTS = 9, /* invalid curvilinear LNS coefficients        */
  TLR_ERR_CHARACTERISTIC = 10, /* far-field decomposition failed           */
  TLR_ERR_CUDA = 11,
  TLR_ERR_NOMEM = 12,
  TLR_ERR_NOT_CONVERGED = 13,
  TLR_ERR_TIMEOUT = 14,     /* bounded device wait ran out                 */
  TLR_ERR_SINGULAR = 15,    /* zero pivot in the sparse factorisation      */
  TLR_ERR_RULE = 16         /* FD-q rule generation or validation failed   */
} tlr_status;

/* Numerical part of the reference Recipe (Recipe.hpp:17-61). */
typedef struct {
  int q_y, q_z;
  double mach, reynolds, prandtl, gas_constant, gamma;
  double reference_viscosity;      /* parsed but unused, as in the reference */
  double reference_temperature, sutherland_constant;
  double alpha_re, alpha_im;       /* streamwise wavenumber                  */
  double omega_re, omega_im;       /* search centre; lambda_s = Im w - i Re w */
  int nev;                         /* NumberOfEigenvalues                    */
  double tol;                      /* EigenSolver.Tolerance                  */
  int max_it;                      /* EigenSolver.MaximumIterations          */
} tlr_recipe;

/* One-dimensional FD-q rule (FDQRuleData, ProblemData.hpp:26-96). */
typedef struct {
  int node_count;
  int q;                        /* stencil has q+1 entries                  */
  int periodic;                 /* 0 bounded (xi), 1 periodic (eta)         */
  double period;
  const double *nodes;          /* [node_count]                             */
  const int *stencil_indices;   /* [node_count][q+1] wrapped node index     */
  const int *stencil_offsets;   /* [node_count][q+1] unwrapped displacement */
  const double *weights;        /* [3][node_count][q+1]: d0, d1, d2         */
} tlr_rule;

/* MetricDiagnostics (Metrics.hpp:40-50). */
typedef struct {
  double min_jacobian, max_jacobian, max_grid_imaginary;
  double norms[10];
} tlr_metric_diag;

/* BaseFlowDerivativeDiagnostics (BaseFlowDerivatives.hpp:67-75). */
typedef struct {
  double max_baseflow_imaginary;
  double norms[25];
} tlr_deriv_diag;

/* GlobalOperatorDiagnostics (GlobalOperator.hpp:12-32). */
typedef struct {
  long rows, columns, block_size;
  double mass_used_blocks, mass_allocated_blocks;
  double spatial_used_blocks, spatial_allocated_blocks;
  double mass_frobenius_norm, spatial_frobenius_norm;
  float assemble_ms;            /* device time of the numeric assembly      */
} tlr_operator_diag;

/* BoundaryConditionDiagnostics (BoundaryConditions.hpp:12-34). */
typedef struct {
  int wall_nodes, farfield_nodes;
  int incoming_modes, neutral_modes;
  int min_incoming_per_node, max_incoming_per_node;
  double max_characteristic_imaginary, max_eigenvector_condition;
  double eigen_frobenius_norm, eigen_mass_frobenius_norm;
} tlr_bc_diag;

/* Matrices addressable through tlr_spmv / tlr_copy_out. */
enum { TLR_MAT_M = 0, TLR_MAT_L = 1, TLR_MAT_A = 2, TLR_MAT_B = 3 };

/* Arrays addressable through tlr_copy_out. */
enum {
  TLR_OUT_METRICS = 0,      /* [N][10] double                              */
  TLR_OUT_DERIVATIVES = 1,  /* [N][25] double                              */
  TLR_OUT_ROW_PTR = 2,      /* [N+1] int (pattern of L and A_bc)           */
  TLR_OUT_COL_IDX = 3,      /* [nnzb] int                                  */
  TLR_OUT_M_VALUES = 4,     /* [N][5][5] complex (M_Gamma, block diagonal) */
  TLR_OUT_L_VALUES = 5,     /* [nnzb][5][5] complex                        */
  TLR_OUT_A_VALUES = 6,     /* [nnzb][5][5] complex (A_bc)                 */
  TLR_OUT_B_VALUES = 7      /* [N][5][5] complex (B_bc, block diagonal)    */
};

typedef struct tlr_ctx tlr_ctx;

/* Create a context for an ny x nz problem (Prepare::initialize's checks on
 * the rules: sizes, degrees, stencil indices).  device < 0 uses the
 * current device. */
int tlr_ctx_create(const tlr_recipe *recipe, const tlr_rule *xi,
                   const tlr_rule *eta, int ny, int nz,
                   double spanwise_period, int device, tlr_ctx **out);
void tlr_ctx_destroy(tlr_ctx *ctx);

/* Replace the streamwise wavenumber and search centre of a context; the
 * derived operators must be re-assembled afterwards. */
int tlr_set_alpha(tlr_ctx *ctx, double alpha_re, double alpha_im,
                  double omega_re, double omega_im);

/* Replace every numerical recipe value (physics, wavenumber, target,
 * solver settings) of a context; q_y / q_z must not change.  The grid,
 * rules, symbolic analysis and buffers are kept; the derived operators
 * must be re-assembled (sweeps over alpha, Re, Mach reuse one context). */
int tlr_set_physics(tlr_ctx *ctx, const tlr_recipe *recipe);

/* Host arrays in natural order: grid [N][3] complex (x, y, z), baseflow
 * [N][5] complex (rho, U, V, W, T) (Prepare.cpp:537-586). */
int tlr_load_fields(tlr_ctx *ctx, const double *grid, const double *baseflow);

int tlr_metrics(tlr_ctx *ctx, tlr_metric_diag *diag);
int tlr_baseflow_derivatives(tlr_ctx *ctx, tlr_deriv_diag *diag);
int tlr_assemble(tlr_ctx *ctx, tlr_operator_diag *diag);
int tlr_apply_bc(tlr_ctx *ctx, tlr_bc_diag *diag);

/* y = Mat x for Mat in {M, L, A_bc, B_bc}; x, y complex [5N].  With
 * device_pointers = 0 both are host arrays and the call copies them. */
int tlr_spmv(tlr_ctx *ctx, int which, const double *x, double *y,
             int device_pointers);

/* Copy one context array to host memory; bytes must match exactly. */
int tlr_copy_out(tlr_ctx *ctx, int what, void *dst, size_t bytes);
size_t tlr_out_bytes(tlr_ctx *ctx, int what);

/* Pointwise entry points used by the golden tests.
 * tlr_lns_points: LNSCoefficients::evaluate (LNSCoefficients.cpp:173-404)
 *   q [np][10][5] (value, dx, dy, dz, dxx, dyy, dzz, dxy, dxz, dyz),
 *   blocks [np][11][5][5] real (Gamma, A, B, C, D, Vxx, Vxy, Vxz, Vyy, Vyz,
 *   Vzz), status [np] CoefficientStatus codes.
 * tlr_transform_points: StreamwiseFourier::apply + CurvilinearTransform::
 *   apply (StreamwiseFourier.cpp:16-44, CurvilinearTransform.cpp:62-101):
 *   alpha [np] complex, phys [np][11][25], metrics [np][10]; fourier and
 *   curvilinear [np][7][25] complex. */
int tlr_lns_points(const tlr_recipe *recipe, int np, const double *q,
                   double *blocks, int *status);
int tlr_transform_points(int np, const double *alpha, const double *phys,
                         const double *metrics, double *fourier,
                         double *curvilinear, int *status);

/* Shift-and-invert Krylov-Schur solve (EigenSolver.cpp:31-89). */
typedef struct {
  int nev;                /* 0: recipe value                                */
  int ncv;                /* 0: max(2 nev, nev + 15) (SLEPc default)        */
  double tol;             /* 0: recipe value                                */
  int max_it;             /* 0: recipe value                                */
  int precision;          /* 0: FP64 factorisation (drop-in form);
                             1: FP32 factorisation + FP64 refinement       */
  double sigma_re, sigma_im; /* used when use_sigma != 0                    */
  int use_sigma;          /* 0: sigma = lambda target from omega            */
  const double *start;    /* optional complex [5N] host start vector        */
  int cuda_core_schur;    /* Schur-update kernel.  0 (default): the fastest
                             measured -- mixed form: tcgen05 (3xTF32) fed by
                             bulk copies of operand planes split once per
                             panel step, in a persistent warp-specialised
                             kernel (one CTA per SM: a copy thread, an MMA
                             thread and eight epilogue warps, two TMEM
                             accumulators, so a tile's F22 update overlaps
                             the next tile's MMAs); FP64 form: CUDA-core
                             FP64 FMA.
                             1: CUDA cores (FP32 / FP64 FMA).  2: mixed form
                             on tcgen05 with every tile staging its own
                             operands (the same bits as 0); FP64 form on the
                             FP64 tensor cores (DMMA, mma.sync m8n8k4 f64;
                             GB300's FP64 tensor rate is no higher than its
                             FP64 FMA rate, and measured 13% slower).  3:
                             mixed form, the bulk-copy kernel with a two-
                             stage ring and three CTAs per SM (the same
                             bits as 0; measured 11% slower: 513 vs 460 ms
                             for a 300 x 192 factorisation).  4: mixed
                             form, the bulk-copy kernel with one tile per
                             CTA, two CTAs per SM (the same bits as 0;
                             measured 6% slower: 351 vs 331 ms)            */
  int solve_block;        /* mixed form: diagonal-block size of the
                             triangular solves, 128, 256 or 512 (0: 256)     */
  int refinement;         /* mixed form: 0 (default) classic iterative
                             refinement; 1 FP64 GMRES-based refinement
                             (right-preconditioned GMRES(4) with the
                             complex64 LU: the same two inner solves per
                             application here, and 9% slower)               */
  int panel_width;        /* panel columns of the factorisation: 32, 64 or
                             128 (0: 32 for complex128, 64 for complex64)    */
  int cluster_panel;      /* pivoting panel over an 8-CTA thread-block
                             cluster per front (candidates exchanged through
                             distributed shared memory) or one CTA; same
                             pivots and factors.  A panel step uses the
                             cluster when at least cluster_panel fully
                             summed rows are left (1: always); 0 (default):
                             256; -1: never.  The cluster keeps the
                             panel in distributed shared memory when its
                             rows fit (up to about 3000 rows at complex64,
                             64 columns)                                */
  int persistent_solve;   /* 0 (default): each triangular solve replays a
                             CUDA graph of per-step launches; 1: one
                             persistent cooperative launch with grid
                             barriers between steps (slower on GB300: 1.82
                             vs 1.23 ms per solve at 200 x 128)              */
  int block;              /* Krylov block size: 0 or 1 (default) the single-
                             vector Krylov-Schur of the reference's SLEPc
                             solver; 2, 4 or 8 block Krylov-Schur, every
                             operator application on `block` vectors at once
                             (in the mixed form one triangular solve then
                             reads the factor once for all of them).  ncv is
                             rounded up to a multiple of block.  No
                             counterpart in the reference.                  */
  int nstart;             /* vectors in `start` ([nstart][5N] complex; 0:
                             one when start is set); at most `block` are
                             used, the rest of the start block is
                             pseudo-random                                 */
  int warm_start;         /* 1: without `start`, begin from the Ritz vectors
                             of the previous solve on this context (a
                             neighbouring point of a sweep), vector i of the
                             start block the sum of Ritz vectors i, i +
                             block, ...                                     */
  int ring_slack_percent; /* nested-dissection ordering of the factor: a box
                             of the periodic ring is cut across xi when that
                             separator has at most ring_slack_percent / 100
                             times the ring cut's nodes (0: 110, slightly
                             wider separators for shallower top fronts; 100:
                             the smallest separator; range [100, 1000]);
                             see tlr_symbolic_analyze                      */
  int conv_check;         /* convergence tests inside a Krylov-Schur
                             expansion: every conv_check operator
                             applications once the basis holds more than
                             nev vectors, the solve stops as soon as nev
                             Ritz pairs meet the tolerance (estimates, then
                             explicit residuals); the test of one basis
                             size runs on the host while the GPU applies
                             the operator to the next vector.  0: every 4
                             (default); -1: only when the basis is full, as
                             SLEPc                                          */
  int solve_wave;         /* triangular solves: 0 (default) one launch per
                             block step; 1 one dependency-driven launch per
                             direction for every level whose fronts have
                             several diagonal blocks (32-row tiles wait only
                             for the blocks they need, bounded waits).  Same
                             bits; measured 6% slower per solve at 300 x
                             192 and 12% at 200 x 128                      */
  int fp64_acceptance;    /* mixed form: the residual that accepts each
                             refined K^-1 application (||r|| <= 1e-12 ||y||)
                             -- 0 (default): a float-float residual (the
                             operator as FP32 hi/lo pairs, 48-bit products
                             and sums on the FP32 pipe, combined in FP64);
                             1: an FP64 residual (FP64 pipe).  A rejected
                             application continues with float-float
                             corrections and an FP64 acceptance either way;
                             eigen residuals are always FP64               */
} tlr_solve_opts;

typedef struct {
  int requested, converged, iterations, reason;
  double target_re, target_im;
  double max_relative_error;
  int factorizations, solves, refinement_steps;
  double factor_ms, krylov_ms, total_ms;
  double factor_flops;    /* algorithmic complex-counted flops of the LU    */
  double solve_ms;        /* time inside K^-1 applications (incl. refinement) */
  double factor_bytes;    /* bytes of the stored L and U factors            */
  double trisolve_ms;     /* device time of the triangular solves (CUDA
                             events around each solve graph)               */
  int trisolves;          /* triangular solves timed in trisolve_ms         */
  double ortho_ms;        /* Gram-Schmidt of the Arnoldi steps (host clock) */
  double dense_ms;        /* projected Schur problem on the host            */
  double residual_ms;     /* Ritz vectors and explicit residuals            */
  double refine_res[3];   /* mixed form: largest ||r|| / ||y|| seen after the
                             first solve, the first and the second correction */
  int block;              /* Krylov block size used (vectors per triangular
                             solve in the mixed form)                       */
  int conv_checks;        /* convergence checks made inside expansions      */
} tlr_eig_diag;

/* lambda [nev] complex, residual [nev]; modes [nev][5N] complex or NULL. */
int tlr_solve(tlr_ctx *ctx, const tlr_solve_opts *opts, double *lambda,
              double *residual, double *modes, tlr_eig_diag *diag);

/* Learned shift / start-vector proposal: a multilayer perceptron with
 * `depth` SiLU hidden layers of `width` units, trained and evaluated on the
 * GPU by hand-written kernels.  No reference counterpart (the reference
 * starts SLEPc from a random vector at the configured target).  Parameters
 * are FP32, flat per layer: W [out][in] row-major, then b [out].  All
 * arrays are host arrays, row-major [rows][features]. */
typedef struct tlr_mlp tlr_mlp;
int tlr_mlp_create(int n_in, int width, int depth, int n_out,
                   unsigned long long seed, tlr_mlp **out);
void tlr_mlp_destroy(tlr_mlp *m);
long long tlr_mlp_num_params(const tlr_mlp *m);
/* set != 0 copies params into the network, else out of it */
int tlr_mlp_params(tlr_mlp *m, float *params, int set);
/* mean-squared-error loss and its parameter gradient on one batch */
int tlr_mlp_gradients(tlr_mlp *m, const float *x, const float *y, int n,
                      float *grads, float *loss);
/* Adam over `epochs` passes in minibatches; loss_history[epochs] optional */
int tlr_mlp_train(tlr_mlp *m, const float *x, const float *y, int n,
                  int epochs, int batch, float lr, float *loss_history);
/* inference; bf16 != 0 rounds weights and activations to bfloat16 */
int tlr_mlp_forward(tlr_mlp *m, const float *x, int n, float *y, int bf16);

/* Frobenius norm sqrt(sum |v|^2) of `count` complex values at the device
 * address `values` (16-byte aligned: TLR_ERR_ARG otherwise), written to the
 * host double `result`, computed on `stream` (NULL: the default stream) --
 * the norm tlr_assemble and tlr_apply_bc report for the operators.  No
 * counterpart in the reference: it serves callers that cannot allocate
 * device memory (hosts whose caching allocator forbids raw cudaMalloc from
 * the libraries they load, or that reserve nearly all of HBM for their own
 * pool).  It allocates nothing: its scratch is a fixed 32 KB device array
 * inside the library, one per device, so count is limited to 2^28 values
 * (TLR_ERR_SIZE beyond that).  It copies the result to the host and
 * synchronises the stream before returning.  The first call on a device
 * looks up that array and should come before any stream capture; every
 * call shares the array, so calls that overlap on the GPU race: serialise
 * them (one stream, or synchronise between calls). */
int tlr_frobenius_noalloc(const double *values, size_t count, double *result,
                          void *stream);

/* The context's CUDA stream (cudaStream_t) -- all device work of the
 * context is ordered on it; callers time or synchronise against it. */
void *tlr_stream(tlr_ctx *ctx);

/* Batched alpha-sweep, no counterpart in the reference (which solves one
 * recipe per run, Process.cpp:34-179): every point is a full pass (metrics,
 * derivatives, assembly, boundary rows, shift-invert Krylov-Schur) of its
 * grid class at its own alpha.  Grid classes share one symbolic analysis
 * each; worker threads own one context per class and run their points
 * concurrently on the GPU. */
typedef struct {
  const tlr_recipe *recipe;   /* physics; alpha is taken from each point       */
  const tlr_rule *xi, *eta;
  int ny, nz;
  double spanwise_period;
  const double *grid;         /* natural-order fields, as for tlr_load_fields */
  const double *baseflow;
} tlr_grid_class;

typedef struct {
  int grid_class;
  double alpha_re, alpha_im;
  const double *start;        /* optional complex [5N] start vector (NULL)    */
  double reynolds;            /* > 0: overrides the class recipe's Reynolds
                                 number (Mach stays a class property: the
                                 base flow depends on it)                      */
} tlr_sweep_point;

typedef struct {
  tlr_solve_opts solve;       /* shared solve options (start is ignored)      */
  int workers;                /* concurrent instances (0: 8)                  */
  int autotune;               /* mixed form: time both Schur-update kernels,
                                 both solve block sizes and panels of 64 and
                                 128 columns on each class's first point and
                                 keep the fastest                             */
  int device;
} tlr_sweep_opts;

typedef struct {
  double wall_ms;
  int points, failed, workers;
  int converged_pairs;        /* pairs with relative residual <= tol          */
  int cuda_core_schur[16];    /* per grid class: chosen Schur kernel          */
  int solve_block[16];        /* per grid class: chosen diagonal-block size   */
  double tune_factor_ms[16][2];   /* tensor cores, CUDA cores                 */
  double tune_trisolve_ms[16][2]; /* block 256, block 128                     */
  int panel_width[16];        /* per grid class: chosen panel width (the
                                 depth of the Schur-update tiles; 0: default) */
  double tune_wide_factor_ms[16]; /* the chosen kernel with 128-wide panels   */
} tlr_sweep_diag;

/* lambda [npoints][nev] complex, residual [npoints][nev] (-1: not solved),
 * status [npoints]; point_diag [npoints] optional.  Returns the first
 * failing point's status (its message in tlr_last_error(NULL)). */
int tlr_sweep(const tlr_grid_class *classes, int nclass, const tlr_sweep_point *points,
              int npoints, const tlr_sweep_opts *opts, double *lambda, double *residual,
              int *status, tlr_eig_diag *point_diag, tlr_sweep_diag *diag);

/* Test hook, no counterpart in the reference: one Schur-complement update
 * F22 -= L21 U12 of a single dense complex64 front (m x m, column-major,
 * interleaved re/im) for the panel columns [k0, k0 + min(w, p - k0)), on
 * the tensor-core (tcgen05, 3xTF32) path the mixed factorisation uses.
 * k0 must be a multiple of w, w <= 64.  lbo/sbo: shared-memory descriptor
 * strides of the operand planes in bytes (0: the library's values).
 * Writes the updated front to out. */
/* Test hook, no counterpart in the reference: x = K^-1 rhs through the
 * context's complex64 factor (left by a mixed-form tlr_solve) for nvec
 * host vectors rhs [nvec][5N] complex (rounded to complex64), written to
 * out [nvec][5N].  multi = 1 solves all of them in one multi-vector solve
 * (nvec 2, 4 or 8; every factor tile read once), multi = 0 one at a time;
 * both give the same bits. */
int tlr_factor_solve(tlr_ctx *ctx, int nvec, const double *rhs, double *out, int multi);

int tlr_schur_update_c64(const float *front, int m, int p, int k0, int w, unsigned lbo,
                         unsigned sbo, float *out);

/* An explicit generalized pencil A x = lambda B x as a solver context
 * (EigenSolver::solve(recipe, eigenMatrix, massMatrix, ...),
 * EigenSolver.hpp:60-67: the overload for small independently known
 * problems).  A and B are dense n x n complex matrices, column-major with
 * interleaved (re, im) doubles; B must be block diagonal in 5 x 5 blocks
 * (TLR_ERR_ARG otherwise).  The recipe supplies the search centre omega,
 * nev, tol and max_it.  The context accepts tlr_solve (FP64 or mixed
 * form), tlr_spmv and tlr_copy_out of A and B, tlr_set_alpha (a new search
 * centre) and tlr_set_physics; the grid stages return TLR_ERR_WRONGSTATE.
 * Modes are returned as 5 * ceil(n / 5) complex entries (the first n are
 * the eigenvector).  1 <= n <= 5000 (TLR_ERR_SIZE otherwise): the pencil
 * is stored densely. */
int tlr_pencil_create(const tlr_recipe *recipe, int n, const double *A, const double *B,
                      int device, tlr_ctx **out);

/* Symbolic analysis on the host, no GPU needed: the nested-dissection
 * ordering and the multifrontal structure that tlr_solve and tlr_sweep use
 * for the grid of the rules xi (bounded, Ny nodes) and eta (periodic, Nz
 * nodes).  The reference leaves this to MUMPS's analysis phase behind
 * PCLU (EigenSolver.cpp:61-71); here it lets a caller size a
 * factorisation (flops, factor and front-pool entries) before creating a
 * context.  leaf_nodes: boxes of at most this many nodes become leaf
 * fronts (0: the solver's 48).  ring_slack_percent: a box of the periodic
 * ring is cut across xi instead of across the ring when that separator
 * has at most this percentage of the ring cut's nodes (0: the solver's
 * 110; 100..1000).  Optional outputs: node_rank[Ny*Nz] (elimination
 * position of node j*Ny + i), node_front[Ny*Nz] (front that eliminates
 * it), front_parent[front_capacity] (-1 for the root; fronts are numbered
 * in postorder).  *info is filled first, so a call with front_parent NULL
 * sizes the array; a front_capacity below info->fronts returns
 * TLR_ERR_SIZE. */
typedef struct {
  int fronts;                /* fronts in the elimination tree               */
  int levels;                /* tree height + 1: batched launches per sweep  */
  int max_front_order;       /* largest front, scalar rows                   */
  int max_pivots;            /* largest pivot block, scalar rows             */
  double flops;              /* factorisation flops, 8 real per complex MAC  */
  long long factor_elems;    /* stored L and U entries: sum p (p + 2 b)      */
  long long pool_elems;      /* front pool entries: sum m^2                  */
} tlr_symbolic_info;

int tlr_symbolic_analyze(const tlr_rule *xi, const tlr_rule *eta, int leaf_nodes,
                         int ring_slack_percent, tlr_symbolic_info *info, int *node_rank,
                         int *node_front, int *front_parent, int front_capacity);

/* FD-q rule generation on the host (src/Python/fdq_nodes.py:280-353,
 * calculate_fdq_rule and calculate_periodic_fdq_rule).  periodic = 0: the
 * equal-error nodes on [-1, 1] with node_count - 1 intervals (period is
 * ignored and taken as 2); periodic = 1: node_count uniform nodes on
 * [-period/2, period/2) with centred stencils.  The caller provides
 * nodes[node_count], stencil_indices and stencil_offsets
 * [node_count][q+1] and weights [3][node_count][q+1] (d0, d1, d2), the
 * layout of tlr_rule; log_error[node_count] (the equal-error amplitudes,
 * zero for periodic rules) may be NULL.  Argument checks as the
 * reference's (TLR_ERR_ARG); a node solve that does not converge or a
 * rule that fails the reference's symmetry, equal-error or polynomial
 * checks returns TLR_ERR_RULE. */
int tlr_fdq_rule(int node_count, int q, int periodic, double period, double *nodes,
                 int *stencil_indices, int *stencil_offsets, double *weights,
                 double *log_error);

/* Test hook, no counterpart in the reference: failure detection without a
 * GPU fault.  which = 0: the tensor-core kernel's bounded mbarrier wait on
 * a barrier that nothing completes; which = 1: the persistent solve's
 * bounded grid barrier waiting for a CTA that does not exist.  limit is the
 * poll count; *timed_out = 1 when the wait gave up and reported it (the
 * context stays usable). */
int tlr_wait_selftest(int which, unsigned limit, int *timed_out);

/* Kernels of this library launched by the process so far (every kernel
 * node of a replayed CUDA graph counts once per replay; cuBLAS kernels are
 * not counted).  No counterpart in the reference: it lets a caller check
 * which device work a region ran. */
long long tlr_kernel_launches(void);

const char *tlr_status_string(int status);
/* Message of the last failure: the context's own for a non-NULL ctx; for
 * NULL, the last failure of a call without a context (creation, sweeps,
 * pencils, rule generation, symbolic analysis) on the calling thread --
 * each host thread keeps its own.  The pointer stays valid until the next
 * call on the same context or thread. */
const char *tlr_last_error(const tlr_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
