// tlr_assemble.cu -- BSR pattern, pointwise coefficients and the numeric
// assembly of M_Gamma and L (K3).
//
// Reference: GlobalOperator.cpp:162-378.  The reference evaluates the
// coefficient pipeline twice per node and makes 97 blocked insertions per
// node; here one kernel evaluates each node's curvilinear blocks once into a
// per-node SoA record (L2-resident), and a second kernel streams the block
// rows out.  In the writer every FP64 operation is lane-dense: a CTA first
// builds, in shared memory, the 17 "line" blocks of a few nodes (centre,
// xi line, eta line: dense complex) and the 6 structural nonzeros of each
// cross block, then writes the nodes' contiguous 77-block rows with
// coalesced 16-byte streaming stores.  Each block entry is accumulated in
// the reference's ADD order (K0, xi-line combination, eta-line
// combination, cross term); this file is compiled with --fmad=false.
#include <cfloat>

#include "tlr_internal.h"
#include "tlr_lns.cuh"

namespace tlr {
namespace {

constexpr int kSub = 4;        // nodes per writer iteration
constexpr int kMaxSx = 12;     // stencil size limits of the writer
constexpr int kMaxSe = 8;
constexpr int kMaxLine = kMaxSx + kMaxSe - 1;
constexpr int kMaxS = kMaxSx * kMaxSe;
constexpr int kWriterThreads = 256;

// rc of the six structural nonzeros of the viscous curvilinear blocks.
__constant__ int c_vpos[6] = {6, 12, 18, 24, 13, 17};
__constant__ int c_vidx[25] = {-1, -1, -1, -1, -1, -1, 0,  -1, -1,
                               -1, -1, -1, 1,  4,  -1, -1, -1, 5,
                               2,  -1, -1, -1, -1, -1, 3};

__device__ inline bool finite(double v) { return isfinite(v); }

// BSR column pattern (GlobalOperator.cpp:209-283): row n = j*ny + i holds
// the tensor product of its eta and xi stencils, eta slots in ascending
// wrapped index, xi slots ascending.
__global__ void k_pattern(int ny, int nz, DevRule xi, DevRule eta,
                          int *row_ptr, int *col) {
  const int S = xi.s * eta.s;
  const long long total = (long long)ny * nz * S;
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < (long long)ny * nz + 1) row_ptr[x] = (int)(x * S);
  if (x >= total) return;
  const int n = (int)(x / S), k = (int)(x % S);
  const int i = n % ny, j = n / ny;
  const int r = k / xi.s, t = k % xi.s;
  const int s = eta.order[j * eta.s + r];
  col[x] = eta.idx[j * eta.s + s] * ny + xi.idx[i * xi.s + t];
}

struct CoefParams {
  int nn;
  double Re, Pr, M, gamma, s;
  double ia_re, ia_im, a2_re, a2_im;
  int alpha_finite;
};

struct CoefBody {
  const FlowPoint &f;
  const Transport &tr;
  const Metric10 &m;
  const CoefParams &p;
  double *coef;
  size_t nn, n;
  bool &ok;
  template <int RC>
  __device__ __forceinline__ void operator()() {
    const Entry e = phys_entry<RC>(f, tr);
    const FourierEntry fe =
        fourier_entry<RC>(e, p.ia_re, p.ia_im, p.a2_re, p.a2_im);
    const CurvEntry c = curv_entry<RC>(fe, m);
    ok = ok && finite(e.A) && finite(e.B) && finite(e.C) && finite(e.D) &&
         finite(e.G) && finite(e.Vxx) && finite(e.Vxy) && finite(e.Vxz) &&
         finite(e.Vyy) && finite(e.Vyz) && finite(e.Vzz) && finite(c.K0r) &&
         finite(c.K0i) && finite(c.Kxr) && finite(c.Kxi) && finite(c.Ker) &&
         finite(c.Kei) && finite(c.Vxx) && finite(c.Vxe) && finite(c.Vee);
    coef[(CF_K0_RE + RC) * nn + n] = c.K0r;
    coef[(CF_K0_IM + RC) * nn + n] = c.K0i;
    coef[(CF_KXI_RE + RC) * nn + n] = c.Kxr;
    coef[(CF_KXI_IM + RC) * nn + n] = c.Kxi;
    coef[(CF_KETA_RE + RC) * nn + n] = c.Ker;
    coef[(CF_KETA_IM + RC) * nn + n] = c.Kei;
    coef[(CF_VXX + RC) * nn + n] = c.Vxx;
    coef[(CF_VXE + RC) * nn + n] = c.Vxe;
    coef[(CF_VEE + RC) * nn + n] = c.Vee;
    coef[(CF_GAMMA + RC) * nn + n] = c.G;
  }
};

// One thread per node: evaluateNode (GlobalOperator.cpp:124-145) into
// the SoA coefficient record; status on any invalid input or output.
__global__ void __launch_bounds__(128)
    k_coefficients(CoefParams p, const double *__restrict__ base_c,
                   const double *__restrict__ der,
                   const double *__restrict__ met, double *__restrict__ coef,
                   int *status) {
  const int nn = p.nn;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  bool ok = p.alpha_finite != 0;
  FlowPoint f{};
  {
    const double *b = base_c + (size_t)n * 10;
    for (int c = 0; c < 5; ++c)
      if (!finite(b[2 * c]) || !finite(b[2 * c + 1]) || b[2 * c + 1] != 0.0)
        ok = false;
    f.rho = b[0]; f.U = b[2]; f.V = b[4]; f.W = b[6]; f.T = b[8];
  }
  auto D = [&](int d, int c) { return der[(d * 5 + c) * (size_t)nn + n]; };
  f.rhoy = D(0, 0); f.Uy = D(0, 1); f.Vy = D(0, 2); f.Wy = D(0, 3); f.Ty = D(0, 4);
  f.rhoz = D(1, 0); f.Uz = D(1, 1); f.Vz = D(1, 2); f.Wz = D(1, 3); f.Tz = D(1, 4);
  f.Uyy = D(2, 1); f.Vyy = D(2, 2); f.Wyy = D(2, 3); f.Tyy = D(2, 4);
  f.Uzz = D(3, 1); f.Vzz = D(3, 2); f.Wzz = D(3, 3); f.Tzz = D(3, 4);
  f.Uyz = D(4, 1); f.Vyz = D(4, 2); f.Wyz = D(4, 3);
  for (int k = 0; k < 25; ++k)
    if (!finite(der[k * (size_t)nn + n])) ok = false;
  if (!(f.rho > 0.0) || !(f.T > 0.0)) ok = false;
  Metric10 m;
  m.xy = met[n]; m.xz = met[(size_t)nn + n];
  m.ey = met[2 * (size_t)nn + n]; m.ez = met[3 * (size_t)nn + n];
  m.xyy = met[4 * (size_t)nn + n]; m.xzz = met[5 * (size_t)nn + n];
  m.xyz = met[6 * (size_t)nn + n]; m.eyy = met[7 * (size_t)nn + n];
  m.ezz = met[8 * (size_t)nn + n]; m.eyz = met[9 * (size_t)nn + n];
  for (int k = 0; k < 10; ++k)
    if (!finite(met[k * (size_t)nn + n])) ok = false;
  const Transport tr = transport(f, p.Re, p.Pr, p.M, p.gamma, p.s);
  CoefBody body{f, tr, m, p, coef, (size_t)nn, (size_t)n, ok};
  for_entries<0>(body);
  if (!ok) atomicMax(status + ST_COEF, 1);
}

struct WriterShared {
  double cf[kSub][CF_COUNT];
  double2 line[kSub][kMaxLine][25];
  double cross[kSub][kMaxS][6];
  double w1x[kSub][kMaxSx], w2x[kSub][kMaxSx];
  double w1e[kSub][kMaxSe], w2e[kSub][kMaxSe];
  int order[kSub][kMaxSe];
  int cx[kSub], ce[kSub];
};

// Writer: M and L block rows for kSub consecutive nodes per iteration.
__global__ void __launch_bounds__(kWriterThreads)
    k_write_rows(int ny, int nz, DevRule xi, DevRule eta,
                 const double *__restrict__ coef, double2 *__restrict__ L,
                 double2 *__restrict__ Mv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WriterShared &sh = *reinterpret_cast<WriterShared *>(smem_raw);
  const int nn = ny * nz;
  const int sx = xi.s, se = eta.s, S = sx * se, NL = sx + se - 1;
  const int tid = threadIdx.x;
  const int groups = (nn + kSub - 1) / kSub;
  for (int g = blockIdx.x; g < groups; g += gridDim.x) {
    const int n0 = g * kSub;
    const int cnt = min(kSub, nn - n0);
    // 1. stage coefficients and stencil data
    for (int x = tid; x < CF_COUNT * kSub; x += kWriterThreads) {
      const int f = x / kSub, u = x % kSub;
      sh.cf[u][f] = u < cnt ? coef[(size_t)f * nn + n0 + u] : 0.0;
    }
    for (int x = tid; x < kSub * (kMaxSx + kMaxSe + 1); x += kWriterThreads) {
      const int u = x / (kMaxSx + kMaxSe + 1), r = x % (kMaxSx + kMaxSe + 1);
      const int n = min(n0 + u, nn - 1);
      const int i = n % ny, j = n / ny;
      if (r < sx) {
        sh.w1x[u][r] = xi.w1[i * sx + r];
        sh.w2x[u][r] = xi.w2[i * sx + r];
      } else if (r >= kMaxSx && r - kMaxSx < se) {
        const int s = r - kMaxSx;
        sh.w1e[u][s] = eta.w1[j * se + s];
        sh.w2e[u][s] = eta.w2[j * se + s];
        sh.order[u][s] = eta.order[j * se + s];
      } else if (r == kMaxSx + kMaxSe) {
        sh.cx[u] = xi.centre[i];
        sh.ce[u] = eta.centre[j];
      }
    }
    __syncthreads();
    // 2. line blocks (dense complex), entry-parallel
    for (int x = tid; x < kSub * NL * 25; x += kWriterThreads) {
      const int u = x / (NL * 25), rem = x % (NL * 25);
      const int lb = rem / 25, rc = rem % 25;
      const double *cf = sh.cf[u];
      const int cx = sh.cx[u], ce = sh.ce[u];
      const double vxe = cf[CF_VXE + rc];
      double re, im;
      if (lb < sx) {  // xi-line block at (eta slot ce, xi slot lb)
        const double w1 = sh.w1x[u][lb], w2 = -sh.w2x[u][lb];
        const double bre = w1 * cf[CF_KXI_RE + rc] + w2 * cf[CF_VXX + rc];
        const double bim = w1 * cf[CF_KXI_IM + rc];
        const double sc = -sh.w1e[u][ce] * w1;
        if (lb == cx) {
          const double w1e = sh.w1e[u][ce], w2e = -sh.w2e[u][ce];
          const double ere = w1e * cf[CF_KETA_RE + rc] + w2e * cf[CF_VEE + rc];
          const double eim = w1e * cf[CF_KETA_IM + rc];
          re = ((cf[CF_K0_RE + rc] + bre) + ere) + sc * vxe;
          im = (cf[CF_K0_IM + rc] + bim) + eim;
        } else {
          re = bre + sc * vxe;
          im = bim;
        }
      } else {  // eta-line block at (eta slot s != ce, xi slot cx)
        int s = lb - sx;
        if (s >= ce) ++s;
        const double w1 = sh.w1e[u][s], w2 = -sh.w2e[u][s];
        const double bre = w1 * cf[CF_KETA_RE + rc] + w2 * cf[CF_VEE + rc];
        const double sc = -w1 * sh.w1x[u][cx];
        re = bre + sc * vxe;
        im = w1 * cf[CF_KETA_IM + rc];
      }
      sh.line[u][lb][rc] = make_double2(re, im);
    }
    // 3. cross blocks: the six structural nonzeros of -(w1e w1x) Vxieta
    for (int x = tid; x < kSub * S; x += kWriterThreads) {
      const int u = x / S, k = x % S;
      const int s = sh.order[u][k / sx], t = k % sx;
      const double sc = -sh.w1e[u][s] * sh.w1x[u][t];
#pragma unroll
      for (int p = 0; p < 6; ++p) sh.cross[u][k][p] = sc * sh.cf[u][CF_VXE + c_vpos[p]];
    }
    __syncthreads();
    // 4. stream the rows out: L rows are contiguous for consecutive nodes
    const long long base = (long long)n0 * S * 25;
    const int total = cnt * S * 25;
    for (int x = tid; x < total; x += kWriterThreads) {
      const int u = x / (S * 25), e = x % (S * 25);
      const int k = e / 25, rc = e % 25;
      const int r = k / sx, t = k % sx;
      const int s = sh.order[u][r];
      const int cx = sh.cx[u], ce = sh.ce[u];
      double2 v;
      if (s == ce) {
        v = sh.line[u][t][rc];
      } else if (t == cx) {
        v = sh.line[u][sx + (s < ce ? s : s - 1)][rc];
      } else {
        const int vi = c_vidx[rc];
        v = make_double2(vi >= 0 ? sh.cross[u][k][vi] : 0.0, 0.0);
      }
      __stcs(L + base + x, v);
    }
    for (int x = tid; x < cnt * 25; x += kWriterThreads) {
      const int u = x / 25, rc = x % 25;
      __stcs(Mv + (long long)n0 * 25 + x, make_double2(sh.cf[u][CF_GAMMA + rc], 0.0));
    }
    __syncthreads();
  }
}

// Writer specialised on the stencil sizes (SX xi slots, SE eta slots).
// Per group of kSub nodes:
//   pass A  every line-block entry: (w1 K_re, w1 K_im)          (lane-dense)
//           every cross block: scale s = -(w1_eta w1_xi) and its 6 nonzeros
//   pass B  the 6 viscous positions of each non-centre line block:
//           re = (w1 K_re + (-w2) V) + s Vxieta                   (lane-dense)
//   pass C  the centre block from scratch: ((K0 + xi) + eta) + cross
//   store   one warp per 5x5 block: the block's line/cross/zero source is
//           decided once per warp, lanes 0..24 store 400 contiguous bytes.
// Dropping the products with structural zeros of V is exact: for finite y,
// x + 0*y equals x (up to the sign of a zero result).
template <int SX, int SE>
struct WriterSharedT {
  static constexpr int S = SX * SE, NL = SX + SE - 1;
  double cf[kSub][CF_COUNT];
  double2 line[kSub][NL][25];
  double cross[kSub][S][6];
  double scl[kSub][S];
  double w1x[kSub][SX], w2x[kSub][SX];
  double w1e[kSub][SE], w2e[kSub][SE];
  int order[kSub][SE];
  int rank[kSub][SE];  // rank[u][slot] = sorted position of eta slot
  int cx[kSub], ce[kSub];
};

template <int SX, int SE>
__global__ void __launch_bounds__(kWriterThreads)
    k_write_rows_t(int ny, int nz, DevRule xi, DevRule eta, const double *__restrict__ coef,
                   double2 *__restrict__ L, double2 *__restrict__ Mv) {
  using SH = WriterSharedT<SX, SE>;
  constexpr int S = SH::S, NL = SH::NL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SH &sh = *reinterpret_cast<SH *>(smem_raw);
  const int nn = ny * nz;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int groups = (nn + kSub - 1) / kSub;
  for (int g = blockIdx.x; g < groups; g += gridDim.x) {
    const int n0 = g * kSub;
    const int cnt = min(kSub, nn - n0);
    for (int x = tid; x < CF_COUNT * kSub; x += kWriterThreads) {
      const int f = x / kSub, u = x % kSub;
      sh.cf[u][f] = u < cnt ? coef[(size_t)f * nn + n0 + u] : 0.0;
    }
    for (int x = tid; x < kSub * (SX + SE + 1); x += kWriterThreads) {
      const int u = x / (SX + SE + 1), r = x % (SX + SE + 1);
      const int n = min(n0 + u, nn - 1);
      const int i = n % ny, j = n / ny;
      if (r < SX) {
        sh.w1x[u][r] = xi.w1[i * SX + r];
        sh.w2x[u][r] = xi.w2[i * SX + r];
      } else if (r < SX + SE) {
        const int q = r - SX;
        sh.w1e[u][q] = eta.w1[j * SE + q];
        sh.w2e[u][q] = eta.w2[j * SE + q];
        sh.order[u][q] = eta.order[j * SE + q];
        sh.rank[u][eta.order[j * SE + q]] = q;
      } else {
        sh.cx[u] = xi.centre[i];
        sh.ce[u] = eta.centre[j];
      }
    }
    __syncthreads();
    // pass A: w1 K for every line entry; cross scales and nonzeros
    for (int x = tid; x < kSub * NL * 25; x += kWriterThreads) {
      const int u = x / (NL * 25), rem = x % (NL * 25);
      const int lb = rem / 25, rc = rem % 25;
      const double *cf = sh.cf[u];
      double w1, kr, ki;
      if (lb < SX) {
        w1 = sh.w1x[u][lb];
        kr = cf[CF_KXI_RE + rc];
        ki = cf[CF_KXI_IM + rc];
      } else {
        int q = lb - SX;
        if (q >= sh.ce[u]) ++q;
        w1 = sh.w1e[u][q];
        kr = cf[CF_KETA_RE + rc];
        ki = cf[CF_KETA_IM + rc];
      }
      sh.line[u][lb][rc] = make_double2(w1 * kr, w1 * ki);
    }
    for (int x = tid; x < kSub * S; x += kWriterThreads) {
      const int u = x / S, k = x % S;
      const int q = sh.order[u][k / SX], t = k % SX;
      const double sc = -sh.w1e[u][q] * sh.w1x[u][t];
      sh.scl[u][k] = sc;
#pragma unroll
      for (int p = 0; p < 6; ++p) sh.cross[u][k][p] = sc * sh.cf[u][CF_VXE + c_vpos[p]];
    }
    __syncthreads();
    // pass B: viscous positions of the non-centre line blocks
    for (int x = tid; x < kSub * NL * 6; x += kWriterThreads) {
      const int u = x / (NL * 6), rem = x % (NL * 6);
      const int lb = rem / 6, pidx = rem % 6, rc = c_vpos[pidx];
      const int cx = sh.cx[u], ce = sh.ce[u];
      const double *cf = sh.cf[u];
      double w2, v, sc;
      if (lb < SX) {
        if (lb == cx) continue;
        w2 = -sh.w2x[u][lb];
        v = cf[CF_VXX + rc];
        sc = sh.scl[u][sh.rank[u][ce] * SX + lb];  // block (eta slot ce, xi slot lb)
      } else {
        int q = lb - SX;
        if (q >= ce) ++q;
        w2 = -sh.w2e[u][q];
        v = cf[CF_VEE + rc];
        sc = sh.scl[u][sh.rank[u][q] * SX + cx];  // block (eta slot q, xi slot cx)
      }
      double2 &e = sh.line[u][lb][rc];
      e.x = (e.x + w2 * v) + sc * cf[CF_VXE + rc];
    }
    // pass C: the centre block
    for (int x = tid; x < kSub * 25; x += kWriterThreads) {
      const int u = x / 25, rc = x % 25;
      const int cx = sh.cx[u], ce = sh.ce[u];
      const double *cf = sh.cf[u];
      const double w1x = sh.w1x[u][cx], w2x = -sh.w2x[u][cx];
      const double w1e = sh.w1e[u][ce], w2e = -sh.w2e[u][ce];
      const double sc = -w1e * w1x;
      const double bre = w1x * cf[CF_KXI_RE + rc] + w2x * cf[CF_VXX + rc];
      const double ere = w1e * cf[CF_KETA_RE + rc] + w2e * cf[CF_VEE + rc];
      const double re = ((cf[CF_K0_RE + rc] + bre) + ere) + sc * cf[CF_VXE + rc];
      const double im = (cf[CF_K0_IM + rc] + w1x * cf[CF_KXI_IM + rc]) + w1e * cf[CF_KETA_IM + rc];
      sh.line[u][cx][rc] = make_double2(re, im);
    }
    __syncthreads();
    // store: one warp per block
    for (int b = warp; b < cnt * S; b += kWriterThreads / 32) {
      const int u = b / S, k = b % S;
      const int r = k / SX, t = k % SX;
      const int q = sh.order[u][r];
      const int cx = sh.cx[u], ce = sh.ce[u];
      const int lb = q == ce ? t : (t == cx ? SX + (q < ce ? q : q - 1) : -1);
      if (lane < 25) {
        double2 v;
        if (lb >= 0) {
          v = sh.line[u][lb][lane];
        } else {
          const int vi = c_vidx[lane];
          v = make_double2(vi >= 0 ? sh.cross[u][k][vi] : 0.0, 0.0);
        }
        __stcs(L + ((long long)(n0 + u) * S + k) * 25 + lane, v);
      }
    }
    for (int u = warp; u < cnt; u += kWriterThreads / 32)
      if (lane < 25)
        __stcs(Mv + (long long)(n0 + u) * 25 + lane, make_double2(sh.cf[u][CF_GAMMA + lane], 0.0));
    __syncthreads();
  }
}

template <int SX, int SE>
int launch_writer_t(tlr_ctx *ctx) {
  const size_t smem = sizeof(WriterSharedT<SX, SE>);
  TLR_CUDA(ctx, cudaFuncSetAttribute(k_write_rows_t<SX, SE>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int sms = 0, per_sm = 0;
  TLR_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  TLR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_write_rows_t<SX, SE>,
                                                              kWriterThreads, smem));
  const int groups = (ctx->nn + kSub - 1) / kSub;
  const int grid = std::max(1, std::min(groups, sms * std::max(per_sm, 1)));
  { k_write_rows_t<SX, SE><<<grid, kWriterThreads, smem, ctx->stream>>>(
      ctx->ny, ctx->nz, ctx->xi, ctx->eta, ctx->coef, ctx->L, ctx->M); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

// Specialised writer for the common stencils; -1 when none applies.
int launch_writer(tlr_ctx *ctx) {
  if (ctx->sx == 11 && ctx->se == 7) return launch_writer_t<11, 7>(ctx);
  if (ctx->sx == 11 && ctx->se == 5) return launch_writer_t<11, 5>(ctx);
  if (ctx->sx == 5 && ctx->se == 5) return launch_writer_t<5, 5>(ctx);
  if (ctx->sx == 5 && ctx->se == 7) return launch_writer_t<5, 7>(ctx);
  return -1;
}

}  // namespace

int run_pattern(tlr_ctx *ctx) {
  const long long total = (long long)ctx->nn * ctx->S;
  const long long threads = total > ctx->nn + 1 ? total : ctx->nn + 1;
  { k_pattern<<<blocks_for(threads, 256), 256, 0, ctx->stream>>>(
      ctx->ny, ctx->nz, ctx->xi, ctx->eta, ctx->row_ptr, ctx->col); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int run_assemble(tlr_ctx *ctx, tlr_operator_diag *diag) {
  const tlr_recipe &r = ctx->recipe;
  if (ctx->sx > kMaxSx || ctx->se > kMaxSe)
    return fail(ctx, TLR_ERR_ARG, "stencil wider than the assembly kernel supports");
  CoefParams p;
  p.nn = ctx->nn;
  p.Re = r.reynolds;
  p.Pr = r.prandtl;
  p.M = r.mach;
  p.gamma = r.gamma;
  p.s = r.sutherland_constant / r.reference_temperature;
  const double ar = r.alpha_re, ai = r.alpha_im;
  // PETSC_i * alpha and alpha * alpha in the reference's complex products.
  p.ia_re = 0.0 * ar - 1.0 * ai;
  p.ia_im = 0.0 * ai + 1.0 * ar;
  p.a2_re = ar * ar - ai * ai;
  p.a2_im = ar * ai + ai * ar;
  p.alpha_finite = std::isfinite(ar) && std::isfinite(ai);
  TLR_CUDA(ctx, cudaMemsetAsync(ctx->status, 0, sizeof(int) * ST_COUNT, ctx->stream));
  { k_coefficients<<<blocks_for(ctx->nn, 32), 32, 0, ctx->stream>>>(
      p, ctx->base_c, ctx->derivs, ctx->metrics, ctx->coef, ctx->status); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  int st[ST_COUNT];
  TLR_CUDA(ctx, cudaMemcpyAsync(st, ctx->status, sizeof(st), cudaMemcpyDeviceToHost,
                                ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (st[ST_COEF])
    return fail(ctx, TLR_ERR_COEFFICIENTS,
                "At least one node produced invalid curvilinear LNS coefficients "
                "during global operator validation");
  static bool attr = false;
  const size_t smem = sizeof(WriterShared);
  if (!attr) {
    TLR_CUDA(ctx, cudaFuncSetAttribute(k_write_rows,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    attr = true;
  }
  int sms = 0, per_sm = 0;
  TLR_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  TLR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_write_rows,
                                                              kWriterThreads, smem));
  const int groups = (ctx->nn + kSub - 1) / kSub;
  const int grid = std::max(1, std::min(groups, sms * std::max(per_sm, 1)));
  TLR_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  const int wr = launch_writer(ctx);
  if (wr > 0) return wr;
  if (wr < 0) {
    { k_write_rows<<<grid, kWriterThreads, smem, ctx->stream>>>(
        ctx->ny, ctx->nz, ctx->xi, ctx->eta, ctx->coef, ctx->L, ctx->M); count_launches(); }
    TLR_CUDA(ctx, cudaGetLastError());
  }
  TLR_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (diag) {
    tlr_operator_diag d{};
    d.rows = d.columns = 5L * ctx->nn;
    d.block_size = 5;
    d.mass_used_blocks = d.mass_allocated_blocks = ctx->nn;
    d.spatial_used_blocks = d.spatial_allocated_blocks = (double)ctx->nnzb;
    cudaEventElapsedTime(&d.assemble_ms, ctx->ev0, ctx->ev1);
    int rc = frobenius(ctx, ctx->M, (long long)ctx->nn * 25, &d.mass_frobenius_norm);
    if (rc) return rc;
    rc = frobenius(ctx, ctx->L, ctx->nnzb * 25, &d.spatial_frobenius_norm);
    if (rc) return rc;
    *diag = d;
  }
  return TLR_OK;
}

// Launch only the writer (coefficients already evaluated) and return its
// device time; used by the benchmark to time the HBM-bound kernel alone.
int time_writer(tlr_ctx *ctx, float *ms) {
  const size_t smem = sizeof(WriterShared);
  int sms = 0, per_sm = 0;
  TLR_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  TLR_CUDA(ctx, cudaFuncSetAttribute(k_write_rows,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
  TLR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_write_rows,
                                                              kWriterThreads, smem));
  const int groups = (ctx->nn + kSub - 1) / kSub;
  const int grid = std::max(1, std::min(groups, sms * std::max(per_sm, 1)));
  TLR_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  { k_write_rows<<<grid, kWriterThreads, smem, ctx->stream>>>(
      ctx->ny, ctx->nz, ctx->xi, ctx->eta, ctx->coef, ctx->L, ctx->M); count_launches(); }
  TLR_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  TLR_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
  cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1);
  return TLR_OK;
}

}  // namespace tlr
