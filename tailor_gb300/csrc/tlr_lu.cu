// tlr_lu.cu -- multifrontal LU of K = A_bc - sigma B_bc and its
// triangular solves, level-batched, in FP64 (the drop-in form) or FP32
// (the mixed form, refined in FP64 by the caller).
//
// Every front is a dense column-major m x m matrix in one device pool.
// Fronts of one elimination-tree level are processed together: one launch
// assembles all their K blocks, one launch per child slot extend-adds the
// children's Schur complements, and each panel step of width w runs five
// launches over all fronts that still have pivots left:
//   k_panel        partial pivoting over the fully summed rows (one CTA/front)
//   k_swap         the step's row interchanges on the other columns
//   k_trsm_border  L21 = F21 U_kk^-1 for the front's border rows
//   k_trsm_urow    U12 = L_kk^-1 F12
//   k_gemm         trailing update F22 -= L21 U12 (the Schur complement)
// Pivot search is restricted to fully summed rows (no delayed pivots); an
// exactly zero pivot column is perturbed and counted, and the caller
// refines.  After the last level every pivot block's SW x SW diagonal
// blocks are inverted explicitly (k_tri_inv), so each solve step is a
// parallel GEMV plus one small dense product instead of a serial
// substitution; the solves walk the same levels.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "tlr_complex.cuh"
#include "tlr_internal.h"
#include "tlr_lu.h"

namespace tlr {
namespace {

constexpr int kTile = 64;


// ------------------------------------------------------------ factorization

template <class C>
__global__ void k_asm(const AsmEntry *__restrict__ e, long long n,
                      const double2 *__restrict__ A, const double2 *__restrict__ B,
                      double sr, double si, C *__restrict__ pool,
                      const DevFront *__restrict__ fr) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n * 25) return;
  const AsmEntry en = e[x / 25];
  const int rc = (int)(x % 25), r = rc / 5, c = rc % 5;
  double2 v = A[(long long)en.k * 25 + rc];
  if (en.bnode >= 0) {
    const double2 b = B[(long long)en.bnode * 25 + rc];
    v.x -= sr * b.x - si * b.y;
    v.y -= sr * b.y + si * b.x;
  }
  const DevFront f = fr[en.front];
  pool[f.off + (long long)(en.col * 5 + c) * f.m + en.row * 5 + r] = from64<C>(v);
}

template <class C>
__global__ void k_extend(const int *__restrict__ kids, const DevFront *__restrict__ fr,
                         const int *__restrict__ cmap, C *__restrict__ pool) {
  const int child = kids[blockIdx.y];
  const DevFront fc = fr[child];
  const DevFront fp = fr[fc.parent];
  const int bc = fc.m - fc.p;
  const long long total = (long long)bc * bc;
  const int *map = cmap + fc.cmap_off;
  const C *cb = pool + fc.off;
  C *pf = pool + fp.off;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const int rr = (int)(x % bc), cc = (int)(x / bc);
    const int pr = map[rr / 5] * 5 + rr % 5, pc = map[cc / 5] * 5 + cc % 5;
    const C v = cb[(long long)(fc.p + cc) * fc.m + fc.p + rr];
    C &d = pf[(long long)pc * fp.m + pr];
    d = cadd(d, v);
  }
}

// Block-wide argmax of (value, row) pairs: largest value, ties to the
// smaller row; warp shuffles, then one warp over the warp winners.  The
// result is returned to every thread.
template <class T>
__device__ __forceinline__ void block_argmax(T &best, int &bi, T *wval, int *widx) {
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T a = __shfl_down_sync(0xffffffffu, best, o);
    const int ia = __shfl_down_sync(0xffffffffu, bi, o);
    if (a > best || (a == best && ia < bi)) {
      best = a;
      bi = ia;
    }
  }
  if (lane == 0) {
    wval[wp] = best;
    widx[wp] = bi;
  }
  __syncthreads();
  if (wp == 0) {
    best = lane < nw ? wval[lane] : T(-2);
    bi = lane < nw ? widx[lane] : 0x7fffffff;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T a = __shfl_down_sync(0xffffffffu, best, o);
      const int ia = __shfl_down_sync(0xffffffffu, bi, o);
      if (a > best || (a == best && ia < bi)) {
        best = a;
        bi = ia;
      }
    }
    if (lane == 0) {
      wval[0] = best;
      widx[0] = bi;
    }
  }
  __syncthreads();
  best = wval[0];
  bi = widx[0];
  __syncthreads();  // wval/widx are reused by the next call
}

// Panel factorisation of step s for one front per CTA: columns k0..k0+ww,
// partial pivoting over the fully summed rows k0..p-1.  The panel is
// processed in sub-panels of kSB columns: pivoting, scaling and rank-1
// updates stay inside the sub-panel, then the rest of the panel is updated
// once per sub-panel (a unit-lower solve for its U rows and a rank-kSB
// update below), so each panel element crosses L2 ww/kSB times instead of
// ww times.
constexpr int kSB = 8;

template <class C>
__global__ void __launch_bounds__(512)
    k_panel(const int *__restrict__ fl, int s, int w, C *__restrict__ pool,
            const DevFront *__restrict__ fr, int *__restrict__ ipiv,
            int *__restrict__ pert, double tiny) {
  using T = typename Real<C>::T;
  __shared__ T sval[32];
  __shared__ int sidx[32];
  __shared__ C lsub[kSB][kSB];
  const DevFront f = fr[fl[blockIdx.x]];
  C *F = pool + f.off;
  const int m = f.m, p = f.p;
  const int k0 = s * w, ww = min(w, p - k0);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int jb = 0; jb < ww; jb += kSB) {
    const int nb = min(kSB, ww - jb);
    const int c0 = k0 + jb, c1 = c0 + nb;  // sub-panel columns [c0, c1)
    for (int col = c0; col < c1; ++col) {
      T best = -1;
      int bi = col;
      for (int r = col + tid; r < p; r += nt) {
        const T a = cabs1(F[(long long)col * m + r]);
        if (a > best) { best = a; bi = r; }
      }
      block_argmax(best, bi, sval, sidx);
      if (tid == 0) ipiv[f.toff + col] = bi;
      const int pr = bi;
      if (pr != col)
        for (int c = k0 + tid; c < k0 + ww; c += nt) {
          const C t = F[(long long)c * m + col];
          F[(long long)c * m + col] = F[(long long)c * m + pr];
          F[(long long)c * m + pr] = t;
        }
      __syncthreads();
      C pv = F[(long long)col * m + col];
      if (cabs1(pv) == T(0)) {
        pv = cmake<C>((T)tiny, 0);
        if (tid == 0) {
          F[(long long)col * m + col] = pv;
          atomicAdd(pert, 1);
        }
      }
      const C inv = cinv(pv);
      for (int r = col + 1 + tid; r < p; r += nt)
        F[(long long)col * m + r] = cmul(F[(long long)col * m + r], inv);
      __syncthreads();
      const int nr = p - col - 1, nc = c1 - col - 1;
      for (int x = tid; x < nr * nc; x += nt) {
        const int r = col + 1 + x % nr, c = col + 1 + x / nr;
        F[(long long)c * m + r] =
            cfms(F[(long long)c * m + r], F[(long long)col * m + r], F[(long long)c * m + col]);
      }
      __syncthreads();
    }
    if (c1 >= k0 + ww) break;
    // U rows of the sub-panel for the remaining panel columns: unit-lower solve
    for (int x = tid; x < nb * nb; x += nt) lsub[x / nb][x % nb] = F[(long long)(c0 + x % nb) * m + c0 + x / nb];
    __syncthreads();
    for (int c = c1 + tid; c < k0 + ww; c += nt) {
      C xr[kSB];
#pragma unroll
      for (int r = 0; r < kSB; ++r) {
        if (r >= nb) break;
        C v = F[(long long)c * m + c0 + r];
        for (int rp = 0; rp < r; ++rp) v = cfms(v, lsub[r][rp], xr[rp]);
        xr[r] = v;
        F[(long long)c * m + c0 + r] = v;
      }
    }
    __syncthreads();
    // rank-nb update of the rest of the panel below the sub-panel
    const int nr = p - c1, nc = k0 + ww - c1;
    for (int x = tid; x < nr * nc; x += nt) {
      const int r = c1 + x % nr, c = c1 + x / nr;
      C v = F[(long long)c * m + r];
#pragma unroll
      for (int t = 0; t < kSB; ++t)
        if (t < nb) v = cfms(v, F[(long long)(c0 + t) * m + r], F[(long long)c * m + c0 + t]);
      F[(long long)c * m + r] = v;
    }
    __syncthreads();
  }
}

// The cluster-wide pivot: the largest candidate value over the KC CTAs,
// ties to the smaller row (the order of a sequential scan over the CTAs).
// Warp 0 reads one candidate per lane from the other CTAs' shared memory
// and reduces with shuffles; the winner is broadcast through shared memory.
template <class T, int KC>
__device__ __forceinline__ int cluster_argmax(cooperative_groups::cluster_group &cluster,
                                              T *cval, int *cidx, int none, int *gsel) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    T a = -1;
    int ia = none;
    if (lane < KC) {
      a = *cluster.map_shared_rank(cval, lane);
      ia = *cluster.map_shared_rank(cidx, lane);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T a2 = __shfl_down_sync(0xffffffffu, a, o);
      const int i2 = __shfl_down_sync(0xffffffffu, ia, o);
      if (a2 > a || (a2 == a && i2 < ia)) {
        a = a2;
        ia = i2;
      }
    }
    if (lane == 0) gsel[0] = ia;
  }
  __syncthreads();
  return gsel[0];
}

// The same panel factorisation spread over a thread-block cluster of
// kPanelCluster CTAs (one cluster per front): CTA 0 owns the panel's top ww
// rows (where pivots land, and the U rows of every sub-panel), CTAs 1..7
// split the remaining fully summed rows.  Per column each CTA finds its
// local pivot candidate, the candidates are exchanged through distributed
// shared memory after a cluster barrier (every CTA picks the same winner:
// largest |a|, then the smallest row), CTA 0 swaps the rows, and after a
// second barrier every CTA scales and updates its own rows.  Pivots and
// arithmetic are those of k_panel, so the factors are identical.  Panel
// data written by other CTAs is read past L1.
constexpr int kPanelCluster = 8;
constexpr int kPanelW = 128;  // widest panel (complex64)
// dynamic shared memory of the shared-memory cluster panel (its rows x w columns)
constexpr size_t kPanelSmemMax = 200 * 1024;

template <class C>
__global__ void __cluster_dims__(kPanelCluster, 1, 1) __launch_bounds__(256)
    k_panel_cluster(const int *__restrict__ fl, int s, int w, C *__restrict__ pool,
                    const DevFront *__restrict__ fr, int *__restrict__ ipiv,
                    int *__restrict__ pert, double tiny) {
  namespace cg = cooperative_groups;
  using T = typename Real<C>::T;
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank();
  __shared__ T sval[32];
  __shared__ int sidx[32];
  __shared__ T cval;
  __shared__ int cidx;
  __shared__ int gsel[1];
  __shared__ C lsub[kSB][kSB];
  const DevFront f = fr[fl[blockIdx.x / kPanelCluster]];
  C *F = pool + f.off;
  const int m = f.m, p = f.p;
  const int k0 = s * w, ww = min(w, p - k0);
  const int tid = threadIdx.x, nt = blockDim.x;
  // rows of this CTA: CTA 0 the top rows, CTAs 1.. contiguous chunks of the rest
  const int top_end = k0 + ww;
  const int rest = p - top_end;
  const int chunk = (rest + kPanelCluster - 2) / (kPanelCluster - 1);
  const int ra = q == 0 ? k0 : min(p, top_end + (q - 1) * chunk);
  const int rb = q == 0 ? top_end : min(p, ra + chunk);
  for (int jb = 0; jb < ww; jb += kSB) {
    const int nb = min(kSB, ww - jb);
    const int c0 = k0 + jb, c1 = c0 + nb;
    for (int col = c0; col < c1; ++col) {
      // local candidate over owned rows >= col
      T best = -1;
      int bi = p;
      for (int r = max(ra, col) + tid; r < rb; r += nt) {
        const T a = cabs1(__ldcg(F + (long long)col * m + r));
        if (a > best) { best = a; bi = r; }
      }
      block_argmax(best, bi, sval, sidx);
      if (tid == 0) {
        cval = best;
        cidx = bi;
      }
      cluster.sync();
      // every CTA reads the kPanelCluster candidates and picks the same pivot
      const int gi = cluster_argmax<T, kPanelCluster>(cluster, &cval, &cidx, p, gsel);
      const int pr = gi < p ? gi : col;
      if (q == 0) {
        if (tid == 0) ipiv[f.toff + col] = pr;
        if (pr != col)
          for (int c = k0 + tid; c < k0 + ww; c += nt) {
            const C t = __ldcg(F + (long long)c * m + col);
            F[(long long)c * m + col] = __ldcg(F + (long long)c * m + pr);
            F[(long long)c * m + pr] = t;
          }
        __syncthreads();  // the pivot's own column may have been swapped by another thread
        if (tid == 0 && cabs1(__ldcg(F + (long long)col * m + col)) == T(0)) {
          F[(long long)col * m + col] = cmake<C>((T)tiny, 0);
          atomicAdd(pert, 1);
        }
      }
      __threadfence();
      cluster.sync();
      const C inv = cinv(__ldcg(F + (long long)col * m + col));
      const int r0 = max(ra, col + 1);
      for (int r = r0 + tid; r < rb; r += nt)
        F[(long long)col * m + r] = cmul(__ldcg(F + (long long)col * m + r), inv);
      __syncthreads();
      const int nr = rb - r0, nc = c1 - col - 1;
      for (int x = tid; x < nr * nc; x += nt) {
        const int r = r0 + x % nr, c = col + 1 + x / nr;
        F[(long long)c * m + r] = cfms(__ldcg(F + (long long)c * m + r),
                                       __ldcg(F + (long long)col * m + r),
                                       __ldcg(F + (long long)c * m + col));
      }
      __syncthreads();
    }
    if (c1 >= k0 + ww) break;
    // CTA 0: U rows of the sub-panel for the remaining panel columns
    if (q == 0) {
      for (int x = tid; x < nb * nb; x += nt)
        lsub[x / nb][x % nb] = __ldcg(F + (long long)(c0 + x % nb) * m + c0 + x / nb);
      __syncthreads();
      for (int c = c1 + tid; c < k0 + ww; c += nt) {
        C xr[kSB];
#pragma unroll
        for (int r = 0; r < kSB; ++r) {
          if (r >= nb) break;
          C v = __ldcg(F + (long long)c * m + c0 + r);
          for (int rp = 0; rp < r; ++rp) v = cfms(v, lsub[r][rp], xr[rp]);
          xr[r] = v;
          F[(long long)c * m + c0 + r] = v;
        }
      }
    }
    __threadfence();
    cluster.sync();
    // rank-nb update of the owned rows below the sub-panel
    const int r0 = max(ra, c1);
    const int nr = rb - r0, nc = k0 + ww - c1;
    for (int x = tid; x < nr * nc; x += nt) {
      const int r = r0 + x % nr, c = c1 + x / nr;
      C v = __ldcg(F + (long long)c * m + r);
#pragma unroll
      for (int t = 0; t < kSB; ++t)
        if (t < nb)
          v = cfms(v, __ldcg(F + (long long)(c0 + t) * m + r),
                   __ldcg(F + (long long)c * m + c0 + t));
      F[(long long)c * m + r] = v;
    }
    __syncthreads();
  }
  cluster.sync();  // no CTA leaves while others may still read its candidates
}

// The cluster panel with the panel held in distributed shared memory: each
// CTA loads its rows of the ww panel columns once (column-major, leading
// dimension ldp), factors them in shared memory and writes them back at the
// end, so a column step costs two cluster barriers and a few shared-memory
// passes instead of several round trips through L2.  CTA 0 owns the top ww
// rows (pivot rows land there and the sub-panels' U rows live there);
// CTAs 1.. own contiguous chunks of the rest.  The pivot row swap is done
// by CTA 0 alone (its own row and the remote row through DSMEM); the other
// CTAs read the pivot and the sub-panel's U entries from CTA 0.  Pivots,
// tie-breaking and every arithmetic operation are those of k_panel.
template <class C>
__global__ void __cluster_dims__(kPanelCluster, 1, 1) __launch_bounds__(256)
    k_panel_cluster_sm(const int *__restrict__ fl, int s, int w, C *__restrict__ pool,
                       const DevFront *__restrict__ fr, int *__restrict__ ipiv,
                       int *__restrict__ pert, double tiny, int ldp) {
  namespace cg = cooperative_groups;
  using T = typename Real<C>::T;
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *P = reinterpret_cast<C *>(smem_raw);  // P[(c - k0) * ldp + (r - ra)]
  __shared__ T sval[32];
  __shared__ int sidx[32];
  __shared__ T cval;
  __shared__ int cidx;
  __shared__ int gsel[1];
  __shared__ C lsub[kSB][kSB];
  __shared__ C urow[kSB];               // pivot row entries of the sub-panel
  __shared__ C ublk[kSB][kPanelW];      // sub-panel U rows for the rank-nb update
  __shared__ C piv;
  const DevFront f = fr[fl[blockIdx.x / kPanelCluster]];
  C *F = pool + f.off;
  const int m = f.m, p = f.p;
  const int k0 = s * w, ww = min(w, p - k0);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int top_end = k0 + ww;
  const int rest = p - top_end;
  const int chunk = (rest + kPanelCluster - 2) / (kPanelCluster - 1);
  const int ra = q == 0 ? k0 : min(p, top_end + (q - 1) * chunk);
  const int rb = q == 0 ? top_end : min(p, ra + chunk);
  const int nown = rb - ra;
  C *P0 = cluster.map_shared_rank(P, 0);  // CTA 0's panel rows
  // load the owned rows of the panel
  for (int x = tid; x < nown * ww; x += nt) {
    const int rr = x % nown, cc = x / nown;
    P[cc * ldp + rr] = F[(long long)(k0 + cc) * m + ra + rr];
  }
  __syncthreads();
  for (int jb = 0; jb < ww; jb += kSB) {
    const int nb = min(kSB, ww - jb);
    const int c0 = k0 + jb, c1 = c0 + nb;
    for (int col = c0; col < c1; ++col) {
      const int cc = col - k0;
      T best = -1;
      int bi = p;
      for (int r = max(ra, col) + tid; r < rb; r += nt) {
        const T a = cabs1(P[cc * ldp + r - ra]);
        if (a > best) { best = a; bi = r; }
      }
      block_argmax(best, bi, sval, sidx);
      if (tid == 0) {
        cval = best;
        cidx = bi;
      }
      cluster.sync();
      const int gi = cluster_argmax<T, kPanelCluster>(cluster, &cval, &cidx, p, gsel);
      const int pr = gi < p ? gi : col;
      if (q == 0) {
        if (tid == 0) ipiv[f.toff + col] = pr;
        if (pr != col) {
          // owner of row pr and its local row (CTA 0 owns [k0, top_end))
          const int qo = pr < top_end ? 0 : 1 + (pr - top_end) / chunk;
          const int ro = pr - (qo == 0 ? k0 : top_end + (qo - 1) * chunk);
          C *Po = cluster.map_shared_rank(P, qo);
          for (int c = tid; c < ww; c += nt) {
            const C t = P[c * ldp + col - k0];
            P[c * ldp + col - k0] = Po[c * ldp + ro];
            Po[c * ldp + ro] = t;
          }
        }
        __syncthreads();  // the pivot's own column may have been swapped by another thread
        if (tid == 0 && cabs1(P[cc * ldp + col - k0]) == T(0)) {
          P[cc * ldp + col - k0] = cmake<C>((T)tiny, 0);
          atomicAdd(pert, 1);
        }
      }
      cluster.sync();
      if (tid == 0) piv = P0[cc * ldp + col - k0];
      if (tid < c1 - col - 1) urow[tid] = P0[(cc + 1 + tid) * ldp + col - k0];
      __syncthreads();
      const C inv = cinv(piv);
      const int r0 = max(ra, col + 1);
      for (int r = r0 + tid; r < rb; r += nt)
        P[cc * ldp + r - ra] = cmul(P[cc * ldp + r - ra], inv);
      __syncthreads();
      const int nr = rb - r0, nc = c1 - col - 1;
      for (int x = tid; x < nr * nc; x += nt) {
        const int r = r0 + x % nr, c = col + 1 + x / nr;
        P[(c - k0) * ldp + r - ra] =
            cfms(P[(c - k0) * ldp + r - ra], P[cc * ldp + r - ra], urow[c - col - 1]);
      }
      __syncthreads();
    }
    if (c1 >= k0 + ww) break;
    if (q == 0) {
      for (int x = tid; x < nb * nb; x += nt)
        lsub[x / nb][x % nb] = P[(c0 - k0 + x % nb) * ldp + c0 - k0 + x / nb];
      __syncthreads();
      for (int c = c1 + tid; c < k0 + ww; c += nt) {
        C xr[kSB];
#pragma unroll
        for (int r = 0; r < kSB; ++r) {
          if (r >= nb) break;
          C v = P[(c - k0) * ldp + c0 - k0 + r];
          for (int rp = 0; rp < r; ++rp) v = cfms(v, lsub[r][rp], xr[rp]);
          xr[r] = v;
          P[(c - k0) * ldp + c0 - k0 + r] = v;
        }
      }
    }
    cluster.sync();
    // the sub-panel's U rows (CTA 0) for the rank-nb update of the owned rows
    const int ncr = k0 + ww - c1;
    for (int x = tid; x < nb * ncr; x += nt) {
      const int t = x / ncr, c = c1 + x % ncr;
      ublk[t][c - c1] = P0[(c - k0) * ldp + c0 - k0 + t];
    }
    __syncthreads();
    const int r0 = max(ra, c1);
    const int nr = rb - r0;
    for (int x = tid; x < nr * ncr; x += nt) {
      const int r = r0 + x % nr, c = c1 + x / nr;
      C v = P[(c - k0) * ldp + r - ra];
#pragma unroll
      for (int t = 0; t < kSB; ++t)
        if (t < nb) v = cfms(v, P[(c0 - k0 + t) * ldp + r - ra], ublk[t][c - c1]);
      P[(c - k0) * ldp + r - ra] = v;
    }
    __syncthreads();
  }
  cluster.sync();  // every remote read and swap is done
  for (int x = tid; x < nown * ww; x += nt) {
    const int rr = x % nown, cc = x / nown;
    F[(long long)(k0 + cc) * m + ra + rr] = P[cc * ldp + rr];
  }
}

template <class C>
__global__ void k_swap(const int *__restrict__ fl, int s, int w, C *__restrict__ pool,
                       const DevFront *__restrict__ fr, const int *__restrict__ ipiv) {
  const DevFront f = fr[fl[blockIdx.y]];
  const int k0 = s * w, ww = min(w, f.p - k0);
  const int c0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (c0 >= f.m - ww) return;
  const int c = c0 < k0 ? c0 : c0 + ww;
  C *col = pool + f.off + (long long)c * f.m;
  for (int j = 0; j < ww; ++j) {
    const int r1 = k0 + j, r2 = ipiv[f.toff + k0 + j];
    if (r2 != r1) {
      const C t = col[r1];
      col[r1] = col[r2];
      col[r2] = t;
    }
  }
}

// L21 = F21 U_kk^-1 on the border rows p..m-1 of the panel columns.  CTA =
// 32 border rows x all ww columns staged in shared memory; column-oriented
// substitution with all 256 threads: x_c = t_c / U_cc, then t_c' -= x_c U_cc'
// for every later column c' (one barrier per step).
template <class C>
__global__ void __launch_bounds__(256)
    k_trsm_border(const int *__restrict__ fl, int s, int w, C *__restrict__ pool,
                  const DevFront *__restrict__ fr) {
  extern __shared__ __align__(16) unsigned char sm[];
  C *U = reinterpret_cast<C *>(sm);  // ww x ww, column-major U[c * w + r]
  C *T = U + w * w;                  // [ww][33]: T[c * 33 + rr]
  const DevFront f = fr[fl[blockIdx.y]];
  const int k0 = s * w, ww = min(w, f.p - k0);
  const int m = f.m;
  const int r0 = f.p + blockIdx.x * 32;
  if (r0 >= m) return;
  const int nr = min(32, m - r0);
  C *F = pool + f.off;
  for (int x = threadIdx.x; x < ww * ww; x += blockDim.x) {
    const int r = x % ww, c = x / ww;
    U[c * w + r] = F[(long long)(k0 + c) * m + k0 + r];
  }
  for (int x = threadIdx.x; x < ww * 32; x += blockDim.x) {
    const int rr = x & 31, c = x >> 5;
    T[c * 33 + rr] = rr < nr ? F[(long long)(k0 + c) * m + r0 + rr] : czero<C>();
  }
  __syncthreads();
  for (int c = 0; c < ww; ++c) {
    if (threadIdx.x < 32) T[c * 33 + threadIdx.x] = cmul(T[c * 33 + threadIdx.x], cinv(U[c * w + c]));
    __syncthreads();
    for (int x = threadIdx.x; x < (ww - 1 - c) * 32; x += blockDim.x) {
      const int cp = c + 1 + (x >> 5), rr = x & 31;
      T[cp * 33 + rr] = cfms(T[cp * 33 + rr], T[c * 33 + rr], U[cp * w + c]);
    }
    __syncthreads();
  }
  for (int x = threadIdx.x; x < ww * 32; x += blockDim.x) {
    const int rr = x & 31, c = x >> 5;
    if (rr < nr) F[(long long)(k0 + c) * m + r0 + rr] = T[c * 33 + rr];
  }
}

// U12 = L_kk^-1 F12 for columns k0+ww..m-1 (unit lower L_kk).  CTA = 32
// columns x all ww rows staged in shared memory; column-oriented forward
// substitution with all 256 threads: row q final, then t_r -= L_rq t_q for
// r > q (one barrier per step).
template <class C>
__global__ void __launch_bounds__(256)
    k_trsm_urow(const int *__restrict__ fl, int s, int w, C *__restrict__ pool,
                const DevFront *__restrict__ fr) {
  extern __shared__ __align__(16) unsigned char sm[];
  C *Lk = reinterpret_cast<C *>(sm);  // ww x ww, column-major Lk[c * w + r]
  C *T = Lk + w * w;                  // [ww][33]: T[q * 33 + cc]
  const DevFront f = fr[fl[blockIdx.y]];
  const int k0 = s * w, ww = min(w, f.p - k0);
  const int m = f.m;
  const int c0 = k0 + ww + blockIdx.x * 32;
  if (c0 >= m) return;
  const int nc = min(32, m - c0);
  C *F = pool + f.off;
  for (int x = threadIdx.x; x < ww * ww; x += blockDim.x) {
    const int r = x % ww, c = x / ww;
    Lk[c * w + r] = F[(long long)(k0 + c) * m + k0 + r];
  }
  for (int x = threadIdx.x; x < ww * 32; x += blockDim.x) {
    const int q = x % ww, cc = x / ww;
    T[q * 33 + cc] = cc < nc ? F[(long long)(c0 + cc) * m + k0 + q] : czero<C>();
  }
  __syncthreads();
  for (int q = 0; q + 1 < ww; ++q) {
    for (int x = threadIdx.x; x < (ww - 1 - q) * 32; x += blockDim.x) {
      const int r = q + 1 + (x >> 5), cc = x & 31;
      T[r * 33 + cc] = cfms(T[r * 33 + cc], Lk[q * w + r], T[q * 33 + cc]);
    }
    __syncthreads();
  }
  for (int x = threadIdx.x; x < ww * 32; x += blockDim.x) {
    const int q = x % ww, cc = x / ww;
    if (cc < nc) F[(long long)(c0 + cc) * m + k0 + q] = T[q * 33 + cc];
  }
}

// Trailing update F[k0+ww:m, k0+ww:m] -= F[k0+ww:m, k0:k0+ww] F[k0:k0+ww, k0+ww:m]
// over a flat list of 64x64 tiles of all participating fronts.
template <class C>
__global__ void __launch_bounds__(256)
    k_gemm(const int *__restrict__ fl, const int *__restrict__ prefix, int nf, int s,
           int w, C *__restrict__ pool, const DevFront *__restrict__ fr) {
  constexpr int KC = 16;
  __shared__ C As[KC][kTile];
  __shared__ C Bs[KC][kTile + 1];
  const int t = blockIdx.x;
  int lo = 0, hi = nf;  // find the front owning tile t
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  const DevFront f = fr[fl[lo]];
  const int m = f.m, k0 = s * w, ww = min(w, f.p - k0);
  const int base = k0 + ww, ext = m - base;
  const int nt = (ext + kTile - 1) / kTile;
  const int lt = t - prefix[lo];
  const int R0 = base + (lt % nt) * kTile, C0 = base + (lt / nt) * kTile;
  C *F = pool + f.off;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  C acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = czero<C>();
  for (int kk = 0; kk < ww; kk += KC) {
    for (int x = threadIdx.x; x < KC * kTile; x += 256) {
      const int r = x % kTile, k = x / kTile;
      const int gr = R0 + r, gk = k0 + kk + k;
      As[k][r] = (gr < m && kk + k < ww) ? F[(long long)gk * m + gr] : czero<C>();
      const int cc = x / KC, kb = x % KC;
      const int gc = C0 + cc;
      Bs[kb][cc] = (gc < m && kk + kb < ww) ? F[(long long)gc * m + k0 + kk + kb] : czero<C>();
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < KC; ++k) {
      C a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cfma(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gc = C0 + ty + 16 * j;
    if (gc >= m) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int gr = R0 + tx + 16 * i;
      if (gr >= m) continue;
      C &d = F[(long long)gc * m + gr];
      d = csub(d, acc[i][j]);
    }
  }
}

// FP64 trailing update on the FP64 tensor cores (DMMA: mma.sync m8n8k4
// f64; tcgen05 has no FP64 kind).  Same 64x64 complex tiles and tile list as
// k_gemm.  The panel's K columns are staged KC at a time as separate real
// and imaginary planes in shared memory (rows padded to 68 doubles: the
// fragment loads of a half-warp hit 16 distinct banks); warp (wr, wc) owns
// rows 16 wr .. +15 and columns 32 wc .. +31 of the tile, i.e. 2 x 4 real
// 8x8 accumulator tiles for each of Re and Im.  A complex product is four
// real products: Cr += Ar Br - Ai Bi, Ci += Ar Bi + Ai Br.
__device__ __forceinline__ void dmma(double &d0, double &d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(256)
    k_gemm_dmma(const int *__restrict__ fl, const int *__restrict__ prefix, int nf, int s, int w,
                double2 *__restrict__ pool, const DevFront *__restrict__ fr) {
  constexpr int KC = 16, LD = kTile + 4;
  __shared__ double Ar[KC][LD], Ai[KC][LD], Br[KC][LD], Bi[KC][LD];
  const int t = blockIdx.x;
  int lo = 0, hi = nf;  // find the front owning tile t
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  const DevFront f = fr[fl[lo]];
  const int m = f.m, k0 = s * w, ww = min(w, f.p - k0);
  const int base = k0 + ww, ext = m - base;
  const int nt = (ext + kTile - 1) / kTile;
  const int lt = t - prefix[lo];
  const int R0 = base + (lt % nt) * kTile, C0 = base + (lt / nt) * kTile;
  double2 *F = pool + f.off;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wr = warp & 3, wc = warp >> 2;
  const int g = lane >> 2, q = lane & 3;  // fragment row / column group, k index
  double cr[2][4][2], ci[2][4][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) cr[i][j][0] = cr[i][j][1] = ci[i][j][0] = ci[i][j][1] = 0.0;
  for (int kk = 0; kk < ww; kk += KC) {
    for (int x = threadIdx.x; x < KC * kTile; x += 256) {
      const int r = x % kTile, k = x / kTile;
      const int gr = R0 + r;
      const double2 a = (gr < m && kk + k < ww) ? F[(long long)(k0 + kk + k) * m + gr]
                                                : make_double2(0.0, 0.0);
      Ar[k][r] = a.x;
      Ai[k][r] = a.y;
      const int cc = x / KC, kb = x % KC;
      const int gc = C0 + cc;
      const double2 b = (gc < m && kk + kb < ww) ? F[(long long)gc * m + k0 + kk + kb]
                                                 : make_double2(0.0, 0.0);
      Br[kb][cc] = b.x;
      Bi[kb][cc] = b.y;
    }
    __syncthreads();
#pragma unroll
    for (int k4 = 0; k4 < KC; k4 += 4) {
      double ar[2], ai[2], br[4], bi[4];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        ar[i] = Ar[k4 + q][16 * wr + 8 * i + g];
        ai[i] = Ai[k4 + q][16 * wr + 8 * i + g];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        br[j] = Br[k4 + q][32 * wc + 8 * j + g];
        bi[j] = Bi[k4 + q][32 * wc + 8 * j + g];
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          dmma(cr[i][j][0], cr[i][j][1], ar[i], br[j]);
          dmma(cr[i][j][0], cr[i][j][1], -ai[i], bi[j]);
          dmma(ci[i][j][0], ci[i][j][1], ar[i], bi[j]);
          dmma(ci[i][j][0], ci[i][j][1], ai[i], br[j]);
        }
    }
    __syncthreads();
  }
  // accumulator element (g, 2 q + e) of the 8x8 tile (i, j)
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int gr = R0 + 16 * wr + 8 * i + g;
    if (gr >= m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int gc = C0 + 32 * wc + 8 * j + 2 * q + e;
        if (gc < m) {
          double2 &d = F[(long long)gc * m + gr];
          d.x -= cr[i][j][e];
          d.y -= ci[i][j][e];
        }
      }
  }
}

// FP32 trailing update: 128x64 tiles, 256 threads, 8x4 complex register
// tile per thread (rows tx + 16 i, columns ty + 16 j), K staged 16 at a time
// through double-buffered shared memory.  Per k step a thread issues 12
// 8-byte shared loads for 32 complex FMAs (128 FFMA), so the FFMA pipe, not
// shared memory, is the limit.
constexpr int kTM32 = 128, kTN32 = 64;

__global__ void __launch_bounds__(256)
    k_gemm32(const int *__restrict__ fl, const int *__restrict__ prefix, int nf, int s,
             int w, float2 *__restrict__ pool, const DevFront *__restrict__ fr) {
  constexpr int KC = 8;
  __shared__ float2 As[2][KC][kTM32];
  __shared__ float2 Bs[2][KC][kTN32 + 1];
  const int t = blockIdx.x;
  int lo = 0, hi = nf;
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  const DevFront f = fr[fl[lo]];
  const int m = f.m, k0 = s * w, ww = min(w, f.p - k0);
  const int base = k0 + ww, ext = m - base;
  const int ntm = (ext + kTM32 - 1) / kTM32;
  const int lt = t - prefix[lo];
  const int R0 = base + (lt % ntm) * kTM32, C0 = base + (lt / ntm) * kTN32;
  float2 *F = pool + f.off;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float2 acc[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);
  auto load = [&](int buf, int kk) {
    for (int x = threadIdx.x; x < KC * kTM32; x += 256) {
      const int r = x % kTM32, k = x / kTM32;
      const int gr = R0 + r;
      As[buf][k][r] = (gr < m && kk + k < ww) ? F[(long long)(k0 + kk + k) * m + gr]
                                              : make_float2(0.f, 0.f);
    }
    for (int x = threadIdx.x; x < KC * kTN32; x += 256) {
      const int cc = x / KC, kb = x % KC;
      const int gc = C0 + cc;
      Bs[buf][kb][cc] = (gc < m && kk + kb < ww) ? F[(long long)gc * m + k0 + kk + kb]
                                                 : make_float2(0.f, 0.f);
    }
  };
  int buf = 0;
  load(0, 0);
  __syncthreads();
  for (int kk = 0; kk < ww; kk += KC) {
    if (kk + KC < ww) load(buf ^ 1, kk + KC);
#pragma unroll
    for (int k = 0; k < KC; ++k) {
      float2 a[8], b[4];
#pragma unroll
      for (int i = 0; i < 8; ++i) a[i] = As[buf][k][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[buf][k][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc[i][j].x = fmaf(a[i].x, b[j].x, acc[i][j].x);
          acc[i][j].x = fmaf(-a[i].y, b[j].y, acc[i][j].x);
          acc[i][j].y = fmaf(a[i].x, b[j].y, acc[i][j].y);
          acc[i][j].y = fmaf(a[i].y, b[j].x, acc[i][j].y);
        }
    }
    __syncthreads();
    buf ^= 1;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gc = C0 + ty + 16 * j;
    if (gc >= m) continue;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int gr = R0 + tx + 16 * i;
      if (gr >= m) continue;
      float2 &d = F[(long long)gc * m + gr];
      d.x -= acc[i][j].x;
      d.y -= acc[i][j].y;
    }
  }
}

// ------------------------------------------------------------------ solves

// Programmatic dependent launch: a solve kernel lets the next one launch
// right away (launch_dependents) and waits for its predecessor's results
// only where it reads them (wait); loads of factor data go out before the
// wait.  Both are no-ops for a kernel launched without the attribute.
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Forward gather of one level: t[i] = b[unknown of front row perm[i]] for
// pivot rows (0 for border rows), plus the children's updated border rows
// that map to row i (cinv: absolute work index per child slot, -1: none),
// added in child-slot order.
template <class C>
__global__ void k_sgather(const int *__restrict__ fl, const DevFront *__restrict__ fr,
                          const int *__restrict__ nodes, const int *__restrict__ perm,
                          const int2 *__restrict__ cinv, const C *__restrict__ b,
                          C *__restrict__ work) {
  pdl_launch_dependents();
  pdl_wait();
  const DevFront f = fr[fl[blockIdx.y]];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.m) return;
  C v = czero<C>();
  if (i < f.p) {
    const int q = perm[f.toff + i];
    v = b[(long long)nodes[f.node_off + q / 5] * 5 + q % 5];
  }
  const int2 c = cinv[f.toff + i];
  if (c.x >= 0) v = cadd(v, work[c.x]);
  if (c.y >= 0) v = cadd(v, work[c.y]);
  work[f.toff + i] = v;
}

// ---- block-scaled triangular solves ---------------------------------------
// After factorisation each front's pivot block is cut into diagonal blocks
// of SW rows (SW = 128 or 256).  With Dl = blockdiag(L_bb) and Du = blockdiag(U_bb), the
// factors are rewritten in place as L' = L Dl^-1 (every block column right-
// multiplied by inv(L_bb), border rows included) and U' = Du^-1 U (every
// block row left-multiplied by inv(U_bb), border columns included), and
// D_b = inv(U_bb) inv(L_bb) is stored.  L' and U' have identity diagonal
// blocks, so
//   forward:  z_b = t_b, then t_r -= L'(r, b) z_b for the rows below;
//   backward: t = D z - U'12 x_border, then for b from the last block
//             x_b = t_b and t_r -= U'(r, b) x_b for the rows above.
// Every solve step is one fully parallel launch (rows split over CTAs, no
// reductions across CTAs, no serial part); only the border product of the
// backward pass reduces across column chunks.

// inverses of diagonal block fb.y of front fb.x: blockIdx.y = 0 gives
// inv(L_bb) (unit lower), 1 gives inv(U_bb).  Thread r owns row r of the
// inverse for a chunk of kIC columns in registers; step q publishes the
// final row q through shared memory and the other rows take its multiple
// (column-oriented substitution).  Stored column-major, leading dim nb.
constexpr int kIC = 32;

template <class C, int SW>
__global__ void __launch_bounds__(SW)
    k_tri_inv(const int2 *__restrict__ blocks, const C *__restrict__ pool,
              const DevFront *__restrict__ fr, const long long *__restrict__ inv_off,
              C *__restrict__ Linv, C *__restrict__ Uinv) {
  __shared__ C rowq[kIC];
  const int2 fb = blocks[blockIdx.x];
  const DevFront f = fr[fb.x];
  const int b0 = fb.y * SW, nb = min(SW, f.p - b0);
  const C *F = pool + f.off + (long long)b0 * f.m + b0;  // F[c * m + r] = K_bb(r, c)
  const int m = f.m, r = threadIdx.x;
  const bool lower = blockIdx.y == 0;
  C *out = (lower ? Linv : Uinv) + inv_off[fb.x] + (long long)fb.y * SW * SW;
  for (int c0 = 0; c0 < nb; c0 += kIC) {
    C x[kIC];
#pragma unroll
    for (int j = 0; j < kIC; ++j) x[j] = r == c0 + j ? cmake<C>(1, 0) : czero<C>();
    if (lower) {
      for (int q = c0; q < nb; ++q) {
        if (r == q)
#pragma unroll
          for (int j = 0; j < kIC; ++j) rowq[j] = x[j];
        __syncthreads();
        if (r > q && r < nb) {
          const C l = F[(long long)q * m + r];
#pragma unroll
          for (int j = 0; j < kIC; ++j) x[j] = cfms(x[j], l, rowq[j]);
        }
        __syncthreads();
      }
    } else {
      for (int q = min(nb - 1, c0 + kIC - 1); q >= 0; --q) {
        if (r == q) {
          const C d = cinv(F[(long long)q * m + q]);
#pragma unroll
          for (int j = 0; j < kIC; ++j) {
            x[j] = cmul(x[j], d);
            rowq[j] = x[j];
          }
        }
        __syncthreads();
        if (r < q) {
          const C u = F[(long long)q * m + r];
#pragma unroll
          for (int j = 0; j < kIC; ++j) x[j] = cfms(x[j], u, rowq[j]);
        }
        __syncthreads();
      }
    }
    if (r < nb)
#pragma unroll
      for (int j = 0; j < kIC; ++j)
        if (c0 + j < nb) out[(long long)(c0 + j) * nb + r] = x[j];
  }
}

// L'(rows, c) = L(rows, c) inv(L_cc) in place: CTA = 32 rows of block
// column c (all nb columns, staged in shared memory before any write);
// thread (row, g) forms columns g, g+8, ... of its row.
// tiles: {front, block c, first row, -}.
constexpr int kRT = 32;

template <class C, int SW>
__global__ void __launch_bounds__(256)
    k_scale_l(const int4 *__restrict__ tiles, C *__restrict__ pool,
              const DevFront *__restrict__ fr, const long long *__restrict__ inv_off,
              const C *__restrict__ Linv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *As = reinterpret_cast<C *>(smem_raw);  // [SW][kRT], As[q * kRT + r]
  const int4 tl = tiles[blockIdx.x];
  const DevFront f = fr[tl.x];
  const int c0 = tl.y * SW, nb = min(SW, f.p - c0);
  const int r0 = tl.z, nr = min(kRT, f.m - r0);
  C *F = pool + f.off;
  for (int x = threadIdx.x; x < nb * kRT; x += blockDim.x) {
    const int q = x / kRT, r = x % kRT;
    As[x] = r < nr ? F[(long long)(c0 + q) * f.m + r0 + r] : czero<C>();
  }
  __syncthreads();
  const C *Li = Linv + inv_off[tl.x] + (long long)tl.y * SW * SW;  // (q, j) at j nb + q
  const int r = threadIdx.x & (kRT - 1), g = threadIdx.x / kRT;
  C acc[SW / 8];
#pragma unroll
  for (int k = 0; k < SW / 8; ++k) acc[k] = czero<C>();
  for (int q = 0; q < nb; ++q) {
    const C a = As[q * kRT + r];
#pragma unroll
    for (int k = 0; k < SW / 8; ++k) {
      const int j = g + 8 * k;
      if (j <= q) acc[k] = cfma(acc[k], a, Li[(long long)j * nb + q]);
    }
  }
  if (r < nr)
#pragma unroll
    for (int k = 0; k < SW / 8; ++k) {
      const int j = g + 8 * k;
      if (j < nb) F[(long long)(c0 + j) * f.m + r0 + r] = acc[k];
    }
}

// Left product by inv(U_bb), in place over a tile of 32 columns (staged in
// shared memory before any write); max(SW, 256) threads, thread (row i,
// group h of the 256 / SW groups when SW < 256) forms columns h, h + H, ...
// of row i.  tiles: {front, block b, first column, kind}:
//   kind 0: U'(b rows, cols) = inv(U_bb) U(b rows, cols) inside the front;
//   kind 1: D_b(:, cols) = inv(U_bb) inv(L_bb)(:, cols) into dmat.
template <class C, int SW>
__global__ void __launch_bounds__(SW > 256 ? SW : 256)
    k_scale_u(const int4 *__restrict__ tiles, C *__restrict__ pool,
              const DevFront *__restrict__ fr, const long long *__restrict__ inv_off,
              const C *__restrict__ Linv, const C *__restrict__ Uinv, C *__restrict__ dmat) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *As = reinterpret_cast<C *>(smem_raw);  // [SW][kRT], As[q * kRT + cc]
  const int4 tl = tiles[blockIdx.x];
  const DevFront f = fr[tl.x];
  const int b0 = tl.y * SW, nb = min(SW, f.p - b0);
  const long long io = inv_off[tl.x] + (long long)tl.y * SW * SW;
  const C *src;
  C *dst;
  long long ld, ncol;
  if (tl.w == 0) {
    dst = pool + f.off + b0;
    src = dst;
    ld = f.m;
    ncol = f.m;
  } else {
    src = Linv + io;
    dst = dmat + io;
    ld = nb;
    ncol = nb;
  }
  const int col0 = tl.z, nc = (int)min((long long)kRT, ncol - col0);
  for (int x = threadIdx.x; x < nb * kRT; x += blockDim.x) {
    const int cc = x / nb, q = x % nb;
    As[q * kRT + cc] = cc < nc ? src[(long long)(col0 + cc) * ld + q] : czero<C>();
  }
  __syncthreads();
  const C *Ui = Uinv + io;  // (i, q) at q nb + i, upper triangular
  constexpr int H = SW >= 256 ? 1 : 256 / SW;  // column groups (max(SW, 256) threads)
  const int i = threadIdx.x % SW, h = threadIdx.x / SW;
  C acc[kRT / H];
#pragma unroll
  for (int k = 0; k < kRT / H; ++k) acc[k] = czero<C>();
  if (i < nb) {
    for (int q = i & ~31; q < nb; ++q) {
      const C u = q >= i ? Ui[(long long)q * nb + i] : czero<C>();
#pragma unroll
      for (int k = 0; k < kRT / H; ++k) acc[k] = cfma(acc[k], u, As[q * kRT + h + H * k]);
    }
#pragma unroll
    for (int k = 0; k < kRT / H; ++k) {
      const int cc = h + H * k;
      if (cc < nc) dst[(long long)(col0 + cc) * ld + i] = acc[k];
    }
  }
}

// sum over k < min(kQ, nv) of fv[k] v[k], in k order (v in shared memory,
// 16-byte aligned; complex64 pairs are read 16 bytes at a time when all
// kQ columns exist)
template <class C, int kQ>
__device__ __forceinline__ C dot_cols(const C (&fv)[kQ], const C *v, bool full, int nv) {
  C acc = czero<C>();
  if (full) {
    if constexpr (sizeof(C) == sizeof(float2) && kQ % 2 == 0) {
      const float4 *v4 = reinterpret_cast<const float4 *>(v);
#pragma unroll
      for (int k = 0; k < kQ; k += 2) {
        const float4 pv = v4[k / 2];
        acc = cfma(acc, fv[k], make_float2(pv.x, pv.y));
        acc = cfma(acc, fv[k + 1], make_float2(pv.z, pv.w));
      }
    } else {
#pragma unroll
      for (int k = 0; k < kQ; ++k) acc = cfma(acc, fv[k], v[k]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < kQ; ++k)
      if (k < nv) acc = cfma(acc, fv[k], v[k]);
  }
  return acc;
}

// One solve step of every front of the level that owns block b: rows
// [lo, hi) take t[r] -= F(r, b0:b1) t[b0:b1] (forward: lo = b1, hi = m;
// backward: lo = 0, hi = b0).  CTA = 32 rows x 8 warps of SW/8 columns.
// Backward steps run on the pivot-row vector of the backward pass; rows of
// block b-1 are final after step b and are written to the solution x.
template <class C, int SW>
__global__ void __launch_bounds__(256, (SW <= 256 && sizeof(C) == 8) ? 3 : 1)
    k_blk_update(const int *__restrict__ fl, int b, int backward, const C *__restrict__ pool,
                 const DevFront *__restrict__ fr, C *__restrict__ work,
                 const int *__restrict__ nodes, C *__restrict__ x) {
  __shared__ __align__(16) C vs[SW];
  __shared__ C red[8][32];
  pdl_launch_dependents();
  const DevFront f = fr[fl[blockIdx.y]];
  const int b0 = b * SW, b1 = min(f.p, b0 + SW), nb = b1 - b0;
  const int lo = backward ? 0 : b1, hi = backward ? b0 : f.m;
  const int r0 = lo + blockIdx.x * 32;
  if (nb <= 0 || r0 >= hi) return;
  C *t = work + f.toff;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int r = r0 + lane;
  const C *F = pool + f.off + (long long)b0 * f.m;
  // the matrix loads go out before the vector is staged (independent)
  constexpr int kQ = SW / 8;
  const int q0 = wp * kQ;
  const bool full = q0 + kQ <= nb;  // every column of this warp exists
  C fv[kQ];
  if (full && r < hi) {  // unpredicated stream down the warp's columns
    const C *Fp = F + (long long)q0 * f.m + r;
#pragma unroll
    for (int k = 0; k < kQ; ++k, Fp += f.m) fv[k] = *Fp;
  } else {
#pragma unroll
    for (int k = 0; k < kQ; ++k)
      fv[k] = (r < hi && q0 + k < nb) ? F[(long long)(q0 + k) * f.m + r] : czero<C>();
  }
  pdl_wait();
  // complex64: the row's own value goes out with the vector loads (only
  // this CTA writes row r in this step, and no row of block b); the
  // complex128 kernel keeps its registers for three CTAs per SM
  C v = czero<C>();
  if constexpr (sizeof(C) == sizeof(float2))
    if (wp == 0 && r < hi) v = t[r];
  for (int q = threadIdx.x; q < nb; q += blockDim.x) vs[q] = t[b0 + q];
  __syncthreads();
  const C acc = dot_cols<C, kQ>(fv, vs + q0, full, nb - q0);
  red[wp][lane] = acc;
  __syncthreads();
  if (wp == 0 && r < hi) {
    if constexpr (sizeof(C) != sizeof(float2)) v = t[r];
#pragma unroll
    for (int k = 0; k < 8; ++k) v = csub(v, red[k][lane]);
    t[r] = v;
    if (backward && r >= b0 - SW) x[(long long)nodes[f.node_off + r / 5] * 5 + r % 5] = v;
  }
}

// ---- dependency-driven level solve ---------------------------------------
// A level whose fronts have several diagonal blocks needs, step by step,
// one launch per block, and the top of the elimination tree is a chain of
// such launches with little work in each.  k_wave solves a whole level in
// one launch.  CTAs take 32-row tiles from a counter, in dependency order;
// a tile applies the updates of the blocks it depends on one after the
// other, each as soon as that block is final, and a tile of block b counts
// itself into done[front][b] once its own rows are final.  Block b is final
// when all of its tiles have counted in.
//   forward:  rows of block bt (border rows: bt = number of blocks) take
//             the updates of blocks 0 .. bt-1;
//   backward: pivot rows of block bt take the updates of blocks nblk-1 down
//             to bt+1 and are then written to the solution.
// Tiles are numbered forward by block and backward by decreasing block, so
// a tile waits only for tiles taken before it, by CTAs that are already
// running: the level completes with any number of CTAs resident.  Each row
// takes the same updates in the same order with the same arithmetic as in
// k_blk_update, so the results are bitwise those of the step launches.
// Waits are bounded: a wait that runs out raises the solve's error flag and
// the abort word, and every CTA stops waiting (the host rejects the solve).
// Measured slower than the step launches (option solve_wave): with
// programmatic dependent launch a step already costs little more than the
// memory round trips of a hand-over (flag, vector, reduction), which the
// wave pays too, and its CTAs stream less of the factor at a time.
// ctr: [0] next tile, [1] CTAs done, [2] abort, [4 + q maxblk + b] final
// tiles of block b of the level's front q; the last CTA out clears them.
constexpr unsigned kWaveLimit = 1u << 22;

__device__ __forceinline__ int ld_acquire_int(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <class C, int SW, bool BWD>
__global__ void __launch_bounds__(256, (SW <= 256 && sizeof(C) == 8) ? 2 : 1)
    k_wave(const int *__restrict__ fl, const int4 *__restrict__ tiles, int ntiles,
           int *__restrict__ ctr, int nctr, int maxblk, const C *__restrict__ pool,
           const DevFront *__restrict__ fr, C *__restrict__ work, const int *__restrict__ nodes,
           C *__restrict__ x, int *__restrict__ err) {
  __shared__ __align__(16) C vs[SW];
  __shared__ C red[8][32];
  __shared__ int s_tile, s_abort;
  pdl_launch_dependents();
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  constexpr int kQ = SW / 8;
  const int q0 = wp * kQ;
  int *done = ctr + 4;
  bool waited = false, aborted = false;
  while (!aborted) {
    if (threadIdx.x == 0) s_tile = atomicAdd(ctr, 1);
    __syncthreads();
    const int ti = s_tile;
    if (ti >= ntiles) break;
    const int4 tl = tiles[ti];  // {front slot, first row, rows, block}
    const DevFront f = fr[fl[tl.x]];
    const int nblk = (f.p + SW - 1) / SW;
    C *t = work + f.toff;
    const bool rowok = lane < tl.z;
    const int r = tl.y + lane;
    const int nupd = BWD ? nblk - 1 - tl.w : min(tl.w, nblk);
    C v = czero<C>();
    for (int u = 0; u < nupd; ++u) {
      const int b = BWD ? nblk - 1 - u : u;
      const int b0 = b * SW, b1 = min(f.p, b0 + SW), nb = b1 - b0;
      const C *F = pool + f.off + (long long)b0 * f.m;
      const bool full = q0 + kQ <= nb;
      // the factor does not depend on earlier kernels: its loads go out
      // before any wait
      C fv[kQ];
      if (full && rowok) {
        const C *Fp = F + (long long)q0 * f.m + r;
#pragma unroll
        for (int k = 0; k < kQ; ++k, Fp += f.m) fv[k] = *Fp;
      } else {
#pragma unroll
        for (int k = 0; k < kQ; ++k)
          fv[k] = (rowok && q0 + k < nb) ? F[(long long)(q0 + k) * f.m + r] : czero<C>();
      }
      if (!waited) {
        pdl_wait();
        waited = true;
      }
      if (u == 0 && wp == 0 && rowok) v = __ldcg(t + r);
      if (threadIdx.x == 0) {
        const int *c = done + tl.x * maxblk + b;
        const int target = (nb + 31) / 32;
        unsigned it = 0;
        int ab = 0;
        while (ld_acquire_int(c) < target) {
          if (*reinterpret_cast<volatile int *>(ctr + 2)) {
            ab = 1;
            break;
          }
          if (++it > kWaveLimit) {
            atomicExch(ctr + 2, 1);
            atomicExch(err, 1);
            ab = 1;
            break;
          }
          __nanosleep(32);
        }
        s_abort = ab;
      }
      __syncthreads();
      if (s_abort) {
        aborted = true;
        break;
      }
      for (int q = threadIdx.x; q < nb; q += blockDim.x) vs[q] = __ldcg(t + b0 + q);
      __syncthreads();
      const C acc = dot_cols<C, kQ>(fv, vs + q0, full, nb - q0);
      red[wp][lane] = acc;
      __syncthreads();
      if (wp == 0 && rowok) {
#pragma unroll
        for (int k = 0; k < 8; ++k) v = csub(v, red[k][lane]);
      }
      __syncthreads();  // vs and red are reused
    }
    if (aborted) break;
    if (nupd > 0 && wp == 0 && rowok) {
      t[r] = v;
      if (BWD) x[(long long)nodes[f.node_off + r / 5] * 5 + r % 5] = v;
    }
    if (tl.w < nblk) {  // a pivot tile: its rows are final
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(done + tl.x * maxblk + tl.w, 1);
      }
    }
    __syncthreads();  // s_tile is rewritten
  }
  // the last CTA out clears the counters for the next replay
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(ctr + 1, 1) == (int)gridDim.x - 1) {
      ctr[0] = 0;
      ctr[2] = 0;
      for (int i = 4; i < nctr; ++i) ctr[i] = 0;
      __threadfence();
      ctr[1] = 0;
    }
  }
}

// Backward border product, pass 1: partial[front][chunk][i] = sum over a
// kBC-column chunk of the border of U'(i, c) x[unknown of border row c],
// pivot rows i (the border unknowns belong to ancestors, already solved).
// CTA = 32 rows x 8 warps of kBC/8 columns.
constexpr int kBC = 256;

template <class C>
__global__ void __launch_bounds__(256)
    k_border_gemv(const int *__restrict__ fl, const C *__restrict__ pool,
                  const DevFront *__restrict__ fr, const int *__restrict__ nodes,
                  const C *__restrict__ x, double2 *__restrict__ partial, int nck, int pmax) {
  __shared__ C xs[kBC];
  __shared__ C red[8][32];
  pdl_launch_dependents();
  pdl_wait();
  const int fq = blockIdx.z;
  const DevFront f = fr[fl[fq]];
  const int r0 = blockIdx.x * 32;
  const int c0 = f.p + blockIdx.y * kBC;
  if (r0 >= f.p || c0 >= f.m) return;
  const int nc = min(kBC, f.m - c0);
  for (int k = threadIdx.x; k < nc; k += blockDim.x) {
    const int c = c0 + k;
    xs[k] = x[(long long)nodes[f.node_off + c / 5] * 5 + c % 5];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int r = r0 + lane;
  C acc = czero<C>();
  if (r < f.p) {
    const int ka = wp * (kBC / 8), kb = min(nc, ka + kBC / 8);
    const C *F = pool + f.off + (long long)c0 * f.m + r;
#pragma unroll 8
    for (int k = ka; k < kb; ++k) acc = cfma(acc, F[(long long)k * f.m], xs[k]);
  }
  red[wp][lane] = acc;
  __syncthreads();
  if (wp == 0 && r < f.p) {
    C v = czero<C>();
#pragma unroll
    for (int k = 0; k < 8; ++k) v = cadd(v, red[k][lane]);
    partial[((long long)fq * nck + blockIdx.y) * pmax + r] = to64(v);
  }
}

// The same border product for complex64 factors, with the warp's kBC/8
// columns loaded before the programmatic-launch wait (the factor does not
// depend on earlier kernels of the solve) and summed in the same order.
__global__ void __launch_bounds__(256, 3)
    k_border_gemv_pf(const int *__restrict__ fl, const float2 *__restrict__ pool,
                     const DevFront *__restrict__ fr, const int *__restrict__ nodes,
                     const float2 *__restrict__ x, double2 *__restrict__ partial, int nck,
                     int pmax) {
  using C = float2;
  __shared__ __align__(16) C xs[kBC];
  __shared__ C red[8][32];
  pdl_launch_dependents();
  const int fq = blockIdx.z;
  const DevFront f = fr[fl[fq]];
  const int r0 = blockIdx.x * 32;
  const int c0 = f.p + blockIdx.y * kBC;
  if (r0 >= f.p || c0 >= f.m) return;
  const int nc = min(kBC, f.m - c0);
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int r = r0 + lane;
  constexpr int kQ = kBC / 8;
  const int ka = wp * kQ;
  const bool full = ka + kQ <= nc;
  const C *F = pool + f.off + (long long)c0 * f.m + r;
  C fv[kQ];
  if (full && r < f.p) {
    const C *Fp = F + (long long)ka * f.m;
#pragma unroll
    for (int k = 0; k < kQ; ++k, Fp += f.m) fv[k] = *Fp;
  } else {
#pragma unroll
    for (int k = 0; k < kQ; ++k)
      fv[k] = (r < f.p && ka + k < nc) ? F[(long long)(ka + k) * f.m] : czero<C>();
  }
  pdl_wait();
  for (int k = threadIdx.x; k < nc; k += blockDim.x) {
    const int c = c0 + k;
    xs[k] = x[(long long)nodes[f.node_off + c / 5] * 5 + c % 5];
  }
  __syncthreads();
  C acc = czero<C>();
  if (r < f.p) acc = dot_cols<C, kQ>(fv, xs + ka, full, nc - ka);
  red[wp][lane] = acc;
  __syncthreads();
  if (wp == 0 && r < f.p) {
    C v = czero<C>();
#pragma unroll
    for (int k = 0; k < 8; ++k) v = cadd(v, red[k][lane]);
    partial[((long long)fq * nck + blockIdx.y) * pmax + r] = to64(v);
  }
}

// Start of a front's backward pass: rows of block b = blockIdx.x / 4
// (32 per CTA) take w = D_b z_b minus the border chunks of pass 1 (summed
// in chunk order), written to the backward vector (z stays in work for the
// other CTAs of the block).  The last block's rows are final and go to x.
template <class C, int SW>
__global__ void __launch_bounds__(256)
    k_bwd_start(const int *__restrict__ fl, const DevFront *__restrict__ fr,
                const long long *__restrict__ inv_off, const C *__restrict__ dmat,
                const C *__restrict__ work, C *__restrict__ work2,
                const double2 *__restrict__ partial, int nck, int pmax,
                const int *__restrict__ nodes, C *__restrict__ x) {
  __shared__ __align__(16) C zs[SW];
  __shared__ C red[8][32];
  pdl_launch_dependents();
  const int fq = blockIdx.y, fid = fl[fq];
  const DevFront f = fr[fid];
  const int blk = blockIdx.x / (SW / 32), quarter = blockIdx.x % (SW / 32);
  const int b0 = blk * SW, nb = min(SW, f.p - b0);
  const int rr0 = quarter * 32;
  if (nb <= 0 || rr0 >= nb) return;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int rr = rr0 + lane;  // row inside the block
  const C *Dm = dmat + inv_off[fid] + (long long)blk * SW * SW;
  constexpr int kQ = SW / 8;
  const int q0 = wp * kQ;
  const bool full = q0 + kQ <= nb;
  C dv[kQ];
  if (full && rr < nb) {
    const C *Dp = Dm + (long long)q0 * nb + rr;
#pragma unroll
    for (int k = 0; k < kQ; ++k, Dp += nb) dv[k] = *Dp;
  } else {
#pragma unroll
    for (int k = 0; k < kQ; ++k)
      dv[k] = (rr < nb && q0 + k < nb) ? Dm[(long long)(q0 + k) * nb + rr] : czero<C>();
  }
  pdl_wait();
  // warp 0 sums its rows' border partials (in chunk order) while the other
  // warps stage z
  const int r = b0 + rr;
  double2 s = make_double2(0, 0);
  if (wp == 0 && rr < nb) {
    // up to 36 chunks at the top of the tree: the loads go out 8 at a time,
    // the sums stay in chunk order
    const int nchf = f.m > f.p ? (f.m - f.p + kBC - 1) / kBC : 0;
    const double2 *pp = partial + (long long)fq * nck * pmax + r;
    int k = 0;
    for (; k + 8 <= nchf; k += 8) {
      double2 pv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) pv[u] = pp[(long long)(k + u) * pmax];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        s.x += pv[u].x;
        s.y += pv[u].y;
      }
    }
    for (; k < nchf; ++k) {
      const double2 pv = pp[(long long)k * pmax];
      s.x += pv.x;
      s.y += pv.y;
    }
  }
  const C *z = work + f.toff + b0;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) zs[q] = z[q];
  __syncthreads();
  const C acc = dot_cols<C, kQ>(dv, zs + q0, full, nb - q0);
  red[wp][lane] = acc;
  __syncthreads();
  if (wp == 0 && rr < nb) {
    C w = czero<C>();
#pragma unroll
    for (int k = 0; k < 8; ++k) w = cadd(w, red[k][lane]);
    w = csub(w, from64<C>(s));
    work2[f.toff + r] = w;
    if (b0 + SW >= f.p) x[(long long)nodes[f.node_off + r / 5] * 5 + r % 5] = w;
  }
}

// ---- multi-RHS triangular solves (complex64) --------------------------------
// The solve steps above on NR right-hand sides at once.  Every CTA loads its
// factor (or D_b) tile into registers once and applies it to all NR vectors,
// so one solve of NR vectors streams the factor from HBM once instead of NR
// times.  Vector r of x lives at x + r * xs, of work / work2 at + r * ws, and
// its border partial sums at partial + r * ps.  Per vector, the arithmetic
// and its order are those of the single-vector kernels, so every vector's
// result is bitwise the single-vector solve's.

template <int NR>
__global__ void k_sgather_m(const int *__restrict__ fl, const DevFront *__restrict__ fr,
                            const int *__restrict__ nodes, const int *__restrict__ perm,
                            const int2 *__restrict__ cinv, const float2 *__restrict__ b,
                            long long xs, float2 *__restrict__ work, long long ws) {
  pdl_launch_dependents();
  pdl_wait();
  const DevFront f = fr[fl[blockIdx.y]];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.m) return;
  long long src = -1;
  if (i < f.p) {
    const int q = perm[f.toff + i];
    src = (long long)nodes[f.node_off + q / 5] * 5 + q % 5;
  }
  const int2 c = cinv[f.toff + i];
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const float2 *br = b + r * xs;
    float2 *wr = work + r * ws;
    float2 v = src >= 0 ? br[src] : czero<float2>();
    if (c.x >= 0) v = cadd(v, wr[c.x]);
    if (c.y >= 0) v = cadd(v, wr[c.y]);
    wr[f.toff + i] = v;
  }
}

template <int SW, int NR>
__global__ void __launch_bounds__(256)
    k_blk_update_m(const int *__restrict__ fl, int b, int backward, const float2 *__restrict__ pool,
                   const DevFront *__restrict__ fr, float2 *__restrict__ work, long long ws,
                   const int *__restrict__ nodes, float2 *__restrict__ x, long long xs) {
  using C = float2;
  __shared__ __align__(16) C vs[NR][SW];
  __shared__ C red[NR][8][32];
  pdl_launch_dependents();
  const DevFront f = fr[fl[blockIdx.y]];
  const int b0 = b * SW, b1 = min(f.p, b0 + SW), nb = b1 - b0;
  const int lo = backward ? 0 : b1, hi = backward ? b0 : f.m;
  const int r0 = lo + blockIdx.x * 32;
  if (nb <= 0 || r0 >= hi) return;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int r = r0 + lane;
  const C *F = pool + f.off + (long long)b0 * f.m;
  constexpr int kQ = SW / 8;
  const int q0 = wp * kQ;
  const bool full = q0 + kQ <= nb;
  C fv[kQ];
  if (full && r < hi) {
    const C *Fp = F + (long long)q0 * f.m + r;
#pragma unroll
    for (int k = 0; k < kQ; ++k, Fp += f.m) fv[k] = *Fp;
  } else {
#pragma unroll
    for (int k = 0; k < kQ; ++k)
      fv[k] = (r < hi && q0 + k < nb) ? F[(long long)(q0 + k) * f.m + r] : czero<C>();
  }
  pdl_wait();
  for (int t = threadIdx.x; t < NR * nb; t += blockDim.x) {
    const int v = t / nb, q = t - v * nb;
    vs[v][q] = work[v * ws + f.toff + b0 + q];
  }
  __syncthreads();
#pragma unroll
  for (int v = 0; v < NR; ++v) red[v][wp][lane] = dot_cols<C, kQ>(fv, vs[v] + q0, full, nb - q0);
  __syncthreads();
  if (r < hi)
    for (int v = wp; v < NR; v += 8) {  // warp v finishes vector v
      C *t = work + v * ws + f.toff;
      C acc = t[r];
#pragma unroll
      for (int k = 0; k < 8; ++k) acc = csub(acc, red[v][k][lane]);
      t[r] = acc;
      if (backward && r >= b0 - SW)
        x[v * xs + (long long)nodes[f.node_off + r / 5] * 5 + r % 5] = acc;
    }
}

template <int NR>
__global__ void __launch_bounds__(256)
    k_border_gemv_m(const int *__restrict__ fl, const float2 *__restrict__ pool,
                    const DevFront *__restrict__ fr, const int *__restrict__ nodes,
                    const float2 *__restrict__ x, long long xs, double2 *__restrict__ partial,
                    long long ps, int nck, int pmax) {
  using C = float2;
  __shared__ __align__(16) C xsh[NR][kBC];
  __shared__ C red[NR][8][32];
  pdl_launch_dependents();
  const int fq = blockIdx.z;
  const DevFront f = fr[fl[fq]];
  const int r0 = blockIdx.x * 32;
  const int c0 = f.p + blockIdx.y * kBC;
  if (r0 >= f.p || c0 >= f.m) return;
  const int nc = min(kBC, f.m - c0);
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int r = r0 + lane;
  constexpr int kQ = kBC / 8;
  const int ka = wp * kQ;
  const bool full = ka + kQ <= nc;
  const C *F = pool + f.off + (long long)c0 * f.m + r;
  C fv[kQ];
  if (full && r < f.p) {
    const C *Fp = F + (long long)ka * f.m;
#pragma unroll
    for (int k = 0; k < kQ; ++k, Fp += f.m) fv[k] = *Fp;
  } else {
#pragma unroll
    for (int k = 0; k < kQ; ++k)
      fv[k] = (r < f.p && ka + k < nc) ? F[(long long)(ka + k) * f.m] : czero<C>();
  }
  pdl_wait();
  for (int t = threadIdx.x; t < NR * nc; t += blockDim.x) {
    const int v = t / nc, k = t - v * nc;
    const int c = c0 + k;
    xsh[v][k] = x[v * xs + (long long)nodes[f.node_off + c / 5] * 5 + c % 5];
  }
  __syncthreads();
#pragma unroll
  for (int v = 0; v < NR; ++v)
    red[v][wp][lane] = r < f.p ? dot_cols<C, kQ>(fv, xsh[v] + ka, full, nc - ka) : czero<C>();
  __syncthreads();
  if (r < f.p)
    for (int v = wp; v < NR; v += 8) {
      C acc = czero<C>();
#pragma unroll
      for (int k = 0; k < 8; ++k) acc = cadd(acc, red[v][k][lane]);
      partial[v * ps + ((long long)fq * nck + blockIdx.y) * pmax + r] = to64(acc);
    }
}

template <int SW, int NR>
__global__ void __launch_bounds__(256)
    k_bwd_start_m(const int *__restrict__ fl, const DevFront *__restrict__ fr,
                  const long long *__restrict__ inv_off, const float2 *__restrict__ dmat,
                  const float2 *__restrict__ work, float2 *__restrict__ work2, long long ws,
                  const double2 *__restrict__ partial, long long ps, int nck, int pmax,
                  const int *__restrict__ nodes, float2 *__restrict__ x, long long xs) {
  using C = float2;
  static_assert(NR <= 8, "one warp per right-hand side finishes the rows");
  __shared__ __align__(16) C zs[NR][SW];
  __shared__ C red[NR][8][32];
  pdl_launch_dependents();
  const int fq = blockIdx.y, fid = fl[fq];
  const DevFront f = fr[fid];
  const int blk = blockIdx.x / (SW / 32), quarter = blockIdx.x % (SW / 32);
  const int b0 = blk * SW, nb = min(SW, f.p - b0);
  const int rr0 = quarter * 32;
  if (nb <= 0 || rr0 >= nb) return;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int rr = rr0 + lane;
  const C *Dm = dmat + inv_off[fid] + (long long)blk * SW * SW;
  constexpr int kQ = SW / 8;
  const int q0 = wp * kQ;
  const bool full = q0 + kQ <= nb;
  C dv[kQ];
  if (full && rr < nb) {
    const C *Dp = Dm + (long long)q0 * nb + rr;
#pragma unroll
    for (int k = 0; k < kQ; ++k, Dp += nb) dv[k] = *Dp;
  } else {
#pragma unroll
    for (int k = 0; k < kQ; ++k)
      dv[k] = (rr < nb && q0 + k < nb) ? Dm[(long long)(q0 + k) * nb + rr] : czero<C>();
  }
  pdl_wait();
  const int r = b0 + rr;
  // warp v (< NR) sums vector v's border partials for its rows, in chunk order
  double2 s = make_double2(0, 0);
  if (wp < NR && rr < nb) {
    const int nchf = f.m > f.p ? (f.m - f.p + kBC - 1) / kBC : 0;
    const double2 *pv = partial + wp * ps;
#pragma unroll 4
    for (int k = 0; k < nchf; ++k) {
      const double2 p = pv[((long long)fq * nck + k) * pmax + r];
      s.x += p.x;
      s.y += p.y;
    }
  }
  for (int t = threadIdx.x; t < NR * nb; t += blockDim.x) {
    const int v = t / nb, q = t - v * nb;
    zs[v][q] = work[v * ws + f.toff + b0 + q];
  }
  __syncthreads();
#pragma unroll
  for (int v = 0; v < NR; ++v) red[v][wp][lane] = dot_cols<C, kQ>(dv, zs[v] + q0, full, nb - q0);
  __syncthreads();
  if (wp < NR && rr < nb) {
    C w = czero<C>();
#pragma unroll
    for (int k = 0; k < 8; ++k) w = cadd(w, red[wp][k][lane]);
    w = csub(w, from64<C>(s));
    work2[wp * ws + f.toff + r] = w;
    if (b0 + SW >= f.p) x[wp * xs + (long long)nodes[f.node_off + r / 5] * 5 + r % 5] = w;
  }
}

// ---- persistent solve ------------------------------------------------------
// The whole triangular solve as one cooperative launch: every phase of the
// graph above (gather of a level, one block step, border product, backward
// start) becomes a list of CTA work items that the resident CTAs stride
// through, with a grid barrier between dependent phases.  Data written by
// other CTAs in earlier phases is read past L1 (__ldcg).  The barrier spins
// with a bound: on timeout it raises the solve's error flag and goes on (the
// host rejects the solve).

enum PhaseType : int { kPhGather = 0, kPhFwd = 1, kPhBorder = 2, kPhBwdStart = 3, kPhBwd = 4 };

constexpr unsigned kBarrierLimit = 1u << 22;

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void grid_barrier(unsigned *count, unsigned target, int *err,
                                             unsigned limit = kBarrierLimit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(count, 1u);
    unsigned it = 0;
    while (ld_acquire(count) < target)
      if (++it > limit) {
        atomicExch(err, 1);
        break;
      }
    __threadfence();
  }
  __syncthreads();
}

// one CTA waits at a grid barrier for a second arrival that never comes
__global__ void k_grid_barrier_probe(unsigned *count, unsigned limit, int *err) {
  grid_barrier(count, 2u, err, limit);
}

template <class C>
__device__ void ps_gather(const int *fl, const DevFront *fr, const int *nodes, const int *perm,
                          const int2 *cinv, const C *b, C *work, int bx, int by) {
  const DevFront f = fr[fl[by]];
  const int i = bx * blockDim.x + threadIdx.x;
  if (i >= f.m) return;
  C v = czero<C>();
  if (i < f.p) {
    const int q = perm[f.toff + i];
    v = __ldcg(b + (long long)nodes[f.node_off + q / 5] * 5 + q % 5);
  }
  const int2 c = cinv[f.toff + i];
  if (c.x >= 0) v = cadd(v, __ldcg(work + c.x));
  if (c.y >= 0) v = cadd(v, __ldcg(work + c.y));
  work[f.toff + i] = v;
}

template <class C, int SW>
__device__ void ps_step(const int *fl, int b, int backward, const C *pool, const DevFront *fr,
                        C *work, const int *nodes, C *x, int bx, int by, C *vs, C (*red)[32]) {
  const DevFront f = fr[fl[by]];
  const int b0 = b * SW, b1 = min(f.p, b0 + SW), nb = b1 - b0;
  const int lo = backward ? 0 : b1, hi = backward ? b0 : f.m;
  const int r0 = lo + bx * 32;
  if (nb <= 0 || r0 >= hi) return;
  C *t = work + f.toff;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int r = r0 + lane;
  const C *F = pool + f.off + (long long)b0 * f.m;
  constexpr int kQ = SW / 8;
  const int q0 = wp * kQ;
  C fv[kQ];
#pragma unroll
  for (int k = 0; k < kQ; ++k)
    fv[k] = (r < hi && q0 + k < nb) ? F[(long long)(q0 + k) * f.m + r] : czero<C>();
  for (int q = threadIdx.x; q < nb; q += blockDim.x) vs[q] = __ldcg(t + b0 + q);
  __syncthreads();
  C acc = czero<C>();
#pragma unroll
  for (int k = 0; k < kQ; ++k)
    if (q0 + k < nb) acc = cfma(acc, fv[k], vs[q0 + k]);
  red[wp][lane] = acc;
  __syncthreads();
  if (wp == 0 && r < hi) {
    C v = __ldcg(t + r);
#pragma unroll
    for (int k = 0; k < 8; ++k) v = csub(v, red[k][lane]);
    t[r] = v;
    if (backward && r >= b0 - SW) x[(long long)nodes[f.node_off + r / 5] * 5 + r % 5] = v;
  }
  __syncthreads();  // vs and red are reused by the next item
}

template <class C>
__device__ void ps_border(const int *fl, const C *pool, const DevFront *fr, const int *nodes,
                          const C *x, double2 *partial, int nck, int pmax, int bx, int by, int bz,
                          C *xs, C (*red)[32]) {
  const DevFront f = fr[fl[bz]];
  const int r0 = bx * 32;
  const int c0 = f.p + by * kBC;
  if (r0 >= f.p || c0 >= f.m) return;
  const int nc = min(kBC, f.m - c0);
  for (int k = threadIdx.x; k < nc; k += blockDim.x) {
    const int c = c0 + k;
    xs[k] = __ldcg(x + (long long)nodes[f.node_off + c / 5] * 5 + c % 5);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int r = r0 + lane;
  C acc = czero<C>();
  if (r < f.p) {
    const int ka = wp * (kBC / 8), kb = min(nc, ka + kBC / 8);
    const C *F = pool + f.off + (long long)c0 * f.m + r;
#pragma unroll 8
    for (int k = ka; k < kb; ++k) acc = cfma(acc, F[(long long)k * f.m], xs[k]);
  }
  red[wp][lane] = acc;
  __syncthreads();
  if (wp == 0 && r < f.p) {
    C v = czero<C>();
#pragma unroll
    for (int k = 0; k < 8; ++k) v = cadd(v, red[k][lane]);
    partial[((long long)bz * nck + by) * pmax + r] = to64(v);
  }
  __syncthreads();
}

template <class C, int SW>
__device__ void ps_bwd_start(const int *fl, const DevFront *fr, const long long *inv_off,
                             const C *dmat, const C *work, C *work2, const double2 *partial,
                             int nck, int pmax, const int *nodes, C *x, int bx, int by, C *zs,
                             C (*red)[32]) {
  const int fid = fl[by];
  const DevFront f = fr[fid];
  const int blk = bx / (SW / 32), quarter = bx % (SW / 32);
  const int b0 = blk * SW, nb = min(SW, f.p - b0);
  const int rr0 = quarter * 32;
  if (nb <= 0 || rr0 >= nb) return;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int rr = rr0 + lane;
  const C *Dm = dmat + inv_off[fid] + (long long)blk * SW * SW;
  constexpr int kQ = SW / 8;
  const int q0 = wp * kQ;
  C dv[kQ];
#pragma unroll
  for (int k = 0; k < kQ; ++k)
    dv[k] = (rr < nb && q0 + k < nb) ? Dm[(long long)(q0 + k) * nb + rr] : czero<C>();
  const C *z = work + f.toff + b0;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) zs[q] = __ldcg(z + q);
  __syncthreads();
  C acc = czero<C>();
#pragma unroll
  for (int k = 0; k < kQ; ++k)
    if (q0 + k < nb) acc = cfma(acc, dv[k], zs[q0 + k]);
  red[wp][lane] = acc;
  __syncthreads();
  if (wp == 0 && rr < nb) {
    C w = czero<C>();
#pragma unroll
    for (int k = 0; k < 8; ++k) w = cadd(w, red[k][lane]);
    const int r = b0 + rr;
    const int nchf = f.m > f.p ? (f.m - f.p + kBC - 1) / kBC : 0;
    double2 s = make_double2(0, 0);
    for (int k = 0; k < nchf; ++k) {
      const double2 pv = __ldcg(partial + ((long long)by * nck + k) * pmax + r);
      s.x += pv.x;
      s.y += pv.y;
    }
    w = csub(w, from64<C>(s));
    work2[f.toff + r] = w;
    if (b0 + SW >= f.p) x[(long long)nodes[f.node_off + r / 5] * 5 + r % 5] = w;
  }
  __syncthreads();
}

template <class C, int SW>
__global__ void __launch_bounds__(256)
    k_solve_persistent(const Phase *__restrict__ phases, int nphases, const int *__restrict__ sched,
                       const C *__restrict__ pool, const DevFront *__restrict__ fr,
                       const int *__restrict__ nodes, const int *__restrict__ perm,
                       const int2 *__restrict__ cinv, const long long *__restrict__ inv_off,
                       const C *__restrict__ dmat, C *work, C *work2, double2 *partial, C *x,
                       unsigned *barrier, int *err) {
  __shared__ C vec_s[SW > kBC ? SW : kBC];
  __shared__ C red_s[8][32];
  unsigned target = 0;
  for (int ph = 0; ph < nphases; ++ph) {
    const Phase P = phases[ph];
    const int *fl = sched + P.fl_off;
    const int nitems = P.nx * P.ny * P.nz;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
      const int bx = it % P.nx, rest = it / P.nx, by = rest % P.ny, bz = rest / P.ny;
      switch (P.type) {
        case kPhGather: ps_gather<C>(fl, fr, nodes, perm, cinv, x, work, bx, by); break;
        case kPhFwd: ps_step<C, SW>(fl, P.b, 0, pool, fr, work, nodes, x, bx, by, vec_s, red_s); break;
        case kPhBorder:
          ps_border<C>(fl, pool, fr, nodes, x, partial, P.nck, P.pmax, bx, by, bz, vec_s, red_s);
          break;
        case kPhBwdStart:
          ps_bwd_start<C, SW>(fl, fr, inv_off, dmat, work, work2, partial, P.nck, P.pmax, nodes, x,
                              bx, by, vec_s, red_s);
          break;
        default: ps_step<C, SW>(fl, P.b, 1, pool, fr, work2, nodes, x, bx, by, vec_s, red_s); break;
      }
    }
    if (ph + 1 < nphases) {
      target += gridDim.x;
      grid_barrier(barrier, target, err);
    }
  }
}

// launch, with programmatic stream serialisation when pdl (captured into
// the graph as a programmatic dependency on the previous kernel)
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace

// ------------------------------------------------------------------- host

int Factor::setup(tlr_ctx *ctx, int precision, int leaf, int solve_block, int panel_width,
                  int ring_slack_percent) {
  prec = precision;
  ring_slack = ring_slack_percent > 0 ? ring_slack_percent : kRingSlackDefault;
  // complex128 panels stop at 64 columns: the TRSM tiles (w x w + w x 33
  // values) must fit in shared memory
  w = panel_width == 32 || panel_width == 64 || (panel_width == 128 && precision == 1)
          ? panel_width
          : (precision == 0 ? 32 : 64);
  sw = precision == 0 ? 128 : (solve_block == 128 || solve_block == 512 ? solve_block : 256);
  int rc;
  if (ctx->shared_sym) {
    sym = *ctx->shared_sym;  // analysis shared by every context of the grid class
  } else {
    std::vector<int> rp(ctx->nn + 1), cl((size_t)ctx->nnzb);
    TLR_CUDA(ctx, cudaMemcpy(rp.data(), ctx->row_ptr, rp.size() * sizeof(int),
                             cudaMemcpyDeviceToHost));
    TLR_CUDA(ctx, cudaMemcpy(cl.data(), ctx->col, cl.size() * sizeof(int),
                             cudaMemcpyDeviceToHost));
    rc = build_symbolic(ctx->ny, ctx->nz, ctx->h_xi_idx, ctx->sx, ctx->h_eta_off, ctx->se, rp,
                        cl, leaf, sym, ring_slack);
    if (rc) {
      char buf[96];
      snprintf(buf, sizeof(buf), "symbolic analysis failed (code %d)", rc);
      return fail(ctx, TLR_ERR_ARG, buf);
    }
  }
  const int nf = (int)sym.fronts.size();
  std::vector<DevFront> df(nf);
  std::vector<int> nodes;
  nodes.reserve(sym.work_elems / 5);
  for (int t = 0; t < nf; ++t) {
    const FrontInfo &f = sym.fronts[t];
    DevFront &d = df[t];
    d.off = f.off;
    d.toff = f.toff;
    d.p = f.p;
    d.m = f.m;
    d.parent = f.parent;
    d.cmap_off = sym.cmap_off[t] < 0 ? 0 : sym.cmap_off[t];
    d.node_off = (int)(f.toff / 5);
  }
  nodes.assign(sym.work_elems / 5, 0);
  for (int t = 0; t < nf; ++t) {
    const FrontInfo &f = sym.fronts[t];
    int a = df[t].node_off;
    for (int u : f.piv) nodes[a++] = u;
    for (int v : f.border) nodes[a++] = v;
  }
  // schedules: per level, fronts sorted by p descending; per step prefix
  std::vector<int> sched;
  long long max_plane_tiles = 0;  // largest atiles + btiles of a panel step
  levels.clear();
  for (size_t h = 0; h < sym.levels.size(); ++h) {
    Level L;
    std::vector<int> fl = sym.levels[h];
    std::sort(fl.begin(), fl.end(),
              [&](int a, int b) { return sym.fronts[a].p > sym.fronts[b].p; });
    L.nfronts = (int)fl.size();
    L.fronts_off = (int)sched.size();
    sched.insert(sched.end(), fl.begin(), fl.end());
    L.max_m = 0;
    for (int t : fl) L.max_m = std::max(L.max_m, sym.fronts[t].m);
    for (int slot = 0; slot < 2; ++slot) {
      std::vector<int> kids;
      for (int t : fl)
        if ((int)sym.fronts[t].children.size() > slot) kids.push_back(sym.fronts[t].children[slot]);
      L.kids[slot] = (int)kids.size();
      L.kids_off[slot] = (int)sched.size();
      int mb = 0;
      for (int c : kids) mb = std::max(mb, sym.fronts[c].m - sym.fronts[c].p);
      L.kids_maxb[slot] = mb;
      sched.insert(sched.end(), kids.begin(), kids.end());
    }
    L.entry_begin = sym.level_entry_begin[h];
    L.entry_end = sym.level_entry_begin[h + 1];
    L.pool_begin = sym.fronts[fl.back()].off;
    L.pool_end = 0;
    for (int t : fl) {
      L.pool_begin = std::min(L.pool_begin, sym.fronts[t].off);
      L.pool_end = std::max(L.pool_end, sym.fronts[t].off + (long long)sym.fronts[t].m * sym.fronts[t].m);
    }
    const int pmax = sym.fronts[fl.front()].p;
    const int nsteps = (pmax + w - 1) / w;
    for (int s = 0; s < nsteps; ++s) {
      Step st;
      st.nf = 0;
      for (int t : fl)
        if (sym.fronts[t].p > s * w) ++st.nf;
      st.max_m = 0;
      st.max_b = 0;
      st.max_ext = 0;
      st.prefix_off = (int)sched.size();
      int acc = 0;
      for (int q = 0; q < st.nf; ++q) {
        const FrontInfo &f = sym.fronts[fl[q]];
        const int ww = std::min(w, f.p - s * w);
        const int ext = f.m - s * w - ww;
        const int tm = prec == 0 ? kTile : kTM32, tn = prec == 0 ? kTile : kTN32;
        sched.push_back(acc);
        acc += ((ext + tm - 1) / tm) * ((ext + tn - 1) / tn);
        st.max_m = std::max(st.max_m, f.m);
        st.max_b = std::max(st.max_b, f.m - f.p);
        st.max_ext = std::max(st.max_ext, ext);
      }
      sched.push_back(acc);
      st.tiles = acc;
      if (prec == 1) {  // the operand tiles of the bulk-copy Schur update
        for (int pass = 0; pass < 2; ++pass) {
          (pass ? st.pb_off : st.pa_off) = (int)sched.size();
          int tot = 0;
          for (int q = 0; q < st.nf; ++q) {
            const FrontInfo &f = sym.fronts[fl[q]];
            const int ww = std::min(w, f.p - s * w);
            const int ext = f.m - s * w - ww;
            sched.push_back(tot);
            tot += (ext + (pass ? kTN32 : kTM32) - 1) / (pass ? kTN32 : kTM32);
          }
          sched.push_back(tot);
          (pass ? st.btiles : st.atiles) = tot;
        }
        max_plane_tiles = std::max(max_plane_tiles, (long long)st.atiles + st.btiles);
      }
      L.steps.push_back(st);
    }
    levels.push_back(L);
  }
  long long partial_elems = 0;
  for (auto &L : levels) {
    L.pmax = 0;
    L.bmax = 0;
    for (int q = 0; q < L.nfronts; ++q) {
      const FrontInfo &f = sym.fronts[sched[L.fronts_off + q]];
      L.pmax = std::max(L.pmax, f.p);
      L.bmax = std::max(L.bmax, f.m - f.p);
    }
    L.nck_b = std::max(1, (L.bmax + kBC - 1) / kBC);
    L.blk_nf.clear();
    L.fwd_rows.clear();
    for (int b = 0; b * sw < L.pmax; ++b) {
      int n = 0, rows = 0;
      for (int q = 0; q < L.nfronts; ++q) {
        const FrontInfo &f = sym.fronts[sched[L.fronts_off + q]];
        if (f.p > b * sw) {
          ++n;
          rows = std::max(rows, f.m - std::min(f.p, (b + 1) * sw));
        }
      }
      L.blk_nf.push_back(n);
      L.fwd_rows.push_back(rows);
    }
    partial_elems = std::max(partial_elems, (long long)L.nfronts * L.nck_b * std::max(L.pmax, 1));
  }
  // dependency-driven level solves: 32-row tiles of every level with two or
  // more diagonal blocks, forward in block order (border rows last),
  // backward in decreasing block order; tile = {front slot, first row, rows,
  // block}
  std::vector<int4> wtiles;
  long long wctr = 0;
  for (auto &L : levels) {
    L.wave = L.blk_nf.size() >= 2;
    if (!L.wave) continue;
    L.maxblk = (int)L.blk_nf.size();
    std::vector<std::pair<int, int4>> fw, bw;
    for (int q = 0; q < L.nfronts; ++q) {
      const FrontInfo &f = sym.fronts[sched[L.fronts_off + q]];
      const int nblk = (f.p + sw - 1) / sw;
      for (int bt = 0; bt < nblk; ++bt) {
        const int b0 = bt * sw, b1 = std::min(f.p, b0 + sw);
        for (int r = b0; r < b1; r += 32) {
          const int4 tl = make_int4(q, r, std::min(32, b1 - r), bt);
          fw.push_back({bt, tl});
          bw.push_back({-bt, tl});
        }
      }
      for (int r = f.p; r < f.m; r += 32)
        fw.push_back({nblk, make_int4(q, r, std::min(32, f.m - r), nblk)});
    }
    auto by_key = [](const std::pair<int, int4> &x, const std::pair<int, int4> &y) {
      return x.first < y.first;
    };
    std::stable_sort(fw.begin(), fw.end(), by_key);
    std::stable_sort(bw.begin(), bw.end(), by_key);
    L.wf_off = (long long)wtiles.size();
    L.wf_n = (int)fw.size();
    for (auto &e : fw) wtiles.push_back(e.second);
    L.wb_off = (long long)wtiles.size();
    L.wb_n = (int)bw.size();
    for (auto &e : bw) wtiles.push_back(e.second);
    L.wctr_n = 4 + L.nfronts * L.maxblk;
    L.wcf_off = wctr;
    L.wcb_off = wctr + L.wctr_n;
    wctr += 2LL * L.wctr_n;
  }
  // diagonal blocks (full blocks sw x sw, the last one nb x nb) and the
  // tiles of the factor rewrite L' = L Dl^-1, U' = Du^-1 U, D = Du^-1 Dl^-1
  std::vector<long long> inv_off(nf);
  std::vector<int2> inv_blocks;
  std::vector<int4> ltiles, utiles, ltiles_tc, utiles_tc;
  inv_elems = 0;
  for (int t = 0; t < nf; ++t) {
    const int p = sym.fronts[t].p, m = sym.fronts[t].m;
    inv_off[t] = inv_elems;
    for (int b = 0; b * sw < p; ++b) {
      const int b1 = std::min(p, (b + 1) * sw), nb = b1 - b * sw;
      inv_blocks.push_back(make_int2(t, b));
      inv_elems += (long long)nb * nb;
      for (int r = b1; r < m; r += kRT) ltiles.push_back(make_int4(t, b, r, 0));
      for (int c = b1; c < m; c += kRT) utiles.push_back(make_int4(t, b, c, 0));
      for (int c = 0; c < nb; c += kRT) utiles.push_back(make_int4(t, b, c, 1));
      if (prec == 1 && sw == 256) {
        for (int r = b1; r < m; r += 128) ltiles_tc.push_back(make_int4(t, b, r, 0));
        for (int c = b1; c < m; c += 64) utiles_tc.push_back(make_int4(t, b, c, 0));
        for (int c = 0; c < nb; c += 64) utiles_tc.push_back(make_int4(t, b, c, 1));
      }
    }
  }
  n_ltiles = (long long)ltiles.size();
  n_utiles = (long long)utiles.size();
  n_ltiles_tc = (long long)ltiles_tc.size();
  n_utiles_tc = (long long)utiles_tc.size();
  n_inv_blocks = (int)inv_blocks.size();
  const size_t csize = prec == 0 ? sizeof(double2) : sizeof(float2);
  auto alloc = [&](void **p, size_t bytes) -> int {
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) {
      *p = nullptr;
      return fail(ctx, TLR_ERR_NOMEM, std::string("factor allocation failed: ") +
                                          cudaGetErrorString(e));
    }
    return TLR_OK;
  };
  if ((rc = alloc(&pool, (size_t)sym.pool_elems * csize)) ||
      (rc = alloc(&work, (size_t)sym.work_elems * csize)) ||
      (rc = alloc((void **)&d_fronts, nf * sizeof(DevFront))) ||
      (rc = alloc((void **)&d_entries, sym.entries.size() * sizeof(AsmEntry))) ||
      (rc = alloc((void **)&d_cmap, sym.cmap.size() * sizeof(int))) ||
      (rc = alloc((void **)&d_nodes, nodes.size() * sizeof(int))) ||
      (rc = alloc((void **)&d_ipiv, sym.work_elems * sizeof(int))) ||
      (rc = alloc((void **)&d_perm, sym.work_elems * sizeof(int))) ||
      (rc = alloc((void **)&d_cinv, sym.work_elems * sizeof(int2))) ||
      (rc = alloc(&work2, (size_t)sym.work_elems * csize)) ||
      (rc = alloc((void **)&d_sched, sched.size() * sizeof(int))) ||
      (rc = alloc((void **)&d_partial, (size_t)partial_elems * sizeof(double2))) ||
      (rc = alloc((void **)&d_pert, sizeof(int))) ||
      (rc = alloc((void **)&d_tc_err, sizeof(int))) ||
      (rc = alloc(&linv, (size_t)inv_elems * csize)) ||
      (rc = alloc(&uinv, (size_t)inv_elems * csize)) ||
      (rc = alloc(&dmat, (size_t)inv_elems * csize)) ||
      (rc = alloc((void **)&d_ltiles, ltiles.size() * sizeof(int4))) ||
      (rc = alloc((void **)&d_utiles, utiles.size() * sizeof(int4))) ||
      (rc = alloc((void **)&d_inv_off, nf * sizeof(long long))) ||
      (rc = alloc((void **)&d_inv_blocks, inv_blocks.size() * sizeof(int2))) ||
      (rc = alloc(&vec_a, (size_t)ctx->nn * 5 * csize)) ||
      (rc = alloc((void **)&d_ltiles_tc, ltiles_tc.size() * sizeof(int4))) ||
      (rc = alloc((void **)&d_utiles_tc, utiles_tc.size() * sizeof(int4))) ||
      (rc = alloc((void **)&d_wave_tiles, wtiles.size() * sizeof(int4))) ||
      (rc = alloc((void **)&d_wave_ctr, (size_t)wctr * sizeof(int))))
    return rc;
  {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    wave_grid = std::max(1, sms) * (prec == 1 && sw <= 256 ? 2 : 1);
  }
  if (!wtiles.empty())
    TLR_CUDA(ctx, cudaMemcpy(d_wave_tiles, wtiles.data(), wtiles.size() * sizeof(int4),
                             cudaMemcpyHostToDevice));
  if (wctr) TLR_CUDA(ctx, cudaMemset(d_wave_ctr, 0, (size_t)wctr * sizeof(int)));
  if (prec == 1 &&
      (rc = alloc((void **)&tc_planes, (size_t)max_plane_tiles * ((w + 7) / 8) *
                                           tc_chunk_image_bytes())))
    return rc;
  partial_stride = std::max(partial_elems, 1LL);
  TLR_CUDA(ctx, cudaMemcpy(d_inv_off, inv_off.data(), nf * sizeof(long long),
                           cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d_ltiles, ltiles.data(), ltiles.size() * sizeof(int4),
                           cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d_utiles, utiles.data(), utiles.size() * sizeof(int4),
                           cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d_inv_blocks, inv_blocks.data(), inv_blocks.size() * sizeof(int2),
                           cudaMemcpyHostToDevice));
  if (!ltiles_tc.empty())
    TLR_CUDA(ctx, cudaMemcpy(d_ltiles_tc, ltiles_tc.data(), ltiles_tc.size() * sizeof(int4),
                             cudaMemcpyHostToDevice));
  if (!utiles_tc.empty())
    TLR_CUDA(ctx, cudaMemcpy(d_utiles_tc, utiles_tc.data(), utiles_tc.size() * sizeof(int4),
                             cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d_fronts, df.data(), nf * sizeof(DevFront), cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d_entries, sym.entries.data(), sym.entries.size() * sizeof(AsmEntry),
                           cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d_cmap, sym.cmap.data(), sym.cmap.size() * sizeof(int),
                           cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d_nodes, nodes.data(), nodes.size() * sizeof(int),
                           cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemcpy(d_sched, sched.data(), sched.size() * sizeof(int),
                           cudaMemcpyHostToDevice));
  return build_phases(ctx);
}

int Factor::build_phases(tlr_ctx *ctx) {
  std::vector<Phase> ph;
  for (size_t h = 0; h < levels.size(); ++h) {
    const Level &L = levels[h];
    ph.push_back({kPhGather, L.fronts_off, 0, blocks_for(L.max_m, 256), L.nfronts, 1, 0, 0});
    for (int b = 0; b < (int)L.blk_nf.size(); ++b)
      if (L.fwd_rows[b] > 0)
        ph.push_back({kPhFwd, L.fronts_off, b, blocks_for(L.fwd_rows[b], 32), L.blk_nf[b], 1, 0, 0});
  }
  for (int h = (int)levels.size() - 1; h >= 0; --h) {
    const Level &L = levels[h];
    if (L.bmax > 0)
      ph.push_back({kPhBorder, L.fronts_off, 0, blocks_for(L.pmax, 32), L.nck_b, L.nfronts,
                    L.nck_b, L.pmax});
    ph.push_back({kPhBwdStart, L.fronts_off, 0, (int)L.blk_nf.size() * (sw / 32), L.nfronts, 1,
                  L.nck_b, L.pmax});
    for (int b = (int)L.blk_nf.size() - 1; b >= 1; --b)
      ph.push_back({kPhBwd, L.fronts_off, b, blocks_for(b * sw, 32), L.blk_nf[b], 1, 0, 0});
  }
  nphases = (int)ph.size();
  cudaError_t e;
  if ((e = cudaMalloc(&d_phases, std::max<size_t>(ph.size(), 1) * sizeof(Phase))) != cudaSuccess ||
      (e = cudaMalloc(&d_barrier, sizeof(unsigned))) != cudaSuccess ||
      (e = cudaMalloc(&d_solve_err, sizeof(int))) != cudaSuccess)
    return fail(ctx, TLR_ERR_NOMEM, std::string("factor allocation failed: ") + cudaGetErrorString(e));
  TLR_CUDA(ctx, cudaMemcpy(d_phases, ph.data(), ph.size() * sizeof(Phase), cudaMemcpyHostToDevice));
  TLR_CUDA(ctx, cudaMemset(d_solve_err, 0, sizeof(int)));
  return TLR_OK;
}

int grid_barrier_probe(unsigned *count, unsigned limit, int *err) {
  { k_grid_barrier_probe<<<1, 32>>>(count, limit, err); count_launches(); }
  return cudaGetLastError() == cudaSuccess ? TLR_OK : TLR_ERR_CUDA;
}

int Factor::take_solve_error(tlr_ctx *ctx) {
  if (!d_solve_err) return TLR_OK;
  int h = 0;
  TLR_CUDA(ctx, cudaMemcpyAsync(&h, d_solve_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (!h) return TLR_OK;
  TLR_CUDA(ctx, cudaMemsetAsync(d_solve_err, 0, sizeof(int), ctx->stream));
  return fail(ctx, TLR_ERR_TIMEOUT, "triangular solve: a bounded wait between CTAs timed out");
}

template <class C, int SW>
int Factor::solve_persistent(tlr_ctx *ctx) {
  cudaStream_t st = ctx->stream;
  int grid = persist_grid;
  int dev = 0, sms = 0, occ = 0;
  TLR_CUDA(ctx, cudaGetDevice(&dev));
  TLR_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  TLR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_solve_persistent<C, SW>,
                                                               256, 0));
  const int cap = sms * std::max(occ, 1);
  if (grid <= 0) grid = 2 * sms;
  grid = std::max(1, std::min(grid, cap));
  const Phase *ph = d_phases;
  int np = nphases;
  const int *sc = d_sched;
  const C *P = static_cast<const C *>(pool);
  const DevFront *frp = d_fronts;
  const int *nd = d_nodes, *pm = d_perm;
  const int2 *ci = d_cinv;
  const long long *io = d_inv_off;
  const C *dm = static_cast<const C *>(dmat);
  C *W = static_cast<C *>(work), *W2 = static_cast<C *>(work2), *X = static_cast<C *>(vec_a);
  double2 *pa = d_partial;
  unsigned *bar = d_barrier;
  int *er = d_solve_err;
  void *args[] = {&ph, &np, &sc, &P, &frp, &nd, &pm, &ci, &io, &dm, &W, &W2, &pa, &X, &bar, &er};
  TLR_CUDA(ctx, cudaMemsetAsync(d_barrier, 0, sizeof(unsigned), st));
  TLR_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)k_solve_persistent<C, SW>, dim3(grid),
                                            dim3(256), args, 0, st));
  count_launches(1);
  return TLR_OK;
}

double Factor::take_solve_time(int *count) {
  double ms = 0.0;
  if (ev_used > 0) cudaEventSynchronize(ev_pool[ev_used - 1]);
  for (size_t i = 0; i + 1 < ev_used; i += 2) {
    float e = 0.f;
    if (cudaEventElapsedTime(&e, ev_pool[i], ev_pool[i + 1]) == cudaSuccess) ms += e;
  }
  if (count) *count = (int)(ev_used / 2);
  ev_used = 0;
  return ms;
}

void Factor::release() {
  for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
  ev_pool.clear();
  ev_used = 0;
  cudaFree(pool); cudaFree(work); cudaFree(d_fronts); cudaFree(d_entries);
  cudaFree(d_cmap); cudaFree(d_nodes); cudaFree(d_ipiv); cudaFree(d_perm);
  cudaFree(d_cinv); cudaFree(work2); cudaFree(d_sched); cudaFree(d_partial); cudaFree(d_pert); cudaFree(d_tc_err);
  cudaFree(vec_a); cudaFree(linv); cudaFree(uinv); cudaFree(dmat);
  cudaFree(d_inv_off); cudaFree(d_inv_blocks); cudaFree(d_ltiles); cudaFree(d_utiles);
  cudaFree(d_phases); cudaFree(d_barrier); cudaFree(d_solve_err); cudaFree(tc_planes);
  cudaFree(d_wave_tiles); cudaFree(d_wave_ctr); cudaFree(d_ltiles_tc); cudaFree(d_utiles_tc);
  d_ltiles_tc = d_utiles_tc = nullptr;
  d_wave_tiles = nullptr;
  d_wave_ctr = nullptr;
  tc_planes = nullptr;
  d_phases = nullptr;
  d_barrier = nullptr;
  d_solve_err = nullptr;
  linv = uinv = dmat = nullptr;
  d_ltiles = d_utiles = nullptr;
  d_inv_off = nullptr;
  d_inv_blocks = nullptr;
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  graph_exec = nullptr;
  pool = work = work2 = vec_a = nullptr;
  for (auto &g : graph_m) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  cudaFree(work_m); cudaFree(work2_m); cudaFree(vec_m); cudaFree(partial_m);
  work_m = work2_m = vec_m = nullptr;
  partial_m = nullptr;
  multi_cap = 0;
}

template <class C, int SW>
int Factor::rewrite_factors(tlr_ctx *ctx) {
  cudaStream_t st = ctx->stream;
  C *P = static_cast<C *>(pool);
  C *Li = static_cast<C *>(linv), *Ui = static_cast<C *>(uinv);
  { k_tri_inv<C, SW><<<dim3(n_inv_blocks, 2), SW, 0, st>>>(d_inv_blocks, P, d_fronts, d_inv_off,
                                                          Li, Ui); count_launches(); }
  if constexpr (sizeof(C) == sizeof(float2) && SW == 256) {
    if (tensor_cores)  // the products on the tensor cores, like the Schur updates
      return launch_rewrite_tc(ctx, d_ltiles_tc, n_ltiles_tc, d_utiles_tc, n_utiles_tc,
                               reinterpret_cast<float2 *>(P), d_fronts, d_inv_off,
                               reinterpret_cast<const float2 *>(Li),
                               reinterpret_cast<const float2 *>(Ui),
                               static_cast<float2 *>(dmat), d_tc_err, st);
  }
  const size_t ssm = sizeof(C) * SW * kRT;
  TLR_CUDA(ctx, cudaFuncSetAttribute(k_scale_u<C, SW>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm));
  TLR_CUDA(ctx, cudaFuncSetAttribute(k_scale_l<C, SW>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm));
  if (n_utiles > 0)
    { k_scale_u<C, SW><<<(unsigned)n_utiles, SW > 256 ? SW : 256, ssm, st>>>(d_utiles, P, d_fronts, d_inv_off, Li,
                                                            Ui, static_cast<C *>(dmat)); count_launches(); }
  if (n_ltiles > 0)
    { k_scale_l<C, SW><<<(unsigned)n_ltiles, 256, ssm, st>>>(d_ltiles, P, d_fronts, d_inv_off,
                                                            Li); count_launches(); }
  return TLR_OK;
}

template <class C>
int Factor::factor_impl(tlr_ctx *ctx, double sr, double si, double tiny) {
  cudaStream_t st = ctx->stream;
  C *P = static_cast<C *>(pool);
  TLR_CUDA(ctx, cudaMemsetAsync(d_pert, 0, sizeof(int), st));
  TLR_CUDA(ctx, cudaMemsetAsync(d_tc_err, 0, sizeof(int), st));
  const size_t tsm = sizeof(C) * (size_t)(w * w + w * 33);
  TLR_CUDA(ctx, cudaFuncSetAttribute(k_trsm_border<C>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
  TLR_CUDA(ctx, cudaFuncSetAttribute(k_trsm_urow<C>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
  TLR_CUDA(ctx, cudaFuncSetAttribute(k_panel_cluster_sm<C>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kPanelSmemMax));
  for (size_t h = 0; h < levels.size(); ++h) {
    const Level &L = levels[h];
    TLR_CUDA(ctx, cudaMemsetAsync(P + L.pool_begin, 0,
                                  (size_t)(L.pool_end - L.pool_begin) * sizeof(C), st));
    const long long ne = L.entry_end - L.entry_begin;
    if (ne > 0)
      { k_asm<C><<<blocks_for(ne * 25, 256), 256, 0, st>>>(d_entries + L.entry_begin, ne,
                                                         ctx->A, ctx->B, sr, si, P, d_fronts); count_launches(); }
    for (int slot = 0; slot < 2; ++slot) {
      if (!L.kids[slot]) continue;
      const long long mb = L.kids_maxb[slot];
      dim3 g((unsigned)std::min<long long>(std::max<long long>(blocks_for(mb * mb, 256), 1), 4096),
             L.kids[slot]);
      { k_extend<C><<<g, 256, 0, st>>>(d_sched + L.kids_off[slot], d_fronts, d_cmap, P); count_launches(); }
    }
    const int *fl = d_sched + L.fronts_off;
    for (int s = 0; s < (int)L.steps.size(); ++s) {
      const Step &S = L.steps[s];
      // the cluster panel pays off once the largest front still has many
      // fully summed rows; both give the same pivots and factors
      const int rem = L.pmax - s * w;
      const bool cluster = rem >= cluster_rows;
      // rows per CTA of the cluster (CTA 0: the top w rows)
      const int ldp = std::max(w, (rem + kPanelCluster - 2) / (kPanelCluster - 1));
      const size_t psm = (size_t)w * ldp * sizeof(C);
      if (cluster && psm <= kPanelSmemMax)
        { k_panel_cluster_sm<C><<<S.nf * kPanelCluster, 256, psm, st>>>(fl, s, w, P, d_fronts, d_ipiv, d_pert, tiny, ldp); count_launches(); }
      else if (cluster)
        { k_panel_cluster<C><<<S.nf * kPanelCluster, 256, 0, st>>>(fl, s, w, P, d_fronts, d_ipiv, d_pert, tiny); count_launches(); }
      else
        { k_panel<C><<<S.nf, 512, 0, st>>>(fl, s, w, P, d_fronts, d_ipiv, d_pert, tiny); count_launches(); }
      { k_swap<C><<<dim3(blocks_for(S.max_m, 128), S.nf), 128, 0, st>>>(fl, s, w, P, d_fronts,
                                                                       d_ipiv); count_launches(); }
      if (S.max_b > 0)
        { k_trsm_border<C><<<dim3(blocks_for(S.max_b, 32), S.nf), 256, tsm, st>>>(fl, s, w, P,
                                                                                 d_fronts); count_launches(); }
      if (S.max_ext > 0) {
        { k_trsm_urow<C><<<dim3(blocks_for(S.max_ext, 32), S.nf), 256, tsm, st>>>(fl, s, w, P,
                                                                                 d_fronts); count_launches(); }
        if (S.tiles > 0) {
          if constexpr (sizeof(C) == sizeof(float2)) {
            if (tensor_cores && tc_bulk) {
              const int rc = launch_gemm_tc_bulk(
                  ctx, fl, d_sched + S.prefix_off, d_sched + S.pa_off, d_sched + S.pb_off, S.nf,
                  s, w, reinterpret_cast<float2 *>(P), d_fronts, S.tiles, S.atiles, S.btiles,
                  tc_planes, d_tc_err, st, tc_variant);
              if (rc) return rc;
            } else if (tensor_cores) {
              const int rc = launch_gemm_tc(ctx, fl, d_sched + S.prefix_off, S.nf, s, w,
                                            reinterpret_cast<float2 *>(P), d_fronts, S.tiles,
                                            d_tc_err, st);
              if (rc) return rc;
            } else
              { k_gemm32<<<S.tiles, 256, 0, st>>>(fl, d_sched + S.prefix_off, S.nf, s, w,
                                                reinterpret_cast<float2 *>(P), d_fronts); count_launches(); }
          }
          else if (tensor_cores)
            { k_gemm_dmma<<<S.tiles, 256, 0, st>>>(fl, d_sched + S.prefix_off, S.nf, s, w,
                                                  reinterpret_cast<double2 *>(P), d_fronts); count_launches(); }
          else
            { k_gemm<C><<<S.tiles, 256, 0, st>>>(fl, d_sched + S.prefix_off, S.nf, s, w, P,
                                               d_fronts); count_launches(); }
        }
      }
    }
  }
  if (n_inv_blocks > 0) {
    int rc;
    if constexpr (sizeof(C) == sizeof(float2))
      rc = sw == 512   ? rewrite_factors<C, 512>(ctx)
           : sw == 256 ? rewrite_factors<C, 256>(ctx)
                       : rewrite_factors<C, 128>(ctx);
    else
      rc = rewrite_factors<C, 128>(ctx);
    if (rc) return rc;
  }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int Factor::factor(tlr_ctx *ctx, double sr, double si, double tiny) {
  int rc = prec == 0 ? factor_impl<double2>(ctx, sr, si, tiny)
                     : factor_impl<float2>(ctx, sr, si, tiny);
  if (rc) return rc;
  // row permutations of every front, and the children's maps through them
  std::vector<int> ipiv(sym.work_elems), perm(sym.work_elems), pmap(sym.work_elems, 0);
  TLR_CUDA(ctx, cudaMemcpyAsync(ipiv.data(), d_ipiv, ipiv.size() * sizeof(int),
                                cudaMemcpyDeviceToHost, ctx->stream));
  TLR_CUDA(ctx, cudaMemcpyAsync(&perturbed, d_pert, sizeof(int), cudaMemcpyDeviceToHost,
                                ctx->stream));
  int tc_err = 0;
  TLR_CUDA(ctx, cudaMemcpyAsync(&tc_err, d_tc_err, sizeof(int), cudaMemcpyDeviceToHost,
                                ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (tc_err)
    return fail(ctx, TLR_ERR_TIMEOUT,
                "tensor-core kernel of the factorisation: an mbarrier wait timed out");
  const int nf = (int)sym.fronts.size();
  std::vector<int> inv;
  for (int t = 0; t < nf; ++t) {
    const FrontInfo &f = sym.fronts[t];
    int *pr = perm.data() + f.toff;
    for (int i = 0; i < f.m; ++i) pr[i] = i;
    for (int c = 0; c < f.p; ++c) std::swap(pr[c], pr[ipiv[f.toff + c]]);
  }
  for (int t = 0; t < nf; ++t) {
    const FrontInfo &f = sym.fronts[t];
    if (f.parent < 0) continue;
    const FrontInfo &pf = sym.fronts[f.parent];
    inv.assign(pf.m, 0);
    for (int i = 0; i < pf.m; ++i) inv[perm[pf.toff + i]] = i;
    const int bc = f.m - f.p;
    for (int x = 0; x < bc; ++x) {
      const int q = sym.cmap[sym.cmap_off[t] + x / 5] * 5 + x % 5;
      pmap[f.toff + x] = inv[q];
    }
  }
  TLR_CUDA(ctx, cudaMemcpyAsync(d_perm, perm.data(), perm.size() * sizeof(int),
                                cudaMemcpyHostToDevice, ctx->stream));
  // per parent row, the work index of each child slot's border row mapped
  // onto it (the forward gather adds them in slot order)
  std::vector<int2> cinv(sym.work_elems, make_int2(-1, -1));
  for (int t = 0; t < nf; ++t) {
    const FrontInfo &f = sym.fronts[t];
    for (size_t slot = 0; slot < f.children.size() && slot < 2; ++slot) {
      const FrontInfo &c = sym.fronts[f.children[slot]];
      for (int x = 0; x < c.m - c.p; ++x) {
        int2 &e = cinv[f.toff + pmap[c.toff + x]];
        (slot == 0 ? e.x : e.y) = (int)(c.toff + c.p + x);
      }
    }
  }
  TLR_CUDA(ctx, cudaMemcpyAsync(d_cinv, cinv.data(), cinv.size() * sizeof(int2),
                                cudaMemcpyHostToDevice, ctx->stream));
  TLR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  factored = true;
  return TLR_OK;
}

template <class C, int SW>
int Factor::solve_impl(tlr_ctx *ctx, void *xv) {
  cudaStream_t st = ctx->stream;
  // programmatic dependent launch pays for the complex64 solve (about 7% at
  // 200 x 128) but not for the register-heavier complex128 kernels
  const bool pdl = sizeof(C) == sizeof(float2);
  const C *P = static_cast<const C *>(pool);
  C *W = static_cast<C *>(work);
  C *W2 = static_cast<C *>(work2);
  C *x = static_cast<C *>(xv);
  for (size_t h = 0; h < levels.size(); ++h) {
    const Level &L = levels[h];
    const int *fl = d_sched + L.fronts_off;
    // the first kernel follows a copy (or an event) node, not a kernel: no
    // programmatic edge for it
    TLR_CUDA(ctx, launch_pdl(pdl && h > 0, k_sgather<C>, dim3(blocks_for(L.max_m, 128), L.nfronts), dim3(128),
                             st, fl, (const DevFront *)d_fronts, (const int *)d_nodes,
                             (const int *)d_perm, (const int2 *)d_cinv, (const C *)x, W));
    count_launches();
    if (wave && L.wave) {
      TLR_CUDA(ctx, launch_pdl(pdl, k_wave<C, SW, false>, dim3(std::min(L.wf_n, wave_grid)),
                               dim3(256), st, fl, (const int4 *)(d_wave_tiles + L.wf_off), L.wf_n,
                               d_wave_ctr + L.wcf_off, L.wctr_n, L.maxblk, P,
                               (const DevFront *)d_fronts, W, (const int *)d_nodes, x,
                               d_solve_err));
      count_launches();
      continue;
    }
    for (int b = 0; b < (int)L.blk_nf.size(); ++b) {
      const int rows = L.fwd_rows[b];
      if (rows > 0) {
        TLR_CUDA(ctx, launch_pdl(pdl, k_blk_update<C, SW>, dim3(blocks_for(rows, 32), L.blk_nf[b]),
                                 dim3(256), st, fl, b, 0, P, (const DevFront *)d_fronts, W,
                                 (const int *)d_nodes, x));
        count_launches();
      }
    }
  }
  for (int h = (int)levels.size() - 1; h >= 0; --h) {
    const Level &L = levels[h];
    const int *fl = d_sched + L.fronts_off;
    if (L.bmax > 0) {
      const dim3 g(blocks_for(L.pmax, 32), L.nck_b, L.nfronts);
      if constexpr (sizeof(C) == sizeof(float2))
        TLR_CUDA(ctx, launch_pdl(pdl, k_border_gemv_pf, g, dim3(256), st, fl, P,
                                 (const DevFront *)d_fronts, (const int *)d_nodes, (const C *)x,
                                 d_partial, L.nck_b, L.pmax));
      else
        TLR_CUDA(ctx, launch_pdl(pdl, k_border_gemv<C>, g, dim3(256), st, fl, P,
                                 (const DevFront *)d_fronts, (const int *)d_nodes, (const C *)x,
                                 d_partial, L.nck_b, L.pmax));
      count_launches();
    }
    TLR_CUDA(ctx, launch_pdl(pdl, k_bwd_start<C, SW>,
                             dim3((unsigned)L.blk_nf.size() * (SW / 32), L.nfronts), dim3(256), st,
                             fl, (const DevFront *)d_fronts, (const long long *)d_inv_off,
                             static_cast<const C *>(dmat), (const C *)W, W2,
                             (const double2 *)d_partial, L.nck_b, L.pmax, (const int *)d_nodes,
                             x));
    count_launches();
    if (wave && L.wave) {
      TLR_CUDA(ctx, launch_pdl(pdl, k_wave<C, SW, true>, dim3(std::min(L.wb_n, wave_grid)),
                               dim3(256), st, fl, (const int4 *)(d_wave_tiles + L.wb_off), L.wb_n,
                               d_wave_ctr + L.wcb_off, L.wctr_n, L.maxblk, P,
                               (const DevFront *)d_fronts, W2, (const int *)d_nodes, x,
                               d_solve_err));
      count_launches();
      continue;
    }
    for (int b = (int)L.blk_nf.size() - 1; b >= 1; --b) {
      TLR_CUDA(ctx, launch_pdl(pdl, k_blk_update<C, SW>, dim3(blocks_for(b * SW, 32), L.blk_nf[b]),
                               dim3(256), st, fl, b, 1, P, (const DevFront *)d_fronts, W2,
                               (const int *)d_nodes, x));
      count_launches();
    }
  }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int Factor::enqueue_solve(tlr_ctx *ctx, void *x, cudaEvent_t a, cudaEvent_t b) {
  const size_t bytes = (size_t)sym.nn * 5 * (prec == 0 ? sizeof(double2) : sizeof(float2));
  cudaStream_t st = ctx->stream;
  TLR_CUDA(ctx, cudaMemcpyAsync(vec_a, x, bytes, cudaMemcpyDeviceToDevice, st));
  // external event nodes: the events are recorded (with time stamps) on
  // every replay of the caller's graph
  if (a) TLR_CUDA(ctx, cudaEventRecordWithFlags(a, st, cudaEventRecordExternal));
  const int rc = prec == 0 ? solve_impl<double2, 128>(ctx, vec_a)
                           : (sw == 512   ? solve_impl<float2, 512>(ctx, vec_a)
                              : sw == 256 ? solve_impl<float2, 256>(ctx, vec_a)
                                          : solve_impl<float2, 128>(ctx, vec_a));
  if (rc) return rc;
  if (b) TLR_CUDA(ctx, cudaEventRecordWithFlags(b, st, cudaEventRecordExternal));
  TLR_CUDA(ctx, cudaMemcpyAsync(x, vec_a, bytes, cudaMemcpyDeviceToDevice, st));
  return TLR_OK;
}

int Factor::solve(tlr_ctx *ctx, void *x) {
  const size_t bytes = (size_t)sym.nn * 5 * (prec == 0 ? sizeof(double2) : sizeof(float2));
  cudaStream_t st = ctx->stream;
  TLR_CUDA(ctx, cudaMemcpyAsync(vec_a, x, bytes, cudaMemcpyDeviceToDevice, st));
  if (persistent) {
    if (ev_used + 2 > ev_pool.size()) {
      cudaEvent_t a, b;
      TLR_CUDA(ctx, cudaEventCreate(&a));
      TLR_CUDA(ctx, cudaEventCreate(&b));
      ev_pool.push_back(a);
      ev_pool.push_back(b);
    }
    TLR_CUDA(ctx, cudaEventRecord(ev_pool[ev_used], st));
    const int rc = prec == 0 ? solve_persistent<double2, 128>(ctx)
                             : (sw == 512   ? solve_persistent<float2, 512>(ctx)
                                : sw == 256 ? solve_persistent<float2, 256>(ctx)
                                            : solve_persistent<float2, 128>(ctx));
    if (rc) return rc;
    TLR_CUDA(ctx, cudaEventRecord(ev_pool[ev_used + 1], st));
    ev_used += 2;
    TLR_CUDA(ctx, cudaMemcpyAsync(x, vec_a, bytes, cudaMemcpyDeviceToDevice, st));
    return TLR_OK;
  }
  if (!graph_exec) {
    TLR_CUDA(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc;
    {
      CaptureScope cs;
      rc = prec == 0 ? solve_impl<double2, 128>(ctx, vec_a)
                     : (sw == 512   ? solve_impl<float2, 512>(ctx, vec_a)
                        : sw == 256 ? solve_impl<float2, 256>(ctx, vec_a)
                                    : solve_impl<float2, 128>(ctx, vec_a));
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
    size_t nn = 0;
    graph_kernels = 0;
    if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn > 0) {
      std::vector<cudaGraphNode_t> nodes(nn);
      if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess)
        for (size_t i = 0; i < nn; ++i) {
          cudaGraphNodeType t;
          if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
            ++graph_kernels;
        }
    }
    const cudaError_t e2 = cudaGraphInstantiate(&graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "cudaGraphInstantiate");
  }
  if (ev_used + 2 > ev_pool.size()) {
    cudaEvent_t a, b;
    TLR_CUDA(ctx, cudaEventCreate(&a));
    TLR_CUDA(ctx, cudaEventCreate(&b));
    ev_pool.push_back(a);
    ev_pool.push_back(b);
  }
  TLR_CUDA(ctx, cudaEventRecord(ev_pool[ev_used], st));
  TLR_CUDA(ctx, cudaGraphLaunch(graph_exec, st));
  TLR_CUDA(ctx, cudaEventRecord(ev_pool[ev_used + 1], st));
  ev_used += 2;
  count_launches(graph_kernels);
  TLR_CUDA(ctx, cudaMemcpyAsync(x, vec_a, bytes, cudaMemcpyDeviceToDevice, st));
  return TLR_OK;
}

// ---- multi-RHS solve (host) ---------------------------------------------------
template <int SW, int NR>
int Factor::solve_impl_m(tlr_ctx *ctx) {
  cudaStream_t st = ctx->stream;
  const float2 *P = static_cast<const float2 *>(pool);
  float2 *W = static_cast<float2 *>(work_m);
  float2 *W2 = static_cast<float2 *>(work2_m);
  float2 *x = static_cast<float2 *>(vec_m);
  const long long xs = (long long)sym.nn * 5, ws = sym.work_elems, ps = partial_stride;
  for (size_t h = 0; h < levels.size(); ++h) {
    const Level &L = levels[h];
    const int *fl = d_sched + L.fronts_off;
    TLR_CUDA(ctx, launch_pdl(h > 0, k_sgather_m<NR>, dim3(blocks_for(L.max_m, 128), L.nfronts),
                             dim3(128), st, fl, (const DevFront *)d_fronts, (const int *)d_nodes,
                             (const int *)d_perm, (const int2 *)d_cinv, (const float2 *)x, xs, W,
                             ws));
    count_launches();
    for (int b = 0; b < (int)L.blk_nf.size(); ++b) {
      const int rows = L.fwd_rows[b];
      if (rows > 0) {
        TLR_CUDA(ctx, launch_pdl(true, k_blk_update_m<SW, NR>,
                                 dim3(blocks_for(rows, 32), L.blk_nf[b]), dim3(256), st, fl, b, 0,
                                 P, (const DevFront *)d_fronts, W, ws, (const int *)d_nodes, x,
                                 xs));
        count_launches();
      }
    }
  }
  for (int h = (int)levels.size() - 1; h >= 0; --h) {
    const Level &L = levels[h];
    const int *fl = d_sched + L.fronts_off;
    if (L.bmax > 0) {
      const dim3 g(blocks_for(L.pmax, 32), L.nck_b, L.nfronts);
      TLR_CUDA(ctx, launch_pdl(true, k_border_gemv_m<NR>, g, dim3(256), st, fl, P,
                               (const DevFront *)d_fronts, (const int *)d_nodes, (const float2 *)x,
                               xs, partial_m, ps, L.nck_b, L.pmax));
      count_launches();
    }
    TLR_CUDA(ctx, launch_pdl(true, k_bwd_start_m<SW, NR>,
                             dim3((unsigned)L.blk_nf.size() * (SW / 32), L.nfronts), dim3(256), st,
                             fl, (const DevFront *)d_fronts, (const long long *)d_inv_off,
                             static_cast<const float2 *>(dmat), (const float2 *)W, W2, ws,
                             (const double2 *)partial_m, ps, L.nck_b, L.pmax,
                             (const int *)d_nodes, x, xs));
    count_launches();
    for (int b = (int)L.blk_nf.size() - 1; b >= 1; --b) {
      TLR_CUDA(ctx, launch_pdl(true, k_blk_update_m<SW, NR>,
                               dim3(blocks_for(b * SW, 32), L.blk_nf[b]), dim3(256), st, fl, b, 1,
                               P, (const DevFront *)d_fronts, W2, ws, (const int *)d_nodes, x, xs));
      count_launches();
    }
  }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int Factor::solve_impl_m_dispatch(tlr_ctx *ctx, int nr) {
  switch (sw * 16 + nr) {
    case 128 * 16 + 2: return solve_impl_m<128, 2>(ctx);
    case 128 * 16 + 4: return solve_impl_m<128, 4>(ctx);
    case 128 * 16 + 8: return solve_impl_m<128, 8>(ctx);
    case 256 * 16 + 2: return solve_impl_m<256, 2>(ctx);
    case 256 * 16 + 4: return solve_impl_m<256, 4>(ctx);
    case 256 * 16 + 8: return solve_impl_m<256, 8>(ctx);
    default:
      return fail(ctx, TLR_ERR_ARG,
                  "multi-vector solves need 2, 4 or 8 vectors and diagonal blocks of 128 or 256");
  }
}

int Factor::solve_multi_prepare(tlr_ctx *ctx) {
  if (multi_cap >= kMaxRhs) return TLR_OK;
  // buffers for up to kMaxRhs vectors, allocated once per factor
  const size_t cs = sizeof(float2);
  const size_t we = (size_t)std::max<long long>(sym.work_elems, 1);
  TLR_CUDA(ctx, cudaMalloc(&work_m, (size_t)kMaxRhs * we * cs));
  TLR_CUDA(ctx, cudaMalloc(&work2_m, (size_t)kMaxRhs * we * cs));
  TLR_CUDA(ctx, cudaMalloc(&vec_m, (size_t)kMaxRhs * sym.nn * 5 * cs));
  TLR_CUDA(ctx, cudaMalloc(&partial_m, (size_t)kMaxRhs * partial_stride * sizeof(double2)));
  multi_cap = kMaxRhs;
  return TLR_OK;
}

int Factor::solve_multi(tlr_ctx *ctx, void *x, int nr, cudaEvent_t a, cudaEvent_t b,
                        bool capture) {
  if (prec != 1 || nr < 2 || nr > kMaxRhs || persistent)
    return fail(ctx, TLR_ERR_ARG, "multi-vector solves run on complex64 graph solves only");
  if (multi_cap < kMaxRhs) {
    if (capture) return fail(ctx, TLR_ERR_ARG, "multi-vector buffers must exist before capture");
    const int rc = solve_multi_prepare(ctx);
    if (rc) return rc;
  }
  const size_t bytes = (size_t)nr * sym.nn * 5 * sizeof(float2);
  cudaStream_t st = ctx->stream;
  TLR_CUDA(ctx, cudaMemcpyAsync(vec_m, x, bytes, cudaMemcpyDeviceToDevice, st));
  if (capture) {  // inside the caller's capture: enqueue the kernels directly
    if (a) TLR_CUDA(ctx, cudaEventRecordWithFlags(a, st, cudaEventRecordExternal));
    const int rc = solve_impl_m_dispatch(ctx, nr);
    if (rc) return rc;
    if (b) TLR_CUDA(ctx, cudaEventRecordWithFlags(b, st, cudaEventRecordExternal));
  } else {
    if (!graph_m[nr]) {
      TLR_CUDA(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      int rc;
      {
        CaptureScope cs;
        rc = solve_impl_m_dispatch(ctx, nr);
      }
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(st, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture (multi solve)");
      size_t nn = 0;
      graph_m_kernels[nr] = 0;
      if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn > 0) {
        std::vector<cudaGraphNode_t> nodes(nn);
        if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess)
          for (size_t i = 0; i < nn; ++i) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
              ++graph_m_kernels[nr];
          }
      }
      const cudaError_t e2 = cudaGraphInstantiate(&graph_m[nr], g, 0);
      cudaGraphDestroy(g);
      if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "cudaGraphInstantiate (multi solve)");
    }
    if (ev_used + 2 > ev_pool.size()) {
      cudaEvent_t e0, e1;
      TLR_CUDA(ctx, cudaEventCreate(&e0));
      TLR_CUDA(ctx, cudaEventCreate(&e1));
      ev_pool.push_back(e0);
      ev_pool.push_back(e1);
    }
    TLR_CUDA(ctx, cudaEventRecord(ev_pool[ev_used], st));
    TLR_CUDA(ctx, cudaGraphLaunch(graph_m[nr], st));
    TLR_CUDA(ctx, cudaEventRecord(ev_pool[ev_used + 1], st));
    ev_used += 2;
    count_launches(graph_m_kernels[nr]);
  }
  TLR_CUDA(ctx, cudaMemcpyAsync(x, vec_m, bytes, cudaMemcpyDeviceToDevice, st));
  return TLR_OK;
}

}  // namespace tlr
