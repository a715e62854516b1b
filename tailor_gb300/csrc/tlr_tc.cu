// tlr_tc.cu -- tensor-core (tcgen05) Schur-complement update of complex64
// fronts: F22 -= L21 U12 for one panel step of every front of a level.
//
// A complex product is a real product of doubled inner dimension:
//   A = [Lr | Li]            (128 rows  x 2K)
//   B = [Ur ; -Ui] -> Cr     (first 64 "rows" of the N x 2K operand)
//       [Ui ;  Ur] -> Ci     (last 64)
// so one 128 x 128 x 2K real MMA chain yields [Cr | Ci] for a 128 x 64
// complex tile.  FP32 accuracy on the TF32 pipe comes from the 3xTF32
// split (x = hi + lo, both TF32): A_lo B_hi + A_hi B_lo + A_hi B_hi,
// accumulated in FP32 in tensor memory.
//
// Per CTA (256 threads, one output tile): threads stage K chunks of 16
// complex columns (32 real) as TF32 hi/lo planes in shared memory in the
// canonical K-major no-swizzle layout (8-row x 16-byte core matrices),
// double-buffered; one thread issues tcgen05.mma (M = 128, N = 128, K = 8)
// and commits each chunk to an mbarrier; the accumulator lives in 128 TMEM
// columns and is read back with tcgen05.ld for the F22 -= epilogue.  Every
// mbarrier wait is bounded: on timeout the kernel records an error, waits
// (bounded) once more, frees its TMEM and returns.
#include <algorithm>
#include <cstdint>

#include "tlr_complex.cuh"
#include "tlr_internal.h"
#include "tlr_lu.h"

namespace tlr {
namespace {

constexpr int kTcM = 128;      // complex rows per tile
constexpr int kTcN = 64;       // complex columns per tile
constexpr int kTcKC = 8;       // complex K columns per stage (16 real: re | im)
constexpr int kPlane = 8192;   // bytes of one 128 x 16 TF32 operand plane
constexpr int kStage = 4 * kPlane;  // A_hi, A_lo, B_hi, B_lo
constexpr int kTmemCols = 128;
constexpr unsigned kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// byte offset of element (row, kk) of a 128 x 16 K-major plane: k-step
// kk/8 owns 4 KB; inside, 8-row group g at 256 g, the two core matrices of
// the k-step at +0 / +128, row r % 8 at 16 (r % 8), element kk % 4 at 4 (kk % 4)
__device__ __forceinline__ uint32_t plane_off(int row, int kk) {
  return (uint32_t)((kk >> 3) * 4096 + (row >> 3) * 256 + ((kk >> 2) & 1) * 128 + (row & 7) * 16 +
                    (kk & 3) * 4);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// kind::tf32, D f32, A/B tf32 K-major, M = 128, N = 128
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((128u >> 3) << 17) |
                            ((128u >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          unsigned limit = kWaitLimit) {
  for (unsigned it = 0; it < limit; ++it)
    if (mbar_test(bar, parity)) return true;
  return false;
}

// Bounded-wait check: one thread waits on an mbarrier that nothing will
// complete, with a short poll limit, and reports the timeout.
__global__ void k_mbar_timeout_probe(unsigned limit, int *err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0 && !mbar_wait(&bar, 0, limit)) atomicExch(err, 1);
}

#define TLR_TC_LD16(taddr, r)                                                                    \
  asm volatile(                                                                                  \
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14," \
      "%15}, [%16];"                                                                             \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),     \
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),              \
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])                                                    \
      : "r"(taddr))

#define TLR_TC_LD8(taddr, r)                                                                    \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"        \
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),        \
                 "=r"(r[6]), "=r"(r[7])                                                         \
               : "r"(taddr))

__global__ void __launch_bounds__(256)
    k_gemm_tc(const int *__restrict__ fl, const int *__restrict__ prefix, int nf, int s, int w,
              float2 *__restrict__ pool, const DevFront *__restrict__ fr, int *__restrict__ err,
              uint32_t lbo, uint32_t sbo) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int wait_ok;
  unsigned char *stage0 =
      tc_smem + ((1024 - (smem_addr(tc_smem) & 1023)) & 1023);  // 1 KB aligned
  const int tid = threadIdx.x, warp = tid >> 5;

  // tile decode (same schedule as the CUDA-core kernel: 128 x 64 tiles)
  const int t = blockIdx.x;
  int lo = 0, hi = nf;
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  const DevFront f = fr[fl[lo]];
  const int m = f.m, k0 = s * w, ww = min(w, f.p - k0);
  const int base = k0 + ww, ext = m - base;
  const int ntm = (ext + kTcM - 1) / kTcM;
  const int lt = t - prefix[lo];
  const int R0 = base + (lt % ntm) * kTcM, C0 = base + (lt / ntm) * kTcN;
  float2 *F = pool + f.off;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  const int nch = (ww + kTcKC - 1) / kTcKC;
  // A: thread (row ar, quad aq) stages complex columns 4 aq .. 4 aq + 3 of
  // the chunk; B: thread (column bn, quad bq) stages K rows 4 bq .. 4 bq + 3
  // (threads 128..255 take the second 64 of nothing: B has 64 x 2 quads).
  const int ar = tid & (kTcM - 1), aq = tid >> 7;
  const int bn = tid & 63, bq = (tid >> 6) & 1;
  const bool bact = tid < 128;
  float2 va[4], vb[4];
  auto load = [&](int c) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int kc = c * kTcKC + 4 * aq + j;
      va[j] = (R0 + ar < m && kc < ww) ? F[(long long)(k0 + kc) * m + R0 + ar]
                                        : make_float2(0.f, 0.f);
      const int kb = c * kTcKC + 4 * bq + j;
      vb[j] = (bact && C0 + bn < m && kb < ww) ? F[(long long)(C0 + bn) * m + k0 + kb]
                                               : make_float2(0.f, 0.f);
    }
  };
  auto split4 = [](const float *x, uint4 &hi4, uint4 &lo4) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      h[j] = to_tf32(x[j]);
      l[j] = to_tf32(x[j] - __uint_as_float(h[j]));
    }
    hi4 = make_uint4(h[0], h[1], h[2], h[3]);
    lo4 = make_uint4(l[0], l[1], l[2], l[3]);
  };
  auto store = [&](unsigned char *st) {
    float re[4], im[4];
    uint4 h, l;
#pragma unroll
    for (int j = 0; j < 4; ++j) { re[j] = va[j].x; im[j] = va[j].y; }
    // A row ar: K' 4 aq .. +3 = Lr, K' 8 + 4 aq .. +3 = Li
    split4(re, h, l);
    *reinterpret_cast<uint4 *>(st + plane_off(ar, 4 * aq)) = h;
    *reinterpret_cast<uint4 *>(st + kPlane + plane_off(ar, 4 * aq)) = l;
    split4(im, h, l);
    *reinterpret_cast<uint4 *>(st + plane_off(ar, 8 + 4 * aq)) = h;
    *reinterpret_cast<uint4 *>(st + kPlane + plane_off(ar, 8 + 4 * aq)) = l;
    if (bact) {
      unsigned char *bh = st + 2 * kPlane, *bl = st + 3 * kPlane;
      float ur[4], ui[4], nui[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) { ur[j] = vb[j].x; ui[j] = vb[j].y; nui[j] = -vb[j].y; }
      // Cr row bn: [Ur ; -Ui]; Ci row 64 + bn: [Ui ; Ur]
      split4(ur, h, l);
      *reinterpret_cast<uint4 *>(bh + plane_off(bn, 4 * bq)) = h;
      *reinterpret_cast<uint4 *>(bl + plane_off(bn, 4 * bq)) = l;
      *reinterpret_cast<uint4 *>(bh + plane_off(64 + bn, 8 + 4 * bq)) = h;
      *reinterpret_cast<uint4 *>(bl + plane_off(64 + bn, 8 + 4 * bq)) = l;
      split4(nui, h, l);
      *reinterpret_cast<uint4 *>(bh + plane_off(bn, 8 + 4 * bq)) = h;
      *reinterpret_cast<uint4 *>(bl + plane_off(bn, 8 + 4 * bq)) = l;
      split4(ui, h, l);
      *reinterpret_cast<uint4 *>(bh + plane_off(64 + bn, 4 * bq)) = h;
      *reinterpret_cast<uint4 *>(bl + plane_off(64 + bn, 4 * bq)) = l;
    }
  };
  bool ok = true;
  if (nch > 0) load(0);
  for (int c = 0; c < nch; ++c) {
    const int sb = c & 1;
    unsigned char *st = stage0 + sb * kStage;
    if (c >= 2) {  // the MMAs of chunk c - 2 read this buffer
      if (tid == 0) wait_ok = mbar_wait(&bars[sb], ((c - 2) >> 1) & 1);
      __syncthreads();
      if (!wait_ok) {
        ok = false;
        break;
      }
    }
    store(st);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a_hi = smem_addr(st), a_lo = a_hi + kPlane;
      const uint32_t b_hi = a_hi + 2 * kPlane, b_lo = a_hi + 3 * kPlane;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const uint32_t o = j * 4096;
        const uint32_t acc0 = (c > 0 || j > 0) ? 1u : 0u;
        mma_tf32(tmem, smem_desc(a_lo + o, lbo, sbo), smem_desc(b_hi + o, lbo, sbo), acc0);
        mma_tf32(tmem, smem_desc(a_hi + o, lbo, sbo), smem_desc(b_lo + o, lbo, sbo), 1u);
        mma_tf32(tmem, smem_desc(a_hi + o, lbo, sbo), smem_desc(b_hi + o, lbo, sbo), 1u);
      }
      mma_commit(&bars[sb]);
    }
    if (c + 1 < nch) load(c + 1);  // next chunk's loads overlap these MMAs
  }
  if (tid == 0) {
    // the last commit covers every MMA of the tile
    int fine = ok && nch > 0 ? mbar_wait(&bars[(nch - 1) & 1], ((nch - 1) >> 1) & 1) : ok;
    if (!fine) {
      atomicExch(err, 1);
      // let any MMA still in flight land before the memory is released
      if (nch > 0) mbar_wait(&bars[(nch - 1) & 1], ((nch - 1) >> 1) & 1);
    }
    wait_ok = fine;
  }
  __syncthreads();
  ok = wait_ok != 0;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (ok) {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (tile rows), column
    // half w / 4 of Cr (TMEM columns 0..63) and Ci (64..127)
    const int q = warp & 3, h = warp >> 2;
    const int row = 32 * q + (tid & 31);
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      uint32_t cr[16], ci[16];
      const int n0 = 32 * h + 16 * part;
      TLR_TC_LD16(lane_addr + n0, cr);
      TLR_TC_LD16(lane_addr + 64 + n0, ci);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (R0 + row < m) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = n0 + j;
          if (C0 + n < m) {
            float2 &d = F[(long long)(C0 + n) * m + R0 + row];
            d.x -= __uint_as_float(cr[j]);
            d.y -= __uint_as_float(ci[j]);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
}

// ---- operand planes in global memory, bulk-copy Schur update -------------
// The update above converts every operand chunk into TF32 hi/lo planes once
// per output tile, so each row tile of L21 is converted once per column
// tile and vice versa, and the global loads feeding that conversion stall
// the warps.  Here the conversion runs once per panel step: k_tc_split
// writes, for every 128-row tile of L21 and every 64-column tile of U12 of
// every front of the step, each K chunk as a 16 KB image [hi plane | lo
// plane] in exactly the shared-memory layout the MMA descriptors expect.
// k_gemm_tc_bulk then streams those images into a three-stage shared
// memory ring with cp.async.bulk (one thread issues the copies and the
// MMAs; completion by mbarrier transaction counts), while the other
// threads prefetch the F22 tile into registers for the epilogue.
constexpr int kChunkImg = 2 * kPlane;  // one operand chunk: hi + lo planes
constexpr int kBulkStages = 3;  // the default ring: three stages, two CTAs per SM

__device__ __forceinline__ int find_front(const int *__restrict__ prefix, int nf, int t) {
  int lo = 0, hi = nf;
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

// grid (atiles + btiles, nchmax): blockIdx.x < atiles is A tile
// (front, 128-row tile), else B tile (front, 64-column tile); blockIdx.y is
// the K chunk.  pa / pb: per-front prefix of A / B tiles (nf + 1 each).
__global__ void __launch_bounds__(256)
    k_tc_split(const int *__restrict__ fl, const int *__restrict__ pa, const int *__restrict__ pb,
               int nf, int s, int w, const float2 *__restrict__ pool,
               const DevFront *__restrict__ fr, unsigned char *__restrict__ planes, int atiles,
               int nchmax) {
  const int tid = threadIdx.x, c = blockIdx.y;
  const bool is_a = (int)blockIdx.x < atiles;
  const int t = is_a ? blockIdx.x : blockIdx.x - atiles;
  const int lo = find_front(is_a ? pa : pb, nf, t);
  const DevFront f = fr[fl[lo]];
  const int m = f.m, k0 = s * w, ww = min(w, f.p - k0);
  const int base = k0 + ww;
  if (c * kTcKC >= ww) return;  // this front has fewer chunks
  const float2 *F = pool + f.off;
  unsigned char *img = planes + ((long long)blockIdx.x * nchmax + c) * kChunkImg;
  auto split4 = [](const float *x, uint4 &hi4, uint4 &lo4) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      h[j] = to_tf32(x[j]);
      l[j] = to_tf32(x[j] - __uint_as_float(h[j]));
    }
    hi4 = make_uint4(h[0], h[1], h[2], h[3]);
    lo4 = make_uint4(l[0], l[1], l[2], l[3]);
  };
  uint4 h, l;
  if (is_a) {
    // rows R0 + ar, complex columns 4 aq .. 4 aq + 3 of the chunk
    const int R0 = base + (t - pa[lo]) * kTcM;
    const int ar = tid & (kTcM - 1), aq = tid >> 7;
    float re[4], im[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int kc = c * kTcKC + 4 * aq + j;
      const float2 v = (R0 + ar < m && kc < ww) ? F[(long long)(k0 + kc) * m + R0 + ar]
                                                 : make_float2(0.f, 0.f);
      re[j] = v.x;
      im[j] = v.y;
    }
    split4(re, h, l);
    *reinterpret_cast<uint4 *>(img + plane_off(ar, 4 * aq)) = h;
    *reinterpret_cast<uint4 *>(img + kPlane + plane_off(ar, 4 * aq)) = l;
    split4(im, h, l);
    *reinterpret_cast<uint4 *>(img + plane_off(ar, 8 + 4 * aq)) = h;
    *reinterpret_cast<uint4 *>(img + kPlane + plane_off(ar, 8 + 4 * aq)) = l;
  } else if (tid < 128) {
    // columns C0 + bn, K rows 4 bq .. 4 bq + 3 of the chunk:
    // Cr row bn: [Ur ; -Ui]; Ci row 64 + bn: [Ui ; Ur]
    const int C0 = base + (t - pb[lo]) * kTcN;
    const int bn = tid & 63, bq = tid >> 6;
    float ur[4], ui[4], nui[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int kb = c * kTcKC + 4 * bq + j;
      const float2 v = (C0 + bn < m && kb < ww) ? F[(long long)(C0 + bn) * m + k0 + kb]
                                                 : make_float2(0.f, 0.f);
      ur[j] = v.x;
      ui[j] = v.y;
      nui[j] = -v.y;
    }
    unsigned char *bh = img, *bl = img + kPlane;
    split4(ur, h, l);
    *reinterpret_cast<uint4 *>(bh + plane_off(bn, 4 * bq)) = h;
    *reinterpret_cast<uint4 *>(bl + plane_off(bn, 4 * bq)) = l;
    *reinterpret_cast<uint4 *>(bh + plane_off(64 + bn, 8 + 4 * bq)) = h;
    *reinterpret_cast<uint4 *>(bl + plane_off(64 + bn, 8 + 4 * bq)) = l;
    split4(nui, h, l);
    *reinterpret_cast<uint4 *>(bh + plane_off(bn, 8 + 4 * bq)) = h;
    *reinterpret_cast<uint4 *>(bl + plane_off(bn, 8 + 4 * bq)) = l;
    split4(ui, h, l);
    *reinterpret_cast<uint4 *>(bh + plane_off(64 + bn, 4 * bq)) = h;
    *reinterpret_cast<uint4 *>(bl + plane_off(64 + bn, 4 * bq)) = l;
  }
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// global -> shared bulk copy of `bytes` (16-byte aligned addresses, size a
// multiple of 16), completing `bytes` transactions on bar
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// S: ring stages (shared memory S x 32 KB), MINB: CTAs per SM the register
// budget must allow, PF: F22 columns per thread prefetched during the MMAs
// (the rest is read in the epilogue)
template <int S, int MINB, int PF>
__global__ void __launch_bounds__(256, MINB)
    k_gemm_tc_bulk(const int *__restrict__ fl, const int *__restrict__ prefix,
                   const int *__restrict__ pa, const int *__restrict__ pb, int nf, int s, int w,
                   float2 *__restrict__ pool, const DevFront *__restrict__ fr,
                   const unsigned char *__restrict__ planes_a,
                   const unsigned char *__restrict__ planes_b, int nchmax, int *__restrict__ err,
                   uint32_t lbo, uint32_t sbo) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t full[S], empty[S];
  __shared__ uint32_t tmem_slot;
  __shared__ int wait_ok;
  unsigned char *ring = tc_smem + ((1024 - (smem_addr(tc_smem) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5;

  const int t = blockIdx.x;
  const int lo = find_front(prefix, nf, t);
  const DevFront f = fr[fl[lo]];
  const int m = f.m, k0 = s * w, ww = min(w, f.p - k0);
  const int base = k0 + ww, ext = m - base;
  const int ntm = (ext + kTcM - 1) / kTcM;
  const int lt = t - prefix[lo];
  const int rt = lt % ntm, ct = lt / ntm;
  const int R0 = base + rt * kTcM, C0 = base + ct * kTcN;
  float2 *F = pool + f.off;
  const int nch = (ww + kTcKC - 1) / kTcKC;
  const unsigned char *ga = planes_a + (long long)(pa[lo] + rt) * nchmax * kChunkImg;
  const unsigned char *gb = planes_b + (long long)(pb[lo] + ct) * nchmax * kChunkImg;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int q = 0; q < S; ++q) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&full[q])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&empty[q])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  auto issue = [&](int c) {  // chunk c into stage c % S
    unsigned char *st = ring + (c % S) * kStage;
    uint64_t *bar = &full[c % S];
    mbar_expect_tx(bar, 2 * kChunkImg);
    bulk_g2s(st, ga + (long long)c * kChunkImg, kChunkImg, bar);
    bulk_g2s(st + kChunkImg, gb + (long long)c * kChunkImg, kChunkImg, bar);
  };
  int issued = 0;
  if (tid == 0)
    for (; issued < nch && issued < S; ++issued) issue(issued);

  // the F22 entries of the epilogue: warp w owns tile rows 32 (w % 4) + lane
  // and the 32 columns 32 (w / 4) .. +31.  Warps 1..7 fetch theirs while the
  // operands stream in; warp 0, whose first thread drives the copies and
  // MMAs, fetches after them (keeping its registers free for that loop).
  const int q4 = warp & 3, h2 = warp >> 2;
  const int row = 32 * q4 + (tid & 31);
  const bool row_ok = R0 + row < m;
  float2 f22[PF > 0 ? PF : 1];
  auto fetch_f22 = [&]() {
#pragma unroll
    for (int j = 0; j < PF; ++j) {
      const int n = 32 * h2 + j;
      f22[j] = (row_ok && C0 + n < m) ? F[(long long)(C0 + n) * m + R0 + row]
                                      : make_float2(0.f, 0.f);
    }
  };
  if (warp != 0) fetch_f22();

  if (tid == 0) {
    bool ok = true;
    int done = 0;  // chunks whose MMAs were issued
    for (int c = 0; c < nch && ok; ++c) {
      const int sb = c % S;
      if (!mbar_wait(&full[sb], (c / S) & 1)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a_hi = smem_addr(ring + sb * kStage), a_lo = a_hi + kPlane;
      const uint32_t b_hi = a_hi + 2 * kPlane, b_lo = a_hi + 3 * kPlane;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const uint32_t o = j * 4096;
        const uint32_t acc0 = (c > 0 || j > 0) ? 1u : 0u;
        mma_tf32(tmem, smem_desc(a_lo + o, lbo, sbo), smem_desc(b_hi + o, lbo, sbo), acc0);
        mma_tf32(tmem, smem_desc(a_hi + o, lbo, sbo), smem_desc(b_lo + o, lbo, sbo), 1u);
        mma_tf32(tmem, smem_desc(a_hi + o, lbo, sbo), smem_desc(b_hi + o, lbo, sbo), 1u);
      }
      mma_commit(&empty[sb]);
      done = c + 1;
      if (issued < nch) {  // refill this stage once its MMAs have read it
        if (!mbar_wait(&empty[sb], (c / S) & 1)) {
          ok = false;
          break;
        }
        issue(issued++);
      }
    }
    // the last commit covers every MMA issued before it
    bool fine = ok && done == nch &&
                (nch == 0 || mbar_wait(&empty[(nch - 1) % S],
                                       ((nch - 1) / S) & 1));
    if (!fine) {
      atomicExch(err, 1);
      // let copies and MMAs still in flight land before the memory is
      // released: every issued chunk's copy, then the last commit
      for (int c = done; c < issued; ++c)
        mbar_wait(&full[c % S], (c / S) & 1);
      if (done > 0)
        mbar_wait(&empty[(done - 1) % S], ((done - 1) / S) & 1);
    }
    wait_ok = fine;
  }
  __syncthreads();
  const bool ok = wait_ok != 0;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0) fetch_f22();
  if (ok) {
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * q4) << 16);
#pragma unroll
    for (int part = 0; part < 4; ++part) {
      uint32_t cr[8], ci[8];
      const int n0 = 32 * h2 + 8 * part;
      TLR_TC_LD8(lane_addr + n0, cr);
      TLR_TC_LD8(lane_addr + 64 + n0, ci);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row_ok) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int n = n0 + j;
          if (C0 + n < m) {
            float2 d;
            if (8 * part + j < PF)
              d = f22[(8 * part + j) % (PF > 0 ? PF : 1)];
            else
              d = F[(long long)(C0 + n) * m + R0 + row];
            d.x -= __uint_as_float(cr[j]);
            d.y -= __uint_as_float(ci[j]);
            F[(long long)(C0 + n) * m + R0 + row] = d;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
}

// Persistent, warp-specialised variant of k_gemm_tc_bulk.  In the kernel
// above a CTA stages one tile's operands, runs its MMAs and then reads the
// accumulator back for the F22 update, so the copies, the tensor pipe and
// the epilogue of one CTA never overlap.  Here one CTA per SM walks the
// tiles blockIdx.x, blockIdx.x + gridDim.x, ... with three roles:
//   warp 8 (one thread): bulk copies of every chunk of every tile into the
//     S-stage ring (full[] / empty[] mbarriers);
//   warp 9 (one thread): the MMAs of a tile into one of two TMEM
//     accumulators (128 columns each), committing the ring stages (empty[])
//     and, after the tile's last chunk, the accumulator (tfull[]);
//   warps 0..7: the epilogue.  Warp w owns tile rows 32 (w % 4) + lane
//     (its TMEM lane quarter) and the 32 complex columns 32 (w / 4) .. +31;
//     it loads its F22 entries of a tile before that tile's accumulator is
//     ready, then subtracts the accumulator and releases it (tempty[]),
//     while the MMAs of the next tile run on the other accumulator.
// The MMAs and the epilogue arithmetic are those of k_gemm_tc_bulk, so the
// factors are bitwise the same.  Every wait is bounded: a wait that runs
// out raises the error flag and the CTA's abort word, every role stops
// waiting, and the copies and MMAs already issued are awaited (bounded)
// before TMEM is released.
constexpr int kPersistThreads = 320;

template <int S>
__global__ void __launch_bounds__(kPersistThreads, 1)
    k_gemm_tc_persist(const int *__restrict__ fl, const int *__restrict__ prefix,
                      const int *__restrict__ pa, const int *__restrict__ pb, int nf, int s, int w,
                      int tiles, float2 *__restrict__ pool, const DevFront *__restrict__ fr,
                      const unsigned char *__restrict__ planes_a,
                      const unsigned char *__restrict__ planes_b, int nchmax,
                      int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t full[S], empty[S], tfull[2], tempty[2];
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  __shared__ int issued_g, consumed_g, committed_g;  // chunk counters at exit
  unsigned char *ring = tc_smem + ((1024 - (smem_addr(tc_smem) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 8) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(&tmem_slot)),
                 "r"(256));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int q = 0; q < S; ++q) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&full[q])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&empty[q])));
    }
    for (int q = 0; q < 2; ++q) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&tfull[q])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 8;" ::"r"(smem_addr(&tempty[q])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
    issued_g = consumed_g = committed_g = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  // tile t -> front, its first row / column and the operand images
  struct Tile {
    float2 *F;
    int m, R0, C0, nch;
    const unsigned char *ga, *gb;
  };
  auto decode = [&](int t) {
    Tile d;
    const int lo = find_front(prefix, nf, t);
    const DevFront f = fr[fl[lo]];
    const int k0 = s * w, ww = min(w, f.p - k0);
    const int base = k0 + ww, ext = f.m - base;
    const int ntm = (ext + kTcM - 1) / kTcM;
    const int lt = t - prefix[lo];
    const int rt = lt % ntm, ct = lt / ntm;
    d.F = pool + f.off;
    d.m = f.m;
    d.R0 = base + rt * kTcM;
    d.C0 = base + ct * kTcN;
    d.nch = (ww + kTcKC - 1) / kTcKC;
    d.ga = planes_a + (long long)(pa[lo] + rt) * nchmax * kChunkImg;
    d.gb = planes_b + (long long)(pb[lo] + ct) * nchmax * kChunkImg;
    return d;
  };
  // bounded wait that also gives up once another role has aborted
  auto wait_bar = [&](uint64_t *bar, uint32_t parity) -> bool {
    for (unsigned it = 0; it < kWaitLimit; ++it) {
      if (mbar_test(bar, parity)) return true;
      if (abort_flag) return false;
    }
    abort_flag = 1;
    atomicExch(err, 1);
    return false;
  };

  if (warp == 8) {
    if (lane == 0) {  // producer
      int g = 0;
      for (int t = blockIdx.x; t < tiles && !abort_flag; t += gridDim.x) {
        const Tile d = decode(t);
        for (int c = 0; c < d.nch; ++c, ++g) {
          const int st = g % S;
          if (g >= S && !wait_bar(&empty[st], ((g / S) & 1) ^ 1)) break;
          unsigned char *dst = ring + st * kStage;
          mbar_expect_tx(&full[st], 2 * kChunkImg);
          bulk_g2s(dst, d.ga + (long long)c * kChunkImg, kChunkImg, &full[st]);
          bulk_g2s(dst + kChunkImg, d.gb + (long long)c * kChunkImg, kChunkImg, &full[st]);
        }
      }
      issued_g = g;
    }
  } else if (warp == 9) {
    if (lane == 0) {  // MMA issuer
      int g = 0, ti = 0, committed = 0;
      for (int t = blockIdx.x; t < tiles && !abort_flag; t += gridDim.x, ++ti) {
        const Tile d = decode(t);
        const int acc = ti & 1;
        if (ti >= 2 && !wait_bar(&tempty[acc], ((ti >> 1) - 1) & 1)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t tacc = tmem + 128 * acc;
        bool ok = true;
        for (int c = 0; c < d.nch; ++c, ++g) {
          const int st = g % S;
          if (!wait_bar(&full[st], (g / S) & 1)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t a_hi = smem_addr(ring + st * kStage), a_lo = a_hi + kPlane;
          const uint32_t b_hi = a_hi + 2 * kPlane, b_lo = a_hi + 3 * kPlane;
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const uint32_t o = j * 4096;
            const uint32_t acc0 = (c > 0 || j > 0) ? 1u : 0u;
            mma_tf32(tacc, smem_desc(a_lo + o, 128u, 256u), smem_desc(b_hi + o, 128u, 256u), acc0);
            mma_tf32(tacc, smem_desc(a_hi + o, 128u, 256u), smem_desc(b_lo + o, 128u, 256u), 1u);
            mma_tf32(tacc, smem_desc(a_hi + o, 128u, 256u), smem_desc(b_hi + o, 128u, 256u), 1u);
          }
          mma_commit(&empty[st]);
          committed = g + 1;
        }
        if (!ok) break;
        mma_commit(&tfull[acc]);  // covers every MMA of the tile
      }
      consumed_g = g;
      committed_g = committed;
    }
  } else {  // epilogue, warps 0..7
    const int q4 = warp & 3, h2 = warp >> 2;
    const int row = 32 * q4 + lane;
    int ti = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++ti) {
      const Tile d = decode(t);
      const int acc = ti & 1;
      const bool row_ok = d.R0 + row < d.m;
      // this tile's F22 entries, fetched while its MMAs run
      float2 f22[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int n = 32 * h2 + j;
        f22[j] = (row_ok && d.C0 + n < d.m) ? d.F[(long long)(d.C0 + n) * d.m + d.R0 + row]
                                            : make_float2(0.f, 0.f);
      }
      bool ok = true;
      if (lane == 0) ok = wait_bar(&tfull[acc], (ti >> 1) & 1);
      ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t lane_addr = tmem + 128 * acc + ((uint32_t)(32 * q4) << 16);
#pragma unroll
      for (int part = 0; part < 4; ++part) {
        uint32_t cr[8], ci[8];
        const int n0 = 32 * h2 + 8 * part;
        TLR_TC_LD8(lane_addr + n0, cr);
        TLR_TC_LD8(lane_addr + 64 + n0, ci);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row_ok) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int n = n0 + j;
            if (d.C0 + n < d.m) {
              float2 v = f22[8 * part + j];
              v.x -= __uint_as_float(cr[j]);
              v.y -= __uint_as_float(ci[j]);
              d.F[(long long)(d.C0 + n) * d.m + d.R0 + row] = v;
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&tempty[acc]))
                     : "memory");
    }
  }
  __syncthreads();
  if (tid == 0 && abort_flag) {
    // let the copies and MMAs already issued land before TMEM is released
    for (int g = consumed_g; g < issued_g; ++g) mbar_wait(&full[g % S], (g / S) & 1);
    if (committed_g > 0) mbar_wait(&empty[(committed_g - 1) % S], ((committed_g - 1) / S) & 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 8)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
}

}  // namespace

size_t gemm_tc_smem() { return 2 * kStage + 1024; }

size_t gemm_tc_bulk_smem(int stages) { return stages * kStage + 1024; }
size_t tc_chunk_image_bytes() { return kChunkImg; }

namespace {

// ---- factor rewrite on the tensor cores -------------------------------------
// The block-scaled solves need L' = L inv(L_bb) below every 256-row diagonal
// block, U' = inv(U_bb) U right of it and D_b = inv(U_bb) inv(L_bb).  On the
// CUDA cores each output entry costs about 128 complex FMAs, every one fed by
// a load of the inverse (k_scale_l / k_scale_u).  Here the same products run
// as tcgen05 MMAs with the 3xTF32 split and FP32 accumulation in TMEM, the
// operands staged per 8-column K chunk as in k_gemm_tc.  Each CTA owns a
// whole output band and writes it only after its last MMA has read the
// band, so the rewrite stays in place.  The inverses are triangular: output
// tiles that only see zeros of a chunk skip its MMAs.
//   k_scale_l_tc: CTA = 128 rows below block b; C (128 x nb) = L(rows,
//     block) inv(L_bb) as four 64-column tiles in 512 TMEM columns; tile t
//     needs K rows q >= 64 t only (inv(L_bb) is lower triangular).
//   k_scale_u_tc: CTA = 64 columns: kind 0 right of block b, in place
//     (X = U(block rows, cols)); kind 1 of D_b (X = inv(L_bb), written to
//     dmat); C (nb x 64) = inv(U_bb) X as two 128-row tiles in 256 TMEM
//     columns; the second needs K columns q >= 128 only (inv(U_bb) is upper
//     triangular).
// tiles: {front, block, first row (L) / first column (U), kind}.
constexpr int kRwSW = 256;                          // diagonal-block size
constexpr int kRwLStage = 10 * kPlane;              // A hi/lo + four B tiles hi/lo
constexpr int kRwUStage = 6 * kPlane;               // two A tiles hi/lo + B hi/lo

__device__ __forceinline__ void split4_tf32(const float *x, uint4 &hi4, uint4 &lo4) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    h[j] = to_tf32(x[j]);
    l[j] = to_tf32(x[j] - __uint_as_float(h[j]));
  }
  hi4 = make_uint4(h[0], h[1], h[2], h[3]);
  lo4 = make_uint4(l[0], l[1], l[2], l[3]);
}

// A-operand row `row` of a 128-row plane pair: K' 4 q4 .. +3 real parts and
// 8 + 4 q4 .. +3 imaginary parts of four complex K entries
__device__ __forceinline__ void stage_a4(unsigned char *hi, int row, int q4, const float2 *v) {
  float re[4], im[4];
  uint4 h, l;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    re[j] = v[j].x;
    im[j] = v[j].y;
  }
  split4_tf32(re, h, l);
  *reinterpret_cast<uint4 *>(hi + plane_off(row, 4 * q4)) = h;
  *reinterpret_cast<uint4 *>(hi + kPlane + plane_off(row, 4 * q4)) = l;
  split4_tf32(im, h, l);
  *reinterpret_cast<uint4 *>(hi + plane_off(row, 8 + 4 * q4)) = h;
  *reinterpret_cast<uint4 *>(hi + kPlane + plane_off(row, 8 + 4 * q4)) = l;
}

// B-operand column bn of a 64-column output tile (planes of 128 "rows":
// Cr row bn = [Br ; -Bi], Ci row 64 + bn = [Bi ; Br]) for four complex K
// entries 4 q4 .. +3
__device__ __forceinline__ void stage_b4(unsigned char *hi, int bn, int q4, const float2 *v) {
  float br[4], bi[4], nbi[4];
  uint4 h, l;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    br[j] = v[j].x;
    bi[j] = v[j].y;
    nbi[j] = -v[j].y;
  }
  unsigned char *lo = hi + kPlane;
  split4_tf32(br, h, l);
  *reinterpret_cast<uint4 *>(hi + plane_off(bn, 4 * q4)) = h;
  *reinterpret_cast<uint4 *>(lo + plane_off(bn, 4 * q4)) = l;
  *reinterpret_cast<uint4 *>(hi + plane_off(64 + bn, 8 + 4 * q4)) = h;
  *reinterpret_cast<uint4 *>(lo + plane_off(64 + bn, 8 + 4 * q4)) = l;
  split4_tf32(nbi, h, l);
  *reinterpret_cast<uint4 *>(hi + plane_off(bn, 8 + 4 * q4)) = h;
  *reinterpret_cast<uint4 *>(lo + plane_off(bn, 8 + 4 * q4)) = l;
  split4_tf32(bi, h, l);
  *reinterpret_cast<uint4 *>(hi + plane_off(64 + bn, 4 * q4)) = h;
  *reinterpret_cast<uint4 *>(lo + plane_off(64 + bn, 4 * q4)) = l;
}

// the three MMAs of one K step (A_lo B_hi + A_hi B_lo + A_hi B_hi)
__device__ __forceinline__ void mma3(uint32_t tmem, uint32_t a_hi, uint32_t b_hi, uint32_t acc0) {
  const uint32_t a_lo = a_hi + kPlane, b_lo = b_hi + kPlane;
  mma_tf32(tmem, smem_desc(a_lo, 128u, 256u), smem_desc(b_hi, 128u, 256u), acc0);
  mma_tf32(tmem, smem_desc(a_hi, 128u, 256u), smem_desc(b_lo, 128u, 256u), 1u);
  mma_tf32(tmem, smem_desc(a_hi, 128u, 256u), smem_desc(b_hi, 128u, 256u), 1u);
}

// waits for the MMAs of the last chunk (bounded); on a timeout the error is
// recorded and the MMAs still in flight are awaited once more before the
// caller frees TMEM.  Returns whether the results may be written.
__device__ __forceinline__ bool finish_mmas(uint64_t *bars, int nch, bool ok, int *err,
                                            int *wait_ok) {
  if (threadIdx.x == 0) {
    const int fine = ok && nch > 0 ? mbar_wait(&bars[(nch - 1) & 1], ((nch - 1) >> 1) & 1) : ok;
    if (!fine) {
      atomicExch(err, 1);
      if (nch > 0) mbar_wait(&bars[(nch - 1) & 1], ((nch - 1) >> 1) & 1);
    }
    *wait_ok = fine;
  }
  __syncthreads();
  const bool r = *wait_ok != 0;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return r;
}

template <int COLS>
__device__ __forceinline__ void tc_setup(uint32_t *tmem_slot, uint64_t *bars) {
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(tmem_slot)),
                 "r"(COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

template <int COLS>
__device__ __forceinline__ void tc_teardown(uint32_t tmem) {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(COLS));
}

__global__ void __launch_bounds__(256, 1)
    k_scale_l_tc(const int4 *__restrict__ tiles, float2 *__restrict__ pool,
                 const DevFront *__restrict__ fr, const long long *__restrict__ inv_off,
                 const float2 *__restrict__ Linv, int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int wait_ok;
  unsigned char *stage0 = tc_smem + ((1024 - (smem_addr(tc_smem) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int4 tl = tiles[blockIdx.x];
  const DevFront f = fr[tl.x];
  const int m = f.m, b0 = tl.y * kRwSW, nb = min(kRwSW, f.p - b0), R0 = tl.z;
  float2 *F = pool + f.off;
  const float2 *Li = Linv + inv_off[tl.x] + (long long)tl.y * kRwSW * kRwSW;  // (q, j) at j nb + q
  tc_setup<512>(&tmem_slot, bars);
  const uint32_t tmem = tmem_slot;
  const int nch = (nb + kTcKC - 1) / kTcKC;
  const int ntile = (nb + 63) / 64;
  // A: thread (ar, aq) stages K columns 4 aq .. +3 of row ar; B: thread n
  // stages output column n (tile n / 64) for all 8 K rows of the chunk
  const int ar = tid & 127, aq = tid >> 7;
  const int n = tid, bt = n >> 6, bn = n & 63;
  float2 va[4], vb[8];
  auto load = [&](int c) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int kc = c * kTcKC + 4 * aq + j;
      va[j] = (R0 + ar < m && kc < nb) ? F[(long long)(b0 + kc) * m + R0 + ar]
                                        : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int q = c * kTcKC + k;
      vb[k] = (n < nb && q < nb && q >= n) ? Li[(long long)n * nb + q] : make_float2(0.f, 0.f);
    }
  };
  bool ok = true;
  if (nch > 0) load(0);
  for (int c = 0; c < nch; ++c) {
    const int sb = c & 1;
    unsigned char *st = stage0 + sb * kRwLStage;
    if (c >= 2) {  // the MMAs of chunk c - 2 read this buffer
      if (tid == 0) wait_ok = mbar_wait(&bars[sb], ((c - 2) >> 1) & 1);
      __syncthreads();
      if (!wait_ok) {
        ok = false;
        break;
      }
    }
    stage_a4(st, ar, aq, va);
    if (bt < ntile && c >= 8 * bt) {  // tile bt reads this chunk
      unsigned char *bh = st + (2 + 2 * bt) * kPlane;
      stage_b4(bh, bn, 0, vb);
      stage_b4(bh, bn, 1, vb + 4);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a_hi = smem_addr(st);
      for (int t = 0; t < ntile; ++t) {
        if (c < 8 * t) continue;  // inv(L_bb)(q, j) = 0 for q < j
        const uint32_t b_hi = a_hi + (2 + 2 * t) * kPlane;
#pragma unroll
        for (int j = 0; j < 2; ++j)
          mma3(tmem + 128 * t, a_hi + j * 4096, b_hi + j * 4096, (c > 8 * t || j > 0) ? 1u : 0u);
      }
      mma_commit(&bars[sb]);
    }
    if (c + 1 < nch) load(c + 1);  // the next chunk's loads overlap these MMAs
  }
  ok = finish_mmas(bars, nch, ok, err, &wait_ok);
  if (ok) {
    // warp w: TMEM lanes 32 (w % 4) .. +31 (rows), column half w / 4 of each tile
    const int q = warp & 3, h = warp >> 2;
    const int row = 32 * q + (tid & 31);
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
    for (int t = 0; t < ntile; ++t) {
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        uint32_t cr[16], ci[16];
        const int n0 = 32 * h + 16 * part;
        TLR_TC_LD16(lane_addr + 128 * t + n0, cr);
        TLR_TC_LD16(lane_addr + 128 * t + 64 + n0, ci);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (R0 + row < m) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = 64 * t + n0 + j;
            if (col < nb)
              F[(long long)(b0 + col) * m + R0 + row] =
                  make_float2(__uint_as_float(cr[j]), __uint_as_float(ci[j]));
          }
        }
      }
    }
  }
  tc_teardown<512>(tmem);
}

__global__ void __launch_bounds__(256, 2)
    k_scale_u_tc(const int4 *__restrict__ tiles, float2 *__restrict__ pool,
                 const DevFront *__restrict__ fr, const long long *__restrict__ inv_off,
                 const float2 *__restrict__ Linv, const float2 *__restrict__ Uinv,
                 float2 *__restrict__ dmat, int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int wait_ok;
  unsigned char *stage0 = tc_smem + ((1024 - (smem_addr(tc_smem) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int4 tl = tiles[blockIdx.x];
  const DevFront f = fr[tl.x];
  const int b0 = tl.y * kRwSW, nb = min(kRwSW, f.p - b0), col0 = tl.z;
  const long long io = inv_off[tl.x] + (long long)tl.y * kRwSW * kRwSW;
  const float2 *Ui = Uinv + io;  // (i, q) at q nb + i, upper triangular
  // X(q, col) at src[col * ld + q]; the result goes to dst at the same place
  const float2 *src;
  float2 *dst;
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
  tc_setup<256>(&tmem_slot, bars);
  const uint32_t tmem = tmem_slot;
  const int nch = (nb + kTcKC - 1) / kTcKC;
  const int nmt = (nb + 127) / 128;
  // A: thread i stages row i of inv(U_bb) (tile i / 128) for all 8 K
  // columns; B: thread (bn, bq), tid < 128, stages K rows 4 bq .. +3 of
  // output column bn
  const int ai = tid, bn = tid & 63, bq = (tid >> 6) & 1;
  const bool bact = tid < 128;
  float2 va[8], vb[4];
  auto load = [&](int c) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int q = c * kTcKC + k;
      va[k] = (ai < nb && q < nb && q >= ai) ? Ui[(long long)q * nb + ai] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int q = c * kTcKC + 4 * bq + j;
      vb[j] = (bact && col0 + bn < ncol && q < nb) ? src[(long long)(col0 + bn) * ld + q]
                                                   : make_float2(0.f, 0.f);
    }
  };
  bool ok = true;
  if (nch > 0) load(0);
  for (int c = 0; c < nch; ++c) {
    const int sb = c & 1;
    unsigned char *st = stage0 + sb * kRwUStage;
    if (c >= 2) {
      if (tid == 0) wait_ok = mbar_wait(&bars[sb], ((c - 2) >> 1) & 1);
      __syncthreads();
      if (!wait_ok) {
        ok = false;
        break;
      }
    }
    {
      const int mt = ai >> 7;
      if (mt < nmt && (mt == 0 || c >= 16)) {  // tile mt reads this chunk
        unsigned char *ah = st + 2 * mt * kPlane;
        stage_a4(ah, ai & 127, 0, va);
        stage_a4(ah, ai & 127, 1, va + 4);
      }
    }
    if (bact) stage_b4(st + 4 * kPlane, bn, bq, vb);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = smem_addr(st), b_hi = base + 4 * kPlane;
      for (int mt = 0; mt < nmt; ++mt) {
        const int cfirst = mt == 0 ? 0 : 16;  // inv(U_bb)(i, q) = 0 for q < i
        if (c < cfirst) continue;
#pragma unroll
        for (int j = 0; j < 2; ++j)
          mma3(tmem + 128 * mt, base + 2 * mt * kPlane + j * 4096, b_hi + j * 4096,
               (c > cfirst || j > 0) ? 1u : 0u);
      }
      mma_commit(&bars[sb]);
    }
    if (c + 1 < nch) load(c + 1);
  }
  ok = finish_mmas(bars, nch, ok, err, &wait_ok);
  if (ok) {
    const int q = warp & 3, h = warp >> 2;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
    for (int mt = 0; mt < nmt; ++mt) {
      const int row = 128 * mt + 32 * q + (tid & 31);
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        uint32_t cr[16], ci[16];
        const int n0 = 32 * h + 16 * part;
        TLR_TC_LD16(lane_addr + 128 * mt + n0, cr);
        TLR_TC_LD16(lane_addr + 128 * mt + 64 + n0, ci);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row < nb) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = col0 + n0 + j;
            if (col < ncol)
              dst[(long long)col * ld + row] =
                  make_float2(__uint_as_float(cr[j]), __uint_as_float(ci[j]));
          }
        }
      }
    }
  }
  tc_teardown<256>(tmem);
}

}  // namespace

int launch_gemm_tc_bulk(tlr_ctx *ctx, const int *fl, const int *prefix, const int *pa,
                        const int *pb, int nf, int s, int w, float2 *pool, const DevFront *fr,
                        int tiles, int atiles, int btiles, unsigned char *planes, int *err,
                        cudaStream_t st, int variant) {
  const int nchmax = (w + kTcKC - 1) / kTcKC;
  if (atiles + btiles > 0)
    { k_tc_split<<<dim3(atiles + btiles, nchmax), 256, 0, st>>>(fl, pa, pb, nf, s, w, pool, fr,
                                                               planes, atiles, nchmax); count_launches(); }
  const unsigned char *pbp = planes + (long long)atiles * nchmax * kChunkImg;
  if (variant == 2) {  // persistent, warp-specialised: one CTA per SM, four stages
    auto k = k_gemm_tc_persist<4>;
    const int smem = (int)gemm_tc_bulk_smem(4);
    TLR_CUDA(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int grid = std::max(1, std::min(tiles, std::max(sms, 1)));
    { k<<<grid, kPersistThreads, smem, st>>>(fl, prefix, pa, pb, nf, s, w, tiles, pool, fr,
                                             planes, pbp, nchmax, err); count_launches(); }
  } else if (variant == 1) {  // two stages, three CTAs per SM, half the F22 prefetched
    auto k = k_gemm_tc_bulk<2, 3, 16>;
    TLR_CUDA(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)gemm_tc_bulk_smem(2)));
    { k<<<tiles, 256, gemm_tc_bulk_smem(2), st>>>(fl, prefix, pa, pb, nf, s, w, pool, fr, planes,
                                                 pbp, nchmax, err, 128u, 256u); count_launches(); }
  } else {
    auto k = k_gemm_tc_bulk<kBulkStages, 2, 32>;
    TLR_CUDA(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)gemm_tc_bulk_smem(kBulkStages)));
    { k<<<tiles, 256, gemm_tc_bulk_smem(kBulkStages), st>>>(fl, prefix, pa, pb, nf, s, w, pool, fr,
                                                           planes, pbp, nchmax, err, 128u, 256u); count_launches(); }
  }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

int launch_gemm_tc(tlr_ctx *ctx, const int *fl, const int *prefix, int nf, int s, int w,
                   float2 *pool, const DevFront *fr, int tiles, int *err, cudaStream_t st,
                   uint32_t lbo, uint32_t sbo) {
  TLR_CUDA(ctx, cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)gemm_tc_smem()));
  { k_gemm_tc<<<tiles, 256, gemm_tc_smem(), st>>>(fl, prefix, nf, s, w, pool, fr, err, lbo, sbo); count_launches(); }
  return TLR_OK;
}

int launch_rewrite_tc(tlr_ctx *ctx, const int4 *ltiles, long long nl, const int4 *utiles,
                      long long nu, float2 *pool, const DevFront *fr, const long long *inv_off,
                      const float2 *Linv, const float2 *Uinv, float2 *dmat, int *err,
                      cudaStream_t st) {
  const size_t lsm = 2 * kRwLStage + 1024, usm = 2 * kRwUStage + 1024;
  TLR_CUDA(ctx, cudaFuncSetAttribute(k_scale_l_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)lsm));
  TLR_CUDA(ctx, cudaFuncSetAttribute(k_scale_u_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)usm));
  if (nu > 0)
    { k_scale_u_tc<<<(unsigned)nu, 256, usm, st>>>(utiles, pool, fr, inv_off, Linv, Uinv, dmat,
                                                  err); count_launches(); }
  if (nl > 0)
    { k_scale_l_tc<<<(unsigned)nl, 256, lsm, st>>>(ltiles, pool, fr, inv_off, Linv, err); count_launches(); }
  TLR_CUDA(ctx, cudaGetLastError());
  return TLR_OK;
}

}  // namespace tlr

// ---------------------------------------------------------------- test hooks
// Failure detection without a fault: which = 0 runs the tensor-core
// kernel's bounded mbarrier wait on a barrier nothing completes, which = 1
// the persistent solve's bounded grid barrier waiting for a CTA that does
// not exist; *timed_out = 1 when the wait gave up and reported it.
extern "C" int tlr_wait_selftest(int which, unsigned limit, int *timed_out) {
  using namespace tlr;
  if (!timed_out || which < 0 || which > 1 || limit == 0) return TLR_ERR_ARG;
  int *d = nullptr;  // err flag, then the barrier counter
  if (cudaMalloc(&d, 2 * sizeof(int)) != cudaSuccess) return TLR_ERR_NOMEM;
  int rc = TLR_OK;
  if (cudaMemset(d, 0, 2 * sizeof(int)) != cudaSuccess) rc = TLR_ERR_CUDA;
  if (!rc) {
    if (which == 0)
      { k_mbar_timeout_probe<<<1, 32>>>(limit, d); count_launches(); }
    else
      rc = grid_barrier_probe(reinterpret_cast<unsigned *>(d + 1), limit, d);
  }
  int h = 0;
  if (!rc && (cudaDeviceSynchronize() != cudaSuccess ||
              cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess))
    rc = TLR_ERR_CUDA;
  cudaFree(d);
  *timed_out = h;
  return rc;
}

// ---------------------------------------------------------------- test hook
extern "C" int tlr_schur_update_c64(const float *front, int m, int p, int k0, int w,
                                    unsigned lbo, unsigned sbo, float *out) {
  using namespace tlr;
  if (!front || !out || m <= 0 || p <= 0 || p > m || k0 < 0 || k0 >= p || w <= 0 || w > 64 ||
      k0 % w != 0)
    return TLR_ERR_ARG;
  if (lbo == 0) lbo = 128;
  if (sbo == 0) sbo = 256;
  const int ww = std::min(w, p - k0), base = k0 + ww, ext = m - base;
  const size_t bytes = (size_t)m * m * sizeof(float2);
  float2 *F = nullptr;
  DevFront *fr = nullptr;
  int *ints = nullptr;  // fl[1], prefix[2], err[1]
  int rc = TLR_OK;
  cudaStream_t st = nullptr;
  const int tiles = ext > 0 ? ((ext + kTcM - 1) / kTcM) * ((ext + kTcN - 1) / kTcN) : 0;
  DevFront h{};
  h.off = 0;
  h.toff = 0;
  h.cmap_off = 0;
  h.p = p;
  h.m = m;
  h.parent = -1;
  h.node_off = 0;
  const int hi[4] = {0, 0, tiles, 0};
  int herr = 0;
  if (cudaMalloc(&F, bytes) != cudaSuccess || cudaMalloc(&fr, sizeof(DevFront)) != cudaSuccess ||
      cudaMalloc(&ints, 4 * sizeof(int)) != cudaSuccess || cudaStreamCreate(&st) != cudaSuccess) {
    rc = TLR_ERR_NOMEM;
  } else if (cudaMemcpy(F, front, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemcpy(fr, &h, sizeof(h), cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemcpy(ints, hi, sizeof(hi), cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = TLR_ERR_CUDA;
  } else {
    if (tiles > 0) {
      cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)gemm_tc_smem());
      { k_gemm_tc<<<tiles, 256, gemm_tc_smem(), st>>>(ints, ints + 1, 1, k0 / w, w, F, fr, ints + 3, lbo, sbo); count_launches(); }
    }
    if (cudaStreamSynchronize(st) != cudaSuccess ||
        cudaMemcpy(out, F, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&herr, ints + 3, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = TLR_ERR_CUDA;
    else if (herr)
      rc = TLR_ERR_CUDA;
  }
  cudaFree(F);
  cudaFree(fr);
  cudaFree(ints);
  if (st) cudaStreamDestroy(st);
  return rc;
}
