// tlr_noalloc.cu -- Frobenius norm of a complex array with no allocation.
//
// Some callers cannot allocate device memory.  Host frameworks that route
// every device allocation through their own caching pool forbid raw
// cudaMalloc/cudaFree from the libraries they load, and applications that
// reserve nearly all of HBM for their own pool at start-up leave a library
// nothing to allocate from.  tlr_frobenius_noalloc serves them: it computes
// the same Frobenius norm that tlr_assemble and tlr_apply_bc report for the
// operators (sqrt of the sum of |v|^2 over complex values), and its only
// scratch is a file-scope __device__ array of kMaxPartials + 1 doubles
// (32 KB + 8 B) that every GPU which loads the library keeps until exit.
//
// The caller passes the input (a 16-byte aligned device array) and the
// output (a host double).  The entry point calls no cudaMalloc, cudaFree or
// allocating library routine.  It copies the result to the host and
// synchronises the stream before it returns.  The first call on a device
// looks up the array's device address (cudaGetSymbolAddress, with that
// device current) and caches it; make that first call before any stream
// capture begins.  Every call shares the one array, so calls whose kernels
// overlap on the GPU race: serialise them (one stream, or synchronise
// between calls).  Each call overwrites every partial slot it reads, so
// nothing needs clearing between calls.
#include <cstdint>
#include <mutex>

#include "tlr_internal.h"

namespace tlr {
namespace {

constexpr int kMaxPartials = 4096;             // CTAs of the first pass
constexpr long long kPerBlock = 65536;         // complex values per CTA
constexpr long long kMaxCount = kMaxPartials * kPerBlock;  // 2^28 values
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_partial[kMaxPartials + 1];

std::mutex g_mu;
double *g_addr[kMaxDevices] = {nullptr};

__global__ void k_partial(long long n, const double2 *__restrict__ v,
                          double *__restrict__ partial) {
  __shared__ double sh[8];
  const long long b0 = (long long)blockIdx.x * kPerBlock;
  const long long b1 = min(n, b0 + kPerBlock);
  double s = 0.0;
  for (long long x = b0 + threadIdx.x; x < b1; x += blockDim.x) {
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

__global__ void k_final(int nb, double *partial) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double t = 0.0;
  for (int b = 0; b < nb; ++b) t += partial[b];
  partial[kMaxPartials] = sqrt(t);
}

}  // namespace

void set_global_error(const std::string &msg);

}  // namespace tlr

extern "C" int tlr_frobenius_noalloc(const double *values, size_t count, double *result,
                                     void *stream) {
  using namespace tlr;
  if (!values || !result) {
    set_global_error("tlr_frobenius_noalloc: null values or result pointer");
    return TLR_ERR_ARG;
  }
  if ((reinterpret_cast<uintptr_t>(values) & 15u) != 0) {
    // the kernel reads one complex value (two doubles) per 16-byte load
    set_global_error("tlr_frobenius_noalloc: values must be 16-byte aligned "
                     "(the start of a complex128 array)");
    return TLR_ERR_ARG;
  }
  if (count > static_cast<size_t>(kMaxCount)) {
    set_global_error("tlr_frobenius_noalloc: count exceeds the maximum of 268435456 "
                     "complex values (the fixed scratch holds 4096 partial sums)");
    return TLR_ERR_SIZE;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_global_error("tlr_frobenius_noalloc: no usable current CUDA device");
    return TLR_ERR_CUDA;
  }
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
      // one-time set-up on this device, with the device current: the
      // device address of the file-scope array
      e = cudaGetSymbolAddress(reinterpret_cast<void **>(&g_addr[dev]), g_partial);
      if (e != cudaSuccess) {
        g_addr[dev] = nullptr;
        set_global_error(std::string("tlr_frobenius_noalloc: cudaGetSymbolAddress failed: ") +
                         cudaGetErrorString(e));
        return TLR_ERR_CUDA;
      }
    }
    scratch = g_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  (void)cudaGetLastError();  // a stale error from earlier work is not this call's
  const int nb = count == 0 ? 1 : (int)(((long long)count + kPerBlock - 1) / kPerBlock);
  { k_partial<<<nb, 256, 0, st>>>((long long)count, reinterpret_cast<const double2 *>(values),
                                scratch); count_launches(); }
  { k_final<<<1, 32, 0, st>>>(nb, scratch); count_launches(); }
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(result, scratch + kMaxPartials, sizeof(double), cudaMemcpyDeviceToHost,
                        st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_global_error(std::string("tlr_frobenius_noalloc: ") + cudaGetErrorString(e));
    return TLR_ERR_CUDA;
  }
  return TLR_OK;
}
