// tlr_mlp.cu -- the learned shift / start-vector proposal: a small MLP
// (inputs -> depth x width SiLU hidden layers -> outputs) trained and
// evaluated on the GPU by the kernels in this file.  No reference
// counterpart: the reference always starts Krylov-Schur from SLEPc's
// random vector at the configured target (EigenSolver.cpp:46-72).
//
// Parameters are FP32, flat: for each layer l, W_l [out][in] row-major then
// b_l [out].  Training: mean-squared error, full forward/backward per
// minibatch, Adam.  Inference: FP32 or BF16 weights/activations with FP32
// accumulation.
#include <cuda_bf16.h>

#include <cmath>
#include <vector>

#include "tlr_internal.h"

struct tlr_mlp {
  int n_in = 0, width = 0, depth = 0, n_out = 0, n_layers = 0;
  std::vector<int> fan_in, fan_out;
  std::vector<long long> w_off, b_off;
  long long n_params = 0;
  float *params = nullptr, *grads = nullptr, *m1 = nullptr, *m2 = nullptr;
  __nv_bfloat16 *params16 = nullptr;
  float *act = nullptr, *pre = nullptr, *dact = nullptr;  // [layers+1][batch][maxw]
  int cap = 0, maxw = 0;
  float *xbuf = nullptr, *ybuf = nullptr, *loss = nullptr;
  long long adam_t = 0;
  cudaStream_t stream = nullptr;
};

namespace tlr {
namespace {

constexpr int kT = 32;

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

// Y[n][o] = X[n][i] W^T + b (optionally SiLU), pre-activation kept in Z.
__global__ void k_lin_fwd(int n, int in, int out, const float *__restrict__ X, int ldx,
                          const float *__restrict__ W, const float *__restrict__ b,
                          float *__restrict__ Z, float *__restrict__ Y, int ldy, int act) {
  __shared__ float xs[kT][kT + 1], ws[kT][kT + 1];
  const int row = blockIdx.y * kT + threadIdx.y, col = blockIdx.x * kT + threadIdx.x;
  float acc = 0.f;
  for (int k0 = 0; k0 < in; k0 += kT) {
    xs[threadIdx.y][threadIdx.x] =
        (row < n && k0 + threadIdx.x < in) ? X[(long long)row * ldx + k0 + threadIdx.x] : 0.f;
    const int wr = blockIdx.x * kT + threadIdx.y;
    ws[threadIdx.y][threadIdx.x] =
        (wr < out && k0 + threadIdx.x < in) ? W[(long long)wr * in + k0 + threadIdx.x] : 0.f;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kT; ++k) acc = fmaf(xs[threadIdx.y][k], ws[threadIdx.x][k], acc);
    __syncthreads();
  }
  if (row < n && col < out) {
    const float z = acc + b[col];
    if (Z) Z[(long long)row * ldy + col] = z;
    Y[(long long)row * ldy + col] = act ? silu(z) : z;
  }
}

// BF16 inference layer: weights and activations in bf16, FP32 accumulate.
__global__ void k_lin_fwd16(int n, int in, int out, const __nv_bfloat16 *__restrict__ X,
                            const __nv_bfloat16 *__restrict__ W, const __nv_bfloat16 *__restrict__ b,
                            __nv_bfloat16 *__restrict__ Y16, float *__restrict__ Y32, int act) {
  __shared__ float xs[kT][kT + 1], ws[kT][kT + 1];
  const int row = blockIdx.y * kT + threadIdx.y, col = blockIdx.x * kT + threadIdx.x;
  float acc = 0.f;
  for (int k0 = 0; k0 < in; k0 += kT) {
    xs[threadIdx.y][threadIdx.x] = (row < n && k0 + threadIdx.x < in)
                                       ? __bfloat162float(X[(long long)row * in + k0 + threadIdx.x])
                                       : 0.f;
    const int wr = blockIdx.x * kT + threadIdx.y;
    ws[threadIdx.y][threadIdx.x] = (wr < out && k0 + threadIdx.x < in)
                                       ? __bfloat162float(W[(long long)wr * in + k0 + threadIdx.x])
                                       : 0.f;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kT; ++k) acc = fmaf(xs[threadIdx.y][k], ws[threadIdx.x][k], acc);
    __syncthreads();
  }
  if (row < n && col < out) {
    const float z = acc + __bfloat162float(b[col]);
    const float y = act ? silu(z) : z;
    if (Y16) Y16[(long long)row * out + col] = __float2bfloat16(y);
    if (Y32) Y32[(long long)row * out + col] = y;
  }
}

// dX[n][i] = dZ[n][o] W[o][i]
__global__ void k_lin_bwd_data(int n, int in, int out, const float *__restrict__ dZ, int ldz,
                               const float *__restrict__ W, float *__restrict__ dX, int ldx) {
  __shared__ float zs[kT][kT + 1], ws[kT][kT + 1];
  const int row = blockIdx.y * kT + threadIdx.y, col = blockIdx.x * kT + threadIdx.x;
  float acc = 0.f;
  for (int k0 = 0; k0 < out; k0 += kT) {
    zs[threadIdx.y][threadIdx.x] =
        (row < n && k0 + threadIdx.x < out) ? dZ[(long long)row * ldz + k0 + threadIdx.x] : 0.f;
    const int wc = blockIdx.x * kT + threadIdx.x;
    ws[threadIdx.y][threadIdx.x] =
        (k0 + threadIdx.y < out && wc < in) ? W[(long long)(k0 + threadIdx.y) * in + wc] : 0.f;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kT; ++k) acc = fmaf(zs[threadIdx.y][k], ws[k][threadIdx.x], acc);
    __syncthreads();
  }
  if (row < n && col < in) dX[(long long)row * ldx + col] = acc;
}

// dW[o][i] += sum_n dZ[n][o] X[n][i];  db[o] += sum_n dZ[n][o]
__global__ void k_lin_bwd_weight(int n, int in, int out, const float *__restrict__ dZ, int ldz,
                                 const float *__restrict__ X, int ldx, float *__restrict__ dW,
                                 float *__restrict__ db) {
  __shared__ float zs[kT][kT + 1], xs[kT][kT + 1];
  const int o = blockIdx.y * kT + threadIdx.y, i = blockIdx.x * kT + threadIdx.x;
  float acc = 0.f, accb = 0.f;
  for (int r0 = 0; r0 < n; r0 += kT) {
    const int zo = blockIdx.y * kT + threadIdx.x;
    zs[threadIdx.y][threadIdx.x] =
        (r0 + threadIdx.y < n && zo < out) ? dZ[(long long)(r0 + threadIdx.y) * ldz + zo] : 0.f;
    xs[threadIdx.y][threadIdx.x] =
        (r0 + threadIdx.y < n && i < in) ? X[(long long)(r0 + threadIdx.y) * ldx + i] : 0.f;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kT; ++k) {
      acc = fmaf(zs[k][threadIdx.y], xs[k][threadIdx.x], acc);
      accb += zs[k][threadIdx.y];
    }
    __syncthreads();
  }
  if (o < out && i < in) dW[(long long)o * in + i] += acc;
  if (o < out && blockIdx.x == 0 && threadIdx.x == 0) db[o] += accb;
}

__global__ void k_silu_bwd(long long count, int cols, int ld, const float *__restrict__ Z,
                           float *__restrict__ dA) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= count) return;
  const long long r = x / cols, c = x % cols;
  dA[r * ld + c] *= silu_grad(Z[r * ld + c]);
}

// loss = mean((Y - T)^2) over n*o; dY = 2 (Y - T) / (n o)
__global__ void k_mse(int n, int o, int ld, const float *__restrict__ Y, const float *__restrict__ T,
                      float *__restrict__ dY, float *__restrict__ loss) {
  __shared__ float sh[256];
  float s = 0.f;
  const float scale = 2.f / (float)((long long)n * o);
  for (long long x = threadIdx.x; x < (long long)n * o; x += blockDim.x) {
    const long long r = x / o, c = x % o;
    const float d = Y[r * ld + c] - T[x];
    s += d * d;
    dY[r * ld + c] = scale * d;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = sh[0] / (float)((long long)n * o);
}

__global__ void k_adam(long long count, float *__restrict__ p, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, float lr, float b1, float b2,
                       float c1, float c2, float eps) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= count) return;
  const float gi = g[x];
  m[x] = b1 * m[x] + (1.f - b1) * gi;
  v[x] = b2 * v[x] + (1.f - b2) * gi * gi;
  p[x] -= lr * (m[x] / c1) / (sqrtf(v[x] / c2) + eps);
}

__global__ void k_to_bf16(long long count, const float *__restrict__ a, __nv_bfloat16 *__restrict__ b) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < count) b[x] = __float2bfloat16(a[x]);
}

int ensure_capacity(tlr_mlp *m, int n) {
  if (n <= m->cap) return TLR_OK;
  cudaFree(m->act); cudaFree(m->pre); cudaFree(m->dact); cudaFree(m->xbuf); cudaFree(m->ybuf);
  const size_t plane = (size_t)n * m->maxw;
  if (cudaMalloc(&m->act, sizeof(float) * plane * (m->n_layers + 1)) ||
      cudaMalloc(&m->pre, sizeof(float) * plane * (m->n_layers + 1)) ||
      cudaMalloc(&m->dact, sizeof(float) * plane * (m->n_layers + 1)) ||
      cudaMalloc(&m->xbuf, sizeof(float) * (size_t)n * m->n_in) ||
      cudaMalloc(&m->ybuf, sizeof(float) * (size_t)n * m->n_out))
    return TLR_ERR_NOMEM;
  m->cap = n;
  return TLR_OK;
}

// forward of a batch already in xbuf; activations in act planes
void forward(tlr_mlp *m, int n) {
  const size_t plane = (size_t)m->cap * m->maxw;
  const float *X = m->xbuf;
  int ldx = m->n_in;
  for (int l = 0; l < m->n_layers; ++l) {
    const int in = m->fan_in[l], out = m->fan_out[l];
    float *Z = m->pre + plane * (l + 1), *Y = m->act + plane * (l + 1);
    dim3 g((out + kT - 1) / kT, (n + kT - 1) / kT), b(kT, kT);
    { k_lin_fwd<<<g, b, 0, m->stream>>>(n, in, out, X, ldx, m->params + m->w_off[l],
                                      m->params + m->b_off[l], Z, Y, m->maxw,
                                      l + 1 < m->n_layers); count_launches(); }
    X = Y;
    ldx = m->maxw;
  }
}

// backward from dact[last] (dY); accumulates into grads (zeroed by caller)
void backward(tlr_mlp *m, int n) {
  const size_t plane = (size_t)m->cap * m->maxw;
  for (int l = m->n_layers - 1; l >= 0; --l) {
    const int in = m->fan_in[l], out = m->fan_out[l];
    float *dZ = m->dact + plane * (l + 1);
    if (l + 1 < m->n_layers) {
      const long long cnt = (long long)n * out;
      { k_silu_bwd<<<blocks_for(cnt, 256), 256, 0, m->stream>>>(cnt, out, m->maxw,
                                                             m->pre + plane * (l + 1), dZ); count_launches(); }
    }
    const float *X = l == 0 ? m->xbuf : m->act + plane * l;
    const int ldx = l == 0 ? m->n_in : m->maxw;
    dim3 gw((in + kT - 1) / kT, (out + kT - 1) / kT), b(kT, kT);
    { k_lin_bwd_weight<<<gw, b, 0, m->stream>>>(n, in, out, dZ, m->maxw, X, ldx,
                                              m->grads + m->w_off[l], m->grads + m->b_off[l]); count_launches(); }
    if (l > 0) {
      dim3 gd((in + kT - 1) / kT, (n + kT - 1) / kT);
      { k_lin_bwd_data<<<gd, b, 0, m->stream>>>(n, in, out, dZ, m->maxw, m->params + m->w_off[l],
                                              m->dact + plane * l, m->maxw); count_launches(); }
    }
  }
}

}  // namespace
}  // namespace tlr

using namespace tlr;

extern "C" {

int tlr_mlp_create(int n_in, int width, int depth, int n_out, unsigned long long seed,
                   tlr_mlp **out) {
  if (!out || n_in < 1 || width < 1 || depth < 1 || n_out < 1) return TLR_ERR_ARG;
  tlr_mlp *m = new tlr_mlp();
  m->n_in = n_in; m->width = width; m->depth = depth; m->n_out = n_out;
  m->n_layers = depth + 1;
  m->maxw = std::max(width, std::max(n_out, n_in));
  long long off = 0;
  for (int l = 0; l < m->n_layers; ++l) {
    const int in = l == 0 ? n_in : width, o = l + 1 == m->n_layers ? n_out : width;
    m->fan_in.push_back(in);
    m->fan_out.push_back(o);
    m->w_off.push_back(off);
    off += (long long)in * o;
    m->b_off.push_back(off);
    off += o;
  }
  m->n_params = off;
  // He-style initialisation from a deterministic generator
  std::vector<float> h(off, 0.f);
  unsigned long long s = seed ? seed : 0x243F6A8885A308D3ull;
  auto next = [&]() {
    s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
    return (double)((s * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < m->n_layers; ++l) {
    const double a = std::sqrt(6.0 / m->fan_in[l]) * (l + 1 == m->n_layers ? 0.5 : 1.0);
    for (long long k = 0; k < (long long)m->fan_in[l] * m->fan_out[l]; ++k)
      h[m->w_off[l] + k] = (float)((2.0 * next() - 1.0) * a);
  }
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) ||
      cudaMalloc(&m->params, sizeof(float) * off) || cudaMalloc(&m->grads, sizeof(float) * off) ||
      cudaMalloc(&m->m1, sizeof(float) * off) || cudaMalloc(&m->m2, sizeof(float) * off) ||
      cudaMalloc(&m->params16, sizeof(__nv_bfloat16) * off) ||
      cudaMalloc(&m->loss, sizeof(float)) ||
      cudaMemcpy(m->params, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice) ||
      cudaMemset(m->m1, 0, sizeof(float) * off) || cudaMemset(m->m2, 0, sizeof(float) * off)) {
    tlr_mlp_destroy(m);
    return TLR_ERR_NOMEM;
  }
  *out = m;
  return TLR_OK;
}

void tlr_mlp_destroy(tlr_mlp *m) {
  if (!m) return;
  if (m->stream) cudaStreamSynchronize(m->stream);
  cudaFree(m->params); cudaFree(m->grads); cudaFree(m->m1); cudaFree(m->m2);
  cudaFree(m->params16); cudaFree(m->act); cudaFree(m->pre); cudaFree(m->dact);
  cudaFree(m->xbuf); cudaFree(m->ybuf); cudaFree(m->loss);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

long long tlr_mlp_num_params(const tlr_mlp *m) { return m ? m->n_params : 0; }

int tlr_mlp_params(tlr_mlp *m, float *host, int set) {
  if (!m || !host) return TLR_ERR_ARG;
  const size_t bytes = sizeof(float) * m->n_params;
  cudaError_t e = set ? cudaMemcpy(m->params, host, bytes, cudaMemcpyHostToDevice)
                      : cudaMemcpy(host, m->params, bytes, cudaMemcpyDeviceToHost);
  if (set) m->adam_t = 0;
  return e == cudaSuccess ? TLR_OK : TLR_ERR_CUDA;
}

// Loss and parameter gradients of one batch (host arrays), without update.
int tlr_mlp_gradients(tlr_mlp *m, const float *X, const float *Y, int n, float *grads,
                      float *loss) {
  if (!m || !X || !Y || n < 1) return TLR_ERR_ARG;
  int rc = ensure_capacity(m, n);
  if (rc) return rc;
  cudaMemcpyAsync(m->xbuf, X, sizeof(float) * n * m->n_in, cudaMemcpyHostToDevice, m->stream);
  cudaMemcpyAsync(m->ybuf, Y, sizeof(float) * n * m->n_out, cudaMemcpyHostToDevice, m->stream);
  cudaMemsetAsync(m->grads, 0, sizeof(float) * m->n_params, m->stream);
  forward(m, n);
  const size_t plane = (size_t)m->cap * m->maxw;
  { k_mse<<<1, 256, 0, m->stream>>>(n, m->n_out, m->maxw, m->act + plane * m->n_layers, m->ybuf,
                                  m->dact + plane * m->n_layers, m->loss); count_launches(); }
  backward(m, n);
  if (grads)
    cudaMemcpyAsync(grads, m->grads, sizeof(float) * m->n_params, cudaMemcpyDeviceToHost,
                    m->stream);
  if (loss) cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  return cudaStreamSynchronize(m->stream) == cudaSuccess ? TLR_OK : TLR_ERR_CUDA;
}

// Adam training over (X, Y) for `epochs`, minibatches of `batch` rows in a
// fixed cyclic order; loss_history[epoch] = mean minibatch loss (optional).
int tlr_mlp_train(tlr_mlp *m, const float *X, const float *Y, int n, int epochs, int batch,
                  float lr, float *loss_history) {
  if (!m || !X || !Y || n < 1 || epochs < 1 || batch < 1) return TLR_ERR_ARG;
  batch = std::min(batch, n);
  int rc = ensure_capacity(m, batch);
  if (rc) return rc;
  float *dX = nullptr, *dY = nullptr;
  if (cudaMalloc(&dX, sizeof(float) * (size_t)n * m->n_in) ||
      cudaMalloc(&dY, sizeof(float) * (size_t)n * m->n_out)) {
    cudaFree(dX);
    return TLR_ERR_NOMEM;
  }
  cudaMemcpy(dX, X, sizeof(float) * (size_t)n * m->n_in, cudaMemcpyHostToDevice);
  cudaMemcpy(dY, Y, sizeof(float) * (size_t)n * m->n_out, cudaMemcpyHostToDevice);
  const size_t plane = (size_t)m->cap * m->maxw;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  std::vector<float> hl;
  for (int ep = 0; ep < epochs; ++ep) {
    double acc = 0.0;
    int nb = 0;
    for (int r0 = 0; r0 < n; r0 += batch) {
      const int nr = std::min(batch, n - r0);
      cudaMemcpyAsync(m->xbuf, dX + (size_t)r0 * m->n_in, sizeof(float) * nr * m->n_in,
                      cudaMemcpyDeviceToDevice, m->stream);
      cudaMemcpyAsync(m->ybuf, dY + (size_t)r0 * m->n_out, sizeof(float) * nr * m->n_out,
                      cudaMemcpyDeviceToDevice, m->stream);
      cudaMemsetAsync(m->grads, 0, sizeof(float) * m->n_params, m->stream);
      forward(m, nr);
      { k_mse<<<1, 256, 0, m->stream>>>(nr, m->n_out, m->maxw, m->act + plane * m->n_layers,
                                      m->ybuf, m->dact + plane * m->n_layers, m->loss); count_launches(); }
      backward(m, nr);
      ++m->adam_t;
      const float c1 = 1.f - std::pow(b1, (float)m->adam_t), c2 = 1.f - std::pow(b2, (float)m->adam_t);
      { k_adam<<<blocks_for(m->n_params, 256), 256, 0, m->stream>>>(m->n_params, m->params, m->grads,
                                                                  m->m1, m->m2, lr, b1, b2, c1, c2,
                                                                  eps); count_launches(); }
      if (loss_history) {
        float l = 0.f;
        cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
        cudaStreamSynchronize(m->stream);
        acc += l;
        ++nb;
      }
    }
    if (loss_history) loss_history[ep] = (float)(acc / std::max(nb, 1));
  }
  cudaFree(dX);
  cudaFree(dY);
  return cudaStreamSynchronize(m->stream) == cudaSuccess ? TLR_OK : TLR_ERR_CUDA;
}

// Inference: Y [n][n_out] from X [n][n_in] (host arrays); bf16 != 0 runs the
// BF16 path (weights and activations rounded to bf16, FP32 accumulation).
int tlr_mlp_forward(tlr_mlp *m, const float *X, int n, float *Y, int bf16) {
  if (!m || !X || !Y || n < 1) return TLR_ERR_ARG;
  int rc = ensure_capacity(m, n);
  if (rc) return rc;
  cudaMemcpyAsync(m->xbuf, X, sizeof(float) * n * m->n_in, cudaMemcpyHostToDevice, m->stream);
  const size_t plane = (size_t)m->cap * m->maxw;
  if (!bf16) {
    forward(m, n);
    // output plane has leading dimension maxw
    cudaMemcpy2DAsync(Y, sizeof(float) * m->n_out, m->act + plane * m->n_layers,
                      sizeof(float) * m->maxw, sizeof(float) * m->n_out, n,
                      cudaMemcpyDeviceToHost, m->stream);
  } else {
    { k_to_bf16<<<blocks_for(m->n_params, 256), 256, 0, m->stream>>>(m->n_params, m->params,
                                                                   m->params16); count_launches(); }
    __nv_bfloat16 *a = reinterpret_cast<__nv_bfloat16 *>(m->act);
    __nv_bfloat16 *bb = reinterpret_cast<__nv_bfloat16 *>(m->pre);
    { k_to_bf16<<<blocks_for((long long)n * m->n_in, 256), 256, 0, m->stream>>>(
        (long long)n * m->n_in, m->xbuf, a); count_launches(); }
    for (int l = 0; l < m->n_layers; ++l) {
      const int in = m->fan_in[l], o = m->fan_out[l];
      const bool last = l + 1 == m->n_layers;
      dim3 g((o + kT - 1) / kT, (n + kT - 1) / kT), b(kT, kT);
      { k_lin_fwd16<<<g, b, 0, m->stream>>>(n, in, o, a, m->params16 + m->w_off[l],
                                          m->params16 + m->b_off[l], last ? nullptr : bb,
                                          last ? m->dact : nullptr, !last); count_launches(); }
      std::swap(a, bb);
    }
    cudaMemcpyAsync(Y, m->dact, sizeof(float) * n * m->n_out, cudaMemcpyDeviceToHost, m->stream);
  }
  return cudaStreamSynchronize(m->stream) == cudaSuccess ? TLR_OK : TLR_ERR_CUDA;
}

}  // extern "C"
