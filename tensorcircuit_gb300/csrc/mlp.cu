// mlp.cu — the warm-start network's training and inference kernels: dense
// layers with a fused GELU epilogue (float32 weights, bfloat16 activations,
// float32 accumulation), their backward pass, a periodic regression loss for
// circuit angles and the Adam update.
//
// The network is small (31 -> 256 -> 256 -> 186), so every GEMM is a 64x64
// output tile per CTA staged through shared memory in 16-wide k slices, each
// thread accumulating a 4x4 register block; no layer is large enough for a
// tensor-core pipeline to pay for its setup.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.h"

namespace tcg {
namespace {

constexpr int TM = 64, TN = 64, TK = 16;

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
__device__ __forceinline__ float gelu_f(float x) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  return 0.5f * x * (1.f + tanhf(k0 * (x + k1 * x * x * x)));
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  const float u = k0 * (x + k1 * x * x * x);
  const float t = tanhf(u);
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * k0 * (1.f + 3.f * k1 * x * x);
}

template <bool XBF16>
__device__ __forceinline__ float ldx(const void* x, int64_t i) {
  if (XBF16) return __bfloat162float(static_cast<const __nv_bfloat16*>(x)[i]);
  return static_cast<const float*>(x)[i];
}

// Y[b][o] = act(sum_i X[b][i] W[o][i] + bias[o]); pre-activation kept in
// float32 when pre != null; Y in bfloat16 (hidden layers) or float32 (output).
template <bool XBF16, bool YBF16>
__global__ void __launch_bounds__(256) linear_fwd_kernel(const void* __restrict__ X, const float* __restrict__ W,
                                                         const float* __restrict__ bias, int64_t B, int in, int out,
                                                         int act, float* __restrict__ pre, void* __restrict__ Y) {
  __shared__ float sx[TK][TM + 1];
  __shared__ float sw[TK][TN + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t b0 = int64_t(blockIdx.y) * TM;
  const int o0 = blockIdx.x * TN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < in; k0 += TK) {
    for (int e = threadIdx.x; e < TK * TM; e += 256) {
      const int kk = e % TK, r = e / TK;
      const int64_t bb = b0 + r;
      sx[kk][r] = (bb < B && k0 + kk < in) ? ldx<XBF16>(X, bb * in + k0 + kk) : 0.f;
      const int oo = o0 + r;
      sw[kk][r] = (oo < out && k0 + kk < in) ? W[int64_t(oo) * in + k0 + kk] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      float a[4], w[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sx[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) w[j] = sw[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], w[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t bb = b0 + ty * 4 + i;
    if (bb >= B) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int oo = o0 + tx * 4 + j;
      if (oo >= out) continue;
      const float z = acc[i][j] + (bias ? bias[oo] : 0.f);
      if (pre) pre[bb * out + oo] = z;
      const float y = act ? gelu_f(z) : z;
      if (YBF16) static_cast<__nv_bfloat16*>(Y)[bb * out + oo] = __float2bfloat16(y);
      else static_cast<float*>(Y)[bb * out + oo] = y;
    }
  }
}

// dZ[b][o] = dY[b][o] * act'(pre[b][o])   (in place into dz)
__global__ void act_bwd_kernel(const float* __restrict__ dy, const float* __restrict__ pre, int64_t n, int act,
                               float* __restrict__ dz) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    dz[i] = act ? dy[i] * gelu_grad(pre[i]) : dy[i];
}

// dW[o][i] = sum_b dZ[b][o] X[b][i]  (overwritten), one 64x64 tile per CTA,
// the batch is the reduction dimension (fixed order: deterministic).
template <bool XBF16>
__global__ void __launch_bounds__(256) linear_dw_kernel(const float* __restrict__ dZ, const void* __restrict__ X,
                                                        int64_t B, int in, int out, float* __restrict__ dW) {
  __shared__ float sz[TK][TN + 1];
  __shared__ float sx[TK][TM + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int o0 = blockIdx.y * TN;
  const int i0 = blockIdx.x * TM;
  float acc[4][4] = {};
  for (int64_t k0 = 0; k0 < B; k0 += TK) {
    for (int e = threadIdx.x; e < TK * TN; e += 256) {
      const int kk = e / TN, r = e % TN;
      const int64_t bb = k0 + kk;
      sz[kk][r] = (bb < B && o0 + r < out) ? dZ[bb * out + o0 + r] : 0.f;
      sx[kk][r] = (bb < B && i0 + r < in) ? ldx<XBF16>(X, bb * in + i0 + r) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      float a[4], x[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sz[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) x[j] = sx[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], x[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int oo = o0 + ty * 4 + i;
    if (oo >= out) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int ii = i0 + tx * 4 + j;
      if (ii < in) dW[int64_t(oo) * in + ii] = acc[i][j];
    }
  }
}

// db[o] = sum_b dZ[b][o]: one warp per output, fixed lane order.
__global__ void linear_db_kernel(const float* __restrict__ dZ, int64_t B, int out, float* __restrict__ db) {
  const int o = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (o >= out) return;
  float s = 0.f;
  for (int64_t b = lane; b < B; b += 32) s += dZ[b * out + o];
#pragma unroll
  for (int k = 16; k > 0; k >>= 1) s += __shfl_xor_sync(0xffffffffu, s, k);
  if (lane == 0) db[o] = s;
}

// dX[b][i] = sum_o dZ[b][o] W[o][i]
__global__ void __launch_bounds__(256) linear_dx_kernel(const float* __restrict__ dZ, const float* __restrict__ W,
                                                        int64_t B, int in, int out, float* __restrict__ dX) {
  __shared__ float sz[TK][TM + 1];
  __shared__ float sw[TK][TN + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t b0 = int64_t(blockIdx.y) * TM;
  const int i0 = blockIdx.x * TN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < out; k0 += TK) {
    for (int e = threadIdx.x; e < TK * TM; e += 256) {
      const int kk = e % TK, r = e / TK;
      const int64_t bb = b0 + r;
      sz[kk][r] = (bb < B && k0 + kk < out) ? dZ[bb * out + k0 + kk] : 0.f;
      const int ii = i0 + r;
      sw[kk][r] = (ii < in && k0 + kk < out) ? W[int64_t(k0 + kk) * in + ii] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      float a[4], w[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sz[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) w[j] = sw[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], w[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t bb = b0 + ty * 4 + i;
    if (bb >= B) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int ii = i0 + tx * 4 + j;
      if (ii < in) dX[bb * in + ii] = acc[i][j];
    }
  }
}

// Periodic angle loss: per element 1 - cos(pred - target), gradient
// sin(pred - target) / count; per-block partial sums of the loss.
__global__ void periodic_loss_kernel(const float* __restrict__ pred, const float* __restrict__ target, int64_t n,
                                     float inv_count, float* __restrict__ dpred, float* __restrict__ partial) {
  __shared__ float red[256];
  float s = 0.f;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    float sn, cs;
    sincosf(pred[i] - target[i], &sn, &cs);
    s += 1.f - cs;
    dpred[i] = sn * inv_count;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0] * inv_count;
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

unsigned grid_for(int64_t n, int threads, unsigned cap = 2048) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  return (unsigned)(g > cap ? cap : g);
}

}  // namespace
}  // namespace tcg

using namespace tcg;

extern "C" {

int tcg_mlp_linear_forward(const void* x, int32_t x_bf16, const float* w, const float* bias, int64_t batch,
                           int32_t in, int32_t out, int32_t act, float* pre, void* y, int32_t y_bf16,
                           void* stream) {
  if (!x || !w || !y || batch < 0 || in < 1 || out < 1 || act < 0 || act > 1) return TCG_ERR_INVALID_ARG;
  if (batch == 0) return TCG_OK;
  if ((batch + TM - 1) / TM > 65535) return TCG_ERR_INVALID_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  dim3 grid((out + TN - 1) / TN, (unsigned)((batch + TM - 1) / TM));
  count_launch();
  if (x_bf16 && y_bf16) linear_fwd_kernel<true, true><<<grid, 256, 0, st>>>(x, w, bias, batch, in, out, act, pre, y);
  else if (x_bf16) linear_fwd_kernel<true, false><<<grid, 256, 0, st>>>(x, w, bias, batch, in, out, act, pre, y);
  else if (y_bf16) linear_fwd_kernel<false, true><<<grid, 256, 0, st>>>(x, w, bias, batch, in, out, act, pre, y);
  else linear_fwd_kernel<false, false><<<grid, 256, 0, st>>>(x, w, bias, batch, in, out, act, pre, y);
  return cudaGetLastError() == cudaSuccess ? TCG_OK : TCG_ERR_CUDA;
}

int tcg_mlp_linear_backward(const float* dy, const float* pre, int32_t act, const void* x, int32_t x_bf16,
                            const float* w, int64_t batch, int32_t in, int32_t out, float* dz, float* dw,
                            float* db, float* dx, void* stream) {
  if (!dy || !dz || !x || !w || !dw || !db || batch < 1 || in < 1 || out < 1 || (act && !pre))
    return TCG_ERR_INVALID_ARG;
  if ((batch + TM - 1) / TM > 65535) return TCG_ERR_INVALID_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t nz = batch * out;
  count_launch();
  act_bwd_kernel<<<grid_for(nz, 256), 256, 0, st>>>(dy, pre, nz, act, dz);
  dim3 gw((in + TM - 1) / TM, (out + TN - 1) / TN);
  count_launch();
  if (x_bf16) linear_dw_kernel<true><<<gw, 256, 0, st>>>(dz, x, batch, in, out, dw);
  else linear_dw_kernel<false><<<gw, 256, 0, st>>>(dz, x, batch, in, out, dw);
  count_launch();
  linear_db_kernel<<<(out + 7) / 8, 256, 0, st>>>(dz, batch, out, db);
  if (dx) {
    dim3 gx((in + TN - 1) / TN, (unsigned)((batch + TM - 1) / TM));
    count_launch();
    linear_dx_kernel<<<gx, 256, 0, st>>>(dz, w, batch, in, out, dx);
  }
  return cudaGetLastError() == cudaSuccess ? TCG_OK : TCG_ERR_CUDA;
}

int tcg_periodic_loss(const float* pred, const float* target, int64_t n, float* dpred, float* partial,
                      int32_t nblocks, void* stream) {
  if (!pred || !target || !dpred || !partial || n < 1 || nblocks < 1) return TCG_ERR_INVALID_ARG;
  count_launch();
  periodic_loss_kernel<<<nblocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(pred, target, n, 1.f / float(n),
                                                                              dpred, partial);
  return cudaGetLastError() == cudaSuccess ? TCG_OK : TCG_ERR_CUDA;
}

int tcg_adam_update(float* p, const float* g, float* m, float* v, int64_t n, float lr, float beta1, float beta2,
                    float eps, int32_t step, void* stream) {
  if (!p || !g || !m || !v || n < 0 || step < 1) return TCG_ERR_INVALID_ARG;
  if (n == 0) return TCG_OK;
  const float c1 = 1.f - powf(beta1, (float)step);
  const float c2 = 1.f - powf(beta2, (float)step);
  count_launch();
  adam_kernel<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(p, g, m, v, n, lr, beta1, beta2,
                                                                               eps, c1, c2);
  return cudaGetLastError() == cudaSuccess ? TCG_OK : TCG_ERR_CUDA;
}

}  // extern "C"
