// mlp.cu -- the method selector's network: a 3-layer, 64-wide FP32 MLP
//   x (8 features) -> Linear 8x64 -> ReLU -> Linear 64x64 -> ReLU -> Linear 64x7
// that predicts the (standardised) log run time of each candidate algorithm
// (method and tile, xc_algorithm),
// with hand-written inference, gradient and Adam kernels.  New in this
// library: the reference picks algorithms by hand (its YAML sweeps,
// benchmarking/args_test/*.yml).
//
// Parameter layout (XC_MLP_PARAMS floats):
//   W1[64][8], b1[64], W2[64][64], b2[64], W3[7][64], b3[7]
// The forward kernel runs one 64-thread block per sample; the gradient kernel
// recomputes the activations per sample and accumulates the mean-squared
// error gradients (masked: unavailable candidates carry mask 0) with atomics.
#include "xc_common.cuh"
#include "xc_internal.h"

namespace xc {

namespace {

constexpr int IN = XC_MLP_IN, H = XC_MLP_HIDDEN, OUT = XC_MLP_OUT;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * IN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H;
constexpr int OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + OUT * H, NPARAMS = OFF_B3 + OUT;
static_assert(NPARAMS == XC_MLP_PARAMS, "parameter count");

// Activations of one sample in shared memory; thread j owns hidden unit j.
__device__ __forceinline__ void forward_sample(const float* __restrict__ P, const float* __restrict__ x, float* s_x,
                                               float* h1, float* h2, float* y) {
  const int j = threadIdx.x;
  if (j < IN) s_x[j] = x[j];
  __syncthreads();
  float a = P[OFF_B1 + j];
#pragma unroll
  for (int i = 0; i < IN; ++i) a = fmaf(P[OFF_W1 + j * IN + i], s_x[i], a);
  h1[j] = fmaxf(a, 0.0f);
  __syncthreads();
  float b = P[OFF_B2 + j];
#pragma unroll 8
  for (int k = 0; k < H; ++k) b = fmaf(P[OFF_W2 + j * H + k], h1[k], b);
  h2[j] = fmaxf(b, 0.0f);
  __syncthreads();
  if (j < OUT) {
    float c = P[OFF_B3 + j];
#pragma unroll 8
    for (int k = 0; k < H; ++k) c = fmaf(P[OFF_W3 + j * H + k], h2[k], c);
    y[j] = c;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(H) mlp_forward_kernel(const float* __restrict__ P, const float* __restrict__ X,
                                                        int n, float* __restrict__ Y) {
  __shared__ float s_x[IN], h1[H], h2[H], y[OUT];
  const int s = blockIdx.x;
  if (s >= n) return;
  forward_sample(P, X + (long long)s * IN, s_x, h1, h2, y);
  if (threadIdx.x < OUT) Y[(long long)s * OUT + threadIdx.x] = y[threadIdx.x];
}

// loss = sum_s sum_o m[s][o] (y[s][o] - t[s][o])^2 / sum m ; grads of loss.
__global__ void __launch_bounds__(H) mlp_grad_kernel(const float* __restrict__ P, const float* __restrict__ X,
                                                     const float* __restrict__ T, const float* __restrict__ M, int n,
                                                     float inv_count, float* __restrict__ G,
                                                     float* __restrict__ loss) {
  __shared__ float s_x[IN], h1[H], h2[H], y[OUT], dy[OUT], dh2[H];
  const int s = blockIdx.x;
  if (s >= n) return;
  const int j = threadIdx.x;
  forward_sample(P, X + (long long)s * IN, s_x, h1, h2, y);
  if (j < OUT) {
    const float m = M[(long long)s * OUT + j];
    const float d = y[j] - T[(long long)s * OUT + j];
    dy[j] = m * 2.0f * d * inv_count;
    atomicAdd(loss, m * d * d * inv_count);
    atomicAdd(&G[OFF_B3 + j], dy[j]);
  }
  __syncthreads();
  // layer 3: dW3[o][j] = dy[o] * h2[j]; dh2[j] = sum_o W3[o][j] dy[o] (ReLU gate)
  float g2 = 0.0f;
#pragma unroll
  for (int o = 0; o < OUT; ++o) {
    atomicAdd(&G[OFF_W3 + o * H + j], dy[o] * h2[j]);
    g2 = fmaf(P[OFF_W3 + o * H + j], dy[o], g2);
  }
  dh2[j] = h2[j] > 0.0f ? g2 : 0.0f;
  __syncthreads();
  // layer 2: dW2[j][k] = dh2[j] * h1[k]; dh1[j] = sum_i W2[i][j] dh2[i] (ReLU gate)
  atomicAdd(&G[OFF_B2 + j], dh2[j]);
  for (int k = 0; k < H; ++k) atomicAdd(&G[OFF_W2 + j * H + k], dh2[j] * h1[k]);
  float g1 = 0.0f;
  for (int i = 0; i < H; ++i) g1 = fmaf(P[OFF_W2 + i * H + j], dh2[i], g1);
  const float dh1 = h1[j] > 0.0f ? g1 : 0.0f;
  // layer 1
  atomicAdd(&G[OFF_B1 + j], dh1);
#pragma unroll
  for (int i = 0; i < IN; ++i) atomicAdd(&G[OFF_W1 + j * IN + i], dh1 * s_x[i]);
}

// Adam (Kingma & Ba 2015) with bias correction.
__global__ void adam_kernel(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ Mo,
                            float* __restrict__ V, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = G[i];
  const float m = b1 * Mo[i] + (1.0f - b1) * g;
  const float v = b2 * V[i] + (1.0f - b2) * g * g;
  Mo[i] = m;
  V[i] = v;
  P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

}  // namespace

xc_status mlp_forward(const float* params, const float* x, uint32_t n, float* y, cudaStream_t stream) {
  if (n == 0) return XC_OK;
  mlp_forward_kernel<<<n, H, 0, stream>>>(params, x, (int)n, y);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

xc_status mlp_gradient(const float* params, const float* x, const float* target, const float* mask, uint32_t n,
                       float mask_count, float* grad, float* loss, cudaStream_t stream) {
  XC_CUDA_TRY(cudaMemsetAsync(grad, 0, sizeof(float) * NPARAMS, stream));
  XC_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), stream));
  if (n == 0 || mask_count <= 0.0f) return XC_OK;
  mlp_grad_kernel<<<n, H, 0, stream>>>(params, x, target, mask, (int)n, 1.0f / mask_count, grad, loss);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

xc_status mlp_adam(float* params, const float* grad, float* m, float* v, uint32_t step, float lr,
                   cudaStream_t stream) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  adam_kernel<<<(NPARAMS + 255) / 256, 256, 0, stream>>>(params, grad, m, v, NPARAMS, lr, b1, b2, eps, c1, c2);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

}  // namespace xc
