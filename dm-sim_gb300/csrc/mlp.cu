// mlp.cu -- the pass cost model: a 17-32-32-1 ReLU network in FP32, with its
// forward (inference), backward and Adam kernels.  The engine trains it on
// per-pass timings it records on its own random circuits and uses it to score
// candidate fusion plans.
//
// Parameter layout (kMlpParams floats): W1[32][17], b1[32], W2[32][32], b2[32],
// W3[32], b3.  Loss: mean squared error on log(ms).
#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp.h"

namespace dmg {

namespace {
constexpr int I = kMlpIn, Hd = kMlpHidden;
constexpr int oW1 = 0, oB1 = oW1 + Hd * I, oW2 = oB1 + Hd, oB2 = oW2 + Hd * Hd, oW3 = oB2 + Hd, oB3 = oW3 + Hd;
static_assert(oB3 + 1 == kMlpParams, "parameter layout");

__device__ __forceinline__ void forward_one(const float* __restrict__ p, const float* x, float* a1, float* a2, float& out) {
#pragma unroll 4
  for (int j = 0; j < Hd; j++) {
    float z = p[oB1 + j];
#pragma unroll
    for (int k = 0; k < I; k++) z = fmaf(p[oW1 + j * I + k], x[k], z);
    a1[j] = fmaxf(z, 0.f);
  }
#pragma unroll 4
  for (int j = 0; j < Hd; j++) {
    float z = p[oB2 + j];
#pragma unroll 8
    for (int k = 0; k < Hd; k++) z = fmaf(p[oW2 + j * Hd + k], a1[k], z);
    a2[j] = fmaxf(z, 0.f);
  }
  float z = p[oB3];
#pragma unroll 8
  for (int k = 0; k < Hd; k++) z = fmaf(p[oW3 + k], a2[k], z);
  out = z;
}
}  // namespace

// One thread per sample: y[b] = f(X[b]).
__global__ void __launch_bounds__(256) k_mlp_forward(const float* __restrict__ p, const float* __restrict__ X, int B,
                                                     float* __restrict__ y) {
  __shared__ float sp[kMlpParams];
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) sp[i] = p[i];
  __syncthreads();
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  float x[I], a1[Hd], a2[Hd], out;
#pragma unroll
  for (int k = 0; k < I; k++) x[k] = X[b * I + k];
  forward_one(sp, x, a1, a2, out);
  y[b] = out;
}

// Loss gradient of the mean squared error over the batch, accumulated into
// grad (kMlpParams floats, zeroed by the caller); loss sum into *loss.
__global__ void __launch_bounds__(256) k_mlp_backward(const float* __restrict__ p, const float* __restrict__ X,
                                                      const float* __restrict__ T, int B, float* __restrict__ grad,
                                                      float* __restrict__ loss) {
  __shared__ float sp[kMlpParams];
  __shared__ float sg[kMlpParams];
  __shared__ float sl;
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) {
    sp[i] = p[i];
    sg[i] = 0.f;
  }
  if (threadIdx.x == 0) sl = 0.f;
  __syncthreads();
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < B) {
    float x[I], a1[Hd], a2[Hd], out;
#pragma unroll
    for (int k = 0; k < I; k++) x[k] = X[b * I + k];
    forward_one(sp, x, a1, a2, out);
    const float r = out - T[b];
    atomicAdd(&sl, r * r / (float)B);
    const float dout = 2.f * r / (float)B;
    atomicAdd(&sg[oB3], dout);
    float d2[Hd];
#pragma unroll 8
    for (int k = 0; k < Hd; k++) {
      atomicAdd(&sg[oW3 + k], dout * a2[k]);
      d2[k] = a2[k] > 0.f ? dout * sp[oW3 + k] : 0.f;
    }
    float d1[Hd];
#pragma unroll 4
    for (int k = 0; k < Hd; k++) d1[k] = 0.f;
    for (int j = 0; j < Hd; j++) {
      if (d2[j] == 0.f) continue;
      atomicAdd(&sg[oB2 + j], d2[j]);
      for (int k = 0; k < Hd; k++) {
        atomicAdd(&sg[oW2 + j * Hd + k], d2[j] * a1[k]);
        d1[k] = fmaf(sp[oW2 + j * Hd + k], d2[j], d1[k]);
      }
    }
    for (int j = 0; j < Hd; j++) {
      const float g = a1[j] > 0.f ? d1[j] : 0.f;
      if (g == 0.f) continue;
      atomicAdd(&sg[oB1 + j], g);
      for (int k = 0; k < I; k++) atomicAdd(&sg[oW1 + j * I + k], g * x[k]);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x)
    if (sg[i] != 0.f) atomicAdd(&grad[i], sg[i]);
  if (threadIdx.x == 0) atomicAdd(loss, sl);
}

// Adam step t (1-based) on all parameters.
__global__ void k_mlp_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                           float* __restrict__ v, float lr, int t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kMlpParams) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float mi = b1 * m[i] + (1.f - b1) * g[i];
  const float vi = b2 * v[i] + (1.f - b2) * g[i] * g[i];
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.f - powf(b1, (float)t));
  const float vh = vi / (1.f - powf(b2, (float)t));
  p[i] -= lr * mh / (sqrtf(vh) + eps);
}

cudaError_t mlp_forward(const float* d_params, const float* d_X, int B, float* d_y, cudaStream_t s) {
  if (B <= 0) return cudaSuccess;
  k_mlp_forward<<<(B + 255) / 256, 256, 0, s>>>(d_params, d_X, B, d_y);
  return cudaGetLastError();
}

cudaError_t mlp_grad(const float* d_params, const float* d_X, const float* d_T, int B, float* d_grad, float* d_loss,
                     cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(d_grad, 0, kMlpParams * sizeof(float), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(d_loss, 0, sizeof(float), s);
  if (e != cudaSuccess) return e;
  if (B <= 0) return cudaSuccess;
  k_mlp_backward<<<(B + 255) / 256, 256, 0, s>>>(d_params, d_X, d_T, B, d_grad, d_loss);
  return cudaGetLastError();
}

cudaError_t mlp_adam(float* d_params, const float* d_grad, float* d_m, float* d_v, float lr, int t, cudaStream_t s) {
  k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(d_params, d_grad, d_m, d_v, lr, t);
  return cudaGetLastError();
}

}  // namespace dmg
