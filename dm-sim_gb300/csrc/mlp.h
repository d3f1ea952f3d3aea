// mlp.h -- the pass cost model's network (mlp.cu).
#pragma once
#include <cuda_runtime.h>

namespace dmg {

constexpr int kMlpIn = 17;
constexpr int kMlpHidden = 32;
constexpr int kMlpParams = kMlpHidden * kMlpIn + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden + kMlpHidden + 1;

// y[b] = net(X[b]) for b < B (X row-major B x kMlpIn)
cudaError_t mlp_forward(const float* d_params, const float* d_X, int B, float* d_y, cudaStream_t s);
// grad = d(MSE)/d(params) over the batch (overwritten), *d_loss = MSE
cudaError_t mlp_grad(const float* d_params, const float* d_X, const float* d_T, int B, float* d_grad, float* d_loss,
                     cudaStream_t s);
// one Adam step (t >= 1)
cudaError_t mlp_adam(float* d_params, const float* d_grad, float* d_m, float* d_v, float lr, int t, cudaStream_t s);

}  // namespace dmg
