// Launchers of the sizing model's kernels (mlp.cu).  Matrices are row-major fp32; W of a dense
// layer is k x m (input x output).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace omg {

// Y[n, m] = act(X[n, k] W + b), act = ReLU when `relu`.
cudaError_t LaunchDenseForward(const float *X, const float *W, const float *b, float *Y, int n, int k, int m,
    bool relu, cudaStream_t s);
// dY[i] = 0 where Y[i] <= 0 (ReLU backward, in place).
cudaError_t LaunchReluBackward(const float *Y, float *dY, int64_t total, cudaStream_t s);
// dW = X^T dZ * invScale, db = column sums of dZ * invScale.
cudaError_t LaunchDenseWeightGrad(const float *X, const float *dZ, float *dW, float *db, int n, int k, int m,
    float invScale, cudaStream_t s);
// dX = dZ W^T.
cudaError_t LaunchDenseInputGrad(const float *dZ, const float *W, float *dX, int n, int k, int m, cudaStream_t s);
// dY = 2 (Y - T); *loss += sum (Y - T)^2 (loss may be null).
cudaError_t LaunchMseGrad(const float *Y, const float *T, float *dY, int64_t total, float *loss, cudaStream_t s);
// One Adam step (bias-corrected with `step`, counted from 1).
cudaError_t LaunchAdam(float *w, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2,
    float eps, int step, cudaStream_t s);

}  // namespace omg
