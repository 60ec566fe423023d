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

// Fused full-batch training of a network F -> H1 -> H2 -> 1 (ReLU hidden layers, MSE loss, Adam):
// all epochs in one cooperative launch.  Each CTA keeps the weights in shared memory, runs the
// forward and backward passes over tiles of its share of the points and writes its gradient sums;
// after a grid barrier every CTA reduces a slice of the parameters over all CTAs' sums (in CTA
// order, so the result is deterministic) and applies Adam to it; after a second barrier every CTA
// reloads the weights.  Parameter layout as SizingModel: W1 (F x H1), b1, W2 (H1 x H2), b2, W3, b3.
struct MlpFusedArgs {
    const float *X;   // [n, F]
    const float *T;   // [n]
    int32_t n, F, H1, H2;
    int32_t nParams;
    int32_t epochs;
    float *params;    // updated in place
    float *adamM;
    float *adamV;
    float *partial;   // [grid, nParams] scratch
    float *loss;      // sum of squared errors of the last epoch (before its update), may be null
    float *gradOut;   // non-null: write the mean-loss gradient of the first epoch here, update nothing
    float lr, b1, b2, eps;
    double b1Pow, b2Pow;  // b1^step and b2^step before the first epoch
};
// True when the fused trainer takes these dims (F <= 16, H1 and H2 multiples of 4 up to 64).
bool MlpFusedSupported(int F, int H1, int H2);
// Launches the fused trainer; `grid` (<= the SM count, from MlpFusedGrid) CTAs.
int MlpFusedGrid(int n);
cudaError_t LaunchMlpTrainFused(const MlpFusedArgs &a, int grid, cudaStream_t s);

}  // namespace omg
