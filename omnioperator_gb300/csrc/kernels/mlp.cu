// Kernels of the learned sizing model: a small fully connected network (dense layers with ReLU)
// trained by hand-written forward / backward / Adam kernels.
//
// The network is tiny (a few thousand weights) and its batches are a few thousand sketches, so
// the kernels favour simplicity: one thread per output element, fp32 throughout, and every
// reduction over the batch done by one thread in a fixed order, so gradients are deterministic.
#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "mlp.h"

namespace omg {
namespace {

unsigned Blocks(int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    if (b > 65535) {
        b = 65535;
    }
    return static_cast<unsigned>(b < 1 ? 1 : b);
}

// Y[n, m] = act(X[n, k] * W[k, m] + b[m]); W row-major (k rows of m).
__global__ void DenseForwardKernel(const float *X, const float *W, const float *b, float *Y, int n, int k, int m,
    int relu)
{
    const int64_t total = static_cast<int64_t>(n) * m;
    for (int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int r = static_cast<int>(idx / m);
        const int c = static_cast<int>(idx % m);
        float acc = b[c];
        const float *x = X + static_cast<int64_t>(r) * k;
        for (int j = 0; j < k; ++j) {
            acc = fmaf(x[j], W[static_cast<int64_t>(j) * m + c], acc);
        }
        Y[idx] = (relu && acc < 0.f) ? 0.f : acc;
    }
}

// dZ = dY * (Y > 0) for ReLU layers (in place on dY), identity otherwise.
__global__ void ReluBackwardKernel(const float *Y, float *dY, int64_t total)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (Y[i] <= 0.f) {
            dY[i] = 0.f;
        }
    }
}

// dW[k, m] = X^T dZ / scale ;  db[m] = sum_r dZ[r, m] / scale.  One thread per weight.
__global__ void DenseWeightGradKernel(const float *X, const float *dZ, float *dW, float *db, int n, int k, int m,
    float invScale)
{
    const int64_t total = static_cast<int64_t>(k + 1) * m;
    for (int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int j = static_cast<int>(idx / m);
        const int c = static_cast<int>(idx % m);
        float acc = 0.f;
        if (j < k) {
            for (int r = 0; r < n; ++r) {
                acc = fmaf(X[static_cast<int64_t>(r) * k + j], dZ[static_cast<int64_t>(r) * m + c], acc);
            }
            dW[static_cast<int64_t>(j) * m + c] = acc * invScale;
        } else {
            for (int r = 0; r < n; ++r) {
                acc += dZ[static_cast<int64_t>(r) * m + c];
            }
            db[c] = acc * invScale;
        }
    }
}

// dX[n, k] = dZ[n, m] W^T.
__global__ void DenseInputGradKernel(const float *dZ, const float *W, float *dX, int n, int k, int m)
{
    const int64_t total = static_cast<int64_t>(n) * k;
    for (int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int r = static_cast<int>(idx / k);
        const int j = static_cast<int>(idx % k);
        float acc = 0.f;
        const float *dz = dZ + static_cast<int64_t>(r) * m;
        const float *w = W + static_cast<int64_t>(j) * m;
        for (int c = 0; c < m; ++c) {
            acc = fmaf(dz[c], w[c], acc);
        }
        dX[idx] = acc;
    }
}

// Mean squared error: dY = 2 (Y - T) (the 1/n is applied in the weight gradient), loss partials.
__global__ void MseGradKernel(const float *Y, const float *T, float *dY, int64_t total, float *loss)
{
    float local = 0.f;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float d = Y[i] - T[i];
        dY[i] = 2.f * d;
        local += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) {
        local += __shfl_down_sync(0xffffffffu, local, o);
    }
    if ((threadIdx.x & 31) == 0 && loss != nullptr) {
        atomicAdd(loss, local);  // the loss is reported only; its summation order does not matter
    }
}

__global__ void AdamKernel(float *w, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2,
    float eps, float c1, float c2)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace

cudaError_t LaunchDenseForward(const float *X, const float *W, const float *b, float *Y, int n, int k, int m,
    bool relu, cudaStream_t s)
{
    DenseForwardKernel<<<Blocks(static_cast<int64_t>(n) * m, 256), 256, 0, s>>>(X, W, b, Y, n, k, m, relu ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t LaunchReluBackward(const float *Y, float *dY, int64_t total, cudaStream_t s)
{
    ReluBackwardKernel<<<Blocks(total, 256), 256, 0, s>>>(Y, dY, total);
    return cudaGetLastError();
}

cudaError_t LaunchDenseWeightGrad(const float *X, const float *dZ, float *dW, float *db, int n, int k, int m,
    float invScale, cudaStream_t s)
{
    DenseWeightGradKernel<<<Blocks(static_cast<int64_t>(k + 1) * m, 128), 128, 0, s>>>(X, dZ, dW, db, n, k, m,
        invScale);
    return cudaGetLastError();
}

cudaError_t LaunchDenseInputGrad(const float *dZ, const float *W, float *dX, int n, int k, int m, cudaStream_t s)
{
    DenseInputGradKernel<<<Blocks(static_cast<int64_t>(n) * k, 256), 256, 0, s>>>(dZ, W, dX, n, k, m);
    return cudaGetLastError();
}

cudaError_t LaunchMseGrad(const float *Y, const float *T, float *dY, int64_t total, float *loss, cudaStream_t s)
{
    MseGradKernel<<<Blocks(total, 256), 256, 0, s>>>(Y, T, dY, total, loss);
    return cudaGetLastError();
}

cudaError_t LaunchAdam(float *w, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2,
    float eps, int step, cudaStream_t s)
{
    const float c1 = 1.f - powf(b1, static_cast<float>(step));
    const float c2 = 1.f - powf(b2, static_cast<float>(step));
    AdamKernel<<<Blocks(n, 256), 256, 0, s>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

}  // namespace omg
