// Kernels of the learned sizing model: a small fully connected network (dense layers with ReLU)
// trained by hand-written forward / backward / Adam kernels.
//
// The network is tiny (a few thousand weights) and its batches are a few thousand sketches, so
// the layer kernels favour simplicity: one thread per output element, fp32 throughout, and every
// reduction over the batch done by one thread in a fixed order, so gradients are deterministic.
// Training of the two-hidden-layer shapes runs fused: all epochs in one cooperative launch.
#include <cooperative_groups.h>
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

// ------------------------------------------------------------------ fused training
constexpr int kFusedThreads = 256;
constexpr int kFusedP = 64;  // points per tile
constexpr int kFusedMaxF = 16;
constexpr int kFusedMaxH = 64;

__host__ __device__ inline int Pad4(int x) { return (x + 3) & ~3; }

// Shared-memory layout (floats) of the fused trainer.
struct FusedLayout {
    int params, w2t, grads, x, t, a1, a2, d2, d1, y, total;
    __host__ __device__ FusedLayout(int nParams, int F, int H1, int H2)
    {
        params = 0;
        w2t = params + Pad4(nParams);
        grads = w2t + H1 * H2;
        x = grads + Pad4(nParams);
        t = x + Pad4(kFusedP * F);
        a1 = t + kFusedP;
        a2 = a1 + kFusedP * H1;
        d2 = a2 + kFusedP * H2;
        d1 = d2 + kFusedP * H2;
        y = d1 + kFusedP * H1;
        total = y + kFusedP;
    }
};

__global__ void __launch_bounds__(kFusedThreads) MlpTrainFusedKernel(const MlpFusedArgs a)
{
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    extern __shared__ float4 sFusedVec[];
    float *sm = reinterpret_cast<float *>(sFusedVec);
    const int F = a.F, H1 = a.H1, H2 = a.H2, NP = a.nParams;
    const FusedLayout L(NP, F, H1, H2);
    float *P = sm + L.params;
    float *W2T = sm + L.w2t;
    float *G = sm + L.grads;
    float *X = sm + L.x;
    float *Tt = sm + L.t;
    float *A1 = sm + L.a1;
    float *A2 = sm + L.a2;
    float *D2 = sm + L.d2;
    float *D1 = sm + L.d1;
    float *Y = sm + L.y;
    const int oW1 = 0, ob1 = F * H1, oW2 = ob1 + H1, ob2 = oW2 + H1 * H2, oW3 = ob2 + H2, ob3 = oW3 + H2;
    const int t = threadIdx.x;
    const int nCta = gridDim.x;
    const int per = (a.n + nCta - 1) / nCta;
    const int lo = blockIdx.x * per;
    const int hi = min(a.n, lo + per);
    const float invN = 1.f / static_cast<float>(a.n);
    double b1Pow = a.b1Pow;
    double b2Pow = a.b2Pow;
    for (int e = 0; e < a.epochs; ++e) {
        const bool last = e + 1 == a.epochs;
        for (int i = t; i < NP; i += kFusedThreads) {
            P[i] = a.params[i];
            G[i] = 0.f;
        }
        __syncthreads();
        for (int i = t; i < H1 * H2; i += kFusedThreads) {
            const int r = i / H2, c = i % H2;
            W2T[c * H1 + r] = P[oW2 + i];
        }
        float sse = 0.f;
        for (int base = lo; base < hi; base += kFusedP) {
            const int np = min(kFusedP, hi - base);
            for (int i = t; i < kFusedP * F; i += kFusedThreads) {
                const int p = i / F;
                X[i] = p < np ? a.X[static_cast<int64_t>(base + p) * F + (i % F)] : 0.f;
            }
            for (int p = t; p < kFusedP; p += kFusedThreads) {
                Tt[p] = p < np ? a.T[base + p] : 0.f;
            }
            __syncthreads();
            // Layer 1: A1 = relu(X W1 + b1).
            for (int i = t; i < kFusedP * H1; i += kFusedThreads) {
                const int p = i / H1, j = i % H1;
                float acc = P[ob1 + j];
                for (int f = 0; f < F; ++f) {
                    acc = fmaf(X[p * F + f], P[oW1 + f * H1 + j], acc);
                }
                A1[i] = acc > 0.f ? acc : 0.f;
            }
            __syncthreads();
            // Layer 2 in 4 x 4 register tiles: A2 = relu(A1 W2 + b2).
            for (int q = t; q < (kFusedP / 4) * (H2 / 4); q += kFusedThreads) {
                const int p0 = (q / (H2 / 4)) * 4, j0 = (q % (H2 / 4)) * 4;
                float acc[4][4];
                const float4 bb = *reinterpret_cast<const float4 *>(P + ob2 + j0);
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    acc[r][0] = bb.x;
                    acc[r][1] = bb.y;
                    acc[r][2] = bb.z;
                    acc[r][3] = bb.w;
                }
                for (int i = 0; i < H1; ++i) {
                    const float4 w = *reinterpret_cast<const float4 *>(P + oW2 + i * H2 + j0);
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        const float x = A1[(p0 + r) * H1 + i];
                        acc[r][0] = fmaf(x, w.x, acc[r][0]);
                        acc[r][1] = fmaf(x, w.y, acc[r][1]);
                        acc[r][2] = fmaf(x, w.z, acc[r][2]);
                        acc[r][3] = fmaf(x, w.w, acc[r][3]);
                    }
                }
#pragma unroll
                for (int r = 0; r < 4; ++r) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        A2[(p0 + r) * H2 + j0 + c] = acc[r][c] > 0.f ? acc[r][c] : 0.f;
                    }
                }
            }
            __syncthreads();
            // Output and the loss gradient: dY = 2 (y - t) / n (0 for padding rows).
            for (int p = t; p < kFusedP; p += kFusedThreads) {
                float acc = P[ob3];
                for (int j = 0; j < H2; ++j) {
                    acc = fmaf(A2[p * H2 + j], P[oW3 + j], acc);
                }
                const float d = p < np ? acc - Tt[p] : 0.f;
                Y[p] = 2.f * d * invN;
                sse += d * d;
            }
            __syncthreads();
            for (int i = t; i < kFusedP * H2; i += kFusedThreads) {
                const int p = i / H2, j = i % H2;
                D2[i] = A2[i] > 0.f ? Y[p] * P[oW3 + j] : 0.f;
            }
            __syncthreads();
            // D1 = (D2 W2^T) * (A1 > 0), 4 x 4 tiles over (point, input unit).
            for (int q = t; q < (kFusedP / 4) * (H1 / 4); q += kFusedThreads) {
                const int p0 = (q / (H1 / 4)) * 4, i0 = (q % (H1 / 4)) * 4;
                float acc[4][4] = {};
                for (int j = 0; j < H2; ++j) {
                    const float4 w = *reinterpret_cast<const float4 *>(W2T + j * H1 + i0);
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        const float d = D2[(p0 + r) * H2 + j];
                        acc[r][0] = fmaf(d, w.x, acc[r][0]);
                        acc[r][1] = fmaf(d, w.y, acc[r][1]);
                        acc[r][2] = fmaf(d, w.z, acc[r][2]);
                        acc[r][3] = fmaf(d, w.w, acc[r][3]);
                    }
                }
#pragma unroll
                for (int r = 0; r < 4; ++r) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const int idx = (p0 + r) * H1 + i0 + c;
                        D1[idx] = A1[idx] > 0.f ? acc[r][c] : 0.f;
                    }
                }
            }
            __syncthreads();
            // Gradient sums; every entry of G has one owner thread.  dW2 in 4 x 4 tiles.
            for (int q = t; q < (H1 / 4) * (H2 / 4); q += kFusedThreads) {
                const int i0 = (q / (H2 / 4)) * 4, j0 = (q % (H2 / 4)) * 4;
                float acc[4][4] = {};
                for (int p = 0; p < kFusedP; ++p) {
                    const float4 d = *reinterpret_cast<const float4 *>(D2 + p * H2 + j0);
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        const float x = A1[p * H1 + i0 + r];
                        acc[r][0] = fmaf(x, d.x, acc[r][0]);
                        acc[r][1] = fmaf(x, d.y, acc[r][1]);
                        acc[r][2] = fmaf(x, d.z, acc[r][2]);
                        acc[r][3] = fmaf(x, d.w, acc[r][3]);
                    }
                }
#pragma unroll
                for (int r = 0; r < 4; ++r) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        G[oW2 + (i0 + r) * H2 + j0 + c] += acc[r][c];
                    }
                }
            }
            // W1, b1, b2, W3, b3: (F + 1) * H1 + 2 * H2 + 1 entries.
            const int nSmall = (F + 1) * H1 + 2 * H2 + 1;
            for (int q = t; q < nSmall; q += kFusedThreads) {
                float acc = 0.f;
                int dst;
                if (q < F * H1) {
                    const int f = q / H1, j = q % H1;
                    for (int p = 0; p < kFusedP; ++p) {
                        acc = fmaf(X[p * F + f], D1[p * H1 + j], acc);
                    }
                    dst = oW1 + q;
                } else if (q < (F + 1) * H1) {
                    const int j = q - F * H1;
                    for (int p = 0; p < kFusedP; ++p) {
                        acc += D1[p * H1 + j];
                    }
                    dst = ob1 + j;
                } else if (q < (F + 1) * H1 + H2) {
                    const int j = q - (F + 1) * H1;
                    for (int p = 0; p < kFusedP; ++p) {
                        acc += D2[p * H2 + j];
                    }
                    dst = ob2 + j;
                } else if (q < (F + 1) * H1 + 2 * H2) {
                    const int j = q - (F + 1) * H1 - H2;
                    for (int p = 0; p < kFusedP; ++p) {
                        acc = fmaf(A2[p * H2 + j], Y[p], acc);
                    }
                    dst = oW3 + j;
                } else {
                    for (int p = 0; p < kFusedP; ++p) {
                        acc += Y[p];
                    }
                    dst = ob3;
                }
                G[dst] += acc;
            }
            __syncthreads();
        }
        if (last && a.loss != nullptr) {
            for (int o = 16; o > 0; o >>= 1) {
                sse += __shfl_down_sync(0xffffffffu, sse, o);
            }
            if ((t & 31) == 0) {
                atomicAdd(a.loss, sse);  // reported only
            }
        }
        for (int i = t; i < NP; i += kFusedThreads) {
            a.partial[static_cast<int64_t>(blockIdx.x) * NP + i] = G[i];
        }
        grid.sync();
        // Adam on this CTA's slice of the parameters, gradients summed over the CTAs in order.
        b1Pow *= a.b1;
        b2Pow *= a.b2;
        const float c1 = static_cast<float>(1.0 - b1Pow);
        const float c2 = static_cast<float>(1.0 - b2Pow);
        for (int i = blockIdx.x * kFusedThreads + t; i < NP; i += nCta * kFusedThreads) {
            float g = 0.f;
            for (int c = 0; c < nCta; ++c) {
                g += a.partial[static_cast<int64_t>(c) * NP + i];
            }
            if (a.gradOut != nullptr) {
                a.gradOut[i] = g;
                continue;
            }
            const float mi = a.b1 * a.adamM[i] + (1.f - a.b1) * g;
            const float vi = a.b2 * a.adamV[i] + (1.f - a.b2) * g * g;
            a.adamM[i] = mi;
            a.adamV[i] = vi;
            a.params[i] -= a.lr * (mi / c1) / (sqrtf(vi / c2) + a.eps);
        }
        grid.sync();
        if (a.gradOut != nullptr) {
            break;
        }
    }
}

}  // namespace

bool MlpFusedSupported(int F, int H1, int H2)
{
    return F >= 1 && F <= kFusedMaxF && H1 >= 4 && H1 <= kFusedMaxH && H1 % 4 == 0 && H2 >= 4 && H2 <= kFusedMaxH &&
        H2 % 4 == 0;
}

int MlpFusedGrid(int n)
{
    int dev = 0;
    int sms = 1;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 1;
    }
    const int tiles = (n + kFusedP - 1) / kFusedP;
    return tiles < sms ? (tiles > 0 ? tiles : 1) : sms;
}

cudaError_t LaunchMlpTrainFused(const MlpFusedArgs &a, int grid, cudaStream_t s)
{
    const FusedLayout L(a.nParams, a.F, a.H1, a.H2);
    const size_t smem = static_cast<size_t>(L.total) * sizeof(float);
    cudaError_t err = cudaFuncSetAttribute(reinterpret_cast<const void *>(MlpTrainFusedKernel),
        cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (err != cudaSuccess) {
        return err;
    }
    int perSm = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, MlpTrainFusedKernel, kFusedThreads, smem);
    if (err != cudaSuccess) {
        return err;
    }
    if (perSm < 1) {
        return cudaErrorCooperativeLaunchTooLarge;
    }
    MlpFusedArgs args = a;
    void *kargs[] = {&args};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(MlpTrainFusedKernel), dim3(grid),
        dim3(kFusedThreads), kargs, smem, s);
}

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
