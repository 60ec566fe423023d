// Learned sizing model: a small fully connected network that maps the key sketch an aggregation
// operator takes of its first flush to a group-count estimate.  Its parameters live in HBM and
// it is trained and evaluated by the kernels of kernels/mlp.cu.
#pragma once

#include <cstdint>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "host/gpu_runtime.h"

namespace omg {

// Plain group-count estimate from a key sketch (kSketchStats values) of n sampled rows out of
// `rows`: the GEE estimator sqrt(rows / n) * f1 + (d - f1), clamped to [d, rows], plus the
// special groups the sample saw.
uint64_t PlainGroupEstimate(const unsigned long long *sketch, int64_t rows);
// HyperLogLog estimate from 2^kHllBits registers plus the two special-key flags (Flajolet et
// al. 2007: alpha_m m^2 / sum 2^-M[j], with linear counting m ln(m / V) below 2.5 m when V
// registers are zero); at most `rows`.
uint64_t HllGroupEstimate(const unsigned int *regs, int64_t rows);

// Features of a sizing record (the layout written by HashAggregationOperator::GetSizingLog):
// scale-free functions of the rows N, the sampled rows n, the distinct hashes d of the sample,
// its frequency classes and the plain estimate.
constexpr int kSizerFeatures = 12;
void SizerFeatures(const int64_t *log, float *features);
// Estimate from the model output y: d * 2^(16 y), clamped to [d, N].
uint64_t SizerEstimate(const int64_t *log, float y);
// Target of a sizing record with known group count G: log2(G / d) / 16.
float SizerTarget(const int64_t *log, int64_t groups);

// Range-partition splits learned from a key sample, a two-stage model of the keys' CDF: a network
// 1 -> 32 -> 32 -> 1 trained on the GPU (by the same kernels) maps a normalised key to its
// empirical CDF and routes the key to one of K leaves, each a least-squares line of the CDF over
// its keys.  Split i (1 <= i < 2^bits) is the first sample key whose predicted CDF reaches
// i / 2^bits (predictions made monotone by a running maximum).  Writes 2^bits - 1 sorted splits.
void LearnRangeSplits(const int64_t *sample, int64_t n, int32_t bits, int32_t epochs, uint64_t seed, int64_t *splits);
// Exact sample quantiles as 2^bits - 1 range splits: split k is the sorted sample's key at rank
// floor(k * n / 2^bits) (the method without a network, for comparison with the learned splits).
void QuantileSplits(const int64_t *sample, int64_t n, int32_t bits, int64_t *splits);

// Process-wide: train the two-hidden-layer shapes with the fused kernel (default) or layer by
// layer; for tests and measurements.
void SetFusedTraining(bool on);

class SizingModel {
public:
    // dims: input width, hidden widths..., 1.  Weights: He-uniform from `seed`, biases zero.
    SizingModel(const std::vector<int32_t> &dims, uint64_t seed);
    ~SizingModel();
    SizingModel(const SizingModel &) = delete;
    SizingModel &operator=(const SizingModel &) = delete;

    int64_t NumParams() const { return nParams_; }
    const std::vector<int32_t> &Dims() const { return dims_; }
    void GetParams(float *out);
    void SetParams(const float *in);
    // Y[n] = model(X[n, dims[0]]); host pointers.
    void Predict(const float *X, int32_t n, float *Y);
    // Gradient of the mean squared error over the batch w.r.t. every parameter (layout as
    // GetParams); returns the loss.
    float Gradients(const float *X, const float *T, int32_t n, float *grad);
    // `epochs` full-batch Adam steps; returns the loss before the last step.
    float Train(const float *X, const float *T, int32_t n, int32_t epochs, float lr);

private:
    void Forward(int32_t n);
    float Backward(int32_t n);
    void Upload(const float *X, const float *T, int32_t n);
    bool Fused() const;
    float RunFused(int32_t n, int32_t epochs, float lr, float *gradOut);

    std::vector<int32_t> dims_;
    std::vector<int64_t> wOff_, bOff_;  // offsets of each layer's W and b in the parameter vector
    int64_t nParams_ = 0;
    std::mutex mu_;
    cudaStream_t stream_ = nullptr;
    DevArray<float> params_, grads_, adamM_, adamV_;
    DevArray<float> x_, t_, loss_;
    DevArray<float> partial_;  // fused training: per-CTA gradient sums
    std::vector<DevArray<float>> act_;   // activations per layer output
    std::vector<DevArray<float>> dact_;  // their gradients
    int32_t capacity_ = 0;
    int32_t step_ = 0;
};

}  // namespace omg
