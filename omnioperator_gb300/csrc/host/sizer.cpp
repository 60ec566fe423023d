// Learned sizing model (see sizer.h).
#include <atomic>
#include "host/sizer.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "kernels/mlp.h"

namespace omg {

namespace {
// Sizing record fields (HashAggregationOperator::GetSizingLog).
constexpr int kLogRows = 0;
constexpr int kLogSampled = 1;
constexpr int kLogSpecial = 2;
constexpr int kLogDistinct = 3;
constexpr int kLogF1 = 4;
constexpr int kLogF2 = 5;
constexpr int kLogF3 = 6;
constexpr int kLogF4to7 = 7;
constexpr int kLogF8 = 8;
constexpr int kLogMax = 9;
constexpr int kLogHeavy = 10;

double L2(double v) { return std::log2(v + 1.0); }

// SplitMix64 stream for the initial weights.
struct SplitMix {
    uint64_t s;
    uint64_t Next()
    {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double Uniform() { return static_cast<double>(Next() >> 11) * (1.0 / 9007199254740992.0); }
};
}  // namespace

uint64_t HllGroupEstimate(const unsigned int *regs, int64_t rows)
{
    const double m = static_cast<double>(kHllRegs);
    double z = 0.0;
    int64_t zeros = 0;
    for (int i = 0; i < kHllRegs; ++i) {
        z += std::ldexp(1.0, -static_cast<int>(regs[i]));
        zeros += regs[i] == 0 ? 1 : 0;
    }
    const double alpha = 0.7213 / (1.0 + 1.079 / m);
    double e = alpha * m * m / z;
    if (e <= 2.5 * m && zeros > 0) {
        e = m * std::log(m / static_cast<double>(zeros));
    }
    e += static_cast<double>(regs[kHllRegs] + regs[kHllRegs + 1]);
    const double capped = std::min(std::max(e, 1.0), static_cast<double>(std::max<int64_t>(rows, 1)));
    return static_cast<uint64_t>(std::llround(capped));
}

uint64_t PlainGroupEstimate(const unsigned long long *st, int64_t total)
{
    const double n = static_cast<double>(st[0] - st[1]);
    const double d = static_cast<double>(st[2]);
    const double f1 = static_cast<double>(st[3]);
    const double specials = st[1] > 0 ? 2.0 : 0.0;  // the NULL and EMPTY groups at most
    if (n <= 0) {
        return static_cast<uint64_t>(specials) + 1;
    }
    double est = n >= static_cast<double>(total) ? d : std::sqrt(static_cast<double>(total) / n) * f1 + (d - f1);
    est = std::min(std::max(est, d), static_cast<double>(total));
    return static_cast<uint64_t>(est + specials);
}

void SizerFeatures(const int64_t *log, float *x)
{
    const double N = static_cast<double>(std::max<int64_t>(log[kLogRows], 1));
    const double n = static_cast<double>(std::max<int64_t>(log[kLogSampled] - log[kLogSpecial], 1));
    const double d = static_cast<double>(std::max<int64_t>(log[kLogDistinct], 1));
    const double f1 = static_cast<double>(log[kLogF1]);
    const double gee = std::min(std::max(std::sqrt(N / n) * f1 + (d - f1), d), N);
    x[0] = static_cast<float>(L2(N) / 32.0);
    x[1] = static_cast<float>(L2(n) / 32.0);
    x[2] = static_cast<float>(L2(d) / 32.0);
    x[3] = static_cast<float>(f1 / n);
    x[4] = static_cast<float>(static_cast<double>(log[kLogF2]) / n);
    x[5] = static_cast<float>(static_cast<double>(log[kLogF3]) / n);
    x[6] = static_cast<float>(static_cast<double>(log[kLogF4to7]) / n);
    x[7] = static_cast<float>(static_cast<double>(log[kLogF8]) / n);
    x[8] = static_cast<float>(static_cast<double>(log[kLogHeavy]) / n);
    x[9] = static_cast<float>(L2(static_cast<double>(log[kLogMax])) / 16.0);
    x[10] = static_cast<float>(std::log2(N / n) / 16.0);
    x[11] = static_cast<float>(std::log2(gee / d) / 16.0);
}

uint64_t SizerEstimate(const int64_t *log, float y)
{
    const double N = static_cast<double>(std::max<int64_t>(log[kLogRows], 1));
    const double d = static_cast<double>(std::max<int64_t>(log[kLogDistinct], 1));
    const double specials = log[kLogSpecial] > 0 ? 2.0 : 0.0;
    double est = d * std::exp2(16.0 * std::max(0.0, static_cast<double>(y)));
    est = std::min(std::max(est, d), N);
    return static_cast<uint64_t>(est + specials);
}

float SizerTarget(const int64_t *log, int64_t groups)
{
    const double d = static_cast<double>(std::max<int64_t>(log[kLogDistinct], 1));
    const double g = std::max(static_cast<double>(groups), d);
    return static_cast<float>(std::log2(g / d) / 16.0);
}

SizingModel::SizingModel(const std::vector<int32_t> &dims, uint64_t seed) : dims_(dims)
{
    if (dims_.size() < 2 || dims_.back() != 1) {
        throw OmniException("INVALID_ARGUMENT", "sizing model dims must end with 1 output", -1);
    }
    for (size_t l = 0; l + 1 < dims_.size(); ++l) {
        if (dims_[l] <= 0 || dims_[l] > 4096) {
            throw OmniException("INVALID_ARGUMENT", "sizing model layer width out of range", -1);
        }
        wOff_.push_back(nParams_);
        nParams_ += static_cast<int64_t>(dims_[l]) * dims_[l + 1];
        bOff_.push_back(nParams_);
        nParams_ += dims_[l + 1];
    }
    RequireDevice();
    CudaCheck(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    params_.Reset(nParams_, stream_);
    grads_.Reset(nParams_, stream_);
    adamM_.Reset(nParams_, stream_, true);
    adamV_.Reset(nParams_, stream_, true);
    loss_.Reset(1, stream_, true);
    std::vector<float> init(nParams_, 0.f);
    SplitMix rng{seed};
    for (size_t l = 0; l + 1 < dims_.size(); ++l) {
        const double bound = std::sqrt(6.0 / dims_[l]);  // He-uniform for ReLU layers
        for (int64_t i = 0; i < static_cast<int64_t>(dims_[l]) * dims_[l + 1]; ++i) {
            init[wOff_[l] + i] = static_cast<float>((2.0 * rng.Uniform() - 1.0) * bound);
        }
    }
    SetParams(init.data());
}

SizingModel::~SizingModel()
{
    if (stream_ != nullptr) {
        cudaStreamSynchronize(stream_);
        params_.Release();
        grads_.Release();
        adamM_.Release();
        adamV_.Release();
        x_.Release();
        t_.Release();
        loss_.Release();
        partial_.Release();
        act_.clear();
        dact_.clear();
        cudaStreamSynchronize(stream_);
        cudaStreamDestroy(stream_);
    }
}

void SizingModel::GetParams(float *out)
{
    std::lock_guard<std::mutex> g(mu_);
    CudaCheck(cudaMemcpyAsync(out, params_.Get(), sizeof(float) * nParams_, cudaMemcpyDeviceToHost, stream_),
        "read model parameters");
    CudaCheck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
}

void SizingModel::SetParams(const float *in)
{
    std::lock_guard<std::mutex> g(mu_);
    CudaCheck(cudaMemcpyAsync(params_.Get(), in, sizeof(float) * nParams_, cudaMemcpyHostToDevice, stream_),
        "write model parameters");
    CudaCheck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    step_ = 0;
    CudaCheck(cudaMemsetAsync(adamM_.Get(), 0, sizeof(float) * nParams_, stream_), "reset optimiser");
    CudaCheck(cudaMemsetAsync(adamV_.Get(), 0, sizeof(float) * nParams_, stream_), "reset optimiser");
}

void SizingModel::Upload(const float *X, const float *T, int32_t n)
{
    if (n > capacity_) {
        capacity_ = std::max(n, 256);
        x_.Reset(static_cast<size_t>(capacity_) * dims_[0], stream_);
        t_.Reset(capacity_, stream_);
        act_.clear();
        dact_.clear();
        for (size_t l = 1; l < dims_.size(); ++l) {
            act_.emplace_back(static_cast<size_t>(capacity_) * dims_[l], stream_);
            dact_.emplace_back(static_cast<size_t>(capacity_) * dims_[l], stream_);
        }
    }
    CudaCheck(cudaMemcpyAsync(x_.Get(), X, sizeof(float) * n * dims_[0], cudaMemcpyHostToDevice, stream_),
        "upload features");
    if (T != nullptr) {
        CudaCheck(cudaMemcpyAsync(t_.Get(), T, sizeof(float) * n, cudaMemcpyHostToDevice, stream_), "upload targets");
    }
}

void SizingModel::Forward(int32_t n)
{
    const float *in = x_.Get();
    const size_t layers = dims_.size() - 1;
    for (size_t l = 0; l < layers; ++l) {
        const float *W = params_.Get() + wOff_[l];
        const float *b = params_.Get() + bOff_[l];
        CudaCheck(LaunchDenseForward(in, W, b, act_[l].Get(), n, dims_[l], dims_[l + 1], l + 1 < layers, stream_),
            "dense forward");
        in = act_[l].Get();
    }
}

float SizingModel::Backward(int32_t n)
{
    const size_t layers = dims_.size() - 1;
    CudaCheck(cudaMemsetAsync(loss_.Get(), 0, sizeof(float), stream_), "reset loss");
    CudaCheck(LaunchMseGrad(act_[layers - 1].Get(), t_.Get(), dact_[layers - 1].Get(), n, loss_.Get(), stream_),
        "loss gradient");
    const float invScale = 1.0f / static_cast<float>(n);
    for (size_t l = layers; l-- > 0;) {
        if (l + 1 < layers) {
            CudaCheck(LaunchReluBackward(act_[l].Get(), dact_[l].Get(), static_cast<int64_t>(n) * dims_[l + 1], stream_),
                "relu backward");
        }
        const float *in = l == 0 ? x_.Get() : act_[l - 1].Get();
        CudaCheck(LaunchDenseWeightGrad(in, dact_[l].Get(), grads_.Get() + wOff_[l], grads_.Get() + bOff_[l], n,
                      dims_[l], dims_[l + 1], invScale, stream_),
            "weight gradient");
        if (l > 0) {
            CudaCheck(LaunchDenseInputGrad(dact_[l].Get(), params_.Get() + wOff_[l], dact_[l - 1].Get(), n, dims_[l],
                          dims_[l + 1], stream_),
                "input gradient");
        }
    }
    float loss = 0.f;
    CudaCheck(cudaMemcpyAsync(&loss, loss_.Get(), sizeof(float), cudaMemcpyDeviceToHost, stream_), "read loss");
    CudaCheck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return loss / static_cast<float>(n);
}

void SizingModel::Predict(const float *X, int32_t n, float *Y)
{
    std::lock_guard<std::mutex> g(mu_);
    if (n <= 0) {
        return;
    }
    Upload(X, nullptr, n);
    Forward(n);
    CudaCheck(cudaMemcpyAsync(Y, act_.back().Get(), sizeof(float) * n, cudaMemcpyDeviceToHost, stream_),
        "read predictions");
    CudaCheck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
}

float SizingModel::Gradients(const float *X, const float *T, int32_t n, float *grad)
{
    std::lock_guard<std::mutex> g(mu_);
    if (n <= 0) {
        throw OmniException("INVALID_ARGUMENT", "empty batch", -1);
    }
    Upload(X, T, n);
    float loss;
    if (Fused()) {
        loss = RunFused(n, 1, 0.f, grads_.Get());
    } else {
        Forward(n);
        loss = Backward(n);
    }
    CudaCheck(cudaMemcpyAsync(grad, grads_.Get(), sizeof(float) * nParams_, cudaMemcpyDeviceToHost, stream_),
        "read gradients");
    CudaCheck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return loss;
}

namespace {
std::atomic<bool> g_fusedTraining{true};
}

void SetFusedTraining(bool on) { g_fusedTraining.store(on); }

bool SizingModel::Fused() const
{
    return g_fusedTraining.load() && dims_.size() == 4 && MlpFusedSupported(dims_[0], dims_[1], dims_[2]);
}

// The fused kernel over the uploaded batch: `epochs` Adam steps, or (gradOut non-null) the
// gradient of one pass into gradOut with nothing updated.  Returns the mean squared error of the
// last pass.
float SizingModel::RunFused(int32_t n, int32_t epochs, float lr, float *gradOut)
{
    const int grid = MlpFusedGrid(n);
    partial_.Reset(static_cast<size_t>(grid) * static_cast<size_t>(nParams_), stream_);
    CudaCheck(cudaMemsetAsync(loss_.Get(), 0, sizeof(float), stream_), "reset loss");
    MlpFusedArgs a{};
    a.X = x_.Get();
    a.T = t_.Get();
    a.n = n;
    a.F = dims_[0];
    a.H1 = dims_[1];
    a.H2 = dims_[2];
    a.nParams = static_cast<int32_t>(nParams_);
    a.epochs = epochs;
    a.params = params_.Get();
    a.adamM = adamM_.Get();
    a.adamV = adamV_.Get();
    a.partial = partial_.Get();
    a.loss = loss_.Get();
    a.gradOut = gradOut;
    a.lr = lr;
    a.b1 = 0.9f;
    a.b2 = 0.999f;
    a.eps = 1e-8f;
    a.b1Pow = std::pow(static_cast<double>(a.b1), step_);
    a.b2Pow = std::pow(static_cast<double>(a.b2), step_);
    CudaCheck(LaunchMlpTrainFused(a, grid, stream_), "fused training");
    float loss = 0.f;
    CudaCheck(cudaMemcpyAsync(&loss, loss_.Get(), sizeof(float), cudaMemcpyDeviceToHost, stream_), "read loss");
    CudaCheck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return loss / static_cast<float>(n);
}

float SizingModel::Train(const float *X, const float *T, int32_t n, int32_t epochs, float lr)
{
    std::lock_guard<std::mutex> g(mu_);
    if (n <= 0 || epochs <= 0) {
        throw OmniException("INVALID_ARGUMENT", "empty batch or no epochs", -1);
    }
    Upload(X, T, n);
    if (Fused()) {
        // All epochs in one cooperative launch.
        const float loss = RunFused(n, epochs, lr, nullptr);
        step_ += epochs;
        return loss;
    }
    float loss = 0.f;
    for (int32_t e = 0; e < epochs; ++e) {
        Forward(n);
        // The loss is read back only on the last epoch; other epochs stay on the device.
        const size_t layers = dims_.size() - 1;
        if (e + 1 == epochs) {
            loss = Backward(n);
        } else {
            CudaCheck(LaunchMseGrad(act_[layers - 1].Get(), t_.Get(), dact_[layers - 1].Get(), n, nullptr, stream_),
                "loss gradient");
            const float invScale = 1.0f / static_cast<float>(n);
            for (size_t l = layers; l-- > 0;) {
                if (l + 1 < layers) {
                    CudaCheck(LaunchReluBackward(act_[l].Get(), dact_[l].Get(), static_cast<int64_t>(n) * dims_[l + 1],
                                  stream_),
                        "relu backward");
                }
                const float *in = l == 0 ? x_.Get() : act_[l - 1].Get();
                CudaCheck(LaunchDenseWeightGrad(in, dact_[l].Get(), grads_.Get() + wOff_[l], grads_.Get() + bOff_[l],
                              n, dims_[l], dims_[l + 1], invScale, stream_),
                    "weight gradient");
                if (l > 0) {
                    CudaCheck(LaunchDenseInputGrad(dact_[l].Get(), params_.Get() + wOff_[l], dact_[l - 1].Get(), n,
                                  dims_[l], dims_[l + 1], stream_),
                        "input gradient");
                }
            }
        }
        ++step_;
        CudaCheck(LaunchAdam(params_.Get(), grads_.Get(), adamM_.Get(), adamV_.Get(), nParams_, lr, 0.9f, 0.999f,
                      1e-8f, step_, stream_),
            "adam step");
    }
    CudaCheck(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return loss;
}

void QuantileSplits(const int64_t *sample, int64_t n, int32_t bits, int64_t *splits)
{
    if (n <= 0 || bits < 1 || bits > 12) {
        throw OmniException("INVALID_ARGUMENT", "quantile splits need a sample and 1 <= bits <= 12", -1);
    }
    std::vector<int64_t> keys(sample, sample + n);
    std::sort(keys.begin(), keys.end());
    const int64_t P = int64_t(1) << bits;
    for (int64_t k = 1; k < P; ++k) {
        splits[k - 1] = keys[std::min<int64_t>(n - 1, (k * n) / P)];
    }
}

void LearnRangeSplits(const int64_t *sample, int64_t n, int32_t bits, int32_t epochs, uint64_t seed, int64_t *splits)
{
    if (n <= 0 || bits < 1 || bits > 12) {
        throw OmniException("INVALID_ARGUMENT", "learned splits need a sample and 1 <= bits <= 12", -1);
    }
    std::vector<int64_t> keys(sample, sample + n);
    std::sort(keys.begin(), keys.end());
    const double lo = static_cast<double>(keys.front());
    const double span = std::max(static_cast<double>(keys.back()) - lo, 1.0);
    // Training points: up to 16,384 evenly spaced sample ranks, target = empirical CDF.
    const int64_t m = std::min<int64_t>(n, 16384);
    std::vector<float> X(m), T(m);
    for (int64_t j = 0; j < m; ++j) {
        const int64_t i = (j * n) / m;
        X[j] = static_cast<float>((static_cast<double>(keys[i]) - lo) / span);
        T[j] = static_cast<float>((static_cast<double>(i) + 0.5) / static_cast<double>(n));
    }
    SizingModel model({1, 32, 32, 1}, seed);
    model.Train(X.data(), T.data(), static_cast<int32_t>(m), std::max(epochs, 1), 3e-3f);
    // Two stages (a recursive model index): the network's CDF routes each key to one of K leaf
    // models, each a least-squares line of the empirical CDF over the keys routed to it.  The
    // network alone cannot resolve the CDF finely enough for thousands of equal ranges.
    std::vector<float> xs(n), y1(n);
    for (int64_t i = 0; i < n; ++i) {
        xs[i] = static_cast<float>((static_cast<double>(keys[i]) - lo) / span);
    }
    model.Predict(xs.data(), static_cast<int32_t>(n), y1.data());
    const int64_t K = std::min<int64_t>(4096, std::max<int64_t>(16, n / 32));
    std::vector<int64_t> leaf(n);
    std::vector<double> sx(K, 0), sy(K, 0), sxx(K, 0), sxy(K, 0), cnt(K, 0);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t l = std::min<int64_t>(K - 1, std::max<int64_t>(0, static_cast<int64_t>(y1[i] * K)));
        leaf[i] = l;
        const double x = xs[i];
        const double y = (static_cast<double>(i) + 0.5) / static_cast<double>(n);
        sx[l] += x;
        sy[l] += y;
        sxx[l] += x * x;
        sxy[l] += x * y;
        cnt[l] += 1;
    }
    std::vector<double> a(K, 0), b(K, 0);
    for (int64_t l = 0; l < K; ++l) {
        if (cnt[l] == 0) {
            continue;
        }
        const double mx = sx[l] / cnt[l];
        const double my = sy[l] / cnt[l];
        const double vx = sxx[l] / cnt[l] - mx * mx;
        b[l] = (cnt[l] >= 2 && vx > 1e-18) ? (sxy[l] / cnt[l] - mx * my) / vx : 0.0;
        a[l] = my - b[l] * mx;
    }
    // Predicted CDF of every sample key (made monotone), then the crossing points.
    std::vector<double> ys(n);
    double run = -1e300;
    for (int64_t i = 0; i < n; ++i) {
        run = std::max(run, a[leaf[i]] + b[leaf[i]] * xs[i]);
        ys[i] = run;
    }
    const int32_t P = 1 << bits;
    int64_t i = 0;
    for (int32_t k = 1; k < P; ++k) {
        const double q = static_cast<double>(k) / static_cast<double>(P);
        while (i < n && ys[i] < q) {
            ++i;
        }
        splits[k - 1] = i < n ? keys[i] : keys.back();
    }
}

}  // namespace omg
