// Batched aggregation of many independent tasks (see omniop/batched_agg.h).
#include "omniop/batched_agg.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "host/gpu_runtime.h"
#include "host/sizer.h"
#include "kernels/launch.h"

namespace omniruntime {
namespace op {

using exception::OmniException;
using omg::CudaCheck;
using omg::DevArray;
using omg::PinnedArray;
using vec::VectorBatch;

namespace {
constexpr uint64_t kMinTaskSlots = 64;
constexpr int32_t kDefaultVariant = 1;  // 256 threads, 4 CTAs per SM
// Probe limit of the task tables (sized for a load of 1/2 or less): a task whose rows need more
// probes has outgrown its table and is re-run exactly.
constexpr int32_t kTaskMaxProbe = 96;

uint64_t NextPow2(uint64_t v)
{
    uint64_t p = 1;
    while (p < v) {
        p <<= 1;
    }
    return p;
}

int64_t NowUs()
{
    return std::chrono::duration_cast<std::chrono::microseconds>(
        std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

int Log2Bucket(uint64_t v)
{
    int b = 0;
    while ((uint64_t(1) << b) < v && b < 62) {
        ++b;
    }
    return b;
}

// Tuned launch shape per (slot words, key kind, accumulators, log2 rows, log2 tasks).
using TuneKey = std::tuple<int, int, int, int, int>;
std::mutex g_tuneMu;
std::map<TuneKey, int32_t> *g_tuned = new std::map<TuneKey, int32_t>();  // process lifetime

// A view of batch b that shares its buffers (for the exact re-run through an operator, which
// takes ownership of what it is given).
VectorBatch *ViewOf(VectorBatch *b)
{
    auto *v = new VectorBatch(b->GetRowCount());
    for (int32_t i = 0; i < b->GetVectorCount(); ++i) {
        vec::BaseVector *x = b->Get(i);
        v->Append(new vec::BaseVector(x->GetTypeId(), x->GetWidth(), x->GetSize(), x->ValuesBuffer(),
            x->ValuesOffset(), x->NullsBufferPtr(), x->NullsOffset(), x->NullFlag() || x->HasNull()));
    }
    return v;
}
}  // namespace

struct BatchedAggregation::Impl {
    HashAggregationOperatorFactory *factory = nullptr;
    AggPlan plan;
    std::vector<VectorBatch *> tasks;
    omg::SizingModel *sizer = nullptr;
    int32_t flags = 0;
    omg::OpStream stream;
    omg::KernelTimer timer;
    bool prepared = false;

    omg::BatchTable bt;
    int32_t n = 0;
    int64_t rows = 0;
    std::vector<unsigned long long> sketch;  // n * kSketchStats
    std::vector<uint64_t> estimate, plainEstimate;
    std::vector<uint64_t> capacity;
    uint64_t totalSlots = 0;
    uint64_t outBound = 0;  // output rows allocated (sum of per-task bounds, 64-row padded)

    DevArray<uint64_t> slab;
    DevArray<uint32_t> specials;
    DevArray<omg::AggTable> tables;
    DevArray<uint32_t> failed;
    DevArray<uint32_t> counts;  // padded to 64 rows per task (output regions)
    DevArray<uint32_t> groups;  // exact groups per task
    DevArray<int64_t> offsets;
    DevArray<int64_t> blockSums;
    DevArray<long long> total;
    DevArray<unsigned long long> scratch;  // extraction's error / ambiguity words
    std::vector<omg::OutColumn> outCols;
    PinnedArray<uint32_t> hGroups, hFailed;
    PinnedArray<int64_t> hOffsets;

    int32_t variant = kDefaultVariant;
    int64_t tuneUs = 0, prepareUs = 0, lastRunNs = 0, runs = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;

    // Results of the last run.
    std::vector<int64_t> taskGroups;
    std::vector<bool> taskRerun;  // the task outgrew its first table
    std::vector<bool> taskGrown;  // ... and was finished by the grow pass
    std::vector<std::vector<VectorBatch *>> rerunOutputs;
    // The grow pass: one more batched run over the tasks that outgrew their tables, each with a
    // table of at least twice its rows (forcedCapacity), so none can outgrow it; a task that
    // still fails (its probe limit) is re-run through a regular operator.
    std::vector<uint64_t> forcedCapacity;
    std::unique_ptr<Impl> grow;
    std::vector<int32_t> growTasks;

    ~Impl()
    {
        if (exec != nullptr) {
            cudaGraphExecDestroy(exec);
        }
        if (graph != nullptr) {
            cudaGraphDestroy(graph);
        }
        for (auto &v : rerunOutputs) {
            for (auto *b : v) {
                vec::VectorHelper::FreeVecBatch(b);
            }
        }
    }

    omg::AggLaunch Launch()
    {
        omg::AggLaunch p = MakeAggLaunch(plan, slab.Get(), totalSlots - 2, specials.Get(), nullptr);
        p.maxProbe = kTaskMaxProbe;
        p.error = reinterpret_cast<int32_t *>(scratch.Get());
        p.batches = bt.DeviceBatches();
        p.tiles = bt.DeviceTiles();
        p.nTiles = bt.NumTiles();
        p.taskTables = tables.Get();
        p.taskFailed = failed.Get();
        return p;
    }

    // The per-run sequence: reset, aggregate, count, place and extract every task's groups.
    void Sequence(cudaStream_t s)
    {
        omg::AggLaunch p = Launch();
        CudaCheck(cudaMemsetAsync(specials.Get(), 0, sizeof(uint32_t) * 2 * n, s), "reset special slots");
        CudaCheck(cudaMemsetAsync(failed.Get(), 0, sizeof(uint32_t) * n, s), "reset task flags");
        CudaCheck(omg::LaunchAggInitTable(p, s), "init task tables");
        CudaCheck(omg::LaunchAggTasks(p, variant, s), "batched aggregation");
        CudaCheck(omg::LaunchAggTaskCount(tables.Get(), n, plan.key.kind, groups.Get(), s), "count task groups");
        CudaCheck(omg::LaunchAggTaskPad(groups.Get(), n, counts.Get(), s), "pad task regions");
        CudaCheck(omg::LaunchScanCounts(counts.Get(), n, offsets.Get(), blockSums.Get(), total.Get(), s),
            "place task outputs");
        for (auto &c : outCols) {
            if (c.nulls) {
                CudaCheck(cudaMemsetAsync(c.nulls->Data(), 0, omg::NullBitmapBytes(static_cast<int64_t>(outBound)), s),
                    "reset output nulls");
            }
        }
        omg::AggExtract e;
        std::memset(&e, 0, sizeof(e));
        e.key = plan.key;
        e.nAccs = static_cast<int32_t>(plan.accs.size());
        for (int i = 0; i < e.nAccs; ++i) {
            e.accs[i] = plan.accs[i];
        }
        e.nOut = static_cast<int32_t>(plan.outs.size());
        for (int32_t o = 0; o < e.nOut; ++o) {
            e.out[o] = plan.outs[o];
            e.out[o].values = outCols[o].values->Data();
            e.out[o].nulls = static_cast<uint8_t *>(outCols[o].nulls->Data());
        }
        e.overflowAsNull = plan.overflowAsNull ? 1 : 0;
        e.outCount = scratch.Get() + 1;
        e.error = reinterpret_cast<int32_t *>(scratch.Get() + 2);
        e.nAmbiguous = scratch.Get() + 3;
        e.ambiguousSlots = scratch.Get() + 4;
        e.ambiguousCap = 0;
        CudaCheck(omg::LaunchAggTaskExtract(e, tables.Get(), n, offsets.Get(), s), "extract task groups");
    }

    void Prepare(cudaStream_t s)
    {
        const int64_t t0 = NowUs();
        n = static_cast<int32_t>(tasks.size());
        bt.Build(tasks, plan.inputCols, omg::kTileRows, &plan.inputMasks);
        bt.Upload(s);
        rows = bt.TotalRows();
        scratch.Reset(8, s, true);
        // Sizing: one sketch per task, then the plain estimate or the model's, batched (the grow
        // pass has its capacities already).
        sketch.assign(static_cast<size_t>(n) * omg::kSketchStats, 0);
        if (forcedCapacity.empty()) {
            DevArray<unsigned long long> st(static_cast<size_t>(n) * omg::kSketchStats, s);
            omg::AggLaunch p = MakeAggLaunch(plan, nullptr, 0, nullptr, nullptr);
            p.batches = bt.DeviceBatches();
            CudaCheck(omg::LaunchAggTaskSketch(p, n, st.Get(), s), "task sketches");
            CudaCheck(cudaMemcpyAsync(sketch.data(), st.Get(), sizeof(unsigned long long) * sketch.size(),
                          cudaMemcpyDeviceToHost, s),
                "read task sketches");
            CudaCheck(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        }
        estimate.resize(n);
        plainEstimate.resize(n);
        std::vector<float> X;
        std::vector<int64_t> logs;
        for (int32_t t = 0; t < n; ++t) {
            const int64_t r = tasks[t]->GetRowCount();
            plainEstimate[t] = forcedCapacity.empty()
                ? omg::PlainGroupEstimate(&sketch[static_cast<size_t>(t) * omg::kSketchStats], r)
                : forcedCapacity[t] / 2;
            estimate[t] = plainEstimate[t];
        }
        if (sizer != nullptr && forcedCapacity.empty()) {
            X.resize(static_cast<size_t>(n) * omg::kSizerFeatures);
            std::vector<int64_t> log(1 + omg::kSketchStats);
            std::vector<std::vector<int64_t>> allLogs(n);
            for (int32_t t = 0; t < n; ++t) {
                log[0] = tasks[t]->GetRowCount();
                for (int i = 0; i < omg::kSketchStats; ++i) {
                    log[1 + i] = static_cast<int64_t>(sketch[static_cast<size_t>(t) * omg::kSketchStats + i]);
                }
                omg::SizerFeatures(log.data(), &X[static_cast<size_t>(t) * omg::kSizerFeatures]);
                allLogs[t] = log;
            }
            std::vector<float> y(n);
            sizer->Predict(X.data(), n, y.data());
            for (int32_t t = 0; t < n; ++t) {
                estimate[t] = omg::SizerEstimate(allLogs[t].data(), y[t]);
            }
        }
        // Tables: nextpow2(2 x estimate) slots each (at least 64), one slab.
        capacity.resize(n);
        std::vector<omg::AggTable> hostTables(n);
        totalSlots = 0;
        outBound = 0;
        for (int32_t t = 0; t < n; ++t) {
            uint64_t want = (flags & (kBatchTinyTables | kBatchTinyGrow)) ? kMinTaskSlots
                                                                          : NextPow2(2 * std::max<uint64_t>(estimate[t], 1));
            if (!forcedCapacity.empty()) {
                want = forcedCapacity[t];
            }
            capacity[t] = std::max(want, kMinTaskSlots);
            const uint64_t bound = std::min<uint64_t>(capacity[t] + 2, static_cast<uint64_t>(tasks[t]->GetRowCount()));
            outBound += (bound + 63) / 64 * 64;
            totalSlots += capacity[t] + 2;
        }
        slab.Reset(totalSlots * plan.slotWords, s);
        specials.Reset(2 * static_cast<size_t>(n), s, true);
        uint64_t off = 0;
        for (int32_t t = 0; t < n; ++t) {
            omg::AggTable &tab = hostTables[t];
            std::memset(&tab, 0, sizeof(tab));
            tab.slots = slab.Get() + off * plan.slotWords;
            tab.capacity = capacity[t];
            tab.slotWords = plan.slotWords;
            tab.keyWords = plan.keyWords;
            tab.specialUsed = specials.Get() + 2 * t;
            off += capacity[t] + 2;
        }
        tables.Reset(n, s);
        CudaCheck(cudaMemcpyAsync(tables.Get(), hostTables.data(), sizeof(omg::AggTable) * n, cudaMemcpyHostToDevice, s),
            "upload task tables");
        failed.Reset(n, s, true);
        counts.Reset(n, s);
        groups.Reset(n, s);
        offsets.Reset(n, s);
        blockSums.Reset(static_cast<size_t>(n) / 1024 + 2, s);
        total.Reset(1, s, true);
        hGroups.Reset(n);
        hFailed.Reset(n);
        hOffsets.Reset(n);
        outCols.assign(plan.outs.size(), omg::OutColumn{});
        for (size_t o = 0; o < plan.outs.size(); ++o) {
            outCols[o].type = plan.outTypes[o]->GetId();
            outCols[o].width = plan.outs[o].outWidth;
            outCols[o].values = omg::Buffer::NewDevice(outBound * plan.outs[o].outWidth + 16, s, false);
            outCols[o].nulls = omg::Buffer::NewDevice(omg::NullBitmapBytes(static_cast<int64_t>(outBound)), s, true);
            outCols[o].hasNull = plan.outs[o].kind != omg::OUT_COUNT && plan.outs[o].kind != omg::OUT_IS_EMPTY;
        }
        CudaCheck(cudaStreamSynchronize(s), "cudaStreamSynchronize");  // hostTables is on the stack
        prepareUs = NowUs() - t0;
        Tune(s);
        // Capture the per-run sequence once (a private stream is needed for capture).
        if (!(flags & kBatchNoGraph) && s != nullptr) {
            CudaCheck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin graph capture");
            try {
                Sequence(s);
            } catch (...) {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(s, &g);
                if (g != nullptr) {
                    cudaGraphDestroy(g);
                }
                throw;
            }
            CudaCheck(cudaStreamEndCapture(s, &graph), "end graph capture");
            CudaCheck(cudaGraphInstantiate(&exec, graph, 0), "instantiate graph");
        }
        prepared = true;
    }

    // Time every launch shape of the persistent kernel once (each on freshly initialised tables)
    // and keep the fastest; cached per plan shape and workload size.
    void Tune(cudaStream_t s)
    {
        const TuneKey key{plan.slotWords, plan.key.kind, static_cast<int>(plan.accs.size()),
            Log2Bucket(static_cast<uint64_t>(std::max<int64_t>(rows, 1))), Log2Bucket(static_cast<uint64_t>(n))};
        {
            std::lock_guard<std::mutex> g(g_tuneMu);
            auto it = g_tuned->find(key);
            if (it != g_tuned->end()) {
                variant = it->second;
                return;
            }
        }
        if (flags & kBatchNoTune) {
            variant = kDefaultVariant;
            return;
        }
        const int64_t t0 = NowUs();
        omg::AggLaunch p = Launch();
        float best = 1e30f;
        int32_t bestV = kDefaultVariant;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        CudaCheck(cudaEventCreate(&e0), "cudaEventCreate");
        CudaCheck(cudaEventCreate(&e1), "cudaEventCreate");
        for (int32_t v = 0; v < omg::AggTasksVariants(); ++v) {
            CudaCheck(cudaMemsetAsync(specials.Get(), 0, sizeof(uint32_t) * 2 * n, s), "reset special slots");
            CudaCheck(omg::LaunchAggInitTable(p, s), "init task tables");
            CudaCheck(cudaEventRecord(e0, s), "cudaEventRecord");
            CudaCheck(omg::LaunchAggTasks(p, v, s), "batched aggregation (tuning)");
            CudaCheck(cudaEventRecord(e1, s), "cudaEventRecord");
            CudaCheck(cudaEventSynchronize(e1), "cudaEventSynchronize");
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                bestV = v;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        variant = bestV;
        tuneUs = NowUs() - t0;
        std::lock_guard<std::mutex> g(g_tuneMu);
        (*g_tuned)[key] = bestV;
    }
};

BatchedAggregation::BatchedAggregation(HashAggregationOperatorFactory &factory, std::vector<VectorBatch *> tasks,
    omg::SizingModel *sizer, int32_t flags)
    : impl_(new Impl())
{
    factory.Init();
    impl_->factory = &factory;
    impl_->plan = factory.Plan();
    impl_->sizer = sizer;
    impl_->flags = flags;
    if (impl_->plan.orderDependent) {
        throw OmniException("UNSUPPORTED_ERROR",
            "batched aggregation does not run plans with sticky-overflow sums; use one operator per task", -2);
    }
    for (int32_t c : impl_->plan.outContainer) {
        if (c > 0) {
            throw OmniException("UNSUPPORTED_ERROR",
                "batched aggregation does not emit container vectors; use one operator per task", -2);
        }
    }
    if (!impl_->plan.dictInputs.empty() || !impl_->plan.varlenInputs.empty()) {
        throw OmniException("UNSUPPORTED_ERROR",
            "batched aggregation does not run plans with VARCHAR/CHAR columns; use one operator per task", -2);
    }
    if (sizer != nullptr && sizer->Dims()[0] != omg::kSizerFeatures) {
        throw OmniException("INVALID_ARGUMENT", "sizing model input width must be 12", -1);
    }
    for (auto *b : tasks) {
        if (b == nullptr || b->GetRowCount() <= 0) {
            throw OmniException("INVALID_ARGUMENT", "every task needs a non-empty batch", -1);
        }
    }
    impl_->tasks = std::move(tasks);
}

BatchedAggregation::~BatchedAggregation()
{
    impl_->stream.Sync();
}

void BatchedAggregation::Run(void *stream)
{
    omg::RequireDevice();
    Impl &im = *impl_;
    if (stream != nullptr) {
        im.stream.SetUser(stream);
    }
    cudaStream_t s = im.stream.Get();
    if (!im.prepared) {
        im.Prepare(s);
    }
    for (auto &v : im.rerunOutputs) {
        for (auto *b : v) {
            vec::VectorHelper::FreeVecBatch(b);
        }
    }
    im.timer.Start(s);
    if (im.exec != nullptr) {
        CudaCheck(cudaGraphLaunch(im.exec, s), "graph launch");
    } else {
        im.Sequence(s);
    }
    im.timer.Stop(s);
    CudaCheck(cudaMemcpyAsync(im.hGroups.Get(), im.groups.Get(), sizeof(uint32_t) * im.n, cudaMemcpyDeviceToHost, s),
        "read task groups");
    CudaCheck(cudaMemcpyAsync(im.hFailed.Get(), im.failed.Get(), sizeof(uint32_t) * im.n, cudaMemcpyDeviceToHost, s),
        "read task flags");
    CudaCheck(cudaMemcpyAsync(im.hOffsets.Get(), im.offsets.Get(), sizeof(int64_t) * im.n, cudaMemcpyDeviceToHost, s),
        "read task offsets");
    unsigned long long err[3] = {0, 0, 0};
    CudaCheck(cudaMemcpyAsync(err, im.scratch.Get(), sizeof(err), cudaMemcpyDeviceToHost, s), "read errors");
    im.stream.Sync();
    im.lastRunNs = im.timer.ElapsedNs();
    ++im.runs;
    if (err[0] != 0 || err[2] != 0) {
        const int32_t code = static_cast<int32_t>(err[0] != 0 ? err[0] : err[2]);
        throw OmniException("OPERATOR_RUNTIME_ERROR", "batched aggregation kernel error " + std::to_string(code),
            code == 7 ? -7 : (code == 5 ? -5 : -9));
    }
    im.taskGroups.assign(im.n, 0);
    im.taskRerun.assign(im.n, false);
    im.taskGrown.assign(im.n, false);
    im.rerunOutputs.assign(im.n, {});
    const bool device = (im.flags & kBatchDeviceOutput) != 0;
    std::vector<int32_t> failedTasks;
    for (int32_t t = 0; t < im.n; ++t) {
        im.taskGroups[t] = im.hGroups[t];
        if (im.hFailed[t] != 0) {
            im.taskRerun[t] = true;
            failedTasks.push_back(t);
        }
    }
    if (!failedTasks.empty() && !(im.flags & kBatchTinyTables)) {
        // The grow pass (prepared once per set of failed tasks; graph replays fail the same tasks).
        if (!im.grow || im.growTasks != failedTasks) {
            std::unique_ptr<Impl> g(new Impl());
            g->factory = im.factory;
            g->plan = im.plan;
            g->flags = (im.flags & kBatchDeviceOutput) | kBatchNoGraph | kBatchNoTune;
            for (int32_t t : failedTasks) {
                g->tasks.push_back(im.tasks[t]);
                g->forcedCapacity.push_back(
                    std::max(kMinTaskSlots, NextPow2(2 * static_cast<uint64_t>(im.tasks[t]->GetRowCount()))));
            }
            g->Prepare(s);
            g->variant = im.variant;
            im.grow = std::move(g);
            im.growTasks = failedTasks;
        }
        Impl &g = *im.grow;
        g.timer.Start(s);
        g.Sequence(s);
        g.timer.Stop(s);
        CudaCheck(cudaMemcpyAsync(g.hGroups.Get(), g.groups.Get(), sizeof(uint32_t) * g.n, cudaMemcpyDeviceToHost, s),
            "read grown task groups");
        CudaCheck(cudaMemcpyAsync(g.hFailed.Get(), g.failed.Get(), sizeof(uint32_t) * g.n, cudaMemcpyDeviceToHost, s),
            "read grown task flags");
        CudaCheck(cudaMemcpyAsync(g.hOffsets.Get(), g.offsets.Get(), sizeof(int64_t) * g.n, cudaMemcpyDeviceToHost, s),
            "read grown task offsets");
        unsigned long long gerr[3] = {0, 0, 0};
        CudaCheck(cudaMemcpyAsync(gerr, g.scratch.Get(), sizeof(gerr), cudaMemcpyDeviceToHost, s), "read errors");
        im.stream.Sync();
        im.lastRunNs += g.timer.ElapsedNs();
        if (gerr[0] != 0 || gerr[2] != 0) {
            const int32_t code = static_cast<int32_t>(gerr[0] != 0 ? gerr[0] : gerr[2]);
            throw OmniException("OPERATOR_RUNTIME_ERROR", "batched aggregation kernel error " + std::to_string(code),
                code == 7 ? -7 : (code == 5 ? -5 : -9));
        }
        for (int32_t i = 0; i < g.n; ++i) {
            if (g.hFailed[i] == 0) {
                im.taskGrown[failedTasks[i]] = true;
                im.taskGroups[failedTasks[i]] = g.hGroups[i];
            }
        }
    }
    for (int32_t t = 0; t < im.n; ++t) {
        if (im.hFailed[t] == 0 || im.taskGrown[t]) {
            continue;
        }
        // The task outgrew its tables: aggregate it through a regular operator (exact resize path).
        std::unique_ptr<Operator> op(im.factory->CreateOperator());
        op->SetStream(s);
        op->SetDeviceOutput(device);
        op->AddInput(ViewOf(im.tasks[t]));
        int64_t g = 0;
        while (true) {
            VectorBatch *b = nullptr;
            op->GetOutput(&b);
            if (b == nullptr) {
                break;
            }
            g += b->GetRowCount();
            im.rerunOutputs[t].push_back(b);
        }
        op->Close();
        im.taskGroups[t] = g;
    }
}

void BatchedAggregation::Outputs(std::vector<VectorBatch *> &batches, std::vector<int32_t> &taskOf)
{
    Impl &im = *impl_;
    batches.clear();
    taskOf.clear();
    if (im.runs == 0) {
        return;
    }
    cudaStream_t s = im.stream.Get();
    std::vector<omg::OutColumn> cols = im.outCols;
    if (!(im.flags & kBatchDeviceOutput)) {
        int64_t used = 0;
        for (int32_t t = 0; t < im.n; ++t) {
            used = std::max<int64_t>(used, im.hOffsets[t] + static_cast<int64_t>(im.hGroups[t]));
        }
        cols = omg::CopyColumnsToHost(im.outCols, used, s, 0);
        im.stream.Sync();
        for (auto &c : cols) {
            c.hasNull = false;  // host vectors: HasNull() scans the bitmap
        }
    }
    // Grown tasks: their rows from the grow pass's output columns.
    std::vector<omg::OutColumn> growCols;
    std::vector<int32_t> growIndex(im.n, -1);
    if (im.grow) {
        Impl &g = *im.grow;
        growCols = g.outCols;
        if (!(im.flags & kBatchDeviceOutput)) {
            int64_t used = 0;
            for (int32_t i = 0; i < g.n; ++i) {
                used = std::max<int64_t>(used, g.hOffsets[i] + static_cast<int64_t>(g.hGroups[i]));
            }
            growCols = omg::CopyColumnsToHost(g.outCols, used, s, 0);
            im.stream.Sync();
            for (auto &c : growCols) {
                c.hasNull = false;
            }
        }
        for (int32_t i = 0; i < g.n; ++i) {
            growIndex[im.growTasks[i]] = i;
        }
    }
    for (int32_t t = 0; t < im.n; ++t) {
        if (im.taskGrown[t]) {
            const int32_t i = growIndex[t];
            for (auto *b : omg::CarveBatches(growCols, im.grow->hGroups[i], im.plan.rowsPerBatch, im.grow->hOffsets[i])) {
                batches.push_back(b);
                taskOf.push_back(t);
            }
            continue;
        }
        if (im.taskRerun[t]) {
            for (auto *b : im.rerunOutputs[t]) {
                batches.push_back(b);
                taskOf.push_back(t);
            }
            im.rerunOutputs[t].clear();
            continue;
        }
        for (auto *b : omg::CarveBatches(cols, im.hGroups[t], im.plan.rowsPerBatch, im.hOffsets[t])) {
            batches.push_back(b);
            taskOf.push_back(t);
        }
    }
}

std::vector<int64_t> BatchedAggregation::Info() const
{
    const Impl &im = *impl_;
    int32_t threads = 0, perSM = 0;
    omg::AggTasksVariantShape(im.variant, &threads, &perSM);
    int64_t reruns = 0, groups = 0, grown = 0;
    for (size_t t = 0; t < im.taskGroups.size(); ++t) {
        reruns += im.taskRerun[t] ? 1 : 0;
        grown += im.taskGrown[t] ? 1 : 0;
        groups += im.taskGroups[t];
    }
    return {im.n, im.rows, static_cast<int64_t>(im.totalSlots), reruns, threads, perSM, im.runs, groups, im.tuneUs,
        im.prepareUs, im.lastRunNs / 1000, im.sizer != nullptr ? 1 : 0, im.exec != nullptr ? 1 : 0, grown,
        reruns - grown};
}

std::vector<int64_t> BatchedAggregation::SizingLogs() const
{
    const Impl &im = *impl_;
    std::vector<int64_t> out;
    for (int32_t t = 0; t < im.n; ++t) {
        out.push_back(im.tasks[t]->GetRowCount());
        for (int i = 0; i < omg::kSketchStats; ++i) {
            out.push_back(static_cast<int64_t>(im.sketch[static_cast<size_t>(t) * omg::kSketchStats + i]));
        }
        out.push_back(static_cast<int64_t>(im.estimate[t]));
        out.push_back(-1);
        out.push_back(t < static_cast<int32_t>(im.taskGroups.size()) ? im.taskGroups[t] : 0);
        out.push_back(static_cast<int64_t>(im.plainEstimate[t]));
        out.push_back(im.sizer != nullptr ? 1 : 0);
        out.push_back(0);
    }
    return out;
}

}  // namespace op
}  // namespace omniruntime
