// Host-side launch helpers (see gpu_runtime.h).
#include "host/gpu_runtime.h"
#include "kernels/launch.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>

namespace omg {

using omniruntime::vec::BaseVector;
using omniruntime::vec::VectorBatch;

void BatchTable::Build(const std::vector<VectorBatch *> &batches, const std::vector<int32_t> &inputCols,
    int32_t tileRows, const std::vector<int32_t> *inputMasks)
{
    maskSlots_.clear();
    maskJobs_.clear();
    maskWords_ = 0;
    masksDone_ = false;
    if (inputCols.size() > static_cast<size_t>(kMaxInputs)) {
        throw OmniException("UNSUPPORTED_ERROR", "too many input columns for one kernel", -2);
    }
    descs_.Reset(batches.size());
    anyNulls_.assign(inputCols.size(), false);
    allDevice_.assign(inputCols.size(), true);
    size_t nTiles = 0;
    for (auto *b : batches) {
        nTiles += (static_cast<size_t>(b->GetRowCount()) + tileRows - 1) / tileRows;
    }
    tiles_.Reset(nTiles);
    tileOut_.Reset(nTiles);
    totalRows_ = 0;
    size_t t = 0;
    for (size_t bi = 0; bi < batches.size(); ++bi) {
        VectorBatch *b = batches[bi];
        BatchDesc &d = descs_[bi];
        std::memset(&d, 0, sizeof(d));
        d.rows = b->GetRowCount();
        d.rowBase = totalRows_;
        for (size_t i = 0; i < inputCols.size(); ++i) {
            const bool fieldRef = inputCols[i] >= kFieldRefBase;
            const int32_t c = fieldRef ? FieldRefColumn(inputCols[i]) : inputCols[i];
            if (c < 0 || c >= b->GetVectorCount()) {
                throw OmniException("OPERATOR_RUNTIME_ERROR",
                    "input batch has " + std::to_string(b->GetVectorCount()) + " vectors, column " +
                        std::to_string(c) + " requested",
                    -1);
            }
            BaseVector *v = b->Get(c);
            if (fieldRef) {
                const int32_t f = FieldRefField(inputCols[i]);
                if (v->GetEncoding() != omniruntime::vec::OMNI_ENCODING_CONTAINER || f >= v->NumFields()) {
                    throw OmniException("OPERATOR_RUNTIME_ERROR",
                        "column " + std::to_string(c) + " is not a container vector with field " + std::to_string(f), -1);
                }
                v = v->Field(f);
            }
            if (v->GetEncoding() != omniruntime::vec::OMNI_FLAT) {
                throw OmniException("OPERATOR_RUNTIME_ERROR",
                    v->GetEncoding() == omniruntime::vec::OMNI_DICTIONARY ? "dictionary vector reached a kernel unflattened"
                                                                           : "container vector used as a plain column",
                    -1);
            }
            if (v->GetSize() < b->GetRowCount()) {
                throw OmniException("OPERATOR_RUNTIME_ERROR", "vector shorter than the batch row count", -1);
            }
            d.cols[i] = v->RawValues();
            d.offs[i] = v->RawOffsets();
            if (!v->IsDevice()) {
                allDevice_[i] = false;
            }
            const bool hasNull = v->RawNulls() != nullptr && v->HasNull();
            d.nulls[i] = hasNull ? v->RawNulls() : nullptr;
            if (hasNull) {
                anyNulls_[i] = true;
            }
            const int32_t entry = inputMasks != nullptr && i < inputMasks->size() ? (*inputMasks)[i] : -1;
            if (entry == -1) {
                continue;
            }
            const int mode = entry < -1 ? 1 : (entry >= kNullsOfMaskBase ? 2 : 0);
            const int32_t m = mode == 1 ? -2 - entry : (mode == 2 ? entry - kNullsOfMaskBase : entry);
            if (m >= b->GetVectorCount()) {
                throw OmniException("OPERATOR_RUNTIME_ERROR",
                    "input batch has " + std::to_string(b->GetVectorCount()) + " vectors, mask column " +
                        std::to_string(m) + " requested",
                    -1);
            }
            BaseVector *mv = b->Get(m);
            if (mv->GetEncoding() != omniruntime::vec::OMNI_FLAT || mv->GetSize() < b->GetRowCount()) {
                throw OmniException("OPERATOR_RUNTIME_ERROR", "mask column is not a flat vector of the batch's rows", -1);
            }
            MaskJob job{};
            job.valueNulls = d.nulls[i];
            job.maskValues = static_cast<const uint8_t *>(mv->RawValues());
            job.maskNulls = mv->RawNulls() != nullptr && mv->HasNull() ? mv->RawNulls() : nullptr;
            job.out = nullptr;
            job.rows = d.rows;
            job.mode = mode;
            maskJobs_.push_back(job);
            maskSlots_.push_back(MaskSlot{bi, static_cast<int32_t>(i), maskWords_});
            maskWords_ += (d.rows + 31) / 32;
            d.nulls[i] = nullptr;  // set at Upload, once the bitmap exists
            anyNulls_[i] = true;
        }
        for (int64_t r = 0; r < d.rows; r += tileRows) {
            TileDesc &td = tiles_[t];
            td.batch = static_cast<int32_t>(bi);
            td.row0 = static_cast<int32_t>(r);
            td.rows = static_cast<int32_t>(std::min<int64_t>(tileRows, d.rows - r));
            td.pad = 0;
            tileOut_[t] = totalRows_ + r;
            ++t;
        }
        totalRows_ += d.rows;
    }
}

namespace {
class BatchReaper {
public:
    BatchReaper() : thread_([this] { Run(); }) {}
    ~BatchReaper()
    {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_one();
        thread_.join();
    }
    void Add(std::vector<VectorBatch *> &&batches)
    {
        {
            std::lock_guard<std::mutex> g(mu_);
            queue_.push_back(std::move(batches));
        }
        cv_.notify_one();
    }

private:
    void Run()
    {
        std::unique_lock<std::mutex> lock(mu_);
        while (true) {
            cv_.wait(lock, [this] { return stop_ || !queue_.empty(); });
            while (!queue_.empty()) {
                std::vector<VectorBatch *> work = std::move(queue_.front());
                queue_.pop_front();
                lock.unlock();
                for (auto *b : work) {
                    omniruntime::vec::VectorHelper::FreeVecBatch(b);
                }
                lock.lock();
            }
            if (stop_) {
                return;
            }
        }
    }
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<std::vector<VectorBatch *>> queue_;
    bool stop_ = false;
    std::thread thread_;  // last member: starts after the others exist
};
}  // namespace

void FreeBatchesLater(std::vector<VectorBatch *> &&batches)
{
    static BatchReaper reaper;
    if (!batches.empty()) {
        reaper.Add(std::move(batches));
    }
}

void BatchTable::Upload(cudaStream_t s)
{
    if (!maskJobs_.empty() && !masksDone_) {
        maskBits_.Reset(static_cast<size_t>(std::max<int64_t>(maskWords_, 1)), s);
        hMaskJobs_.Reset(maskJobs_.size());
        for (size_t j = 0; j < maskJobs_.size(); ++j) {
            const MaskSlot &ms = maskSlots_[j];
            MaskJob job = maskJobs_[j];
            job.out = maskBits_.Get() + ms.word;
            hMaskJobs_[j] = job;
            descs_[ms.batch].nulls[ms.input] = reinterpret_cast<const uint8_t *>(job.out);
        }
        dMaskJobs_.Reset(maskJobs_.size(), s);
        CudaCheck(cudaMemcpyAsync(dMaskJobs_.Get(), hMaskJobs_.Get(), sizeof(MaskJob) * maskJobs_.size(),
                      cudaMemcpyHostToDevice, s),
            "upload mask jobs");
        CudaCheck(LaunchMaskNulls(dMaskJobs_.Get(), static_cast<int32_t>(maskJobs_.size()), s), "mask NULL bitmaps");
        masksDone_ = true;
    }
    dBatches_.Reset(std::max<size_t>(descs_.Size(), 1), s);
    dTiles_.Reset(std::max<size_t>(tiles_.Size(), 1), s);
    dTileOut_.Reset(std::max<size_t>(tileOut_.Size(), 1), s);
    if (descs_.Size() > 0) {
        CudaCheck(cudaMemcpyAsync(dBatches_.Get(), descs_.Get(), sizeof(BatchDesc) * descs_.Size(),
                      cudaMemcpyHostToDevice, s),
            "upload batch descriptors");
    }
    if (tiles_.Size() > 0) {
        CudaCheck(cudaMemcpyAsync(dTiles_.Get(), tiles_.Get(), sizeof(TileDesc) * tiles_.Size(),
                      cudaMemcpyHostToDevice, s),
            "upload tile descriptors");
        CudaCheck(cudaMemcpyAsync(dTileOut_.Get(), tileOut_.Get(), sizeof(int64_t) * tileOut_.Size(),
                      cudaMemcpyHostToDevice, s),
            "upload tile offsets");
    }
}

std::vector<int64_t> BatchTable::RegionRows(int32_t nRegions) const
{
    std::vector<int64_t> rows(static_cast<size_t>(nRegions > 0 ? nRegions : 1), 0);
    const TileDesc *t = tiles_.Get();
    for (size_t i = 0; i < tiles_.Size(); ++i) {
        rows[i % rows.size()] += t[i].rows;
    }
    return rows;
}

size_t NullBitmapBytes(int64_t rows) { return static_cast<size_t>(((rows + 31) / 32) * 4 + 8); }

namespace {
std::atomic<long long> g_waitBudget{0};
std::mutex g_poolMu;
std::vector<cudaStream_t> *g_streamPool = new std::vector<cudaStream_t>();  // never freed, like its streams
}

cudaStream_t AcquirePooledStream()
{
    {
        std::lock_guard<std::mutex> g(g_poolMu);
        if (!g_streamPool->empty()) {
            cudaStream_t s = g_streamPool->back();
            g_streamPool->pop_back();
            return s;
        }
    }
    cudaStream_t s = nullptr;
    CudaCheck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    return s;
}

void ReleasePooledStream(cudaStream_t s)
{
    std::lock_guard<std::mutex> g(g_poolMu);
    g_streamPool->push_back(s);
}
long long WaitBudget()
{
    const long long b = g_waitBudget.load();
    return b > 0 ? b : kDefaultWaitBudget;
}
void SetWaitBudget(long long ticks) { g_waitBudget.store(ticks); }

namespace {
std::atomic<int64_t> g_aggFlushRows{0};
}
int64_t AggFlushRows()
{
    const int64_t r = g_aggFlushRows.load();
    return r > 0 ? r : (int64_t(1) << 28);
}
void SetAggFlushRows(int64_t rows) { g_aggFlushRows.store(rows); }

namespace {
std::atomic<int64_t> g_probeChunkRows{0};
}
int64_t ProbeChunkRows()
{
    const int64_t r = g_probeChunkRows.load();
    return r > 0 ? r : (int64_t(1) << 22);
}
void SetProbeChunkRows(int64_t rows) { g_probeChunkRows.store(rows); }

std::vector<VectorBatch *> CarveBatches(const std::vector<OutColumn> &cols, int64_t rows, int32_t rowsPerBatch,
    int64_t firstRow)
{
    std::vector<VectorBatch *> out;
    if (rows <= 0) {
        return out;
    }
    const int32_t step = AlignedBatchRows(rowsPerBatch);
    for (int64_t r0 = 0; r0 < rows; r0 += step) {
        const int32_t n = static_cast<int32_t>(std::min<int64_t>(step, rows - r0));
        auto *b = new VectorBatch(n);
        auto view = [&](const OutColumn &c) -> BaseVector * {
            const size_t nOff = static_cast<size_t>((firstRow + r0) / 8);
            if (c.width == 0) {
                const size_t oOff = static_cast<size_t>(firstRow + r0) * sizeof(int32_t);
                return new BaseVector(c.type, n, c.values, c.dataBytes, c.offsets, oOff, c.nulls, nOff, c.hasNull);
            }
            const size_t vOff = static_cast<size_t>(firstRow + r0) * c.width;
            return new BaseVector(c.type, c.width, n, c.values, vOff, c.nulls, nOff, c.hasNull);
        };
        for (size_t i = 0; i < cols.size(); ++i) {
            if (cols[i].containerFields > 0) {
                std::vector<BaseVector *> fields;
                for (int32_t f = 0; f < cols[i].containerFields; ++f) {
                    fields.push_back(view(cols.at(i + f)));
                }
                b->Append(new BaseVector(fields));
                i += static_cast<size_t>(cols[i].containerFields - 1);
                continue;
            }
            b->Append(view(cols[i]));
        }
        out.push_back(b);
    }
    return out;
}

std::vector<OutColumn> CopyColumnsToHost(const std::vector<OutColumn> &cols, int64_t rows, cudaStream_t s,
    int64_t firstRow)
{
    std::vector<OutColumn> host;
    for (const auto &c : cols) {
        OutColumn h = c;
        if (c.width == 0) {
            // VARCHAR: the offsets of these rows, then the characters they span, rebased to 0.
            const size_t ob = (static_cast<size_t>(rows) + 1) * sizeof(int32_t);
            h.offsets = Buffer::NewHost(ob, false);
            CudaCheck(cudaMemcpyAsync(h.offsets->Data(),
                          static_cast<const char *>(c.offsets->Data()) + static_cast<size_t>(firstRow) * sizeof(int32_t),
                          ob, cudaMemcpyDeviceToHost, s),
                "copy output offsets to host");
            CudaCheck(cudaStreamSynchronize(s), "copy output offsets to host");
            int32_t *o = static_cast<int32_t *>(h.offsets->Data());
            const int32_t base = o[0];
            const int64_t bytes = static_cast<int64_t>(o[rows]) - base;
            h.values = Buffer::NewHost(static_cast<size_t>(bytes) + 16, false);
            h.dataBytes = bytes;
            if (bytes > 0) {
                CudaCheck(cudaMemcpyAsync(h.values->Data(), static_cast<const char *>(c.values->Data()) + base,
                              static_cast<size_t>(bytes), cudaMemcpyDeviceToHost, s),
                    "copy output characters to host");
            }
            for (int64_t i = 0; i <= rows; ++i) {
                o[i] -= base;
            }
        } else {
        const size_t vb = static_cast<size_t>(rows) * c.width;
        h.values = Buffer::NewHost(vb == 0 ? 16 : vb, false);
        if (vb > 0) {
            const char *src = static_cast<const char *>(c.values->Data()) + static_cast<size_t>(firstRow) * c.width;
            CudaCheck(cudaMemcpyAsync(h.values->Data(), src, vb, cudaMemcpyDeviceToHost, s),
                "copy output values to host");
        }
        }
        const size_t nb = NullBitmapBytes(rows);
        if (c.nulls != nullptr && c.hasNull) {
            // The source bitmap holds NullBitmapBytes(firstRow + rows) bytes or more.
            h.nulls = Buffer::NewHost(nb, false);
            const char *src = static_cast<const char *>(c.nulls->Data()) + static_cast<size_t>(firstRow / 8);
            CudaCheck(cudaMemcpyAsync(h.nulls->Data(), src, nb, cudaMemcpyDeviceToHost, s),
                "copy output nulls to host");
        } else {
            h.nulls = Buffer::NewHost(nb, true);
            h.hasNull = false;
        }
        host.push_back(h);
    }
    return host;
}

BaseVector *FlattenDictionary(const BaseVector &v, cudaStream_t s)
{
    using omniruntime::vec::OMNI_DICTIONARY;
    if (v.GetEncoding() != OMNI_DICTIONARY) {
        throw OmniException("INVALID_ARGUMENT", "not a dictionary-encoded vector", -1);
    }
    RequireDevice();
    const BaseVector &d = *v.Dictionary();
    const int64_t n = v.GetSize();
    const int32_t *ids = v.RawIds();
    DevArray<int32_t> err(1, s, true);
    const size_t nullBytes = static_cast<size_t>(((n + 31) / 32) * 4 + 8);
    BufferPtr nulls = Buffer::NewDevice(nullBytes, s, true);
    BaseVector *out = nullptr;
    if (d.IsVarlen()) {
        DevArray<uint32_t> lens(static_cast<size_t>(n), s);
        CudaCheck(LaunchDictGatherLens(ids, n, d.RawOffsets(), d.RawNulls(), d.GetSize(), lens.Get(),
                      static_cast<uint32_t *>(nulls->Data()), err.Get(), s),
            "dictionary string lengths");
        DevArray<int64_t> offs64;
        const int64_t total = ScanLengths(lens.Get(), n, offs64, s);
        if (total >= (int64_t(1) << 31)) {
            throw OmniException("UNSUPPORTED_ERROR", "more than 2 GiB of characters in one vector", -2);
        }
        BufferPtr chars = Buffer::NewDevice(static_cast<size_t>(total) + 16, s, false);
        BufferPtr offs = Buffer::NewDevice((static_cast<size_t>(n) + 1) * sizeof(int32_t), s, true);
        CudaCheck(LaunchDictGatherChars(ids, n, d.RawOffsets(), d.RawValues(), d.RawNulls(), d.GetSize(),
                      offs64.Get(), static_cast<uint8_t *>(chars->Data()), static_cast<int32_t *>(offs->Data()), total,
                      s),
            "dictionary strings");
        out = new BaseVector(v.GetTypeId(), v.GetSize(), chars, total, offs, 0, nulls, 0, d.NullFlag());
    } else {
        const int w = d.GetWidth();
        if (w != 1 && w != 2 && w != 4 && w != 8 && w != 16) {
            throw OmniException("UNSUPPORTED_ERROR", "dictionary vectors of " + std::to_string(w) + "-byte values", -2);
        }
        BufferPtr values = Buffer::NewDevice(((static_cast<size_t>(d.GetWidth()) * (n < 1 ? 1 : n)) + 15) & ~size_t(15),
            s, false);
        CudaCheck(LaunchDictGatherFixed(ids, n, d.RawValues(), d.RawNulls(), d.GetSize(), d.GetWidth(),
                      static_cast<uint8_t *>(values->Data()), static_cast<uint32_t *>(nulls->Data()), err.Get(), s),
            "dictionary values");
        out = new BaseVector(v.GetTypeId(), v.GetWidth(), v.GetSize(), values, 0, nulls, 0, d.NullFlag());
    }
    int32_t h = 0;
    CudaCheck(cudaMemcpyAsync(&h, err.Get(), sizeof(h), cudaMemcpyDeviceToHost, s), "read dictionary check");
    CudaCheck(cudaStreamSynchronize(s), "read dictionary check");
    if (h != 0) {
        delete out;
        throw OmniException("INVALID_ARGUMENT", "dictionary id out of range", -1);
    }
    return out;
}

bool HasDictionary(const VectorBatch *batch)
{
    for (int32_t i = 0; i < batch->GetVectorCount(); ++i) {
        if (batch->Get(i)->GetEncoding() == omniruntime::vec::OMNI_DICTIONARY) {
            return true;
        }
    }
    return false;
}

void FlattenTaken(VectorBatch *batch)
{
    if (!HasDictionary(batch)) {
        return;
    }
    cudaStream_t s = nullptr;
    try {
        RequireDevice();
        s = AcquirePooledStream();
        FlattenDictionaries(batch, s);
    } catch (...) {
        if (s != nullptr) {
            ReleasePooledStream(s);
        }
        omniruntime::vec::VectorHelper::FreeVecBatch(batch);
        throw;
    }
    ReleasePooledStream(s);
}

void FlattenDictionaries(VectorBatch *batch, cudaStream_t s)
{
    for (int32_t i = 0; i < batch->GetVectorCount(); ++i) {
        if (batch->Get(i)->GetEncoding() == omniruntime::vec::OMNI_DICTIONARY) {
            batch->Set(i, FlattenDictionary(*batch->Get(i), s));
        }
    }
}

// A VARCHAR column from per-row lengths: exclusive offsets (n + 1, 64-bit) and the total.
int64_t ScanLengths(const uint32_t *lens, int64_t n, DevArray<int64_t> &offs, cudaStream_t s)
{
    offs.Reset(static_cast<size_t>(n) + 1, s);
    DevArray<int64_t> blockSums(static_cast<size_t>((n + 1023) / 1024 + 1), s);
    DevArray<long long> total(1, s, true);
    if (n > 0) {
        CudaCheck(LaunchScanCounts(lens, n, offs.Get(), blockSums.Get(), total.Get(), s), "scan lengths");
    }
    CudaCheck(LaunchOffsetsTail(offs.Get(), n, total.Get(), s), "offsets tail");
    long long h = 0;
    CudaCheck(cudaMemcpyAsync(&h, total.Get(), sizeof(h), cudaMemcpyDeviceToHost, s), "read total length");
    CudaCheck(cudaStreamSynchronize(s), "read total length");
    return h;
}

}  // namespace omg
