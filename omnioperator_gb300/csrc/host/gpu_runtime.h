// Host-side helpers for launching the operator kernels: error checks, streams, scratch
// buffers and the batch/tile descriptor tables that let one launch cover many VectorBatches.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "kernels/plan.h"
#include "omniop/memory.h"
#include "omniop/types.h"
#include "omniop/vector.h"

namespace omg {

using omniruntime::exception::OmniException;

inline void CudaCheck(cudaError_t err, const char *what)
{
    if (err != cudaSuccess) {
        cudaGetLastError();
        throw OmniException("CUDA_ERROR", std::string(what) + ": " + cudaGetErrorString(err), -3);
    }
}

inline void RequireDevice()
{
    if (!DeviceAvailable()) {
        throw OmniException("CUDA_ERROR", "no CUDA device is available; the GB300 operators do not run on the CPU", -8);
    }
}

// Operator-owned streams come from a process-wide pool and are never destroyed: device buffers
// are freed stream-ordered on the stream they were allocated on, and such a buffer (an output
// batch, a factory's packed payload) may outlive the operator that allocated it.
cudaStream_t AcquirePooledStream();
void ReleasePooledStream(cudaStream_t s);

// The stream an operator issues its work on: the caller's (which must stay valid while any
// device batch the operator produced is alive), or one from the pool.
class OpStream {
public:
    OpStream() = default;
    ~OpStream()
    {
        if (own_ != nullptr) {
            cudaStreamSynchronize(own_);
            ReleasePooledStream(own_);
        }
    }
    OpStream(const OpStream &) = delete;
    OpStream &operator=(const OpStream &) = delete;
    // Set the caller's stream; a previous call's stream counts as "unset" only via ClearUser.
    void SetUser(void *s)
    {
        user_ = static_cast<cudaStream_t>(s);
        userSet_ = true;
    }
    void ClearUser() { userSet_ = false; }
    cudaStream_t Get()
    {
        if (userSet_) {
            return user_;
        }
        if (own_ == nullptr) {
            RequireDevice();
            own_ = AcquirePooledStream();
        }
        return own_;
    }
    void Sync() { CudaCheck(cudaStreamSynchronize(Get()), "cudaStreamSynchronize"); }

private:
    cudaStream_t user_ = nullptr;
    bool userSet_ = false;
    cudaStream_t own_ = nullptr;
};

// Times one kernel launch with CUDA events recorded on the launching stream; the elapsed
// time is read after the stream has been synchronised (ElapsedNs).
class KernelTimer {
public:
    ~KernelTimer()
    {
        if (start_ != nullptr) {
            cudaEventDestroy(start_);
            cudaEventDestroy(stop_);
        }
    }
    void Start(cudaStream_t s)
    {
        if (start_ == nullptr) {
            CudaCheck(cudaEventCreate(&start_), "cudaEventCreate");
            CudaCheck(cudaEventCreate(&stop_), "cudaEventCreate");
        }
        CudaCheck(cudaEventRecord(start_, s), "cudaEventRecord");
    }
    void Stop(cudaStream_t s) { CudaCheck(cudaEventRecord(stop_, s), "cudaEventRecord"); }
    int64_t ElapsedNs() const
    {
        float ms = 0.f;
        if (start_ == nullptr || cudaEventElapsedTime(&ms, start_, stop_) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return static_cast<int64_t>(static_cast<double>(ms) * 1e6);
    }

private:
    cudaEvent_t start_ = nullptr;
    cudaEvent_t stop_ = nullptr;
};

// A device scratch allocation, stream-ordered.
template <typename T> class DevArray {
public:
    DevArray() = default;
    DevArray(size_t n, cudaStream_t s, bool zero = false) { Reset(n, s, zero); }
    void Reset(size_t n, cudaStream_t s, bool zero = false)
    {
        n_ = n;
        buf_ = Buffer::NewDevice(sizeof(T) * (n == 0 ? 1 : n), s, zero);
    }
    void Release() { buf_.reset(); n_ = 0; }
    T *Get() const { return buf_ ? static_cast<T *>(buf_->Data()) : nullptr; }
    size_t Size() const { return n_; }
    const BufferPtr &Buf() const { return buf_; }

private:
    BufferPtr buf_;
    size_t n_ = 0;
};

// Pinned host staging array (kept alive until the stream work that reads it has finished).
template <typename T> class PinnedArray {
public:
    explicit PinnedArray(size_t n = 0) { Reset(n); }
    void Reset(size_t n)
    {
        n_ = n;
        buf_ = Buffer::NewHost(sizeof(T) * (n == 0 ? 1 : n), true);
    }
    T *Get() const { return static_cast<T *>(buf_->Data()); }
    T &operator[](size_t i) { return Get()[i]; }
    size_t Size() const { return n_; }

private:
    BufferPtr buf_;
    size_t n_ = 0;
};

// Descriptors of a list of batches for one launch.  Kernel input i of batch b is column
// inputCols[i] of the batch.  With inputMasks (one entry per input, -1 = none), an input whose
// entry is column m >= 0 reads its values as usual but its NULL bitmap is computed on the device
// at Upload: the value column's NULLs plus every row whose BOOLEAN column m is NULL or FALSE
// (aggregation mask columns).  An entry InvertedMask(m) drops the rows whose column m is TRUE
// instead (the isEmpty column of partial decimal sums), without reading m's NULLs; an entry
// NullsOfMask(m) drops the rows where column m is NULL (a partial count whose partial sum is).
constexpr int32_t InvertedMask(int32_t col) { return -2 - col; }
constexpr int32_t kNullsOfMaskBase = 1 << 24;
constexpr int32_t NullsOfMask(int32_t col) { return kNullsOfMaskBase + col; }
// Kernel inputs that are field `f` of the container vector in column `c` (BatchTable::Build).
constexpr int32_t kFieldRefBase = int32_t(1) << 29;
inline int32_t FieldRef(int32_t c, int32_t f) { return kFieldRefBase + (c << 4) + f; }
inline int32_t FieldRefColumn(int32_t ref) { return (ref - kFieldRefBase) >> 4; }
inline int32_t FieldRefField(int32_t ref) { return (ref - kFieldRefBase) & 15; }

class BatchTable {
public:
    void Build(const std::vector<omniruntime::vec::VectorBatch *> &batches, const std::vector<int32_t> &inputCols,
        int32_t tileRows = kTileRows, const std::vector<int32_t> *inputMasks = nullptr);
    // Copy descriptors to the device on `s` (again after SetInput).
    void Upload(cudaStream_t s);
    // Point input `input` of batch `batch` at other fixed-width values (e.g. dictionary ids of
    // a VARCHAR column; the NULL bitmap stays the column's own).
    void SetInput(size_t batch, int32_t input, const void *values)
    {
        descs_[batch].cols[input] = values;
        descs_[batch].offs[input] = nullptr;
    }
    // Point the NULL bitmap of input `input` of batch `batch` elsewhere (nullptr: no NULLs).
    void SetInputNulls(size_t batch, int32_t input, const uint8_t *nulls) { descs_[batch].nulls[input] = nulls; }
    int64_t BatchRows(size_t batch) { return descs_[batch].rows; }
    int64_t BatchRowBase(size_t batch) { return descs_[batch].rowBase; }
    size_t NumBatches() const { return descs_.Size(); }
    const BatchDesc *DeviceBatches() const { return dBatches_.Get(); }
    const TileDesc *DeviceTiles() const { return dTiles_.Get(); }
    const int64_t *DeviceTileOutRows() const { return dTileOut_.Get(); }
    int32_t NumTiles() const { return static_cast<int32_t>(tiles_.Size()); }
    // Rows of the tiles t with t % nRegions == r, per r.
    std::vector<int64_t> RegionRows(int32_t nRegions) const;
    int64_t TotalRows() const { return totalRows_; }
    bool AnyNulls(int32_t input) const { return input < static_cast<int32_t>(anyNulls_.size()) && anyNulls_[input]; }
    // True when input `input` of every batch is device memory (no pinned host vectors).
    bool AllOnDevice(int32_t input) const
    {
        return input >= 0 && input < static_cast<int32_t>(allDevice_.size()) && allDevice_[input];
    }

private:
    struct MaskSlot {
        size_t batch;
        int32_t input;
        int64_t word;  // offset of the input's bitmap in maskBits_ (32-bit words)
    };
    std::vector<MaskSlot> maskSlots_;
    std::vector<MaskJob> maskJobs_;
    int64_t maskWords_ = 0;
    bool masksDone_ = false;
    DevArray<uint32_t> maskBits_;
    PinnedArray<MaskJob> hMaskJobs_;
    DevArray<MaskJob> dMaskJobs_;
    PinnedArray<BatchDesc> descs_;
    PinnedArray<TileDesc> tiles_;
    PinnedArray<int64_t> tileOut_;
    DevArray<BatchDesc> dBatches_;
    DevArray<TileDesc> dTiles_;
    DevArray<int64_t> dTileOut_;
    std::vector<bool> anyNulls_;
    std::vector<bool> allDevice_;
    int64_t totalRows_ = 0;
};

// Round a row count per output batch down so every batch starts on a 64-row boundary,
// which keeps every batch's null bitmap a byte-aligned view of one large bitmap.
inline int32_t AlignedBatchRows(int32_t maxRows)
{
    return maxRows >= 128 ? (maxRows / 64) * 64 : maxRows;
}

size_t NullBitmapBytes(int64_t rows);

// Frees batches an operator is done with on a background thread, off the operator's path: a
// pipelined probe takes thousands of small host batches per step, and each free returns its
// pinned buffers to the pool.  The batches must no longer be read by any kernel.
void FreeBatchesLater(std::vector<omniruntime::vec::VectorBatch *> &&batches);

// A VARCHAR column from per-row lengths: exclusive offsets (n + 1, 64-bit, the total last) and
// the total, read back to the host (synchronises `s`).
int64_t ScanLengths(const uint32_t *lens, int64_t n, DevArray<int64_t> &offs, cudaStream_t s);

// A dictionary-encoded vector as a new flat DEVICE vector (gathered on `s`; synchronises `s` to
// check the ids).  Throws INVALID_ARGUMENT for an id outside the dictionary.
omniruntime::vec::BaseVector *FlattenDictionary(const omniruntime::vec::BaseVector &v, cudaStream_t s);
// Replace every dictionary-encoded vector of `batch` by its flat device form.
void FlattenDictionaries(omniruntime::vec::VectorBatch *batch, cudaStream_t s);
bool HasDictionary(const omniruntime::vec::VectorBatch *batch);
// For a batch an operator has taken: flatten it on a pooled stream, freeing the batch if that
// fails (the error is rethrown).
void FlattenTaken(omniruntime::vec::VectorBatch *batch);

// Budget of device-side bounded waits (clock64 ticks); 0 restores the default.
long long WaitBudget();
void SetWaitBudget(long long ticks);
// Staged rows at which an aggregation operator flushes its queued batches; 0 restores 2^28.
int64_t AggFlushRows();
void SetAggFlushRows(int64_t rows);
// Queued probe rows at which a pipelined probe operator launches a chunk; 0 restores 2^22.
int64_t ProbeChunkRows();
void SetProbeChunkRows(int64_t rows);

// Cut `rows` rows of contiguous output columns into VectorBatches of at most
// `rowsPerBatch` rows that are views of the given buffers (host or device).
struct OutColumn {
    omniruntime::type::DataTypeId type;
    int32_t width;    // 0: VARCHAR/CHAR (values = characters, offsets = rows + 1 int32)
    BufferPtr values;
    BufferPtr nulls;  // may be null
    bool hasNull;
    BufferPtr offsets;       // VARCHAR/CHAR: absolute positions in `values`
    int64_t dataBytes = 0;   // VARCHAR/CHAR: size of `values`
    // > 0: this column and the next containerFields - 1 columns are the fields of one container
    // vector in the output batches (a partial AVG under the container-vector policy).
    int32_t containerFields = 0;
};
// The rows start at row `firstRow` of the buffers (a multiple of 8).
std::vector<omniruntime::vec::VectorBatch *> CarveBatches(const std::vector<OutColumn> &cols, int64_t rows,
    int32_t rowsPerBatch, int64_t firstRow = 0);

// Copy rows [firstRow, firstRow + rows) of device output columns to new pinned host buffers
// (one copy per column) on `s`; firstRow is a multiple of 8.
std::vector<OutColumn> CopyColumnsToHost(const std::vector<OutColumn> &cols, int64_t rows, cudaStream_t s,
    int64_t firstRow = 0);

}  // namespace omg
