// Hash aggregation of one device-resident batch that allocates no memory.
//
// For callers that cannot let a library allocate device memory: a host engine that accounts
// for every byte of HBM in its own pre-reserved pool, or a caller running where allocation calls
// are not permitted.  The group table, the launch descriptors and the counters live in one
// file-scope device array of fixed size (kNoAllocScratchBytes); every GPU that loads this
// library keeps that array for the life of the process.  The caller passes the input columns
// and pre-allocated output columns.
//
// The array is shared by every call: a call re-initialises what it uses, so calls must not
// overlap on the GPU (calls issued concurrently on different streams race on the array).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "kernels/agg_noalloc.h"
#include "kernels/launch.h"
#include "kernels/plan.h"

namespace omg {
namespace {

constexpr size_t kScratchWords = kNoAllocScratchBytes / sizeof(uint64_t);
static __device__ __align__(256) uint64_t g_noallocScratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_setupMu;
uint64_t *g_scratchPtr[kMaxDevices] = {};

// Device address of the scratch array for the current device, looked up once per device.  In
// host code `g_noallocScratch` names a host-side stand-in, not device memory; only the address
// returned by cudaGetSymbolAddress may be handed to a kernel.
cudaError_t ScratchForCurrentDevice(uint64_t **out)
{
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) {
        return err;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        return cudaErrorInvalidDevice;
    }
    std::lock_guard<std::mutex> g(g_setupMu);
    if (g_scratchPtr[dev] == nullptr) {
        void *p = nullptr;
        err = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (err != cudaSuccess) {
            return err;
        }
        g_scratchPtr[dev] = static_cast<uint64_t *>(p);
    }
    *out = g_scratchPtr[dev];
    return cudaSuccess;
}

struct DescArgs {
    const void *cols[kMaxInputs];
    const uint8_t *nulls[kMaxInputs];
    int64_t rows;
};

// One batch descriptor and its 4096-row tiles, written on the device (no host staging buffer).
__global__ void FillDescKernel(const __grid_constant__ DescArgs a, BatchDesc *batch, TileDesc *tiles, int32_t nTiles)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int i = 0; i < kMaxInputs; ++i) {
            batch->cols[i] = a.cols[i];
            batch->nulls[i] = a.nulls[i];
        }
        batch->rows = a.rows;
        batch->rowBase = 0;
    }
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nTiles; t += gridDim.x * blockDim.x) {
        const int64_t r0 = static_cast<int64_t>(t) * kTileRows;
        tiles[t].batch = 0;
        tiles[t].row0 = static_cast<int32_t>(r0);
        tiles[t].rows = static_cast<int32_t>(a.rows - r0 < kTileRows ? a.rows - r0 : kTileRows);
        tiles[t].pad = 0;
    }
}

uint64_t NextPow2(uint64_t v)
{
    uint64_t p = 1;
    while (p < v) {
        p <<= 1;
    }
    return p;
}

size_t AlignWords(size_t bytes) { return (bytes + 255) / 256 * 32; }  // 256-byte aligned, in words

}  // namespace

NoAllocStatus RunAggNoAlloc(const NoAllocPlan &plan, const void *const *cols, const uint8_t *const *nulls,
    int32_t nCols, int64_t nRows, void *const *outValues, uint8_t *const *outNulls, int32_t nOut, int64_t maxGroups,
    int64_t *numGroups, cudaStream_t stream)
{
    NoAllocStatus st;
    auto error = [&st](int32_t code, const char *fmt, long long a = 0, long long b = 0) {
        st.code = code;
        std::snprintf(st.message, sizeof(st.message), fmt, a, b);
        return st;
    };
    if (nRows < 0 || maxGroups <= 0 || nRows > (int64_t(1) << 31) - 1 || nOut != plan.nOut || numGroups == nullptr ||
        cols == nullptr || outValues == nullptr || outNulls == nullptr) {
        return error(-1, "invalid arguments");
    }
    for (int32_t i = 0; i < plan.nInputs; ++i) {
        const int32_t c = plan.inputCols[i];
        if (c < 0 || c >= nCols || cols[c] == nullptr) {
            return error(-1, "missing input column %lld", c);
        }
    }
    // Scratch layout: [table (cap + 2) * slotWords][special + stats][batch desc][tiles].
    const uint64_t cap = NextPow2(std::max<uint64_t>(2 * static_cast<uint64_t>(maxGroups), 1024));
    const int32_t nTiles = static_cast<int32_t>((nRows + kTileRows - 1) / kTileRows);
    const size_t tableWords = AlignWords((cap + 2) * plan.slotWords * sizeof(uint64_t));
    const size_t ctrWords = AlignWords(16 * sizeof(uint64_t));
    const size_t descWords = AlignWords(sizeof(BatchDesc));
    const size_t tileWords = AlignWords(static_cast<size_t>(nTiles > 0 ? nTiles : 1) * sizeof(TileDesc));
    if (tableWords + ctrWords + descWords + tileWords > kScratchWords) {
        return error(-1, "max_groups %lld with %lld rows exceeds the 64 MiB no-alloc scratch", maxGroups, nRows);
    }
    uint64_t *base = nullptr;
    cudaError_t err = ScratchForCurrentDevice(&base);
    if (err != cudaSuccess) {
        std::snprintf(st.message, sizeof(st.message), "cudaGetSymbolAddress: %s", cudaGetErrorString(err));
        st.code = -3;
        return st;
    }
    uint64_t *slots = base;
    unsigned long long *ctr = reinterpret_cast<unsigned long long *>(base + tableWords);
    BatchDesc *desc = reinterpret_cast<BatchDesc *>(base + tableWords + ctrWords);
    TileDesc *tiles = reinterpret_cast<TileDesc *>(base + tableWords + ctrWords + descWords);
    // ctr: [0] groups inserted, [1] retry count, [2] spill count, [3] error, [4] group count,
    //      [5] rows written, [6] extract error, [7] ambiguous groups, [8..9] special-slot flags.
    uint32_t *special = reinterpret_cast<uint32_t *>(ctr + 8);

    auto fail = [&st](cudaError_t e, const char *what) {
        st.code = -3;
        std::snprintf(st.message, sizeof(st.message), "%s: %s", what, cudaGetErrorString(e));
        return st;
    };
    if ((err = cudaMemsetAsync(ctr, 0, 16 * sizeof(uint64_t), stream)) != cudaSuccess) {
        return fail(err, "clear counters");
    }
    DescArgs da;
    std::memset(&da, 0, sizeof(da));
    for (int32_t i = 0; i < plan.nInputs; ++i) {
        da.cols[i] = cols[plan.inputCols[i]];
        da.nulls[i] = nulls != nullptr ? nulls[plan.inputCols[i]] : nullptr;
    }
    da.rows = nRows;
    FillDescKernel<<<std::max(1, std::min(nTiles / 256 + 1, 64)), 256, 0, stream>>>(da, desc, tiles, nTiles);
    if ((err = cudaGetLastError()) != cudaSuccess) {
        return fail(err, "descriptor kernel");
    }

    AggLaunch p;
    std::memset(&p, 0, sizeof(p));
    p.key = plan.key;
    p.nAccs = plan.nAccs;
    for (int i = 0; i < p.nAccs; ++i) {
        p.accs[i] = plan.accs[i];
    }
    p.nRegInputs = plan.nRegInputs;
    for (int i = 0; i < p.nRegInputs; ++i) {
        p.regInput[i] = plan.regInput[i];
        p.regWidth[i] = plan.regWidth[i];
    }
    p.stateWords = plan.stateWords;
    // At most half full by construction, so a row is placed long before this many probes;
    // more groups than max_groups show up as the error below.
    p.maxProbe = static_cast<int32_t>(std::min<uint64_t>(cap, 4096));
    p.table.slots = slots;
    p.table.capacity = cap;
    p.table.slotWords = plan.slotWords;
    p.table.keyWords = plan.keyWords;
    p.table.specialUsed = special;
    p.table.groupCount = ctr;
    p.nRetry = reinterpret_cast<unsigned int *>(ctr + 1);
    p.retryCap = 0;  // nowhere to queue a row: an unplaceable row is an error
    p.error = reinterpret_cast<int32_t *>(ctr + 3);
    p.waitBudget = plan.waitBudget > 0 ? plan.waitBudget : kDefaultWaitBudget;
    p.batches = desc;
    p.tiles = tiles;
    p.nTiles = nTiles;
    p.smemSlots = plan.smemSlots;
    if ((err = LaunchAggInitTable(p, stream)) != cudaSuccess) {
        return fail(err, "init table");
    }
    if (nTiles > 0) {
        if ((err = LaunchAgg(p, nullptr, reinterpret_cast<unsigned int *>(ctr + 2), 0, nullptr, 0, 0, stream)) !=
            cudaSuccess) {
            return fail(err, "aggregation kernel");
        }
    }
    if ((err = LaunchAggCount(p.table, p.key.kind, ctr + 4, stream)) != cudaSuccess) {
        return fail(err, "count groups");
    }
    unsigned long long h[8];
    if ((err = cudaMemcpyAsync(h, ctr, sizeof(h), cudaMemcpyDeviceToHost, stream)) != cudaSuccess ||
        (err = cudaStreamSynchronize(stream)) != cudaSuccess) {
        return fail(err, "read counters");
    }
    // h[3] is the device error word: 7 = a bounded wait for another thread's slot publication
    // ran out; 4 = a row found no slot within the probe limit (no retry queue here, so the table
    // of 2 * max_groups slots overflowed).
    if (h[3] == 7) {
        return error(-7, "a bounded device-side wait ran out (slot publication)");
    }
    if (h[3] == 4 || h[1] != 0 || static_cast<int64_t>(h[4]) > maxGroups) {
        return error(-1, "the input has more than max_groups = %lld groups", maxGroups);
    }
    if (h[3] != 0 || h[2] != 0) {
        return error(-9, "internal error %lld in the aggregation kernel", static_cast<long long>(h[3]));
    }
    const int64_t groups = static_cast<int64_t>(h[4]);
    AggExtract e;
    std::memset(&e, 0, sizeof(e));
    e.table = p.table;
    e.key = plan.key;
    e.nAccs = p.nAccs;
    for (int i = 0; i < p.nAccs; ++i) {
        e.accs[i] = plan.accs[i];
    }
    e.nOut = nOut;
    const size_t nullBytes = static_cast<size_t>((maxGroups + 31) / 32) * 4;
    for (int32_t o = 0; o < nOut; ++o) {
        if (outValues[o] == nullptr || outNulls[o] == nullptr) {
            return error(-1, "missing output column %lld", o);
        }
        e.out[o] = plan.outs[o];
        e.out[o].values = outValues[o];
        e.out[o].nulls = outNulls[o];
        if ((err = cudaMemsetAsync(outNulls[o], 0, nullBytes, stream)) != cudaSuccess) {
            return fail(err, "clear output nulls");
        }
    }
    e.outCount = ctr + 5;
    e.overflowAsNull = plan.overflowAsNull ? 1 : 0;
    e.error = reinterpret_cast<int32_t *>(ctr + 6);
    e.nAmbiguous = ctr + 7;
    e.ambiguousSlots = nullptr;
    e.ambiguousCap = 0;
    if ((err = LaunchAggExtract(e, stream)) != cudaSuccess) {
        return fail(err, "extract groups");
    }
    if ((err = cudaMemcpyAsync(h, ctr, sizeof(h), cudaMemcpyDeviceToHost, stream)) != cudaSuccess ||
        (err = cudaStreamSynchronize(stream)) != cudaSuccess) {
        return fail(err, "read counters");
    }
    if (h[7] != 0) {
        return error(-2, "a group's sticky-overflow result depends on row order; use the operator API");
    }
    if (h[6] != 0) {
        return error(-5, "sum_aggregator overflow.");
    }
    *numGroups = groups;
    return st;
}

}  // namespace omg
