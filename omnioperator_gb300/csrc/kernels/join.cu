// Hash join build and probe kernels for sm_103a.
//
// Build replaces JoinHashTableVariants::BuildHashTable (operator/join/join_hash_table_variants.cpp:
// 695-863): min/max scan of the keys, then either a direct-index ARRAY table (dense keys) or an
// open-addressing HASH table.  Duplicate build keys, which the reference chains in RowRefList
// blocks (operator/join/row_ref.h:27-169), become a CSR of build rows per key.
//
// Probe replaces LookupJoinOperator::ProbeBatchForInnerJoin / ArrayJoinProbeSIMDNeon and the
// output builder (operator/join/lookup_join.cpp:847-1035,1667-1985): a CTA takes a tile of up to
// 4096 probe rows, looks every non-null key up in registers, prefix-sums the match counts per
// (round, warp) so that the tile's matches get one contiguous output range from a single
// atomicAdd, and writes probe columns plus gathered build columns in probe-row order within the
// tile.
#include <algorithm>
#include <atomic>
#include <type_traits>
#include <cstdint>
#include <cuda_runtime.h>

#include "bulk_copy.cuh"
#include "device_common.cuh"
#include "launch.h"
#include "plan.h"

namespace omg {
namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeRounds = kTileRows / kProbeThreads;  // 16

int SMs() { return DeviceSMCount(); }

unsigned GridFor(int64_t n, int threads, int perSM)
{
    int64_t blocks = (n + threads - 1) / threads;
    const int64_t cap = static_cast<int64_t>(SMs()) * perSM;
    if (blocks > cap) {
        blocks = cap;
    }
    return static_cast<unsigned>(blocks < 1 ? 1 : blocks);
}

__device__ __forceinline__ void CopyValue(void *dst, uint64_t dpos, const void *src, int64_t spos, int width)
{
    switch (width) {
        case 1:
            static_cast<uint8_t *>(dst)[dpos] = static_cast<const uint8_t *>(src)[spos];
            break;
        case 2:
            static_cast<uint16_t *>(dst)[dpos] = static_cast<const uint16_t *>(src)[spos];
            break;
        case 4:
            static_cast<uint32_t *>(dst)[dpos] = static_cast<const uint32_t *>(src)[spos];
            break;
        case 8:
            static_cast<uint64_t *>(dst)[dpos] = static_cast<const uint64_t *>(src)[spos];
            break;
        case 16: {
            const uint64_t *s = static_cast<const uint64_t *>(src) + 2 * spos;
            uint64_t *d = static_cast<uint64_t *>(dst) + 2 * dpos;
            d[0] = s[0];
            d[1] = s[1];
            break;
        }
        default: {
            const uint8_t *s = static_cast<const uint8_t *>(src) + static_cast<int64_t>(width) * spos;
            uint8_t *d = static_cast<uint8_t *>(dst) + static_cast<uint64_t>(width) * dpos;
            for (int i = 0; i < width; ++i) {
                d[i] = s[i];
            }
        }
    }
}

__device__ __forceinline__ void StoreKey(void *dst, uint64_t pos, int width, int64_t v)
{
    switch (width) {
        case 1:
            static_cast<int8_t *>(dst)[pos] = static_cast<int8_t>(v);
            break;
        case 2:
            static_cast<int16_t *>(dst)[pos] = static_cast<int16_t>(v);
            break;
        case 4:
            static_cast<int32_t *>(dst)[pos] = static_cast<int32_t>(v);
            break;
        default:
            static_cast<int64_t *>(dst)[pos] = v;
    }
}

__device__ __forceinline__ void SetBit(uint8_t *bitmap, uint64_t pos)
{
    atomicOr(reinterpret_cast<unsigned int *>(bitmap) + (pos >> 5), 1u << (pos & 31));
}

__global__ void GatherColumnKernel(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, int32_t input, int32_t width, void *valuesOut, uint8_t *nullsOut)
{
    for (int t = blockIdx.x; t < nTiles; t += gridDim.x) {
        const TileDesc tile = tiles[t];
        const BatchDesc &b = batches[tile.batch];
        const int64_t out0 = tileOutRow[t];
        const void *col = b.cols[input];
        const uint8_t *nulls = b.nulls[input];
        for (int r = threadIdx.x; r < tile.rows; r += blockDim.x) {
            const int64_t row = static_cast<int64_t>(tile.row0) + r;
            CopyValue(valuesOut, static_cast<uint64_t>(out0 + r), col, row, width);
            if (nullsOut != nullptr && RowIsNull(nulls, row)) {
                SetBit(nullsOut, static_cast<uint64_t>(out0 + r));
            }
        }
    }
}

__global__ void KeyStatsKernel(const void *keys, const uint8_t *nulls, int64_t n, int32_t width, long long *stats)
{
    long long mn = 0x7fffffffffffffffll;
    long long mx = static_cast<long long>(0x8000000000000000ull);
    unsigned long long cnt = 0;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (RowIsNull(nulls, i)) {
            continue;
        }
        const long long k = LoadInt(keys, i, width);
        mn = k < mn ? k : mn;
        mx = k > mx ? k : mx;
        ++cnt;
    }
    for (int o = 16; o > 0; o >>= 1) {
        long long omn = __shfl_down_sync(0xffffffffu, mn, o);
        long long omx = __shfl_down_sync(0xffffffffu, mx, o);
        unsigned long long oc = __shfl_down_sync(0xffffffffu, cnt, o);
        mn = omn < mn ? omn : mn;
        mx = omx > mx ? omx : mx;
        cnt += oc;
    }
    if ((threadIdx.x & 31) == 0 && cnt != 0) {
        atomicMin(&stats[0], mn);
        atomicMax(&stats[1], mx);
        atomicAdd(reinterpret_cast<unsigned long long *>(&stats[2]), cnt);
    }
}

// Find the hash slot of `key` (inserting it when `insert`), -1 if absent.
__device__ __forceinline__ int64_t HashSlot(uint64_t *keys, uint64_t capacity, uint64_t key, bool insert)
{
    const uint64_t mask = capacity - 1;
    uint64_t i = Mix64(key) & mask;
    for (uint64_t probe = 0; probe < capacity; ++probe) {
        unsigned long long *kp = reinterpret_cast<unsigned long long *>(keys + i);
        unsigned long long cur = *reinterpret_cast<volatile unsigned long long *>(kp);
        if (cur == key) {
            return static_cast<int64_t>(i);
        }
        if (cur == kEmptyKey) {
            if (!insert) {
                return -1;
            }
            unsigned long long prev = atomicCAS(kp, kEmptyKey, key);
            if (prev == kEmptyKey || prev == key) {
                return static_cast<int64_t>(i);
            }
        }
        i = (i + 1) & mask;
    }
    return -1;
}

__global__ void BuildCountKernel(JoinTable t, const void *keys, const uint8_t *nulls, int64_t n, int32_t width,
    uint64_t *hashKeys, uint32_t *counts, uint32_t *sentinelCount, unsigned int *maxCount, int32_t *error)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (RowIsNull(nulls, i)) {
            continue;
        }
        const uint64_t key = static_cast<uint64_t>(LoadInt(keys, i, width));
        uint32_t old;
        if (t.mode == JOIN_ARRAY) {
            old = atomicAdd(&counts[key - static_cast<uint64_t>(t.minKey)], 1u);
        } else if (key == kEmptyKey) {
            old = atomicAdd(sentinelCount, 1u);
        } else {
            const int64_t s = HashSlot(hashKeys, t.capacity, key, true);
            if (s < 0) {
                SetError(error, 4);
                continue;
            }
            old = atomicAdd(&counts[s], 1u);
        }
        if (old >= 1) {
            atomicMax(maxCount, old + 1);
        }
    }
}

__global__ void BuildFillKernel(JoinTable t, const void *keys, const uint8_t *nulls, int64_t n, int32_t width,
    const uint32_t *counts, const int64_t *offsets, uint32_t *cursor, int64_t *entries, int32_t *csrRows,
    uint32_t sentinelCount, int64_t sentinelOffset, unsigned int *sentinelCursor, int64_t *sentinelEntryOut,
    int32_t *error)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (RowIsNull(nulls, i)) {
            continue;
        }
        const uint64_t key = static_cast<uint64_t>(LoadInt(keys, i, width));
        int64_t slot;
        if (t.mode == JOIN_ARRAY) {
            slot = static_cast<int64_t>(key - static_cast<uint64_t>(t.minKey));
        } else if (key == kEmptyKey) {
            slot = -2;
        } else {
            slot = HashSlot(const_cast<uint64_t *>(t.hashKeys), t.capacity, key, false);
            if (slot < 0) {
                SetError(error, 4);
                continue;
            }
        }
        if (t.unique) {
            if (slot >= 0) {
                entries[slot] = i;
            } else {
                *sentinelEntryOut = i;
            }
            continue;
        }
        if (slot == -2) {
            const uint32_t c = atomicAdd(sentinelCursor, 1u);
            csrRows[sentinelOffset + c] = static_cast<int32_t>(i);
            continue;
        }
        const uint32_t c = atomicAdd(&cursor[slot], 1u);
        const int64_t off = offsets[slot];
        csrRows[off + c] = static_cast<int32_t>(i);
        if (c == 0) {
            entries[slot] = (off << 32) | static_cast<int64_t>(counts[slot]);
        }
    }
}

__global__ void FillI64Kernel(int64_t *p, int64_t v, int64_t n)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        p[i] = v;
    }
}

__global__ void FillU64Kernel(uint64_t *p, uint64_t v, int64_t n)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        p[i] = v;
    }
}

// ---- exclusive scan of uint32 counts (three passes: block sums, scan of sums, block scans)
constexpr int kScanThreads = 1024;

__global__ void ScanBlockSumsKernel(const uint32_t *counts, int64_t n, int64_t *blockSums)
{
    __shared__ long long warpSums[32];
    const int64_t i = static_cast<int64_t>(blockIdx.x) * kScanThreads + threadIdx.x;
    long long v = i < n ? counts[i] : 0;
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_down_sync(0xffffffffu, v, o);
    }
    if ((threadIdx.x & 31) == 0) {
        warpSums[threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long s = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) {
            s += warpSums[w];
        }
        blockSums[blockIdx.x] = s;
    }
}

__global__ void ScanSumsKernel(int64_t *blockSums, int64_t nBlocks, long long *total)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        long long run = 0;
        for (int64_t b = 0; b < nBlocks; ++b) {
            const long long v = blockSums[b];
            blockSums[b] = run;
            run += v;
        }
        *total = run;
    }
}

__global__ void ScanApplyKernel(const uint32_t *counts, int64_t n, const int64_t *blockSums, int64_t *offsets)
{
    __shared__ long long warpSums[32];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int64_t i = static_cast<int64_t>(blockIdx.x) * kScanThreads + threadIdx.x;
    const long long v = i < n ? counts[i] : 0;
    long long inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) {
            inc += y;
        }
    }
    if (lane == 31) {
        warpSums[warp] = inc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long s = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) {
            const long long c = warpSums[w];
            warpSums[w] = s;
            s += c;
        }
    }
    __syncthreads();
    if (i < n) {
        offsets[i] = blockSums[blockIdx.x] + warpSums[warp] + inc - v;
    }
}

// ---- probe
struct Match {
    int64_t entry;  // build row (unique) or CSR offset
    uint32_t count;
    uint64_t slot;  // table slot of the key (the slot payload index)
};

__device__ __forceinline__ Match Lookup(const JoinTable &t, uint64_t key)
{
    Match m{0, 0, 0};
    int64_t e = -1;
    if (t.mode == JOIN_ARRAY) {
        const uint64_t d = key - static_cast<uint64_t>(t.minKey);
        if (static_cast<int64_t>(key) >= t.minKey && d < t.range) {
            e = __ldg(reinterpret_cast<const long long *>(t.arrayEntries) + d);
            m.slot = d;
        }
    } else if (key == kEmptyKey) {
        e = t.sentinelEntry;
        m.slot = t.capacity;
    } else {
        const uint64_t mask = t.capacity - 1;
        uint64_t i = Mix64(key) & mask;
        for (uint64_t probe = 0; probe < t.capacity; ++probe) {
            const uint64_t k = __ldg(reinterpret_cast<const unsigned long long *>(t.hashKeys) + i);
            if (k == key) {
                e = __ldg(reinterpret_cast<const long long *>(t.hashEntries) + i);
                m.slot = i;
                break;
            }
            if (k == kEmptyKey) {
                break;
            }
            i = (i + 1) & mask;
        }
    }
    if (e >= 0) {
        if (t.unique) {
            m.entry = e;
            m.count = 1;
        } else {
            m.entry = e >> 32;
            m.count = static_cast<uint32_t>(e & 0xffffffffll);
        }
    }
    return m;
}

// Read-only loads (non-coherent path): the probe never writes what it reads, so these may be
// issued ahead of the output stores.
__device__ __forceinline__ int64_t LoadIntRO(const void *col, int64_t row, int width)
{
    switch (width) {
        case 1:
            return static_cast<int8_t>(__ldg(static_cast<const char *>(col) + row));
        case 2:
            return __ldg(static_cast<const short *>(col) + row);
        case 4:
            return __ldg(static_cast<const int *>(col) + row);
        default:
            return __ldg(static_cast<const long long *>(col) + row);
    }
}

__device__ __forceinline__ bool RowIsNullRO(const uint8_t *nulls, int64_t row)
{
    return nulls != nullptr && ((__ldg(reinterpret_cast<const unsigned char *>(nulls) + (row >> 3)) >> (row & 7)) & 1u);
}

__device__ __forceinline__ void CopyValueRO(void *dst, uint64_t dpos, const void *src, int64_t spos, int width)
{
    switch (width) {
        case 1:
            static_cast<uint8_t *>(dst)[dpos] = static_cast<uint8_t>(__ldg(static_cast<const char *>(src) + spos));
            break;
        case 2:
            static_cast<uint16_t *>(dst)[dpos] = static_cast<uint16_t>(__ldg(static_cast<const short *>(src) + spos));
            break;
        case 4:
            static_cast<uint32_t *>(dst)[dpos] = static_cast<uint32_t>(__ldg(static_cast<const int *>(src) + spos));
            break;
        case 8:
            static_cast<uint64_t *>(dst)[dpos] = static_cast<uint64_t>(__ldg(static_cast<const long long *>(src) + spos));
            break;
        case 16: {
            const longlong2 v = __ldg(static_cast<const longlong2 *>(src) + spos);
            static_cast<longlong2 *>(dst)[dpos] = v;
            break;
        }
        default:
            CopyValue(dst, dpos, src, spos, width);
    }
}

// Write one output row: probe columns from the probe batch (the key from registers), build
// columns gathered by build row.
// VARCHAR outputs get a handle to the source row (see JoinOutCol).
__device__ __forceinline__ int64_t ProbeHandle(const ProbeLaunch &p, const BatchDesc &b, int64_t row)
{
    return (static_cast<int64_t>(&b - p.batches) << 32) | row;
}

__device__ __forceinline__ void WriteJoinRow(const ProbeLaunch &p, const BatchDesc &b, int64_t row, int64_t key,
    int64_t buildRow, uint64_t pos)
{
    for (int o = 0; o < p.nOut; ++o) {
        const JoinOutCol &oc = p.out[o];
        if (oc.width == 0) {
            static_cast<int64_t *>(oc.values)[pos] = oc.side == 0 ? ProbeHandle(p, b, row) : buildRow;
            if (oc.nulls != nullptr &&
                RowIsNullRO(oc.side == 0 ? b.nulls[oc.src] : oc.buildNulls, oc.side == 0 ? row : buildRow)) {
                SetBit(oc.nulls, pos);
            }
            continue;
        }
        if (oc.side == 0) {
            if (oc.src == p.keyInput) {
                StoreKey(oc.values, pos, oc.width, key);
            } else {
                CopyValueRO(oc.values, pos, b.cols[oc.src], row, oc.width);
                if (oc.nulls != nullptr && RowIsNullRO(b.nulls[oc.src], row)) {
                    SetBit(oc.nulls, pos);
                }
            }
        } else {
            CopyValueRO(oc.values, pos, oc.buildValues, buildRow, oc.width);
            if (oc.nulls != nullptr && RowIsNullRO(oc.buildNulls, buildRow)) {
                SetBit(oc.nulls, pos);
            }
        }
    }
}

// Same as WriteJoinRow with the build columns taken from the packed slot payload.
__device__ __forceinline__ void WriteJoinRowPayload(const ProbeLaunch &p, const BatchDesc &b, int64_t row, int64_t key,
    uint64_t payload, uint64_t pos)
{
    for (int o = 0; o < p.nOut; ++o) {
        const JoinOutCol &oc = p.out[o];
        if (oc.width == 0) {  // a probe VARCHAR column (build ones have no slot payload)
            static_cast<int64_t *>(oc.values)[pos] = ProbeHandle(p, b, row);
            if (oc.nulls != nullptr && RowIsNullRO(b.nulls[oc.src], row)) {
                SetBit(oc.nulls, pos);
            }
            continue;
        }
        if (oc.side == 0) {
            if (oc.src == p.keyInput) {
                StoreKey(oc.values, pos, oc.width, key);
            } else {
                CopyValueRO(oc.values, pos, b.cols[oc.src], row, oc.width);
                if (oc.nulls != nullptr && RowIsNullRO(b.nulls[oc.src], row)) {
                    SetBit(oc.nulls, pos);
                }
            }
        } else {
            StoreKey(oc.values, pos, oc.width, static_cast<int64_t>(payload >> oc.shift));
        }
    }
}

// Packs the build output values of every unique-table slot (<= 8 bytes in total).
__global__ void BuildSlotPayloadKernel(const int64_t *entries, uint64_t nSlots, int64_t sentinelEntry,
    const __grid_constant__ ProbeLaunch p, uint64_t *payload)
{
    for (uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; s <= nSlots;
         s += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const int64_t row = s < nSlots ? entries[s] : sentinelEntry;
        uint64_t v = 0;
        if (row >= 0) {
            for (int o = 0; o < p.nOut; ++o) {
                const JoinOutCol &oc = p.out[o];
                if (oc.side == 1) {
                    const uint64_t bits = LoadBits(oc.buildValues, row, oc.width);
                    const uint64_t mask = oc.width >= 8 ? ~0ull : ((1ull << (8 * oc.width)) - 1);
                    v |= (bits & mask) << oc.shift;
                }
            }
        }
        payload[s] = v;
    }
}

// An output row without a build match: probe columns copied, build columns NULL (value 0),
// the existence flag (side 2) set to `matched`.
__device__ __forceinline__ void WriteProbeOnlyRow(const ProbeLaunch &p, const BatchDesc &b, int64_t row, int64_t key,
    bool matched, uint64_t pos)
{
    for (int o = 0; o < p.nOut; ++o) {
        const JoinOutCol &oc = p.out[o];
        if (oc.width == 0) {
            static_cast<int64_t *>(oc.values)[pos] = oc.side == 0 ? ProbeHandle(p, b, row) : -1;
            if (oc.side != 0 || RowIsNullRO(b.nulls[oc.src], row)) {
                SetBit(oc.nulls, pos);
            }
            continue;
        }
        if (oc.side == 0) {
            // Unlike a matched row, this one may carry a NULL probe key (outer and anti joins).
            if (oc.src == p.keyInput) {
                StoreKey(oc.values, pos, oc.width, key);
            } else {
                CopyValueRO(oc.values, pos, b.cols[oc.src], row, oc.width);
            }
            if (oc.nulls != nullptr && RowIsNullRO(b.nulls[oc.src], row)) {
                SetBit(oc.nulls, pos);
            }
        } else if (oc.side == 1) {
            uint8_t *d = static_cast<uint8_t *>(oc.values) + static_cast<uint64_t>(oc.width) * pos;
            for (int i = 0; i < oc.width; ++i) {
                d[i] = 0;
            }
            SetBit(oc.nulls, pos);
        } else {
            static_cast<uint8_t *>(oc.values)[pos] = matched ? 1 : 0;
        }
    }
}

// Output rows a probe row yields for a join kind, given whether the row exists (inside the
// tile) and its number of matching build rows.
__device__ __forceinline__ uint32_t EmitCount(int kind, bool exists, uint32_t cnt)
{
    switch (kind) {
        case JOIN_KIND_PROBE_OUTER:
        case JOIN_KIND_FULL:
            return exists ? (cnt != 0 ? cnt : 1u) : 0u;
        case JOIN_KIND_SEMI:
            return cnt != 0 ? 1u : 0u;
        case JOIN_KIND_ANTI:
            return exists && cnt == 0 ? 1u : 0u;
        case JOIN_KIND_EXISTENCE:
            return exists ? 1u : 0u;
        default:  // INNER, BUILD_OUTER
            return cnt;
    }
}

// Each warp owns kWarpRounds * 32 consecutive rows of a tile and works on its own: lane i reads
// rows base + 32r + i (coalesced), looks the keys up, reserves its output range with one
// atomicAdd, and writes its matches compacted in row order.  kUnique: every key has at most one
// build row, so a ballot gives the compaction; otherwise counts are prefix-summed per round.
constexpr int kWarpRounds = 16;
constexpr int kRowsPerWarp = kWarpRounds * 32;

// kKinds: any join kind (p.joinKind) -- the rows each probe row yields follow EmitCount, rows
// without a match get NULL build columns, and matched build rows are marked visited when the
// kind keeps unmatched build rows.
template <bool kUnique, bool kPayload, bool kKinds>
__global__ void __launch_bounds__(kProbeThreads, 3) ProbeKernel(const __grid_constant__ ProbeLaunch p)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const unsigned int lanesBelow = (1u << lane) - 1u;
    const bool arrayMode = p.table.mode == JOIN_ARRAY;
    const int kind = kKinds ? p.joinKind : static_cast<int>(JOIN_KIND_INNER);
    const bool emitMatches = kind == JOIN_KIND_INNER || kind == JOIN_KIND_PROBE_OUTER ||
        kind == JOIN_KIND_BUILD_OUTER || kind == JOIN_KIND_FULL;
    for (int t = blockIdx.x; t < p.nTiles; t += gridDim.x) {
        const TileDesc tile = p.tiles[t];
        const int w0 = warp * kRowsPerWarp;
        if (w0 >= tile.rows) {
            continue;
        }
        const BatchDesc &b = p.batches[tile.batch];
        const void *keyCol = b.cols[p.keyInput];
        const uint8_t *keyNulls = b.nulls[p.keyInput];
        const int64_t base = static_cast<int64_t>(tile.row0) + w0;
        const int nRows = min(kRowsPerWarp, tile.rows - w0);
        // Phase 1: all keys and validity bits of the warp's rows (independent loads).
        int64_t key[kWarpRounds];
        uint32_t live = 0;   // bit i: this lane's row of round i exists and its key is not NULL
        uint32_t exist = 0;  // bit i: this lane's row of round i exists
#pragma unroll
        for (int i = 0; i < kWarpRounds; ++i) {
            const int r = i * 32 + lane;
            key[i] = 0;
            if (r < nRows) {
                exist |= 1u << i;
                key[i] = LoadIntRO(keyCol, base + r, p.keyWidth);
                if (!RowIsNullRO(keyNulls, base + r)) {
                    live |= 1u << i;
                }
            }
        }
        // Phase 2: table lookups (independent of each other).
        int32_t entry[kWarpRounds];
        uint32_t cnt[kWarpRounds];
        uint64_t payload[kWarpRounds];  // kPayload: the build output values of the match
        uint32_t hit = 0;
        if (arrayMode) {
#pragma unroll
            for (int i = 0; i < kWarpRounds; ++i) {
                const uint64_t d = static_cast<uint64_t>(key[i]) - static_cast<uint64_t>(p.table.minKey);
                int64_t e = -1;
                payload[i] = 0;
                if (((live >> i) & 1u) && key[i] >= p.table.minKey && d < p.table.range) {
                    e = __ldg(reinterpret_cast<const long long *>(p.table.arrayEntries) + d);
                    if (kPayload) {
                        payload[i] = __ldg(reinterpret_cast<const unsigned long long *>(p.table.slotPayload) + d);
                    }
                }
                entry[i] = kUnique ? static_cast<int32_t>(e) : static_cast<int32_t>(e >> 32);
                cnt[i] = e < 0 ? 0u : (kUnique ? 1u : static_cast<uint32_t>(e & 0xffffffffll));
                hit |= (cnt[i] != 0 ? 1u : 0u) << i;
            }
        } else {
#pragma unroll
            for (int i = 0; i < kWarpRounds; ++i) {
                Match m{0, 0, 0};
                payload[i] = 0;
                if ((live >> i) & 1u) {
                    m = Lookup(p.table, static_cast<uint64_t>(key[i]));
                    if (kPayload && m.count != 0) {
                        payload[i] = __ldg(reinterpret_cast<const unsigned long long *>(p.table.slotPayload) + m.slot);
                    }
                }
                entry[i] = static_cast<int32_t>(m.entry);
                cnt[i] = m.count;
                hit |= (m.count != 0 ? 1u : 0u) << i;
            }
        }
        if (kKinds && p.visited != nullptr) {
#pragma unroll
            for (int i = 0; i < kWarpRounds; ++i) {
                if ((hit >> i) & 1u) {
                    // Most matches hit rows already marked: read first, store only the first time
                    // (a lost race stores the same value twice).
                    if (kUnique) {
                        if (p.visited[entry[i]] == 0) {
                            p.visited[entry[i]] = 1;
                        }
                    } else {
                        for (uint32_t k = 0; k < cnt[i]; ++k) {
                            const int32_t br = __ldg(p.table.csrRows + entry[i] + k);
                            if (p.visited[br] == 0) {
                                p.visited[br] = 1;
                            }
                        }
                    }
                }
            }
        }
        // emitBits (unique tables) / emit[] (duplicates): rows each probe row yields.
        uint32_t emitBits = 0;
        uint32_t total = 0;
        if (kUnique) {
#pragma unroll
            for (int i = 0; i < kWarpRounds; ++i) {
                const bool e = kKinds ? EmitCount(kind, (exist >> i) & 1u, (hit >> i) & 1u) != 0 : ((hit >> i) & 1u);
                emitBits |= (e ? 1u : 0u) << i;
                total += __popc(__ballot_sync(0xffffffffu, e));
            }
        } else {
#pragma unroll
            for (int i = 0; i < kWarpRounds; ++i) {
                total += kKinds ? EmitCount(kind, (exist >> i) & 1u, cnt[i]) : cnt[i];
            }
            total = __reduce_add_sync(0xffffffffu, total);
        }
        const int region = t % p.nRegions;
        unsigned long long pos = 0;
        if (lane == 0 && total != 0) {
            pos = atomicAdd(p.outCount + region * kRegionStride, static_cast<unsigned long long>(total));
        }
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (p.countOnly || total == 0) {
            continue;
        }
        const uint64_t regionBase = static_cast<uint64_t>(region) * p.regionCap;
        // Phase 3: compacted writes in row order.
#pragma unroll
        for (int i = 0; i < kWarpRounds; ++i) {
            const int64_t row = base + i * 32 + lane;
            const bool matched = (hit >> i) & 1u;
            if (kUnique) {
                const bool e = (emitBits >> i) & 1u;
                const unsigned int m = __ballot_sync(0xffffffffu, e);
                if (e) {
                    const uint64_t at = pos + __popc(m & lanesBelow);
                    if (at < p.regionCap) {
                        // The key is re-read (an L1/L2 hit) rather than kept live in registers.
                        const int64_t k = LoadIntRO(keyCol, row, p.keyWidth);
                        if (kKinds && !(matched && emitMatches)) {
                            WriteProbeOnlyRow(p, b, row, k, matched, regionBase + at);
                        } else if (kPayload) {
                            WriteJoinRowPayload(p, b, row, k, payload[i], regionBase + at);
                        } else {
                            WriteJoinRow(p, b, row, k, entry[i], regionBase + at);
                        }
                    }
                }
                pos += __popc(m);
            } else {
                const uint32_t e = kKinds ? EmitCount(kind, (exist >> i) & 1u, cnt[i]) : cnt[i];
                uint32_t inc = e;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) {
                        inc += y;
                    }
                }
                const uint64_t at = pos + inc - e;
                if (kKinds && e != 0 && !(matched && emitMatches)) {
                    if (at < p.regionCap) {
                        WriteProbeOnlyRow(p, b, row, LoadIntRO(keyCol, row, p.keyWidth), matched, regionBase + at);
                    }
                } else {
                    for (uint32_t k = 0; k < e; ++k) {
                        if (at + k >= p.regionCap) {
                            break;
                        }
                        WriteJoinRow(p, b, row, LoadIntRO(keyCol, row, p.keyWidth),
                            __ldg(p.table.csrRows + entry[i] + k), regionBase + at + k);
                    }
                }
                pos += __shfl_sync(0xffffffffu, inc, 31);
            }
        }
    }
}

// Hash of the probe row's key tuple; false when a key column is NULL (never matches).
__device__ __forceinline__ bool ProbeTupleHash(const ProbeLaunch &p, const BatchDesc &b, int64_t row, uint64_t &h)
{
    h = static_cast<uint64_t>(p.nKeyCols);
    for (int k = 0; k < p.nKeyCols; ++k) {
        const JoinKeyCol &kc = p.keyCols[k];
        if (RowIsNullRO(b.nulls[kc.input], row)) {
            return false;
        }
        if (kc.width == 0) {
            const int32_t *offs = b.offs[kc.input];
            h = KeyTupleBytes(h, static_cast<const uint8_t *>(b.cols[kc.input]) + offs[row], offs[row + 1] - offs[row]);
        } else if (kc.width == 16) {
            const longlong2 v = __ldg(static_cast<const longlong2 *>(b.cols[kc.input]) + row);
            h = KeyTupleStep(KeyTupleStep(h, static_cast<uint64_t>(v.x)), static_cast<uint64_t>(v.y));
        } else {
            h = KeyTupleStep(h, LoadBitsRO(b.cols[kc.input], row, kc.width));
        }
    }
    return true;
}

// The probe row's key tuple equals build row `br`'s, column by column.
__device__ __forceinline__ bool TupleEquals(const ProbeLaunch &p, const BatchDesc &b, int64_t row, int64_t br)
{
    for (int k = 0; k < p.nKeyCols; ++k) {
        const JoinKeyCol &kc = p.keyCols[k];
        if (kc.width == 0) {
            const int32_t *offs = b.offs[kc.input];
            const int64_t len = offs[row + 1] - offs[row];
            const int64_t b0 = kc.buildOffs[br];
            if (kc.buildOffs[br + 1] - b0 != len) {
                return false;
            }
            const uint8_t *x = static_cast<const uint8_t *>(b.cols[kc.input]) + offs[row];
            const uint8_t *y = static_cast<const uint8_t *>(kc.buildValues) + b0;
            for (int64_t i = 0; i < len; ++i) {
                if (x[i] != y[i]) {
                    return false;
                }
            }
        } else if (kc.width == 16) {
            const longlong2 x = __ldg(static_cast<const longlong2 *>(b.cols[kc.input]) + row);
            const longlong2 y = __ldg(static_cast<const longlong2 *>(kc.buildValues) + br);
            if (x.x != y.x || x.y != y.y) {
                return false;
            }
        } else if (LoadBitsRO(b.cols[kc.input], row, kc.width) != LoadBitsRO(kc.buildValues, br, kc.width)) {
            return false;
        }
    }
    return true;
}

// Probe for keys of several columns (or one 16-byte column), every join kind
// (lookup_join.cpp:924-1430): the table is keyed by the tuple hash and each candidate is
// compared column by column before it counts as a match.  Each warp takes 32
// consecutive probe rows at a time: lane i looks row i up and decides how many rows it emits
// (by kind), the warp prefix-sums those counts, reserves its output range with one atomicAdd and
// writes the rows in probe-row order.  BUILD_OUTER and FULL also mark every matched build row
// visited (a plain byte store: every writer stores the same value).
// One value of a filter operand: the raw bits (an int64, or a double's bits) and flags.
constexpr uint32_t kFNull = 1;
constexpr uint32_t kFDouble = 2;

__device__ __forceinline__ double FilterAsDouble(uint64_t v, uint32_t fl)
{
    return (fl & kFDouble) ? __longlong_as_double(static_cast<long long>(v))
                           : static_cast<double>(static_cast<int64_t>(v));
}

// A build column that is also a slot-payload field: its value from the candidate's slot payload
// (payload fields are NULL-free), sign-extended from its width.
__device__ __forceinline__ uint64_t PayloadField(const FilterInstr &f, uint64_t payload)
{
    const uint64_t v = payload >> (f.payloadShift - 1);
    if (f.dbl || f.width == 8) {
        return v;
    }
    return static_cast<uint64_t>(SignExtend(v, f.width));
}

// ---- strings in filters: a value is (pointer, byte length) ------------------------------------
constexpr uint32_t kFString = 4;

// Byte offset of the code point `count` places after byte `pos` of s[0, len), or -1 when the
// string ends first (utf8_util.h:22-60): a code point starts at every byte that is not a UTF-8
// continuation byte (10xxxxxx), so the answer is the (count + 1)-th such byte from `pos`.
__device__ int32_t Utf8Offset(const uint8_t *s, int32_t len, int32_t pos, int32_t count)
{
    if (len - pos <= count) {
        return -1;
    }
    if (count == 0) {
        return pos;
    }
    int32_t seen = 0;
    for (int32_t i = pos; i < len; ++i) {
        if ((s[i] & 0xC0) != 0x80 && ++seen == count + 1) {
            return i;
        }
    }
    return -1;
}

// Code points of s[0, len): its bytes less its continuation bytes (utf8_util.h:62-91).
__device__ int32_t Utf8Count(const uint8_t *s, int32_t len)
{
    int32_t cont = 0;
    for (int32_t i = 0; i < len; ++i) {
        cont += (s[i] & 0xC0) == 0x80 ? 1 : 0;
    }
    return len - cont;
}

// substr of s[0, len) as a byte range [*from, *from + *outLen) (stringfunctions.h:215-318,
// SubstrVarcharWithStart and SubstrVarchar, start and length in code points, counted from 1 or,
// when negative, from the end).  hasLength false: to the end of the string.  Where the
// reference's result is undefined (a negative start into malformed UTF-8) the result is empty.
__device__ void SubstrRange(const uint8_t *s, int32_t len, int64_t start, bool hasLength, int64_t length,
    int rules, int32_t *from, int32_t *outLen)
{
    *from = 0;
    *outLen = 0;
    if ((rules & kFilterSubstrZero) != 0 && start == 0) {
        start = 1;
    }
    if (start == 0 || (hasLength && length <= 0) || len == 0 || start > len) {
        return;
    }
    int32_t startIndex;
    int32_t endIndex = len;
    if (start > 0) {
        startIndex = Utf8Offset(s, len, 0, static_cast<int32_t>(start - 1));
        if (startIndex < 0) {
            return;
        }
        if (hasLength) {
            endIndex = Utf8Offset(s, len, startIndex, static_cast<int32_t>(length));
            endIndex = endIndex < 0 ? len : endIndex;
        }
    } else {
        const int64_t points = Utf8Count(s, len);
        int64_t startPoint = start + points;
        if (startPoint < 0) {
            if ((rules & kFilterSubstrNegative) == 0 || (hasLength && startPoint + length <= 0)) {
                return;
            }
            length += startPoint;
            startPoint = 0;
        }
        startIndex = Utf8Offset(s, len, 0, static_cast<int32_t>(startPoint));
        if (startIndex < 0) {
            return;
        }
        if (hasLength && startPoint + length < points) {
            endIndex = Utf8Offset(s, len, startIndex, static_cast<int32_t>(length));
            endIndex = endIndex < startIndex ? len : endIndex;
        }
    }
    *from = startIndex;
    *outLen = endIndex - startIndex;
}

// Byte-wise unsigned comparison, then by length: <0, 0 or >0 (stringfunctions.cpp StrCompare).
__device__ int StrCompare(const uint8_t *a, int32_t la, const uint8_t *b, int32_t lb)
{
    const int32_t n = la < lb ? la : lb;
    for (int32_t i = 0; i < n; ++i) {
        if (a[i] != b[i]) {
            return a[i] < b[i] ? -1 : 1;
        }
    }
    return la < lb ? -1 : (la > lb ? 1 : 0);
}

// Byte offset of the first occurrence of sub[0, ls) in s[0, l), or -1.
__device__ int32_t StrFind(const uint8_t *s, int32_t l, const uint8_t *sub, int32_t ls)
{
    for (int32_t pos = 0; pos + ls <= l; ++pos) {
        int32_t i = 0;
        while (i < ls && s[pos + i] == sub[i]) {
            ++i;
        }
        if (i == ls) {
            return pos;
        }
    }
    return -1;
}

// One FOP_STRFN over the stack entries from `a` on; leaves its result at `a`.
__device__ void StrFunction(const FilterInstr &f, uint64_t *v, uint32_t *fl, int32_t *sl, int a)
{
    const bool an = (fl[a] & kFNull) != 0;
    const auto *x = reinterpret_cast<const uint8_t *>(v[a]);
    const int32_t lx = sl[a];
    if (f.width == SFN_LENGTH) {
        v[a] = an ? 0ull : static_cast<uint64_t>(f.imm >= 0 ? f.imm : Utf8Count(x, lx));
        fl[a] = an ? kFNull : 0u;
        sl[a] = 0;
        return;
    }
    const bool bn = (fl[a + 1] & kFNull) != 0;
    const auto *y = reinterpret_cast<const uint8_t *>(v[a + 1]);
    const int32_t ly = sl[a + 1];
    if (f.width == SFN_GREATEST || f.width == SFN_LEAST) {
        // ExtremeStr (stringfunctions.cpp): a NULL side yields the other
        bool right = an;
        if (!an && !bn) {
            const int c = StrCompare(x, lx, y, ly);
            right = f.width == SFN_GREATEST ? c < 0 : c > 0;
        }
        if (right) {
            v[a] = v[a + 1];
            sl[a] = ly;
        }
        fl[a] = (an && bn) ? kFNull : kFString;
        return;
    }
    uint64_t r = 0;
    if (!an && !bn) {
        switch (f.width) {
            case SFN_INSTR: {
                const int32_t pos = ly > lx ? -1 : StrFind(x, lx, y, ly);
                r = pos < 0 ? 0ull : static_cast<uint64_t>(Utf8Count(x, pos) + 1);
                break;
            }
            case SFN_STARTS_WITH:
                r = ly <= lx && StrCompare(x, ly, y, ly) == 0 ? 1ull : 0ull;
                break;
            case SFN_ENDS_WITH:
                r = ly <= lx && StrCompare(x + lx - ly, ly, y, ly) == 0 ? 1ull : 0ull;
                break;
            default:  // SFN_CONTAINS
                r = ly <= lx && StrFind(x, lx, y, ly) >= 0 ? 1ull : 0ull;
                break;
        }
    }
    v[a] = r;
    sl[a] = 0;
    fl[a] = (an || bn) ? kFNull : 0u;
}

// The filter program over the candidate pair (probe row `row` of batch b, build row `br`);
// `payload` (when not null) is the candidate's slot payload.
__device__ bool FilterPasses(const ProbeLaunch &p, const BatchDesc &b, int64_t row, int64_t br,
    bool hasPayload = false, uint64_t payload = 0)
{
    uint64_t v[kMaxFilterDepth];
    uint32_t fl[kMaxFilterDepth];
    int32_t sl[kMaxFilterDepth];  // string values: byte length (v holds the address)
    int sp = 0;
    for (int i = 0; i < p.nFilter; ++i) {
        const FilterInstr &f = p.filter[i];
        const int op = f.op;
        if (op == FOP_PROBE_STR || op == FOP_BUILD_STR || op == FOP_STR_LITERAL) {
            if (sp >= kMaxFilterDepth) {
                return false;  // the host limits the depth; never taken
            }
            const uint8_t *ptr = static_cast<const uint8_t *>(f.values);
            int32_t len = f.input;
            bool isNull = f.isNull != 0;
            if (op == FOP_PROBE_STR) {
                isNull = RowIsNullRO(b.nulls[f.input], row);
                const int32_t *offs = b.offs[f.input];
                const int32_t o0 = isNull ? 0 : offs[row];
                ptr = static_cast<const uint8_t *>(b.cols[f.input]) + o0;
                len = isNull ? 0 : offs[row + 1] - o0;
            } else if (op == FOP_BUILD_STR) {
                isNull = RowIsNullRO(f.nulls, br);
                const int64_t o0 = isNull ? 0 : f.offs[br];
                ptr += o0;
                len = isNull ? 0 : static_cast<int32_t>(f.offs[br + 1] - o0);
            }
            v[sp] = reinterpret_cast<uint64_t>(ptr);
            sl[sp] = len;
            fl[sp] = (isNull ? kFNull : 0u) | kFString;
            ++sp;
            continue;
        }
        if (op == FOP_CAST) {
            if (sp < 1) {
                return false;
            }
            const int a = sp - 1;
            if ((fl[a] & kFNull) == 0) {
                const bool fromDouble = (fl[a] & kFDouble) != 0;
                if (f.dbl) {
                    v[a] = fromDouble ? v[a]
                                      : static_cast<uint64_t>(__double_as_longlong(
                                            static_cast<double>(static_cast<int64_t>(v[a]))));
                } else {
                    int64_t x;
                    if (fromDouble) {
                        // NaN gives 0 and out-of-range values saturate, stated explicitly rather than
                        // left to the conversion instruction
                        const double d = __longlong_as_double(static_cast<long long>(v[a]));
                        const double lim = f.width == 8 ? 9223372036854775808.0 : 2147483648.0;
                        const int64_t hi = f.width == 8 ? INT64_MAX : INT32_MAX;
                        const int64_t lo = f.width == 8 ? INT64_MIN : INT32_MIN;
                        x = d != d ? 0 : (d >= lim ? hi : (d <= -lim ? lo : static_cast<int64_t>(__double2ll_rz(d))));
                    } else {
                        x = static_cast<int64_t>(v[a]);
                    }
                    v[a] = static_cast<uint64_t>(f.width == 8 ? x : SignExtend(static_cast<uint64_t>(x), f.width));
                }
            }
            fl[a] = (fl[a] & kFNull) | (f.dbl ? kFDouble : 0u);
            continue;
        }
        if (op == FOP_STRFN) {
            const int nArgs = f.width == SFN_LENGTH ? 1 : 2;
            if (sp < nArgs) {
                return false;
            }
            StrFunction(f, v, fl, sl, sp - nArgs);
            sp -= nArgs - 1;
            continue;
        }
        if (op == FOP_SUBSTR) {
            const int nArgs = f.width;
            if (sp < nArgs) {
                return false;
            }
            const int base = sp - nArgs;
            bool isNull = false;
            for (int a = 0; a < nArgs; ++a) {
                isNull = isNull || (fl[base + a] & kFNull) != 0;
            }
            int32_t from = 0, len = 0;
            const uint8_t *str = reinterpret_cast<const uint8_t *>(v[base]);
            if (!isNull) {
                SubstrRange(str, sl[base], static_cast<int64_t>(v[base + 1]), nArgs == 3,
                    nArgs == 3 ? static_cast<int64_t>(v[base + 2]) : 0, f.input, &from, &len);
            }
            v[base] = reinterpret_cast<uint64_t>(str + from);
            sl[base] = len;
            fl[base] = (isNull ? kFNull : 0u) | kFString;
            sp = base + 1;
            continue;
        }
        if (op == FOP_IF || op == FOP_BETWEEN) {
            if (sp < 3) {
                return false;
            }
            const int c = sp - 3;
            if (op == FOP_IF) {
                const int pick = ((fl[c] & kFNull) == 0 && v[c] != 0) ? c + 1 : c + 2;
                v[c] = v[pick];
                sl[c] = sl[pick];
                fl[c] = fl[pick];
            } else {
                const uint32_t all = fl[c] | fl[c + 1] | fl[c + 2];
                bool in = false;
                if ((all & kFNull) == 0) {
                    if (fl[c] & kFString) {
                        const auto *x = reinterpret_cast<const uint8_t *>(v[c]);
                        in = StrCompare(reinterpret_cast<const uint8_t *>(v[c + 1]), sl[c + 1], x, sl[c]) <= 0 &&
                            StrCompare(x, sl[c], reinterpret_cast<const uint8_t *>(v[c + 2]), sl[c + 2]) <= 0;
                    } else if (all & kFDouble) {
                        const double x = FilterAsDouble(v[c], fl[c]);
                        in = !(FilterAsDouble(v[c + 1], fl[c + 1]) > x) && !(x > FilterAsDouble(v[c + 2], fl[c + 2]));
                    } else {
                        const int64_t x = static_cast<int64_t>(v[c]);
                        in = static_cast<int64_t>(v[c + 1]) <= x && x <= static_cast<int64_t>(v[c + 2]);
                    }
                }
                v[c] = in ? 1ull : 0ull;
                sl[c] = 0;
                fl[c] = (all & kFNull) ? kFNull : 0u;
            }
            sp = c + 1;
            continue;
        }
        if (op == FOP_COALESCE) {
            if (sp < 2) {
                return false;
            }
            if (fl[sp - 2] & kFNull) {
                v[sp - 2] = v[sp - 1];
                sl[sp - 2] = sl[sp - 1];
                fl[sp - 2] = fl[sp - 1];
            }
            --sp;
            continue;
        }
        if (op == FOP_IN_STEP) {
            if (sp < 3) {
                return false;
            }
            const int t = sp - 1;
            const int x = sp - 2;
            if (fl[t] & kFNull) {
                v[sp - 3] |= 2ull;
            } else if ((fl[x] & kFNull) == 0) {
                bool eq;
                if (fl[x] & kFString) {
                    eq = sl[x] == sl[t] &&
                        StrCompare(reinterpret_cast<const uint8_t *>(v[x]), sl[x],
                            reinterpret_cast<const uint8_t *>(v[t]), sl[t]) == 0;
                } else if ((fl[x] | fl[t]) & kFDouble) {
                    eq = FilterAsDouble(v[x], fl[x]) == FilterAsDouble(v[t], fl[t]);
                } else {
                    eq = v[x] == v[t];
                }
                v[sp - 3] |= eq ? 1ull : 0ull;
            }
            --sp;
            continue;
        }
        if (op == FOP_IN_END) {
            if (sp < 2) {
                return false;
            }
            const uint64_t acc = v[sp - 2];
            const bool isNull = (acc & 1ull) == 0 && ((acc & 2ull) != 0 || (fl[sp - 1] & kFNull) != 0);
            v[sp - 2] = (acc & 1ull) ? 1ull : 0ull;
            sl[sp - 2] = 0;
            fl[sp - 2] = isNull ? kFNull : 0u;
            --sp;
            continue;
        }
        if (op == FOP_PROBE_COL || op == FOP_BUILD_COL || op == FOP_LITERAL || op == FOP_IN_BEGIN) {
            if (sp >= kMaxFilterDepth) {
                return false;  // the host limits the depth; never taken
            }
            if (op == FOP_IN_BEGIN) {
                v[sp] = 0;
                sl[sp] = 0;
                fl[sp] = 0;
                ++sp;
                continue;
            }
            uint64_t bits = static_cast<uint64_t>(f.imm);
            bool isNull = f.isNull != 0;
            if (op == FOP_BUILD_COL && hasPayload && f.payloadShift > 0) {
                bits = PayloadField(f, payload);
                isNull = false;
            } else if (op != FOP_LITERAL) {
                const void *col = op == FOP_PROBE_COL ? b.cols[f.input] : f.values;
                const uint8_t *nulls = op == FOP_PROBE_COL ? b.nulls[f.input] : f.nulls;
                const int64_t r = op == FOP_PROBE_COL ? row : br;
                isNull = RowIsNullRO(nulls, r);
                bits = isNull ? 0ull
                              : (f.dbl ? static_cast<uint64_t>(LoadIntRO(col, r, 8))
                                       : static_cast<uint64_t>(LoadIntRO(col, r, f.width)));
            }
            v[sp] = bits;
            sl[sp] = 0;
            fl[sp] = (isNull ? kFNull : 0u) | (f.dbl ? kFDouble : 0u);
            ++sp;
            continue;
        }
        if (op == FOP_NOT || op == FOP_IS_NULL || op == FOP_IS_NOT_NULL) {
            if (sp < 1) {
                return false;
            }
            const bool n = (fl[sp - 1] & kFNull) != 0;
            if (op == FOP_NOT) {
                v[sp - 1] = n ? 0ull : (v[sp - 1] == 0 ? 1ull : 0ull);
                fl[sp - 1] = n ? kFNull : 0u;
            } else {
                v[sp - 1] = (n == (op == FOP_IS_NULL)) ? 1ull : 0ull;
                fl[sp - 1] = 0u;
            }
            continue;
        }
        if (sp < 2) {
            return false;
        }
        const uint64_t bv = v[sp - 1];
        const uint32_t bf = fl[sp - 1];
        const uint64_t av = v[sp - 2];
        const uint32_t af = fl[sp - 2];
        --sp;
        const bool an = (af & kFNull) != 0;
        const bool bn = (bf & kFNull) != 0;
        uint64_t res = 0;
        bool resNull = false;
        if (op >= FOP_ADD && op <= FOP_TRY_DIV) {
            resNull = an || bn;
            if (!resNull) {
                if (f.dbl) {
                    const double x = FilterAsDouble(av, af);
                    const double y = FilterAsDouble(bv, bf);
                    double r = 0.0;
                    switch (op) {
                        case FOP_ADD:
                        case FOP_TRY_ADD: r = x + y; break;
                        case FOP_SUB:
                        case FOP_TRY_SUB: r = x - y; break;
                        case FOP_MUL:
                        case FOP_TRY_MUL: r = x * y; break;
                        case FOP_MOD:
                            resNull = y == 0.0;
                            r = resNull ? 0.0 : fmod(x, y);
                            break;
                        default:  // FOP_DIV, FOP_TRY_DIV
                            resNull = y == 0.0;
                            r = resNull ? 0.0 : x / y;
                            break;
                    }
                    res = static_cast<uint64_t>(__double_as_longlong(r));
                } else {
                    const int64_t x = static_cast<int64_t>(av);
                    const int64_t y = static_cast<int64_t>(bv);
                    const uint64_t ux = av;
                    const uint64_t uy = bv;
                    int64_t r = 0;
                    bool ovf = false;  // beyond the result width (TRY_* only)
                    switch (op) {
                        case FOP_ADD:
                        case FOP_TRY_ADD:
                            r = static_cast<int64_t>(ux + uy);
                            ovf = f.width == 8 ? ((x >= 0) == (y >= 0) && (r >= 0) != (x >= 0))
                                               : r != static_cast<int32_t>(r);
                            break;
                        case FOP_SUB:
                        case FOP_TRY_SUB:
                            r = static_cast<int64_t>(ux - uy);
                            ovf = f.width == 8 ? ((x >= 0) != (y >= 0) && (r >= 0) != (x >= 0))
                                               : r != static_cast<int32_t>(r);
                            break;
                        case FOP_MUL:
                        case FOP_TRY_MUL:
                            r = static_cast<int64_t>(ux * uy);
                            if (f.width == 8) {
                                ovf = __mul64hi(x, y) != (r >> 63);
                            } else {
                                ovf = r != static_cast<int32_t>(r);
                            }
                            break;
                        case FOP_MOD:
                            resNull = y == 0;
                            r = resNull ? 0 : (y == -1 ? 0 : x % y);
                            break;
                        default:  // FOP_DIV, FOP_TRY_DIV; INT_MIN / -1 wraps
                            resNull = y == 0;
                            r = resNull ? 0 : (y == -1 ? static_cast<int64_t>(0ull - ux) : x / y);
                            break;
                    }
                    if (f.width == 4) {
                        r = static_cast<int32_t>(r);  // wrap at 32 bits
                    }
                    resNull = resNull || (ovf && op >= FOP_TRY_ADD && op != FOP_TRY_DIV);
                    res = static_cast<uint64_t>(r);
                }
            }
            v[sp - 1] = resNull ? 0ull : res;
            fl[sp - 1] = (resNull ? kFNull : 0u) | (f.dbl ? kFDouble : 0u);
            continue;
        }
        if (op == FOP_AND) {
            const bool aFalse = !an && av == 0;
            const bool bFalse = !bn && bv == 0;
            resNull = !(aFalse || bFalse) && (an || bn);
            res = (!aFalse && !bFalse && !resNull) ? 1ull : 0ull;
        } else if (op == FOP_OR) {
            const bool aTrue = !an && av != 0;
            const bool bTrue = !bn && bv != 0;
            resNull = !(aTrue || bTrue) && (an || bn);
            res = (aTrue || bTrue) ? 1ull : 0ull;
        } else if (an || bn) {
            resNull = true;
        } else {
            int c;
            if ((af & bf) & kFString) {
                const uint8_t *x = reinterpret_cast<const uint8_t *>(av);
                const uint8_t *y = reinterpret_cast<const uint8_t *>(bv);
                const int32_t lx = sl[sp - 1];
                const int32_t ly = sl[sp];
                c = (op == FOP_EQ || op == FOP_NEQ) && lx != ly ? 1 : StrCompare(x, lx, y, ly);
                c = c < 0 ? -1 : (c > 0 ? 1 : 0);
            } else if ((af | bf) & kFDouble) {
                const double x = FilterAsDouble(av, af);
                const double y = FilterAsDouble(bv, bf);
                c = x < y ? -1 : (x > y ? 1 : (x == y ? 0 : 2));  // 2: unordered (NaN)
            } else {
                const int64_t x = static_cast<int64_t>(av);
                const int64_t y = static_cast<int64_t>(bv);
                c = x < y ? -1 : (x > y ? 1 : 0);
            }
            bool t = false;
            switch (op) {
                case FOP_EQ: t = c == 0; break;
                case FOP_NEQ: t = c != 0; break;
                case FOP_LT: t = c == -1; break;
                case FOP_LTE: t = c == -1 || c == 0; break;
                case FOP_GT: t = c == 1; break;
                default: t = c == 1 || c == 0; break;  // FOP_GTE
            }
            res = t ? 1ull : 0ull;
        }
        v[sp - 1] = res;
        fl[sp - 1] = resNull ? kFNull : 0u;
    }
    return sp == 1 && (fl[0] & kFNull) == 0 && v[0] != 0;
}

// The filter programs of one comparison between two operands (columns of either side or
// literals): evaluated without the interpreter's stack, with its semantics (NULL fails, doubles
// compare unordered NaN as neither less, greater nor equal).
__device__ __forceinline__ bool SimpleFilterShape(const ProbeLaunch &p)
{
    auto operand = [](int op) { return op == FOP_PROBE_COL || op == FOP_BUILD_COL || op == FOP_LITERAL; };
    return p.nFilter == 3 && operand(p.filter[0].op) && operand(p.filter[1].op) && p.filter[2].op >= FOP_EQ &&
        p.filter[2].op <= FOP_GTE;
}

__device__ __forceinline__ bool FilterOperand(const FilterInstr &f, const BatchDesc &b, int64_t row, int64_t br,
    bool hasPayload, uint64_t payload, uint64_t &bits)
{
    if (f.op == FOP_LITERAL) {
        bits = static_cast<uint64_t>(f.imm);
        return f.isNull == 0;
    }
    if (f.op == FOP_BUILD_COL && hasPayload && f.payloadShift > 0) {
        bits = PayloadField(f, payload);
        return true;
    }
    const bool probe = f.op == FOP_PROBE_COL;
    const int64_t r = probe ? row : br;
    if (RowIsNullRO(probe ? b.nulls[f.input] : f.nulls, r)) {
        return false;
    }
    bits = static_cast<uint64_t>(LoadIntRO(probe ? b.cols[f.input] : f.values, r, f.dbl ? 8 : f.width));
    return true;
}

__device__ __forceinline__ bool SimpleFilterPasses(const ProbeLaunch &p, const BatchDesc &b, int64_t row, int64_t br,
    bool hasPayload, uint64_t payload)
{
    const FilterInstr &fa = p.filter[0];
    const FilterInstr &fb = p.filter[1];
    uint64_t av = 0, bv = 0;
    if (!FilterOperand(fa, b, row, br, hasPayload, payload, av) ||
        !FilterOperand(fb, b, row, br, hasPayload, payload, bv)) {
        return false;  // NULL: the comparison is NULL, which fails
    }
    int c;
    if (fa.dbl || fb.dbl) {
        const double x = FilterAsDouble(av, fa.dbl ? kFDouble : 0u);
        const double y = FilterAsDouble(bv, fb.dbl ? kFDouble : 0u);
        c = x < y ? -1 : (x > y ? 1 : (x == y ? 0 : 2));
    } else {
        const int64_t x = static_cast<int64_t>(av);
        const int64_t y = static_cast<int64_t>(bv);
        c = x < y ? -1 : (x > y ? 1 : 0);
    }
    switch (p.filter[2].op) {
        case FOP_EQ: return c == 0;
        case FOP_NEQ: return c != 0;
        case FOP_LT: return c == -1;
        case FOP_LTE: return c == -1 || c == 0;
        case FOP_GT: return c == 1;
        default: return c == 1 || c == 0;  // FOP_GTE
    }
}

// A candidate build row counts as a match: equal key tuple (multi-column keys) and passing the
// join filter (when there is one).
__device__ __forceinline__ bool Accept(const ProbeLaunch &p, const BatchDesc &b, int64_t row, int64_t br, bool multi)
{
    return (!multi || TupleEquals(p, b, row, br)) && (p.nFilter == 0 || FilterPasses(p, b, row, br));
}

__global__ void __launch_bounds__(kProbeThreads) ProbeKindKernel(const __grid_constant__ ProbeLaunch p)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    constexpr int kWarps = kProbeThreads / 32;
    const int kind = p.joinKind;
    const bool emitMatches = kind == JOIN_KIND_INNER || kind == JOIN_KIND_PROBE_OUTER ||
        kind == JOIN_KIND_BUILD_OUTER || kind == JOIN_KIND_FULL;
    const bool unique = p.table.unique != 0;
    const bool multi = p.nKeyCols > 0;
    const bool check = multi || p.nFilter > 0;  // candidates are tested one by one
    for (int t = blockIdx.x; t < p.nTiles; t += gridDim.x) {
        const TileDesc tile = p.tiles[t];
        const BatchDesc &b = p.batches[tile.batch];
        const void *keyCol = multi ? nullptr : b.cols[p.keyInput];
        const uint8_t *keyNulls = multi ? nullptr : b.nulls[p.keyInput];
        const int region = t % p.nRegions;
        const uint64_t regionBase = static_cast<uint64_t>(region) * p.regionCap;
        for (int r0 = warp * 32; r0 < tile.rows; r0 += kWarps * 32) {
            const int r = r0 + lane;
            const bool exists = r < tile.rows;
            const int64_t row = static_cast<int64_t>(tile.row0) + r;
            int64_t key = 0;
            Match m{0, 0, 0};
            uint32_t nMatch = 0;  // candidates whose key equals the probe key
            if (exists) {
                if (multi) {
                    uint64_t h;
                    if (ProbeTupleHash(p, b, row, h)) {
                        m = Lookup(p.table, h);
                    }
                } else {
                    key = LoadIntRO(keyCol, row, p.keyWidth);
                    if (!RowIsNullRO(keyNulls, row)) {
                        m = Lookup(p.table, static_cast<uint64_t>(key));
                    }
                }
                if (check) {
                    for (uint32_t k = 0; k < m.count; ++k) {
                        const int64_t br = unique ? m.entry : __ldg(p.table.csrRows + m.entry + k);
                        nMatch += Accept(p, b, row, br, multi) ? 1u : 0u;
                    }
                } else {
                    nMatch = m.count;
                }
            }
            const bool matched = nMatch != 0;
            uint32_t emit = 0;
            switch (kind) {
                case JOIN_KIND_PROBE_OUTER:
                case JOIN_KIND_FULL:
                    emit = exists ? (matched ? nMatch : 1u) : 0u;
                    break;
                case JOIN_KIND_SEMI:
                    emit = matched ? 1u : 0u;
                    break;
                case JOIN_KIND_ANTI:
                    emit = exists && !matched ? 1u : 0u;
                    break;
                case JOIN_KIND_EXISTENCE:
                    emit = exists ? 1u : 0u;
                    break;
                default:  // INNER, BUILD_OUTER
                    emit = nMatch;
            }
            if (p.visited != nullptr && matched) {
                for (uint32_t k = 0; k < m.count; ++k) {
                    const int64_t br = unique ? m.entry : __ldg(p.table.csrRows + m.entry + k);
                    if ((!check || Accept(p, b, row, br, multi)) && p.visited[br] == 0) {
                        p.visited[br] = 1;
                    }
                }
            }
            uint32_t inc = emit;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) {
                    inc += y;
                }
            }
            const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
            unsigned long long pos = 0;
            if (lane == 0 && total != 0) {
                pos = atomicAdd(p.outCount + region * kRegionStride, static_cast<unsigned long long>(total));
            }
            pos = __shfl_sync(0xffffffffu, pos, 0);
            if (p.countOnly || emit == 0) {
                continue;
            }
            const uint64_t at = pos + inc - emit;
            if (emitMatches && matched) {
                uint64_t j = at;
                for (uint32_t k = 0; k < m.count && j < p.regionCap; ++k) {
                    const int64_t br = unique ? m.entry : __ldg(p.table.csrRows + m.entry + k);
                    if (!check || Accept(p, b, row, br, multi)) {
                        WriteJoinRow(p, b, row, key, br, regionBase + j);
                        ++j;
                    }
                }
            } else if (at < p.regionCap) {
                WriteProbeOnlyRow(p, b, row, key, matched, regionBase + at);
            }
        }
    }
}

// Build side of a multi-column key: the tuple hash of every build row, NULL when a key column
// is NULL (such rows never enter the table).
__global__ void JoinKeyHashKernel(const JoinKeyCols kc, int64_t n, uint64_t *out, uint8_t *outNulls)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint64_t h = static_cast<uint64_t>(kc.nKeys);
        bool isNull = false;
        for (int k = 0; k < kc.nKeys; ++k) {
            if (RowIsNull(kc.nulls[k], i)) {
                isNull = true;
            } else if (kc.widths[k] == 0) {
                const int64_t o = kc.offs[k][i];
                h = KeyTupleBytes(h, static_cast<const uint8_t *>(kc.cols[k]) + o, kc.offs[k][i + 1] - o);
            } else if (kc.widths[k] == 16) {
                const uint64_t *v = static_cast<const uint64_t *>(kc.cols[k]) + 2 * i;
                h = KeyTupleStep(KeyTupleStep(h, v[0]), v[1]);
            } else {
                h = KeyTupleStep(h, LoadBits(kc.cols[k], i, kc.widths[k]));
            }
        }
        out[i] = isNull ? 0 : h;
        if (isNull) {
            SetBit(outNulls, static_cast<uint64_t>(i));
        }
    }
}

// ------------------------------------------------------------------ packed multi-column keys
// Part k of a packed multi-column key added to `acc` (JoinKeyPack); -1 once any part is outside
// the build's range.
__device__ __forceinline__ int64_t PackKeyPart(const JoinKeyPack &kp, int k, int64_t v, int64_t acc)
{
    const uint64_t d = static_cast<uint64_t>(v) - static_cast<uint64_t>(kp.minv[k]);
    if (acc < 0 || v < kp.minv[k] || d >= kp.span[k]) {
        return -1;
    }
    return acc + static_cast<int64_t>(d * kp.stride[k]);
}

// Build side: the packed key of every build row (contiguous key columns), NULL when a part is.
__global__ void PackBuildKeysKernel(const JoinKeyCols kc, const JoinKeyPack kp, int64_t n, int64_t *out,
    uint32_t *outNulls)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i0 = static_cast<int64_t>(blockIdx.x) * blockDim.x; i0 < n; i0 += stride) {
        const int64_t i = i0 + threadIdx.x;
        bool isNull = false;
        int64_t key = 0;
        if (i < n) {
            for (int k = 0; k < kp.nParts; ++k) {
                isNull = isNull || RowIsNullRO(kc.nulls[k], i);
                key = PackKeyPart(kp, k, LoadInt(kc.cols[k], i, kc.widths[k]), key);
            }
            out[i] = isNull ? 0 : key;
        }
        const unsigned int m = __ballot_sync(0xffffffffu, isNull);
        if (outNulls != nullptr && (threadIdx.x & 31) == 0 && i < n) {
            outNulls[i >> 5] = m;  // i is a multiple of 32 here
        }
    }
}

// Probe side: the packed key of every probe row into input kp.outInput of its batch (a scratch
// column), with its NULL bitmap when that input has one.  One CTA per tile.
__global__ void PackProbeKeysKernel(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles, const JoinKeyPack kp)
{
    for (int32_t t = blockIdx.x; t < nTiles; t += gridDim.x) {
        const TileDesc tile = tiles[t];
        const BatchDesc &b = batches[tile.batch];
        int64_t *out = static_cast<int64_t *>(const_cast<void *>(b.cols[kp.outInput]));
        uint32_t *outNulls = reinterpret_cast<uint32_t *>(const_cast<uint8_t *>(b.nulls[kp.outInput]));
        for (int r0 = 0; r0 < tile.rows; r0 += blockDim.x) {
            const int r = r0 + static_cast<int>(threadIdx.x);
            const int64_t row = static_cast<int64_t>(tile.row0) + r;
            bool isNull = false;
            int64_t key = 0;
            if (r < tile.rows) {
                for (int k = 0; k < kp.nParts; ++k) {
                    isNull = isNull || RowIsNullRO(b.nulls[kp.input[k]], row);
                    key = PackKeyPart(kp, k, LoadInt(b.cols[kp.input[k]], row, kp.width[k]), key);
                }
                out[row] = isNull ? 0 : key;
            }
            const unsigned int m = __ballot_sync(0xffffffffu, isNull);
            if (outNulls != nullptr && (threadIdx.x & 31) == 0 && r < tile.rows) {
                outNulls[row >> 5] = m;  // tiles and warps start on 32-row boundaries
            }
        }
    }
}

// Build rows no probe matched (lookup_outer_join.cpp:270-374): flags, then their row numbers in
// build-row order after a scan of the flags.
__global__ void UnvisitedFlagsKernel(const uint8_t *visited, int64_t n, uint32_t *flags)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        flags[i] = visited[i] == 0 ? 1u : 0u;
    }
}

__global__ void UnvisitedRowsKernel(const uint8_t *visited, const int64_t *offsets, int64_t n, int32_t *rows)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (visited[i] == 0) {
            rows[offsets[i]] = static_cast<int32_t>(i);
        }
    }
}

// dst[i] = src[rows[i]] with its NULL bit.
__global__ void GatherRowsKernel(const void *src, const uint8_t *srcNulls, const int32_t *rows, int64_t n, int32_t width,
    void *dst, uint8_t *dstNulls)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t r = rows[i];
        CopyValueRO(dst, static_cast<uint64_t>(i), src, r, width);
        if (dstNulls != nullptr && RowIsNullRO(srcNulls, r)) {
            SetBit(dstNulls, static_cast<uint64_t>(i));
        }
    }
}

// Specialised probe for the common shape: 8-byte key, unique build with a slot payload, and up
// to kFastMaxOut output columns that are each either the probe key or a field of the payload.
// Column metadata lives in registers and no width is dispatched at run time per row.
constexpr int kFastMaxOut = 4;

template <int kNumOut>
__global__ void __launch_bounds__(kProbeThreads, 3) ProbeFastKernel(const __grid_constant__ ProbeLaunch p)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const unsigned int lanesBelow = (1u << lane) - 1u;
    const bool arrayMode = p.table.mode == JOIN_ARRAY;
    const unsigned long long *payloadTab = reinterpret_cast<const unsigned long long *>(p.table.slotPayload);
    void *vals[kNumOut];
    int width[kNumOut];
    int shift[kNumOut];
    bool isKey[kNumOut];
#pragma unroll
    for (int o = 0; o < kNumOut; ++o) {
        vals[o] = p.out[o].values;
        width[o] = p.out[o].width;
        shift[o] = p.out[o].shift;
        isKey[o] = p.out[o].side == 0;
    }
    for (int t = blockIdx.x; t < p.nTiles; t += gridDim.x) {
        const TileDesc tile = p.tiles[t];
        const int w0 = warp * kRowsPerWarp;
        if (w0 >= tile.rows) {
            continue;
        }
        const BatchDesc &b = p.batches[tile.batch];
        const long long *keyCol = static_cast<const long long *>(b.cols[p.keyInput]);
        const uint8_t *keyNulls = b.nulls[p.keyInput];
        const int64_t base = static_cast<int64_t>(tile.row0) + w0;
        const int nRows = min(kRowsPerWarp, tile.rows - w0);
        int64_t key[kWarpRounds];
        uint32_t live = 0;
#pragma unroll
        for (int i = 0; i < kWarpRounds; ++i) {
            const int r = i * 32 + lane;
            key[i] = 0;
            if (r < nRows) {
                key[i] = __ldg(keyCol + base + r);
                if (!RowIsNullRO(keyNulls, base + r)) {
                    live |= 1u << i;
                }
            }
        }
        uint64_t payload[kWarpRounds];
        uint32_t hit = 0;
        if (arrayMode) {
#pragma unroll
            for (int i = 0; i < kWarpRounds; ++i) {
                const uint64_t d = static_cast<uint64_t>(key[i]) - static_cast<uint64_t>(p.table.minKey);
                payload[i] = 0;
                if (((live >> i) & 1u) && key[i] >= p.table.minKey && d < p.table.range) {
                    const long long e = __ldg(reinterpret_cast<const long long *>(p.table.arrayEntries) + d);
                    payload[i] = __ldg(payloadTab + d);
                    hit |= (e >= 0 ? 1u : 0u) << i;
                }
            }
        } else {
#pragma unroll
            for (int i = 0; i < kWarpRounds; ++i) {
                payload[i] = 0;
                if ((live >> i) & 1u) {
                    const Match m = Lookup(p.table, static_cast<uint64_t>(key[i]));
                    if (m.count != 0) {
                        payload[i] = __ldg(payloadTab + m.slot);
                        hit |= 1u << i;
                    }
                }
            }
        }
        uint32_t total = 0;
#pragma unroll
        for (int i = 0; i < kWarpRounds; ++i) {
            total += __popc(__ballot_sync(0xffffffffu, (hit >> i) & 1u));
        }
        const int region = t % p.nRegions;
        unsigned long long pos = 0;
        if (lane == 0 && total != 0) {
            pos = atomicAdd(p.outCount + region * kRegionStride, static_cast<unsigned long long>(total));
        }
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (p.countOnly || total == 0) {
            continue;
        }
        const uint64_t regionBase = static_cast<uint64_t>(region) * p.regionCap;
#pragma unroll
        for (int i = 0; i < kWarpRounds; ++i) {
            const unsigned int m = __ballot_sync(0xffffffffu, (hit >> i) & 1u);
            if ((hit >> i) & 1u) {
                const uint64_t rat = pos + __popc(m & lanesBelow);
                if (rat < p.regionCap) {
                    const uint64_t at = regionBase + rat;
                    // Re-read the key (an L1 hit) rather than keeping 16 keys live in registers.
                    const int64_t kv = __ldg(keyCol + base + i * 32 + lane);
#pragma unroll
                    for (int o = 0; o < kNumOut; ++o) {
                        const int64_t v = isKey[o] ? kv : static_cast<int64_t>(payload[i] >> shift[o]);
                        if (width[o] == 8) {
                            static_cast<int64_t *>(vals[o])[at] = v;
                        } else if (width[o] == 4) {
                            static_cast<int32_t *>(vals[o])[at] = static_cast<int32_t>(v);
                        } else if (width[o] == 2) {
                            static_cast<int16_t *>(vals[o])[at] = static_cast<int16_t>(v);
                        } else {
                            static_cast<int8_t *>(vals[o])[at] = static_cast<int8_t>(v);
                        }
                    }
                }
            }
            pos += __popc(m);
        }
    }
}

// ARRAY-table probe with the slot-occupancy bitmap staged in shared memory.  The hit test is a
// shared-memory load, so only matched rows send a request (the payload fetch) through L1 to L2;
// with the bitmap in L1 or a table entry per row, the random requests of the lookups bound the
// kernel.  Warps take 128-row segments (4 rounds of 32 rows), 32 warps per CTA, one CTA per SM
// (the bitmap is up to kBitsMaxSmem bytes).  Outputs as in ProbeFastKernel.
constexpr int kBitsThreads = 1024;
constexpr int kBitsRounds = 4;
constexpr int kBitsSegRows = kBitsRounds * 32;
constexpr int kBitsSegsPerTile = kTileRows / kBitsSegRows;
constexpr uint32_t kBitsMaxSmem = 200u * 1024u;
constexpr int32_t kBitsMinTiles = 64;  // 256K probe rows

// Output layouts known at compile time: 3 bits per output column (1, 2, 3, 4 = 1, 2, 4, 8
// bytes; 0 = read the width at run time).
constexpr uint32_t OutLayout(int w0, int w1 = 0, int w2 = 0, int w3 = 0)
{
    return static_cast<uint32_t>(w0) | (static_cast<uint32_t>(w1) << 3) | (static_cast<uint32_t>(w2) << 6) |
        (static_cast<uint32_t>(w3) << 9);
}
constexpr int kW1 = 1, kW2 = 2, kW4 = 3, kW8 = 4;

template <uint32_t kLayout, int kO>
__device__ __forceinline__ void StoreOut(void *col, uint64_t at, int width, int64_t v)
{
    constexpr int code = static_cast<int>((kLayout >> (3 * kO)) & 7u);
    const int w = code == 0 ? width : (1 << (code - 1));
    if (w == 8) {
        static_cast<int64_t *>(col)[at] = v;
    } else if (w == 4) {
        static_cast<int32_t *>(col)[at] = static_cast<int32_t>(v);
    } else if (w == 2) {
        static_cast<int16_t *>(col)[at] = static_cast<int16_t>(v);
    } else {
        static_cast<int8_t *>(col)[at] = static_cast<int8_t>(v);
    }
}

// Keys and validity of one warp segment of kBitsSegRows rows starting at `base` (a multiple of
// 32).  The common segment (all rows inside the batch, bitmap absent or 4-byte aligned) runs
// branch-free so that all its loads issue back to back: the validity of 32 rows is one 32-bit
// word.  Other segments check every row and read validity bytes.
__device__ __forceinline__ uint32_t LoadKeySegment(const long long *keyCol, const uint8_t *keyNulls, int64_t base,
    int64_t batchRows, int lane, int64_t (&key)[kBitsRounds])
{
    uint32_t live = 0;
    if (base + kBitsSegRows <= batchRows && (reinterpret_cast<uintptr_t>(keyNulls) & 3u) == 0) {
        if (keyNulls == nullptr) {
#pragma unroll
            for (int i = 0; i < kBitsRounds; ++i) {
                key[i] = __ldg(keyCol + base + i * 32 + lane);
            }
            return (1u << kBitsRounds) - 1u;
        }
        uint32_t w[kBitsRounds];
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            key[i] = __ldg(keyCol + base + i * 32 + lane);
            w[i] = __ldg(reinterpret_cast<const unsigned int *>(keyNulls) + ((base >> 5) + i));
        }
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            live |= (((w[i] >> lane) & 1u) ^ 1u) << i;
        }
        return live;
    }
#pragma unroll
    for (int i = 0; i < kBitsRounds; ++i) {
        const int64_t row = base + i * 32 + lane;
        key[i] = 0;
        if (row < batchRows) {
            key[i] = __ldg(keyCol + row);
            if (!RowIsNullRO(keyNulls, row)) {
                live |= 1u << i;
            }
        }
    }
    return live;
}

// The kernels that pack multi-column keys as they read them take keys of at most this many parts
// (longer keys are packed by a separate pass).
constexpr int kFusedPackParts = 2;

// Part columns of a packed key in one batch.
struct PackCols {
    const void *col[kFusedPackParts];
    const uint8_t *nulls[kFusedPackParts];
};

__device__ __forceinline__ PackCols PackColsOf(const JoinKeyPack &kp, const BatchDesc &b)
{
    PackCols pc;
#pragma unroll
    for (int k = 0; k < kFusedPackParts; ++k) {
        const int in = kp.input[k < kp.nParts ? k : 0];
        pc.col[k] = b.cols[in];
        pc.nulls[k] = b.nulls[in];
    }
    return pc;
}

// Keys of one warp segment packed from (up to kFusedPackParts) key parts, the part values kept in
// v[k][i] and each part's NULL rows in nullBits[k] (bit i: round i).  Whole segments with
// word-aligned NULL bitmaps read a 32-bit validity word per round and part.
// kTwo32: two parts of 4 bytes each (the widths are not read).
template <bool kTwo32, typename PartT>
__device__ __forceinline__ uint32_t LoadPackedSegment(const JoinKeyPack &kp, const PackCols &pc, int64_t base,
    int64_t batchRows, int lane, int64_t (&key)[kBitsRounds], PartT (&v)[kFusedPackParts][kBitsRounds],
    uint32_t (&nullBits)[kFusedPackParts])
{
    const bool whole = base + kBitsSegRows <= batchRows &&
        ((reinterpret_cast<uintptr_t>(pc.nulls[0]) | reinterpret_cast<uintptr_t>(pc.nulls[1])) & 3u) == 0;
    if (kTwo32 && whole) {
        // Two int32 parts: 32-bit offsets into ranges of at most 2^32 values, one wide multiply.
        const int32_t *c0 = static_cast<const int32_t *>(pc.col[0]);
        const int32_t *c1 = static_cast<const int32_t *>(pc.col[1]);
        const unsigned int *n0 = reinterpret_cast<const unsigned int *>(pc.nulls[0]);
        const unsigned int *n1 = reinterpret_cast<const unsigned int *>(pc.nulls[1]);
        uint32_t w0[kBitsRounds];
        uint32_t w1[kBitsRounds];
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            v[0][i] = static_cast<PartT>(__ldg(c0 + base + i * 32 + lane));
            v[1][i] = static_cast<PartT>(__ldg(c1 + base + i * 32 + lane));
            w0[i] = n0 == nullptr ? 0u : __ldg(n0 + (base >> 5) + i);
            w1[i] = n1 == nullptr ? 0u : __ldg(n1 + (base >> 5) + i);
        }
        const uint32_t min0 = static_cast<uint32_t>(kp.minv[0]);
        const uint32_t min1 = static_cast<uint32_t>(kp.minv[1]);
        const uint64_t span0 = kp.span[0];
        const uint64_t span1 = kp.span[1];
        uint32_t live = 0;
        nullBits[0] = 0;
        nullBits[1] = 0;
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            const uint32_t d0 = static_cast<uint32_t>(v[0][i]) - min0;
            const uint32_t d1 = static_cast<uint32_t>(v[1][i]) - min1;
            const bool in = d0 < span0 && d1 < span1;
            key[i] = in ? static_cast<int64_t>(static_cast<uint64_t>(d0) * span1 + d1) : -1;
            const uint32_t b0 = (w0[i] >> lane) & 1u;
            const uint32_t b1 = (w1[i] >> lane) & 1u;
            nullBits[0] |= b0 << i;
            nullBits[1] |= b1 << i;
            live |= ((b0 | b1) ^ 1u) << i;
        }
        return live;
    }
#pragma unroll
    for (int k = 0; k < kFusedPackParts; ++k) {
        nullBits[k] = 0;
        const bool part = kTwo32 || k < kp.nParts;
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            const int64_t row = base + i * 32 + lane;
            v[k][i] = 0;
            if (part && row < batchRows) {
                v[k][i] = kTwo32 ? static_cast<PartT>(__ldg(static_cast<const int32_t *>(pc.col[k]) + row))
                                 : static_cast<PartT>(LoadInt(pc.col[k], row, kp.width[k]));
                bool isNull;
                if (whole) {
                    const uint32_t w = pc.nulls[k] == nullptr
                        ? 0u
                        : __ldg(reinterpret_cast<const unsigned int *>(pc.nulls[k]) + ((base >> 5) + i));
                    isNull = (w >> lane) & 1u;
                } else {
                    isNull = RowIsNullRO(pc.nulls[k], row);
                }
                nullBits[k] |= (isNull ? 1u : 0u) << i;
            }
        }
    }
    uint32_t live = 0;
#pragma unroll
    for (int i = 0; i < kBitsRounds; ++i) {
        const int64_t row = base + i * 32 + lane;
        int64_t acc = 0;
#pragma unroll
        for (int k = 0; k < kFusedPackParts; ++k) {
            if (kTwo32 || k < kp.nParts) {
                acc = PackKeyPart(kp, k, static_cast<int64_t>(v[k][i]), acc);
            }
        }
        key[i] = acc;
        const bool isNull = (((nullBits[0] | nullBits[1]) >> i) & 1u) != 0;
        live |= (row < batchRows && !isNull ? 1u : 0u) << i;
    }
    return live;
}

// kProbeCols: some output is a probe column other than the key (its values, and its NULLs when
// the output column has a bitmap, are read from the probe batch for each emitted row).
// kPacked: the key is packed from the parts of a multi-column key (p.pack) as the rows are read.
// kPack: 0 one key column, 1 a packed key of up to kFusedPackParts parts of run-time widths,
// 2 a packed key of two 4-byte parts.
// kFilter: each candidate pair (probe row, its one build row) must also pass the join filter;
// 1 = any filter program (the interpreter), 2 = one comparison of two operands (no stack).
template <int kPack, int kFilter>
struct BitsThreads {
    // Packed keys and the interpreter: more registers per thread.
    static constexpr int value = kPack != 0 || kFilter == 1 ? 768 : kBitsThreads;
};

template <int kNumOut, uint32_t kLayout, bool kSingle, bool kProbeCols, int kPack, int kFilter = 0>
__global__ void __launch_bounds__(BitsThreads<kPack, kFilter>::value, 1)
    ProbeBitsKernel(const __grid_constant__ ProbeLaunch p)
{
    constexpr int kThreads = BitsThreads<kPack, kFilter>::value;
    constexpr bool kPacked = kPack != 0;
    using PartT = typename std::conditional<kPack == 2, int32_t, int64_t>::type;
    extern __shared__ uint4 sBitsVec[];
    const uint32_t *sBits = reinterpret_cast<const uint32_t *>(sBitsVec);
    {
        // The bitmap buffer holds a whole number of 16-byte vectors (see LaunchBuildSlotBits).
        const uint32_t nVec = static_cast<uint32_t>((p.table.range + 127) / 128);
        const uint4 *g = reinterpret_cast<const uint4 *>(p.table.slotBits);
        for (uint32_t i = threadIdx.x; i < nVec; i += kThreads) {
            sBitsVec[i] = __ldg(g + i);
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const unsigned int lanesBelow = (1u << lane) - 1u;
    const unsigned long long *payloadTab = reinterpret_cast<const unsigned long long *>(p.table.slotPayload);
    const uint64_t minKey = static_cast<uint64_t>(p.table.minKey);
    const uint64_t range = p.table.range;
    void *vals[kNumOut];
    int width[kNumOut];
    int shift[kNumOut];
    bool isKey[kNumOut];
    bool isFlag[kNumOut];
    bool isProbe[kNumOut];
#pragma unroll
    for (int o = 0; o < kNumOut; ++o) {
        vals[o] = p.out[o].values;
        width[o] = p.out[o].width;
        shift[o] = p.out[o].shift;
        isKey[o] = p.out[o].side == 0 && (!kProbeCols || p.out[o].src == p.keyInput);
        isFlag[o] = p.out[o].side == 2;
        isProbe[o] = kProbeCols && p.out[o].side == 0 && p.out[o].src != p.keyInput;
    }
    // Which rows are emitted follows EmitCount; unmatched rows get NULL build fields, emitted rows
    // of a NULL probe key a NULL key; BUILD_OUTER and FULL also mark matched build rows visited.
    const int kind = p.joinKind;
    const bool inner = kind == JOIN_KIND_INNER;
    // kSingle: the segments of the one batch are indexed directly (no descriptor loads per segment).
    const long long *singleKeys = nullptr;
    const uint8_t *singleNulls = nullptr;
    int64_t singleRows = 0;
    if (kSingle) {
        singleKeys = static_cast<const long long *>(p.batches[0].cols[p.keyInput]);
        singleNulls = p.batches[0].nulls[p.keyInput];
        singleRows = p.batches[0].rows;
    }
    const int64_t nItems = kSingle ? (singleRows + kBitsSegRows - 1) / kBitsSegRows
                                   : static_cast<int64_t>(p.nTiles) * kBitsSegsPerTile;
    // Packed keys: which output reads which key part (-1: none) and the part columns.
    int partOf[kNumOut];
#pragma unroll
    for (int o = 0; o < kNumOut; ++o) {
        partOf[o] = -1;
        for (int k = 0; kPacked && k < p.pack.nParts; ++k) {
            if (isProbe[o] && p.out[o].src == p.pack.input[k]) {
                partOf[o] = k;
            }
        }
    }
    PackCols packCols{};
    if (kPacked && kSingle) {
        packCols = PackColsOf(p.pack, p.batches[0]);
    }
    // Filters: whether every build operand comes from the slot payload (then the build row is
    // needed only to mark it visited).
    bool simpleFilter = false;
    bool filterNeedsRow = false;
    if (kFilter != 0) {
        simpleFilter = kFilter == 2 || SimpleFilterShape(p);
        filterNeedsRow = p.visited != nullptr;
        for (int f = 0; f < p.nFilter; ++f) {
            filterNeedsRow = filterNeedsRow || p.filter[f].op == FOP_BUILD_STR ||
                (p.filter[f].op == FOP_BUILD_COL && (payloadTab == nullptr || p.filter[f].payloadShift == 0));
        }
    }
    // One comparison of an integer slot-payload field with a non-NULL integer literal or an integer
    // probe column, in either order, decoded once here: per candidate the field is shifted out,
    // sign-extended and compared without branching on the program (plMask bit 0: passes when the
    // field is less, 1: equal, 2: greater; a NULL probe value fails).
    bool plCmp = false;
    int plShift = 0;
    int plWidth = 8;
    int64_t plLit = 0;
    int plInput = -1;  // >= 0: the other operand is this probe input
    int plInWidth = 8;
    uint32_t plMask = 0;
    if (kFilter == 2 && payloadTab != nullptr && p.nFilter == 3) {
        auto isField = [](const FilterInstr &f) { return f.op == FOP_BUILD_COL && f.payloadShift > 0 && f.dbl == 0; };
        auto isOther = [](const FilterInstr &f) {
            return (f.op == FOP_LITERAL && f.dbl == 0 && f.isNull == 0) || (f.op == FOP_PROBE_COL && f.dbl == 0);
        };
        const bool fieldFirst = isField(p.filter[0]) && isOther(p.filter[1]);
        const bool fieldSecond = !fieldFirst && isOther(p.filter[0]) && isField(p.filter[1]);
        plCmp = fieldFirst || fieldSecond;
        const FilterInstr &fld = fieldFirst ? p.filter[0] : p.filter[1];
        const FilterInstr &oth = fieldFirst ? p.filter[1] : p.filter[0];
        plShift = fld.payloadShift - 1;
        plWidth = fld.width;
        plLit = oth.imm;
        plInput = oth.op == FOP_PROBE_COL ? oth.input : -1;
        plInWidth = oth.width;
        switch (p.filter[2].op) {
            case FOP_EQ: plMask = 2u; break;
            case FOP_NEQ: plMask = 5u; break;
            case FOP_LT: plMask = 1u; break;
            case FOP_LTE: plMask = 3u; break;
            case FOP_GT: plMask = 4u; break;
            default: plMask = 6u; break;  // FOP_GTE
        }
        if (fieldSecond) {  // other OP field: swap the less and greater outcomes
            plMask = (plMask & 2u) | ((plMask & 1u) << 2) | ((plMask >> 2) & 1u);
        }
    }
    const int64_t warpsTotal = static_cast<int64_t>(gridDim.x) * (kThreads / 32);
    for (int64_t item = static_cast<int64_t>(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5); item < nItems;
         item += warpsTotal) {
        const int t = static_cast<int>(item / kBitsSegsPerTile);
        const long long *keyCol;
        const uint8_t *keyNulls;
        int64_t base;
        int64_t batchRows;
        if (kSingle) {
            keyCol = singleKeys;
            keyNulls = singleNulls;
            base = item * kBitsSegRows;
            batchRows = singleRows;
        } else {
            const int s0 = static_cast<int>(item % kBitsSegsPerTile) * kBitsSegRows;
            const TileDesc tile = p.tiles[t];
            if (s0 >= tile.rows) {
                continue;
            }
            const BatchDesc &b = p.batches[tile.batch];
            keyCol = static_cast<const long long *>(b.cols[p.keyInput]);
            keyNulls = b.nulls[p.keyInput];
            base = static_cast<int64_t>(tile.row0) + s0;
            batchRows = static_cast<int64_t>(tile.row0) + tile.rows;  // rows of the batch up to this tile's end
        }
        const BatchDesc *segBatch = nullptr;
        if (kProbeCols || kPacked || kFilter != 0) {
            segBatch = kSingle ? p.batches : p.batches + p.tiles[t].batch;
        }
        int64_t key[kBitsRounds];
        PartT partVal[kFusedPackParts][kBitsRounds];
        uint32_t partNull[kFusedPackParts];
        uint32_t live;
        if (kPacked) {
            if (!kSingle) {
                packCols = PackColsOf(p.pack, *segBatch);
            }
            live = LoadPackedSegment<kPack == 2>(p.pack, packCols, base, batchRows, lane, key, partVal, partNull);
        } else {
            live = LoadKeySegment(keyCol, keyNulls, base, batchRows, lane, key);
        }
        uint32_t hit = 0;
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            const uint64_t d = static_cast<uint64_t>(key[i]) - minKey;
            if (((live >> i) & 1u) && key[i] >= p.table.minKey && d < range) {
                hit |= ((sBits[d >> 5] >> (d & 31)) & 1u) << i;
            }
        }
        if (p.visited != nullptr) {
            // BUILD_OUTER / FULL: the slot's entry is the one build row of the key.
#pragma unroll
            for (int i = 0; i < kBitsRounds; ++i) {
                if (kFilter == 0 && ((hit >> i) & 1u)) {
                    p.visited[p.table.arrayEntries[static_cast<uint64_t>(key[i]) - minKey]] = 1;
                }
            }
        }
        uint64_t payload[kBitsRounds];
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            payload[i] = ((hit >> i) & 1u) && payloadTab != nullptr
                ? __ldg(payloadTab + (static_cast<uint64_t>(key[i]) - minKey))
                : 0ull;
        }
        if (kFilter != 0) {
            // A unique ARRAY table: the slot's entry is the one build row of the key; build columns
            // that are slot-payload fields are read from the payload instead.
#pragma unroll
            for (int i = 0; i < kBitsRounds; ++i) {
                if ((hit >> i) & 1u) {
                    const int64_t br = filterNeedsRow ? p.table.arrayEntries[static_cast<uint64_t>(key[i]) - minKey] : -1;
                    const int64_t row = base + i * 32 + lane;
                    const bool hasPayload = payloadTab != nullptr;
                    bool pass;
                    if (plCmp) {
                        const uint64_t bits = payload[i] >> plShift;
                        const int64_t x = plWidth == 8 ? static_cast<int64_t>(bits) : SignExtend(bits, plWidth);
                        int64_t y = plLit;
                        bool known = true;
                        if (plInput >= 0) {
                            known = !RowIsNullRO(segBatch->nulls[plInput], row);
                            y = known ? LoadIntRO(segBatch->cols[plInput], row, plInWidth) : 0;
                        }
                        const uint32_t c = (x < y ? 1u : 0u) | (x == y ? 2u : 0u) | (x > y ? 4u : 0u);
                        pass = known && (c & plMask) != 0;
                    } else {
                        pass = (kFilter == 2 || simpleFilter)
                            ? SimpleFilterPasses(p, *segBatch, row, br, hasPayload, payload[i])
                            : (kFilter == 1 && FilterPasses(p, *segBatch, row, br, hasPayload, payload[i]));
                    }
                    if (!pass) {
                        hit &= ~(1u << i);
                    } else if (p.visited != nullptr) {
                        p.visited[br] = 1;
                    }
                }
            }
        }
        uint32_t emit = hit;  // bit i: this lane's row of round i yields an output row
        if (!inner) {
            emit = 0;
#pragma unroll
            for (int i = 0; i < kBitsRounds; ++i) {
                const bool exists = base + i * 32 + lane < batchRows;
                emit |= (EmitCount(kind, exists, (hit >> i) & 1u) != 0 ? 1u : 0u) << i;
            }
        }
        uint32_t total = 0;
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            total += __popc(__ballot_sync(0xffffffffu, (emit >> i) & 1u));
        }
        const int region = t % p.nRegions;
        unsigned long long pos = 0;
        if (lane == 0 && total != 0) {
            pos = atomicAdd(p.outCount + region * kRegionStride, static_cast<unsigned long long>(total));
        }
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (p.countOnly || total == 0) {
            continue;
        }
        const uint64_t regionBase = static_cast<uint64_t>(region) * p.regionCap;
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            const unsigned int m = __ballot_sync(0xffffffffu, (emit >> i) & 1u);
            if ((emit >> i) & 1u) {
                const uint64_t rat = pos + __popc(m & lanesBelow);
                if (rat < p.regionCap) {
                    const uint64_t at = regionBase + rat;
                    const bool h = (hit >> i) & 1u;
                    // Unmatched rows of a probe-side outer join carry zero build fields (NULL below).
                    const int64_t flag = h ? 1 : 0;
                    const int64_t row = base + i * 32 + lane;
                    int64_t v[kNumOut];
#pragma unroll
                    for (int o = 0; o < kNumOut; ++o) {
                        v[o] = isKey[o] ? key[i] : (isFlag[o] ? flag : static_cast<int64_t>(payload[i] >> shift[o]));
                        if (kProbeCols && isProbe[o]) {
                            bool srcNull;
                            if (kPacked && partOf[o] >= 0) {
                                const int k = partOf[o];
                                v[o] = static_cast<int64_t>(k == 0 ? partVal[0][i] : partVal[kFusedPackParts - 1][i]);
                                srcNull = (((k == 0 ? partNull[0] : partNull[kFusedPackParts - 1]) >> i) & 1u) != 0;
                            } else {
                                v[o] = LoadInt(segBatch->cols[p.out[o].src], row, width[o]);
                                srcNull = RowIsNullRO(segBatch->nulls[p.out[o].src], row);
                            }
                            if (p.out[o].nulls != nullptr && srcNull) {
                                SetBit(p.out[o].nulls, at);
                            }
                        }
                    }
                    StoreOut<kLayout, 0>(vals[0], at, width[0], v[0]);
                    if (kNumOut > 1) {
                        StoreOut<kLayout, 1>(vals[1], at, width[1], v[1]);
                    }
                    if (kNumOut > 2) {
                        StoreOut<kLayout, 2>(vals[2], at, width[2], v[2]);
                    }
                    if (kNumOut > 3) {
                        StoreOut<kLayout, 3>(vals[3], at, width[3], v[3]);
                    }
                    if (!inner) {
                        const bool nullKey = !((live >> i) & 1u);
#pragma unroll
                        for (int o = 0; o < kNumOut; ++o) {
                            if ((isKey[o] && nullKey) || (!isKey[o] && !isFlag[o] && !isProbe[o] && !h)) {
                                SetBit(p.out[o].nulls, at);
                            }
                        }
                    }
                }
            }
            pos += __popc(m);
        }
    }
}

// ------------------------------------------------------------------ staged inner probe
// Inner joins on an ARRAY table with its occupancy bitmap in shared memory and a packed slot
// payload, outputs being the 8-byte probe key and payload fields.  The CTA's warps form groups
// of kGroupWarps; a group probes a group tile of kGroupRows rows at a time: its warps resolve
// their 128-row segments as ProbeBitsKernel does, the group prefix-sums the warps' match counts,
// reserves the group tile's output range with one atomic, stages the compacted (key, payload)
// rows in shared memory and writes every output column of the group tile as one contiguous run
// with 16-byte stores.  Each output column of a group tile is then written as whole lines (no
// per-warp partial lines, a quarter of the store instructions), which matters most when the
// output is pinned host memory written over the CPU-GPU link.  Groups synchronise on their own
// named barriers, so one group's stores overlap the other groups' loads.
constexpr int kGroupWarps = 8;
constexpr int kGroupThreads = kGroupWarps * 32;
constexpr int kGroupsPerCta = kBitsThreads / kGroupThreads;
constexpr int kGroupRows = kGroupWarps * kBitsSegRows;
constexpr int kGroupTilesPerTile = kTileRows / kGroupRows;
constexpr uint32_t kGroupStageBytes = static_cast<uint32_t>(kGroupRows) * 16u + 64u;
constexpr uint32_t kGroupMaxSmem = 227u * 1024u;
std::atomic<bool> g_stagedProbe{true};
std::atomic<int> g_bulkProbe{0};  // bulk-copy probe: 0 off, 1 bulk key loads, 2 and bulk output stores
std::atomic<int> g_lastProbeKernel{0};  // ProbeKernelId of the latest LaunchProbe

__device__ __forceinline__ void GroupBarrier(int group)
{
    asm volatile("bar.sync %0, %1;" ::"r"(group + 1), "r"(kGroupThreads) : "memory");
}

// Rows [0, n) of one staged output column to `col` rows [at0, at0 + n): rows up to the first
// 16-byte boundary and after the last one singly, the rest 16 bytes per store.
template <uint32_t kLayout, int kO>
__device__ __forceinline__ void WriteStagedColumn(void *col, int width, bool isKey, int shift,
    const long long *sKey, const unsigned long long *sPay, uint64_t at0, uint32_t n, uint32_t t)
{
    constexpr int code = static_cast<int>((kLayout >> (3 * kO)) & 7u);
    const int w = code == 0 ? width : (1 << (code - 1));
    auto value = [&](uint32_t r) -> uint64_t {
        return isKey ? static_cast<uint64_t>(sKey[r]) : (sPay[r] >> shift);
    };
    if (w != 8 && w != 4) {
        for (uint32_t r = t; r < n; r += kGroupThreads) {
            StoreOut<kLayout, kO>(col, at0 + r, width, static_cast<int64_t>(value(r)));
        }
        return;
    }
    uint8_t *dst = static_cast<uint8_t *>(col) + at0 * static_cast<uint64_t>(w);
    const uint32_t mis = static_cast<uint32_t>(reinterpret_cast<uintptr_t>(dst) & 15u);
    uint32_t head = mis == 0 ? 0u : (16u - mis) / static_cast<uint32_t>(w);
    head = head < n ? head : n;
    const uint32_t per = 16u / static_cast<uint32_t>(w);
    const uint32_t nvec = (n - head) / per;
    const uint32_t tail0 = head + nvec * per;
    if (t < head) {
        StoreOut<kLayout, kO>(col, at0 + t, width, static_cast<int64_t>(value(t)));
    }
    if (t < n - tail0) {
        StoreOut<kLayout, kO>(col, at0 + tail0 + t, width, static_cast<int64_t>(value(tail0 + t)));
    }
    uint4 *vdst = reinterpret_cast<uint4 *>(dst + static_cast<uint64_t>(head) * w);
    for (uint32_t v = t; v < nvec; v += kGroupThreads) {
        const uint32_t r = head + v * per;
        uint4 q;
        if (w == 8) {
            const uint64_t a = value(r);
            const uint64_t b = value(r + 1);
            q = make_uint4(static_cast<uint32_t>(a), static_cast<uint32_t>(a >> 32), static_cast<uint32_t>(b),
                static_cast<uint32_t>(b >> 32));
        } else {
            q = make_uint4(static_cast<uint32_t>(value(r)), static_cast<uint32_t>(value(r + 1)),
                static_cast<uint32_t>(value(r + 2)), static_cast<uint32_t>(value(r + 3)));
        }
        vdst[v] = q;
    }
}

template <int kNumOut, uint32_t kLayout, bool kSingle>
__global__ void __launch_bounds__(kBitsThreads, 1) ProbeGroupKernel(const __grid_constant__ ProbeLaunch p,
    uint32_t bitsVecs)
{
    extern __shared__ uint4 sGroupSmem[];
    {
        const uint4 *g = reinterpret_cast<const uint4 *>(p.table.slotBits);
        for (uint32_t i = threadIdx.x; i < bitsVecs; i += kBitsThreads) {
            sGroupSmem[i] = __ldg(g + i);
        }
    }
    __syncthreads();
    const uint32_t *sBits = reinterpret_cast<const uint32_t *>(sGroupSmem);
    const int group = static_cast<int>(threadIdx.x) / kGroupThreads;
    const uint32_t gt = threadIdx.x % kGroupThreads;  // thread within the group
    const int gw = static_cast<int>(gt >> 5);         // warp within the group
    const int lane = threadIdx.x & 31;
    const unsigned int lanesBelow = (1u << lane) - 1u;
    uint8_t *stage = reinterpret_cast<uint8_t *>(sGroupSmem + bitsVecs) + static_cast<size_t>(group) * kGroupStageBytes;
    long long *sKey = reinterpret_cast<long long *>(stage);
    unsigned long long *sPay = reinterpret_cast<unsigned long long *>(stage + kGroupRows * 8);
    unsigned int *sOff = reinterpret_cast<unsigned int *>(stage + kGroupRows * 16);  // [kGroupWarps]
    unsigned long long *sBase = reinterpret_cast<unsigned long long *>(stage + kGroupRows * 16 + 32);
    unsigned int *sTotal = reinterpret_cast<unsigned int *>(stage + kGroupRows * 16 + 40);

    const unsigned long long *payloadTab = reinterpret_cast<const unsigned long long *>(p.table.slotPayload);
    const uint64_t minKey = static_cast<uint64_t>(p.table.minKey);
    const uint64_t range = p.table.range;
    void *vals[kNumOut];
    int width[kNumOut];
    int shift[kNumOut];
    bool isKey[kNumOut];
#pragma unroll
    for (int o = 0; o < kNumOut; ++o) {
        vals[o] = p.out[o].values;
        width[o] = p.out[o].width;
        shift[o] = p.out[o].shift;
        isKey[o] = p.out[o].side == 0;
    }
    const long long *singleKeys = nullptr;
    const uint8_t *singleNulls = nullptr;
    int64_t singleRows = 0;
    if (kSingle) {
        singleKeys = static_cast<const long long *>(p.batches[0].cols[p.keyInput]);
        singleNulls = p.batches[0].nulls[p.keyInput];
        singleRows = p.batches[0].rows;
    }
    const int64_t nItems = kSingle ? (singleRows + kGroupRows - 1) / kGroupRows
                                   : static_cast<int64_t>(p.nTiles) * kGroupTilesPerTile;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * kGroupsPerCta;
    for (int64_t item = static_cast<int64_t>(blockIdx.x) * kGroupsPerCta + group; item < nItems; item += stride) {
        const int t = static_cast<int>(item / kGroupTilesPerTile);
        const long long *keyCol;
        const uint8_t *keyNulls;
        int64_t base;
        int64_t batchRows;
        if (kSingle) {
            keyCol = singleKeys;
            keyNulls = singleNulls;
            base = item * kGroupRows + gw * kBitsSegRows;
            batchRows = singleRows;
        } else {
            const int s0 = static_cast<int>(item % kGroupTilesPerTile) * kGroupRows;
            const TileDesc tile = p.tiles[t];
            if (s0 >= tile.rows) {
                continue;  // the same for every thread of the group
            }
            const BatchDesc &b = p.batches[tile.batch];
            keyCol = static_cast<const long long *>(b.cols[p.keyInput]);
            keyNulls = b.nulls[p.keyInput];
            base = static_cast<int64_t>(tile.row0) + s0 + gw * kBitsSegRows;
            batchRows = static_cast<int64_t>(tile.row0) + tile.rows;
        }
        int64_t key[kBitsRounds];
        const uint32_t live = LoadKeySegment(keyCol, keyNulls, base, batchRows, lane, key);
        uint32_t hit = 0;
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            const uint64_t d = static_cast<uint64_t>(key[i]) - minKey;
            if (((live >> i) & 1u) && key[i] >= p.table.minKey && d < range) {
                hit |= ((sBits[d >> 5] >> (d & 31)) & 1u) << i;
            }
        }
        uint64_t payload[kBitsRounds];
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            payload[i] = ((hit >> i) & 1u) ? __ldg(payloadTab + (static_cast<uint64_t>(key[i]) - minKey)) : 0ull;
        }
        uint32_t count = 0;
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            count += __popc(__ballot_sync(0xffffffffu, (hit >> i) & 1u));
        }
        if (lane == 0) {
            sOff[gw] = count;
        }
        GroupBarrier(group);
        if (gw == 0) {
            // Exclusive offsets of the group's warps and one output reservation for the group.
            unsigned int c = lane < kGroupWarps ? sOff[lane] : 0u;
            unsigned int incl = c;
#pragma unroll
            for (int d = 1; d < kGroupWarps; d <<= 1) {
                const unsigned int v = __shfl_up_sync(0xffffffffu, incl, d);
                incl += lane >= d ? v : 0u;
            }
            const unsigned int total = __shfl_sync(0xffffffffu, incl, kGroupWarps - 1);
            if (lane < kGroupWarps) {
                sOff[lane] = incl - c;
            }
            if (lane == 0) {
                const int region = t % p.nRegions;
                *sBase = total != 0 ? atomicAdd(p.outCount + region * kRegionStride, static_cast<unsigned long long>(total))
                                    : 0ull;
                *sTotal = total;
            }
        }
        GroupBarrier(group);
        const unsigned int total = *sTotal;
        if (p.countOnly || total == 0) {
            continue;  // uniform over the group
        }
        unsigned int off = sOff[gw];
#pragma unroll
        for (int i = 0; i < kBitsRounds; ++i) {
            const unsigned int m = __ballot_sync(0xffffffffu, (hit >> i) & 1u);
            if ((hit >> i) & 1u) {
                const unsigned int r = off + __popc(m & lanesBelow);
                sKey[r] = key[i];
                sPay[r] = payload[i];
            }
            off += __popc(m);
        }
        GroupBarrier(group);
        const uint64_t pos = *sBase;
        const uint32_t n = pos >= p.regionCap ? 0u
            : static_cast<uint32_t>(pos + total <= p.regionCap ? total : p.regionCap - pos);
        const uint64_t at0 = static_cast<uint64_t>(t % p.nRegions) * p.regionCap + pos;
        WriteStagedColumn<kLayout, 0>(vals[0], width[0], isKey[0], shift[0], sKey, sPay, at0, n, gt);
        if (kNumOut > 1) {
            WriteStagedColumn<kLayout, 1>(vals[1], width[1], isKey[1], shift[1], sKey, sPay, at0, n, gt);
        }
        if (kNumOut > 2) {
            WriteStagedColumn<kLayout, 2>(vals[2], width[2], isKey[2], shift[2], sKey, sPay, at0, n, gt);
        }
        if (kNumOut > 3) {
            WriteStagedColumn<kLayout, 3>(vals[3], width[3], isKey[3], shift[3], sKey, sPay, at0, n, gt);
        }
    }
}

// ------------------------------------------------------------------ bulk-copy inner probe
// Inner joins on an ARRAY table (occupancy bitmap in shared memory, packed slot payload) whose
// outputs are the 8-byte probe key and payload fields of compile-time widths, written to device
// memory.  Columns move by the bulk-copy (TMA) engine instead of per-lane requests through L1:
// - keys (kIn): every warp owns two key buffers in shared memory; while it resolves one segment
//   of kRounds * 32 rows, one lane's `cp.async.bulk` fills the other with the next segment (and
//   its validity bytes), completing on that buffer's mbarrier;
// - outputs (kOut): the warp compacts a segment's matches into one of two staging buffers, each
//   column laid out with its destination's 16-byte phase, and one bulk store per column writes
//   the 16-byte aligned middle of the column's run; the rows before and after it (at most 15
//   bytes each) are plain stores.
// Segments that are not whole or whose columns are not 16-byte aligned read their keys with
// plain loads.  A bounded mbarrier wait that runs out sets error 7 and ends the warp after
// waiting (again bounded) for its copies in flight.
template <int kNumOut, uint32_t kLayout, int kRounds, bool kIn, bool kOut>
struct BulkProbeSmem {
    static constexpr int kRows = kRounds * 32;
    static constexpr uint32_t kKeyBytes = kIn ? static_cast<uint32_t>(kRows) * 8u : 0u;
    static constexpr uint32_t kNullBytes = kIn ? 16u : 0u;  // kRows / 8 validity bytes, padded
    static constexpr uint32_t Width(int o)
    {
        return o < kNumOut ? (1u << (((kLayout >> (3 * o)) & 7u) - 1u)) : 0u;
    }
    // A column's staging run: kRows rows plus up to 15 bytes of destination phase.
    static constexpr uint32_t ColBytes(int o) { return o < kNumOut ? static_cast<uint32_t>(kRows) * Width(o) + 16u : 0u; }
    static constexpr uint32_t ColOffset(int o) { return o == 0 ? 0u : ColOffset(o - 1) + ColBytes(o - 1); }
    static constexpr uint32_t kStageBytes = kOut ? ColOffset(4) : 0u;
    static constexpr uint32_t kKeyOff = 0;
    static constexpr uint32_t kNullOff = 2 * kKeyBytes;
    static constexpr uint32_t kStageOff = kNullOff + 2 * kNullBytes;
    static constexpr uint32_t kBarOff = kStageOff + 2 * kStageBytes;
    static constexpr uint32_t kBytes = kBarOff + (kIn ? 16u : 0u);  // two mbarriers
    // With output staging, 128-row segments fit 16 warps beside a 128 KiB bitmap; capping the
    // CTA there leaves each thread up to 128 registers.
    static constexpr int kMaxThreads = kRounds >= 4 && kOut ? 512 : 1024;
};

struct BulkSeg {
    const long long *keys;
    const uint8_t *nulls;
    int64_t base;
    int64_t batchRows;
    int t;
    bool valid;
    bool bulk;
};

template <bool kSingle, int kRows>
__device__ __forceinline__ BulkSeg BulkSegOf(const ProbeLaunch &p, int64_t item)
{
    BulkSeg s;
    if (kSingle) {
        s.keys = static_cast<const long long *>(p.batches[0].cols[p.keyInput]);
        s.nulls = p.batches[0].nulls[p.keyInput];
        s.base = item * kRows;
        s.batchRows = p.batches[0].rows;
        s.t = static_cast<int>(s.base / kTileRows);
        s.valid = true;
    } else {
        constexpr int kSegsPerTile = kTileRows / kRows;
        s.t = static_cast<int>(item / kSegsPerTile);
        const int s0 = static_cast<int>(item % kSegsPerTile) * kRows;
        const TileDesc tile = p.tiles[s.t];
        s.valid = s0 < tile.rows;
        const BatchDesc &b = p.batches[tile.batch];
        s.keys = static_cast<const long long *>(b.cols[p.keyInput]);
        s.nulls = b.nulls[p.keyInput];
        s.base = static_cast<int64_t>(tile.row0) + s0;
        s.batchRows = static_cast<int64_t>(tile.row0) + tile.rows;
    }
    // Whole segments of 16-byte aligned columns move by bulk copy: the key run starts at
    // base * 8 bytes and the validity run at base / 8 bytes (a multiple of 16 for 128-row
    // segments; 64-row segments read validity words with plain loads).
    const uintptr_t nullAlign = kRows % 128 == 0 ? 15u : 3u;
    s.bulk = s.valid && s.base + kRows <= s.batchRows && (reinterpret_cast<uintptr_t>(s.keys) & 15u) == 0 &&
        (reinterpret_cast<uintptr_t>(s.nulls) & nullAlign) == 0;
    return s;
}

template <int kRows>
__device__ __forceinline__ void BulkSegLoad(const BulkSeg &s, long long *keyBuf, uint8_t *nullBuf, uint64_t *bar)
{
    const bool bulkNulls = s.nulls != nullptr && kRows % 128 == 0;
    const uint32_t bytes = static_cast<uint32_t>(kRows) * 8u + (bulkNulls ? static_cast<uint32_t>(kRows / 8) : 0u);
    MbarArmTx(bar, bytes);
    BulkLoad(keyBuf, s.keys + s.base, static_cast<uint32_t>(kRows) * 8u, bar);
    if (bulkNulls) {
        BulkLoad(nullBuf, s.nulls + (s.base >> 3), static_cast<uint32_t>(kRows / 8), bar);
    }
}

// Keys and validity of one segment with plain loads: whole segments with word-aligned validity
// branch-free, others row by row.
template <int kRounds>
__device__ __forceinline__ uint32_t LoadKeysPlain(const BulkSeg &s, int lane, int64_t (&key)[kRounds])
{
    uint32_t live = 0;
    if (s.base + kRounds * 32 <= s.batchRows && (reinterpret_cast<uintptr_t>(s.nulls) & 3u) == 0) {
        uint32_t w[kRounds];
#pragma unroll
        for (int i = 0; i < kRounds; ++i) {
            key[i] = __ldg(s.keys + s.base + i * 32 + lane);
            w[i] = s.nulls == nullptr ? 0u : __ldg(reinterpret_cast<const unsigned int *>(s.nulls) + ((s.base >> 5) + i));
        }
#pragma unroll
        for (int i = 0; i < kRounds; ++i) {
            live |= (((w[i] >> lane) & 1u) ^ 1u) << i;
        }
        return live;
    }
#pragma unroll
    for (int i = 0; i < kRounds; ++i) {
        const int64_t row = s.base + i * 32 + lane;
        key[i] = 0;
        if (row < s.batchRows) {
            key[i] = __ldg(s.keys + row);
            if (!RowIsNullRO(s.nulls, row)) {
                live |= 1u << i;
            }
        }
    }
    return live;
}

// Widths below are compile-time constants once the column loops are unrolled.
__device__ __forceinline__ void StageOut(uint8_t *col, uint32_t byteAt, uint64_t v, uint32_t width)
{
    if (width == 8) {
        *reinterpret_cast<uint64_t *>(col + byteAt) = v;
    } else if (width == 4) {
        *reinterpret_cast<uint32_t *>(col + byteAt) = static_cast<uint32_t>(v);
    } else if (width == 2) {
        *reinterpret_cast<uint16_t *>(col + byteAt) = static_cast<uint16_t>(v);
    } else {
        col[byteAt] = static_cast<uint8_t>(v);
    }
}

__device__ __forceinline__ void CopyStaged(uint8_t *dst, const uint8_t *src, uint32_t width)
{
    if (width == 8) {
        *reinterpret_cast<uint64_t *>(dst) = *reinterpret_cast<const uint64_t *>(src);
    } else if (width == 4) {
        *reinterpret_cast<uint32_t *>(dst) = *reinterpret_cast<const uint32_t *>(src);
    } else if (width == 2) {
        *reinterpret_cast<uint16_t *>(dst) = *reinterpret_cast<const uint16_t *>(src);
    } else {
        *dst = *src;
    }
}

template <int kNumOut, uint32_t kLayout, bool kSingle, int kRounds, bool kIn, bool kOut>
__global__ void __launch_bounds__(BulkProbeSmem<kNumOut, kLayout, kRounds, kIn, kOut>::kMaxThreads, 1)
    ProbeBulkKernel(const __grid_constant__ ProbeLaunch p, uint32_t bitsVecs)
{
    using G = BulkProbeSmem<kNumOut, kLayout, kRounds, kIn, kOut>;
    constexpr int kRows = G::kRows;
    extern __shared__ uint4 sBulkSmem[];
    const int warp = static_cast<int>(threadIdx.x >> 5);
    const int lane = static_cast<int>(threadIdx.x & 31);
    const unsigned int lanesBelow = (1u << lane) - 1u;
    uint8_t *mine = reinterpret_cast<uint8_t *>(sBulkSmem + bitsVecs) + static_cast<size_t>(warp) * G::kBytes;
    uint64_t *bar = reinterpret_cast<uint64_t *>(mine + G::kBarOff);
    if (kIn && lane == 0) {
        MbarInit(bar, 1);
        MbarInit(bar + 1, 1);
        MbarInitFence();
    }
    {
        const uint4 *g = reinterpret_cast<const uint4 *>(p.table.slotBits);
        for (uint32_t i = threadIdx.x; i < bitsVecs; i += blockDim.x) {
            sBulkSmem[i] = __ldg(g + i);
        }
    }
    __syncthreads();
    const uint32_t *sBits = reinterpret_cast<const uint32_t *>(sBulkSmem);
    const unsigned long long *payloadTab = reinterpret_cast<const unsigned long long *>(p.table.slotPayload);
    const uint64_t minKey = static_cast<uint64_t>(p.table.minKey);
    const uint64_t range = p.table.range;
    const long long budget = p.waitBudget;
    uint8_t *vals[kNumOut];
    int shift[kNumOut];
    bool isKey[kNumOut];
#pragma unroll
    for (int o = 0; o < kNumOut; ++o) {
        vals[o] = static_cast<uint8_t *>(p.out[o].values);
        shift[o] = p.out[o].shift;
        isKey[o] = p.out[o].side == 0;
    }
    const int64_t nItems = kSingle ? (p.batches[0].rows + kRows - 1) / kRows
                                   : static_cast<int64_t>(p.nTiles) * (kTileRows / kRows);
    const int warpsPerCta = static_cast<int>(blockDim.x >> 5);
    const int64_t warpsTotal = static_cast<int64_t>(gridDim.x) * warpsPerCta;
    int64_t item = static_cast<int64_t>(blockIdx.x) * warpsPerCta + warp;
    uint32_t parity = 0;        // bit b: the parity of bar[b]'s next phase
    uint32_t pendingLoads = 0;  // bit b: a load into buffer b is in flight
    int buf = 0;
    int stage = 0;
    bool failed = false;
    BulkSeg cur = BulkSegOf<kSingle, kRows>(p, item < nItems ? item : 0);
    if (kIn && item < nItems && cur.bulk) {
        if (lane == 0) {
            BulkSegLoad<kRows>(cur, reinterpret_cast<long long *>(mine + G::kKeyOff), mine + G::kNullOff, bar);
        }
        pendingLoads |= 1u;
    }
    for (; item < nItems; item += warpsTotal) {
        const int64_t nextItem = item + warpsTotal;
        BulkSeg next = cur;
        next.valid = false;
        next.bulk = false;
        if (nextItem < nItems) {
            next = BulkSegOf<kSingle, kRows>(p, nextItem);
            // Prefetch the next segment into the other buffer; its keys were read into
            // registers by every lane in the previous iteration.
            if (kIn && next.bulk) {
                FenceProxyAsyncShared();
                __syncwarp();
                if (lane == 0) {
                    BulkSegLoad<kRows>(next, reinterpret_cast<long long *>(mine + G::kKeyOff + (buf ^ 1) * G::kKeyBytes),
                        mine + G::kNullOff + (buf ^ 1) * G::kNullBytes, bar + (buf ^ 1));
                }
                pendingLoads |= 1u << (buf ^ 1);
            }
        }
        if (cur.valid) {
            int64_t key[kRounds];
            uint32_t live = 0;
            if (kIn && cur.bulk) {
                const bool ok = __all_sync(0xffffffffu, MbarWaitBounded(bar + buf, (parity >> buf) & 1u, budget));
                if (!ok) {
                    failed = true;
                    break;
                }
                parity ^= 1u << buf;
                pendingLoads &= ~(1u << buf);
                const long long *kb = reinterpret_cast<const long long *>(mine + G::kKeyOff + buf * G::kKeyBytes);
#pragma unroll
                for (int i = 0; i < kRounds; ++i) {
                    key[i] = kb[i * 32 + lane];
                }
                if (cur.nulls == nullptr) {
                    live = (1u << kRounds) - 1u;
                } else {
                    const uint32_t *nw = kRows % 128 == 0
                        ? reinterpret_cast<const uint32_t *>(mine + G::kNullOff + buf * G::kNullBytes)
                        : nullptr;
#pragma unroll
                    for (int i = 0; i < kRounds; ++i) {
                        const uint32_t w = nw != nullptr
                            ? nw[i]
                            : __ldg(reinterpret_cast<const unsigned int *>(cur.nulls) + ((cur.base >> 5) + i));
                        live |= (((w >> lane) & 1u) ^ 1u) << i;
                    }
                }
            } else {
                live = LoadKeysPlain<kRounds>(cur, lane, key);
            }
            uint32_t hit = 0;
#pragma unroll
            for (int i = 0; i < kRounds; ++i) {
                const uint64_t d = static_cast<uint64_t>(key[i]) - minKey;
                if (((live >> i) & 1u) && key[i] >= p.table.minKey && d < range) {
                    hit |= ((sBits[d >> 5] >> (d & 31)) & 1u) << i;
                }
            }
            uint64_t payload[kRounds];
#pragma unroll
            for (int i = 0; i < kRounds; ++i) {
                payload[i] = ((hit >> i) & 1u) ? __ldg(payloadTab + (static_cast<uint64_t>(key[i]) - minKey)) : 0ull;
            }
            uint32_t total = 0;
#pragma unroll
            for (int i = 0; i < kRounds; ++i) {
                total += __popc(__ballot_sync(0xffffffffu, (hit >> i) & 1u));
            }
            const int region = cur.t % p.nRegions;
            unsigned long long pos = 0;
            if (lane == 0 && total != 0) {
                pos = atomicAdd(p.outCount + region * kRegionStride, static_cast<unsigned long long>(total));
            }
            pos = __shfl_sync(0xffffffffu, pos, 0);
            const uint32_t n = p.countOnly || pos >= p.regionCap
                ? 0u
                : static_cast<uint32_t>(pos + total <= p.regionCap ? total : p.regionCap - pos);
            const uint64_t at0 = static_cast<uint64_t>(region) * p.regionCap + pos;
            if (!kOut && n != 0) {
                uint32_t off = 0;
#pragma unroll
                for (int i = 0; i < kRounds; ++i) {
                    const unsigned int m = __ballot_sync(0xffffffffu, (hit >> i) & 1u);
                    const uint32_t j = off + __popc(m & lanesBelow);
                    if (((hit >> i) & 1u) && j < n) {
#pragma unroll
                        for (int o = 0; o < kNumOut; ++o) {
                            const uint64_t v = isKey[o] ? static_cast<uint64_t>(key[i]) : (payload[i] >> shift[o]);
                            StageOut(vals[o] + (at0 + j) * G::Width(o), 0u, v, G::Width(o));
                        }
                    }
                    off += __popc(m);
                }
            }
            if (kOut && n != 0) {
                uint8_t *st = mine + G::kStageOff + stage * G::kStageBytes;
                // The staging buffer was last read by the bulk stores of two segments ago.
                if (lane == 0) {
                    BulkWaitRead<1>();
                }
                __syncwarp();
                uint32_t phase[kNumOut];
#pragma unroll
                for (int o = 0; o < kNumOut; ++o) {
                    phase[o] = static_cast<uint32_t>(reinterpret_cast<uintptr_t>(vals[o] + at0 * G::Width(o)) & 15u);
                }
                uint32_t off = 0;
#pragma unroll
                for (int i = 0; i < kRounds; ++i) {
                    const unsigned int m = __ballot_sync(0xffffffffu, (hit >> i) & 1u);
                    const uint32_t j = off + __popc(m & lanesBelow);
                    if (((hit >> i) & 1u) && j < n) {
#pragma unroll
                        for (int o = 0; o < kNumOut; ++o) {
                            const uint64_t v = isKey[o] ? static_cast<uint64_t>(key[i]) : (payload[i] >> shift[o]);
                            StageOut(st + G::ColOffset(o), phase[o] + j * G::Width(o), v, G::Width(o));
                        }
                    }
                    off += __popc(m);
                }
                FenceProxyAsyncShared();
                __syncwarp();
                // Per column: bytes [head, head + mid) of the run go by one bulk store, the rows
                // before it (fewer than 16 bytes) and after it (likewise) by lane l writing row l.
#pragma unroll
                for (int o = 0; o < kNumOut; ++o) {
                    const uint32_t runBytes = n * G::Width(o);
                    const uint32_t head = (16u - phase[o]) & 15u;
                    const uint32_t mid = runBytes > head ? ((runBytes - head) & ~15u) : 0u;
                    if (lane == 0 && mid != 0) {
                        BulkStore(vals[o] + at0 * G::Width(o) + head, st + G::ColOffset(o) + phase[o] + head, mid);
                    }
                    const uint32_t headEnd = head < runBytes ? head : runBytes;
                    const uint32_t tail = headEnd + mid;
                    const uint32_t lb = static_cast<uint32_t>(lane) * G::Width(o);
                    if (lb < headEnd) {
                        CopyStaged(vals[o] + at0 * G::Width(o) + lb, st + G::ColOffset(o) + phase[o] + lb, G::Width(o));
                    }
                    if (tail + lb < runBytes) {
                        CopyStaged(vals[o] + at0 * G::Width(o) + tail + lb, st + G::ColOffset(o) + phase[o] + tail + lb,
                            G::Width(o));
                    }
                }
                if (lane == 0) {
                    BulkCommit();
                }
                stage ^= 1;
            }
        }
        cur = next;
        buf ^= 1;
    }
    if (kIn && failed) {
        if (lane == 0 && p.error != nullptr) {
            atomicExch(p.error, 7);
        }
        // Let the loads still in flight land before the CTA's shared memory is released.
        for (int b = 0; b < 2; ++b) {
            if ((pendingLoads >> b) & 1u) {
                MbarWaitBounded(bar + b, (parity >> b) & 1u, budget);
            }
        }
    }
    if (kOut && lane == 0) {
        BulkWaitAll();
    }
}

// Occupancy bitmap of an ARRAY table: bit d of word d / 32 set iff entries[d] >= 0.  Words past
// the range (up to the 16-byte padding) are zero.
__global__ void BuildSlotBitsKernel(const int64_t *entries, uint64_t range, uint32_t *bits, uint64_t nWords)
{
    for (uint64_t w = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; w < nWords;
         w += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint32_t v = 0;
        for (int j = 0; j < 32; ++j) {
            const uint64_t d = w * 32 + j;
            if (d < range && entries[d] >= 0) {
                v |= 1u << j;
            }
        }
        bits[w] = v;
    }
}

}  // namespace

cudaError_t LaunchGatherColumn(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, int32_t input, int32_t width, void *valuesOut, uint8_t *nullsOut,
    cudaStream_t stream)
{
    if (nTiles <= 0) {
        return cudaSuccess;
    }
    const unsigned grid = static_cast<unsigned>(nTiles < SMs() * 8 ? nTiles : SMs() * 8);
    GatherColumnKernel<<<grid, 256, 0, stream>>>(batches, tiles, nTiles, tileOutRow, input, width, valuesOut,
        nullsOut);
    return cudaGetLastError();
}

cudaError_t LaunchKeyStats(const void *keys, const uint8_t *nulls, int64_t n, int32_t width, long long *stats,
    cudaStream_t stream)
{
    const long long init[3] = {0x7fffffffffffffffll, static_cast<long long>(0x8000000000000000ull), 0};
    cudaError_t err = cudaMemcpyAsync(stats, init, sizeof(init), cudaMemcpyHostToDevice, stream);
    if (err != cudaSuccess || n == 0) {
        return err;
    }
    KeyStatsKernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(keys, nulls, n, width, stats);
    return cudaGetLastError();
}

cudaError_t LaunchBuildCount(JoinTable t, const void *keys, const uint8_t *nulls, int64_t n, int32_t width,
    uint64_t *hashKeysMutable, uint32_t *counts, uint32_t *sentinelCount, unsigned int *maxCount, int32_t *error,
    cudaStream_t stream)
{
    if (n == 0) {
        return cudaSuccess;
    }
    BuildCountKernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(t, keys, nulls, n, width, hashKeysMutable, counts,
        sentinelCount, maxCount, error);
    return cudaGetLastError();
}

cudaError_t LaunchScanCounts(const uint32_t *counts, int64_t n, int64_t *offsets, int64_t *blockSums,
    long long *total, cudaStream_t stream)
{
    const int64_t nBlocks = (n + kScanThreads - 1) / kScanThreads;
    if (nBlocks == 0) {
        return cudaMemsetAsync(total, 0, sizeof(long long), stream);
    }
    ScanBlockSumsKernel<<<static_cast<unsigned>(nBlocks), kScanThreads, 0, stream>>>(counts, n, blockSums);
    ScanSumsKernel<<<1, 32, 0, stream>>>(blockSums, nBlocks, total);
    ScanApplyKernel<<<static_cast<unsigned>(nBlocks), kScanThreads, 0, stream>>>(counts, n, blockSums, offsets);
    return cudaGetLastError();
}

cudaError_t LaunchBuildFill(JoinTable t, const void *keys, const uint8_t *nulls, int64_t n, int32_t width,
    const uint32_t *counts, const int64_t *offsets, uint32_t *cursor, int64_t *entriesMutable,
    int32_t *csrRowsMutable, uint32_t sentinelCount, int64_t sentinelOffset, unsigned int *sentinelCursor,
    int64_t *sentinelEntryOut, int32_t *error, cudaStream_t stream)
{
    if (n == 0) {
        return cudaSuccess;
    }
    BuildFillKernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(t, keys, nulls, n, width, counts, offsets, cursor,
        entriesMutable, csrRowsMutable, sentinelCount, sentinelOffset, sentinelCursor, sentinelEntryOut, error);
    return cudaGetLastError();
}

uint64_t SlotBitsBytes(uint64_t range) { return ((range + 127) / 128) * 16; }

void SetStagedProbe(bool on) { g_stagedProbe.store(on); }

void SetBulkProbe(int mode) { g_bulkProbe.store(mode == 1 || mode == 2 ? mode : 0); }

int LastProbeKernel() { return g_lastProbeKernel.load(); }

// The bitmap kernel takes every join kind (marking a matched build row visited through its slot's
// entry for the kinds that keep unmatched build rows) on a unique ARRAY table whose occupancy
// bitmap fits in shared memory, on launches large enough to amortise staging it into every CTA;
// its outputs are the probe key, other fixed-width probe columns (*probeCols), payload fields
// (a slot payload present) and the existence flag.
bool BitsProbeEligible(const ProbeLaunch &p, bool *probeCols)
{
    const bool visits = p.joinKind == JOIN_KIND_BUILD_OUTER || p.joinKind == JOIN_KIND_FULL;
    const bool bitsKind = p.joinKind == JOIN_KIND_INNER || p.joinKind == JOIN_KIND_PROBE_OUTER ||
        p.joinKind == JOIN_KIND_SEMI || p.joinKind == JOIN_KIND_ANTI || p.joinKind == JOIN_KIND_EXISTENCE ||
        (visits && p.visited != nullptr && p.table.arrayEntries != nullptr);
    bool ok = bitsKind && p.nKeyCols == 0 && p.table.unique && p.keyWidth == 8 && p.nOut >= 1 &&
        p.nOut <= kFastMaxOut && p.table.mode == JOIN_ARRAY && p.table.slotBits != nullptr &&
        SlotBitsBytes(p.table.range) <= kBitsMaxSmem && p.nTiles >= kBitsMinTiles;
    bool cols = false;
    for (int o = 0; ok && o < p.nOut; ++o) {
        const JoinOutCol &oc = p.out[o];
        ok = ((oc.side == 1 && p.table.slotPayload != nullptr) || (oc.side == 0 && oc.src == p.keyInput && oc.width == 8) ||
                 (oc.side == 0 && oc.src != p.keyInput) || oc.side == 2) &&
            (oc.width == 1 || oc.width == 2 || oc.width == 4 || oc.width == 8);
        cols = cols || (oc.side == 0 && oc.src != p.keyInput);
    }
    if (probeCols != nullptr) {
        *probeCols = cols;
    }
    return ok;
}

// SimpleFilterShape on the host.
bool HostSimpleFilterShape(const ProbeLaunch &p)
{
    auto operand = [](int op) { return op == FOP_PROBE_COL || op == FOP_BUILD_COL || op == FOP_LITERAL; };
    return p.nFilter == 3 && operand(p.filter[0].op) && operand(p.filter[1].op) && p.filter[2].op >= FOP_EQ &&
        p.filter[2].op <= FOP_GTE;
}

// Only the bitmap kernel packs multi-column keys as it reads them (keys of up to two parts).
bool ProbePacksKeys(const ProbeLaunch &p)
{
    return p.pack.nParts <= kFusedPackParts && p.nFilter == 0 && BitsProbeEligible(p, nullptr);
}

cudaError_t LaunchProbe(const ProbeLaunch &p, cudaStream_t stream)
{
    if (p.nTiles <= 0) {
        return cudaSuccess;
    }
    if (p.pack.nParts > 0 && !ProbePacksKeys(p)) {
        // The chosen kernel reads the packed keys from the scratch input: fill it first.
        ProbeLaunch q = p;
        cudaError_t err = LaunchPackProbeKeys(p.batches, p.tiles, p.nTiles, p.pack, stream);
        if (err != cudaSuccess) {
            return err;
        }
        q.pack.nParts = 0;
        return LaunchProbe(q, stream);
    }
    if (p.nKeyCols > 0 || (p.nFilter > 0 && !BitsProbeEligible(p, nullptr))) {
        const int maxGrid = SMs() * BlocksPerSM(reinterpret_cast<const void *>(ProbeKindKernel), kProbeThreads, 0);
        g_lastProbeKernel.store(PROBE_KERNEL_KIND);
        ProbeKindKernel<<<p.nTiles < maxGrid ? p.nTiles : maxGrid, kProbeThreads, 0, stream>>>(p);
        return cudaGetLastError();
    }
    // Fast path: 8-byte key, unique build with slot payload, outputs = probe key / payload fields.
    bool fast = p.table.unique && p.table.slotPayload != nullptr && p.keyWidth == 8 && p.nOut >= 1 &&
        p.nOut <= kFastMaxOut;
    for (int o = 0; fast && o < p.nOut; ++o) {
        const JoinOutCol &oc = p.out[o];
        fast = (oc.side == 1 || (oc.side == 0 && oc.src == p.keyInput && oc.width == 8)) &&
            (oc.width == 1 || oc.width == 2 || oc.width == 4 || oc.width == 8);
    }
    bool probeCols = false;  // an output is a probe column other than the key
    const uint64_t bitsBytes = SlotBitsBytes(p.table.range);
    if (BitsProbeEligible(p, &probeCols)) {
        // Instances: run-time widths for 1-4 outputs, and compile-time widths for the common
        // layouts (8-byte key followed by payload fields).
        struct Inst {
            uint32_t layout;
            int nOut;
            const void *single;
            const void *tiled;
        };
#define OMG_GROUP_INST(n, layout)                                                                  \
    {layout, n, reinterpret_cast<const void *>(ProbeGroupKernel<n, layout, true>),                 \
        reinterpret_cast<const void *>(ProbeGroupKernel<n, layout, false>)}
        static const Inst groupInsts[] = {
            OMG_GROUP_INST(3, OutLayout(kW8, kW4, kW4)), OMG_GROUP_INST(2, OutLayout(kW8, kW8)),
            OMG_GROUP_INST(2, OutLayout(kW8, kW4)), OMG_GROUP_INST(1, 0), OMG_GROUP_INST(2, 0), OMG_GROUP_INST(3, 0),
            OMG_GROUP_INST(4, 0),
        };
#undef OMG_GROUP_INST
#define OMG_BITS_INST(n, layout, cols, packed)                                                              \
    {layout, n, reinterpret_cast<const void *>(ProbeBitsKernel<n, layout, true, cols, packed>),            \
        reinterpret_cast<const void *>(ProbeBitsKernel<n, layout, false, cols, packed>)}
#define OMG_FILTER_INST(n, layout, cols, kind)                                                              \
    {layout, n, reinterpret_cast<const void *>(ProbeBitsKernel<n, layout, true, cols, 0, kind>),           \
        reinterpret_cast<const void *>(ProbeBitsKernel<n, layout, false, cols, 0, kind>)}
        static const Inst insts[] = {
            OMG_BITS_INST(3, OutLayout(kW8, kW4, kW4), false, 0), OMG_BITS_INST(2, OutLayout(kW8, kW8), false, 0),
            OMG_BITS_INST(2, OutLayout(kW8, kW4), false, 0), OMG_BITS_INST(1, 0, false, 0),
            OMG_BITS_INST(2, 0, false, 0), OMG_BITS_INST(3, 0, false, 0), OMG_BITS_INST(4, 0, false, 0),
        };
        // Probe columns other than the key among the outputs, or a packed key: run-time widths.
        static const Inst colInsts[] = {
            OMG_BITS_INST(1, 0, true, 0), OMG_BITS_INST(2, 0, true, 0), OMG_BITS_INST(3, 0, true, 0),
            OMG_BITS_INST(4, 0, true, 0),
        };
        static const Inst packedInsts[] = {
            OMG_BITS_INST(1, 0, true, 1), OMG_BITS_INST(2, 0, true, 1), OMG_BITS_INST(3, 0, true, 1),
            OMG_BITS_INST(4, 0, true, 1),
        };
        // Two 4-byte key parts: the two parts and two 4-byte payload fields, or run-time widths.
        static const Inst two32Insts[] = {
            OMG_BITS_INST(4, OutLayout(kW4, kW4, kW4, kW4), true, 2), OMG_BITS_INST(1, 0, true, 2),
            OMG_BITS_INST(2, 0, true, 2), OMG_BITS_INST(3, 0, true, 2), OMG_BITS_INST(4, 0, true, 2),
        };
        static const Inst filterInsts[] = {
            OMG_FILTER_INST(1, 0, true, 1), OMG_FILTER_INST(2, 0, true, 1), OMG_FILTER_INST(3, 0, true, 1),
            OMG_FILTER_INST(4, 0, true, 1),
        };
        // One comparison: run-time widths, and the headline layout (8-byte key, two 4-byte fields).
        static const Inst cmpInsts[] = {
            OMG_FILTER_INST(1, 0, true, 2), OMG_FILTER_INST(2, 0, true, 2), OMG_FILTER_INST(3, 0, true, 2),
            OMG_FILTER_INST(4, 0, true, 2),
        };
        static const Inst cmpKeyInst = OMG_FILTER_INST(3, OutLayout(kW8, kW4, kW4), false, 2);
#undef OMG_BITS_INST
#undef OMG_FILTER_INST
        constexpr int kInsts = static_cast<int>(sizeof(insts) / sizeof(insts[0]));
        int pick = -1;
        for (int i = 0; i < kInsts && pick < 0; ++i) {
            if (insts[i].nOut != p.nOut) {
                continue;
            }
            bool match = true;
            for (int o = 0; o < p.nOut && insts[i].layout != 0; ++o) {
                const int code = static_cast<int>((insts[i].layout >> (3 * o)) & 7u);
                match = match && (1 << (code - 1)) == p.out[o].width;
            }
            pick = match ? i : -1;
        }
        const int single = p.singleBatch ? 0 : 1;
        if (probeCols || p.pack.nParts > 0 || p.nFilter > 0) {
            const bool filter = p.nFilter > 0;
            const bool packed = p.pack.nParts > 0 && !filter;
            const bool two32 = packed && p.pack.nParts == 2 && p.pack.width[0] == 4 && p.pack.width[1] == 4;
            bool cmp = filter && HostSimpleFilterShape(p);
            const Inst *ci = filter ? (cmp ? &cmpInsts[p.nOut - 1] : &filterInsts[p.nOut - 1])
                                    : (packed ? &packedInsts[p.nOut - 1] : &colInsts[p.nOut - 1]);
            if (cmp && !probeCols && !packed && insts[pick].layout == OutLayout(kW8, kW4, kW4)) {
                ci = &cmpKeyInst;
            }
            if (two32) {
                bool w4 = p.nOut == 4;
                for (int o = 0; w4 && o < p.nOut; ++o) {
                    w4 = p.out[o].width == 4;
                }
                ci = w4 ? &two32Insts[0] : &two32Insts[p.nOut];
            }
            const void *ck = single == 0 ? ci->single : ci->tiled;
            cudaError_t cerr = EnsureDynamicSmem(ck, kBitsMaxSmem);
            if (cerr != cudaSuccess) {
                return cerr;
            }
            const int threads = packed || (filter && !cmp) ? BitsThreads<1, 1>::value : BitsThreads<0, 0>::value;
            const int64_t items = static_cast<int64_t>(p.nTiles) * kBitsSegsPerTile;
            const int64_t wanted = (items + threads / 32 - 1) / (threads / 32);
            const int grid = static_cast<int>(wanted < SMs() ? wanted : SMs());
            void *cargs[] = {const_cast<ProbeLaunch *>(&p)};
            g_lastProbeKernel.store(PROBE_KERNEL_BITS);
            return cudaLaunchKernel(ck, dim3(grid), dim3(threads), cargs, static_cast<size_t>(bitsBytes), stream);
        }
        // Inner joins whose outputs are the probe key and payload fields, written to pinned host
        // memory, take the staged kernel when its shared memory (bitmap + the groups' staging)
        // fits: whole-line output runs carry the link at its rate (with HBM output the per-warp
        // kernel, without the group barriers, is faster).
        const uint32_t groupSmem = static_cast<uint32_t>(bitsBytes) + kGroupsPerCta * kGroupStageBytes;
        bool staged = p.joinKind == JOIN_KIND_INNER && p.table.slotPayload != nullptr && groupSmem <= kGroupMaxSmem &&
            p.hostOutput != 0 && g_stagedProbe.load();
        for (int o = 0; staged && o < p.nOut; ++o) {
            staged = p.out[o].side != 2;
        }
        // Opt-in (omg_debug_set_bulk_probe): inner joins with compile-time output widths written
        // to HBM from device-resident keys run the bulk-copy kernel when its columns are 16-byte
        // aligned and at least 8 warps' buffers fit beside the bitmap.  Measured slower than the
        // per-lane kernel on this path (bulk copies travel the same L1-to-L2 request path, and
        // small bulk stores are slow), so it is not the default.
        const int bulkMode = g_bulkProbe.load();
        bool bulk = !staged && p.hostOutput == 0 && p.deviceKeys != 0 && bulkMode != 0 && p.joinKind == JOIN_KIND_INNER &&
            p.table.slotPayload != nullptr && insts[pick].layout != 0;
        for (int o = 0; bulk && o < p.nOut; ++o) {
            bulk = p.out[o].side != 2 && (reinterpret_cast<uintptr_t>(p.out[o].values) & 15u) == 0 &&
                (p.regionCap * static_cast<uint64_t>(p.out[o].width)) % 16u == 0;
        }
        if (bulk) {
            struct BulkInst {
                uint32_t layout;
                int nOut;
                int mode;  // 1: bulk key loads, 2: bulk key loads and output stores
                uint32_t warpBytes;
                int maxWarps;
                const void *single;
                const void *tiled;
            };
#define OMG_BULK_INST(n, layout, out)                                                                       \
    {layout, n, (out) ? 2 : 1, BulkProbeSmem<n, layout, kBitsRounds, true, out>::kBytes,                    \
        BulkProbeSmem<n, layout, kBitsRounds, true, out>::kMaxThreads / 32,                                  \
        reinterpret_cast<const void *>(ProbeBulkKernel<n, layout, true, kBitsRounds, true, out>),           \
        reinterpret_cast<const void *>(ProbeBulkKernel<n, layout, false, kBitsRounds, true, out>)}
            static const BulkInst bulkInsts[] = {
                OMG_BULK_INST(3, OutLayout(kW8, kW4, kW4), false), OMG_BULK_INST(3, OutLayout(kW8, kW4, kW4), true),
                OMG_BULK_INST(2, OutLayout(kW8, kW8), false), OMG_BULK_INST(2, OutLayout(kW8, kW8), true),
                OMG_BULK_INST(2, OutLayout(kW8, kW4), false), OMG_BULK_INST(2, OutLayout(kW8, kW4), true),
            };
#undef OMG_BULK_INST
            const BulkInst *bi = nullptr;
            for (const BulkInst &c : bulkInsts) {
                if (c.layout == insts[pick].layout && c.nOut == p.nOut && c.mode == bulkMode) {
                    bi = &c;
                }
            }
            const uint32_t room = kGroupMaxSmem - static_cast<uint32_t>(bitsBytes);
            const int warps = bi == nullptr ? 0 : static_cast<int>(std::min<uint32_t>(room / bi->warpBytes, bi->maxWarps));
            if (warps >= 8) {
                const void *bk = single == 0 ? bi->single : bi->tiled;
                cudaError_t berr = EnsureDynamicSmem(bk, kGroupMaxSmem);
                if (berr != cudaSuccess) {
                    return berr;
                }
                const int64_t items = static_cast<int64_t>(p.nTiles) * kBitsSegsPerTile;
                const int64_t wanted = (items + warps - 1) / warps;
                const int grid = static_cast<int>(wanted < SMs() ? (wanted > 0 ? wanted : 1) : SMs());
                uint32_t bitsVecs = static_cast<uint32_t>(bitsBytes / 16);
                const size_t smem = static_cast<size_t>(bitsBytes) + static_cast<size_t>(warps) * bi->warpBytes;
                void *bargs[] = {const_cast<ProbeLaunch *>(&p), &bitsVecs};
                g_lastProbeKernel.store(PROBE_KERNEL_BULK);
                return cudaLaunchKernel(bk, dim3(grid), dim3(warps * 32), bargs, smem, stream);
            }
        }
        if (staged) {
            const void *gk = single == 0 ? groupInsts[pick].single : groupInsts[pick].tiled;
            cudaError_t gerr = EnsureDynamicSmem(gk, kGroupMaxSmem);
            if (gerr != cudaSuccess) {
                return gerr;
            }
            const int64_t items = static_cast<int64_t>(p.nTiles) * kGroupTilesPerTile;
            const int64_t wanted = (items + kGroupsPerCta - 1) / kGroupsPerCta;
            const int grid = static_cast<int>(wanted < SMs() ? (wanted > 0 ? wanted : 1) : SMs());
            uint32_t bitsVecs = static_cast<uint32_t>(bitsBytes / 16);
            void *gargs[] = {const_cast<ProbeLaunch *>(&p), &bitsVecs};
            g_lastProbeKernel.store(PROBE_KERNEL_GROUP);
            return cudaLaunchKernel(gk, dim3(grid), dim3(kBitsThreads), gargs, static_cast<size_t>(groupSmem), stream);
        }
        const void *kernel = single == 0 ? insts[pick].single : insts[pick].tiled;
        cudaError_t err = EnsureDynamicSmem(kernel, kBitsMaxSmem);
        if (err != cudaSuccess) {
            return err;
        }
        const int64_t items = static_cast<int64_t>(p.nTiles) * kBitsSegsPerTile;
        const int64_t warpsPerCta = kBitsThreads / 32;
        const int64_t wanted = (items + warpsPerCta - 1) / warpsPerCta;
        const int grid = static_cast<int>(wanted < SMs() ? wanted : SMs());
        void *args[] = {const_cast<ProbeLaunch *>(&p)};
        g_lastProbeKernel.store(PROBE_KERNEL_BITS);
        return cudaLaunchKernel(kernel, dim3(grid), dim3(kBitsThreads), args, static_cast<size_t>(bitsBytes), stream);
    }
    if (p.nKeyCols == 0 && p.joinKind != JOIN_KIND_INNER) {
        auto kk = !p.table.unique ? ProbeKernel<false, false, true>
                                  : (p.table.slotPayload != nullptr ? ProbeKernel<true, true, true>
                                                                    : ProbeKernel<true, false, true>);
        const int maxGrid = SMs() * BlocksPerSM(reinterpret_cast<const void *>(kk), kProbeThreads, 0);
        g_lastProbeKernel.store(PROBE_KERNEL_GENERAL);
        kk<<<p.nTiles < maxGrid ? p.nTiles : maxGrid, kProbeThreads, 0, stream>>>(p);
        return cudaGetLastError();
    }
    auto kernel = !p.table.unique ? ProbeKernel<false, false, false>
                                  : (p.table.slotPayload != nullptr ? ProbeKernel<true, true, false>
                                                                    : ProbeKernel<true, false, false>);
    if (fast) {
        const void *fk[kFastMaxOut] = {reinterpret_cast<const void *>(ProbeFastKernel<1>),
            reinterpret_cast<const void *>(ProbeFastKernel<2>), reinterpret_cast<const void *>(ProbeFastKernel<3>),
            reinterpret_cast<const void *>(ProbeFastKernel<4>)};
        kernel = reinterpret_cast<decltype(kernel)>(fk[p.nOut - 1]);
    }
    const int maxGrid = SMs() * BlocksPerSM(reinterpret_cast<const void *>(kernel), kProbeThreads, 0);
    const int grid = p.nTiles < maxGrid ? p.nTiles : maxGrid;
    g_lastProbeKernel.store(fast ? PROBE_KERNEL_FAST : PROBE_KERNEL_GENERAL);
    kernel<<<grid, kProbeThreads, 0, stream>>>(p);
    return cudaGetLastError();
}

cudaError_t LaunchPackBuildKeys(const JoinKeyCols &kc, const JoinKeyPack &kp, int64_t n, int64_t *out,
    uint8_t *outNulls, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    PackBuildKeysKernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(kc, kp, n, out, reinterpret_cast<uint32_t *>(outNulls));
    return cudaGetLastError();
}

cudaError_t LaunchPackProbeKeys(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles, const JoinKeyPack &kp,
    cudaStream_t stream)
{
    if (nTiles <= 0) {
        return cudaSuccess;
    }
    const int grid = nTiles < SMs() * 8 ? nTiles : SMs() * 8;
    PackProbeKeysKernel<<<grid, 256, 0, stream>>>(batches, tiles, nTiles, kp);
    return cudaGetLastError();
}

cudaError_t LaunchJoinKeyHash(const JoinKeyCols &kc, int64_t n, uint64_t *out, uint8_t *outNulls, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    JoinKeyHashKernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(kc, n, out, outNulls);
    return cudaGetLastError();
}

cudaError_t LaunchUnvisitedFlags(const uint8_t *visited, int64_t n, uint32_t *flags, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    UnvisitedFlagsKernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(visited, n, flags);
    return cudaGetLastError();
}

cudaError_t LaunchUnvisitedRows(const uint8_t *visited, const int64_t *offsets, int64_t n, int32_t *rows,
    cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    UnvisitedRowsKernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(visited, offsets, n, rows);
    return cudaGetLastError();
}

cudaError_t LaunchGatherRows(const void *src, const uint8_t *srcNulls, const int32_t *rows, int64_t n, int32_t width,
    void *dst, uint8_t *dstNulls, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    GatherRowsKernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(src, srcNulls, rows, n, width, dst, dstNulls);
    return cudaGetLastError();
}

cudaError_t LaunchBuildSlotBits(const int64_t *arrayEntries, uint64_t range, uint32_t *bits, cudaStream_t stream)
{
    const uint64_t nWords = SlotBitsBytes(range) / 4;
    BuildSlotBitsKernel<<<GridFor(static_cast<int64_t>(nWords), 256, 8), 256, 0, stream>>>(arrayEntries, range, bits,
        nWords);
    return cudaGetLastError();
}

cudaError_t LaunchBuildSlotPayload(const ProbeLaunch &p, uint64_t nSlots, uint64_t *payload, cudaStream_t stream)
{
    const int64_t n = static_cast<int64_t>(nSlots) + 1;
    const int64_t *entries = p.table.mode == JOIN_ARRAY ? p.table.arrayEntries : p.table.hashEntries;
    BuildSlotPayloadKernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(entries, nSlots, p.table.sentinelEntry, p, payload);
    return cudaGetLastError();
}

cudaError_t LaunchFillI64(int64_t *p, int64_t v, int64_t n, cudaStream_t stream)
{
    if (n == 0) {
        return cudaSuccess;
    }
    FillI64Kernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(p, v, n);
    return cudaGetLastError();
}

cudaError_t LaunchFillU64(uint64_t *p, uint64_t v, int64_t n, cudaStream_t stream)
{
    if (n == 0) {
        return cudaSuccess;
    }
    FillU64Kernel<<<GridFor(n, 256, 8), 256, 0, stream>>>(p, v, n);
    return cudaGetLastError();
}

}  // namespace omg
