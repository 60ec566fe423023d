// Partitioned inner hash join for unique 8-byte build keys (no reference counterpart: the
// reference probes one shared table, operator/join/lookup_join.cpp:924-1035).
//
// Both sides are split into P = 2^bits partitions by one partition function, either a hash of
// the key or a range lookup in P - 1 sorted splits (set from the probe keys' distribution).
// Partitioning is a radix pass per side: per-chunk histograms, one placement scan, a scatter in
// which every row gets a unique slot from its chunk's placement (no per-row global atomics).  The
// build side then gets one small open-addressing table per partition; the probe walks the
// partitioned keys in order, so consecutive rows use the same small table and it stays in cache.
#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "join_part.h"
#include "launch.h"

namespace omg {
namespace {

int SMs() { return DeviceSMCount(); }

constexpr int kPartThreads = 512;

struct RangeLut {
    const int64_t *splits;   // shared memory
    const uint16_t *lut;     // shared memory
    int64_t base;
    int32_t shift;
    int32_t nSplits;
};

__device__ __forceinline__ int PartOfKey(int64_t key, int32_t kind, int32_t bits, const RangeLut &r)
{
    if (kind == JOIN_PART_HASH) {
        return static_cast<int>(Mix64(static_cast<uint64_t>(key)) >> (64 - bits));
    }
    // upper_bound (the number of splits <= key), searched within the key's bucket: the bucket's
    // splits are [lut[b], lut[b + 1]) and every split before lut[b] is <= any key of bucket b.
    uint64_t b = key < r.base ? 0 : ((static_cast<uint64_t>(key) - static_cast<uint64_t>(r.base)) >> r.shift);
    b = b < static_cast<uint64_t>(kJoinLutBuckets) ? b : kJoinLutBuckets - 1;
    int lo = r.lut[b];
    int hi = key < r.base ? lo : r.lut[b + 1];
    const int64_t *splits = r.splits;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (splits[mid] <= key) {
            lo = mid + 1;
        } else {
            hi = mid;
        }
    }
    return lo;
}

// Stage the splits and the bucket table in shared memory (range partitioning).
constexpr size_t kRangeSmem = sizeof(int64_t) * kMaxJoinSplits + sizeof(uint16_t) * (kJoinLutBuckets + 8);

__device__ __forceinline__ RangeLut StageSplits(const JoinPartFn &f, unsigned char *smem)
{
    RangeLut r{nullptr, nullptr, f.lutBase, f.lutShift, f.nSplits};
    if (f.kind != JOIN_PART_RANGE) {
        return r;
    }
    int64_t *sSplits = reinterpret_cast<int64_t *>(smem);
    uint16_t *sLut = reinterpret_cast<uint16_t *>(smem + sizeof(int64_t) * kMaxJoinSplits);
    for (int i = threadIdx.x; i < f.nSplits; i += blockDim.x) {
        sSplits[i] = f.splits[i];
    }
    for (int i = threadIdx.x; i <= kJoinLutBuckets; i += blockDim.x) {
        sLut[i] = f.lut[i];
    }
    __syncthreads();
    r.splits = sSplits;
    r.lut = sLut;
    return r;
}

// Rows [begin, end) of chunk c of a key column.
__device__ __forceinline__ void ChunkRange(int64_t n, int32_t nChunks, int32_t c, int64_t *begin, int64_t *end)
{
    const int64_t per = (n + nChunks - 1) / nChunks;
    *begin = per * c < n ? per * c : n;
    *end = per * (c + 1) < n ? per * (c + 1) : n;
}

// hist[c * P + p] = non-NULL rows of chunk c in partition p.
__global__ void __launch_bounds__(kPartThreads) KeyHistKernel(const int64_t *keys, const uint8_t *nulls, int64_t n,
    const __grid_constant__ JoinPartFn f, int32_t nChunks, uint32_t *hist)
{
    extern __shared__ unsigned char smem[];
    unsigned int *h = reinterpret_cast<unsigned int *>(smem + kRangeSmem);
    const int P = 1 << f.bits;
    const RangeLut rl = StageSplits(f, smem);
    for (int c = blockIdx.x; c < nChunks; c += gridDim.x) {
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            h[i] = 0;
        }
        __syncthreads();
        int64_t b, e;
        ChunkRange(n, nChunks, c, &b, &e);
        // Four rows per thread per step: their loads are in flight together.
        for (int64_t r0 = b + threadIdx.x; r0 < e; r0 += 4 * static_cast<int64_t>(blockDim.x)) {
            int64_t k4[4];
            bool ok[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int64_t r = r0 + j * static_cast<int64_t>(blockDim.x);
                ok[j] = r < e && !NullRO(nulls, r);
                k4[j] = r < e ? __ldg(keys + r) : 0;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (ok[j]) {
                    atomicAdd(&h[PartOfKey(k4[j], f.kind, f.bits, rl)], 1u);
                }
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            hist[static_cast<int64_t>(c) * P + i] = h[i];
        }
        __syncthreads();
    }
}

// Partition totals and starts: total[p] = sum over chunks; start[p] = exclusive prefix of the
// totals (start[P] = all rows).  One block.
__global__ void PartTotalsKernel(const uint32_t *hist, int32_t nChunks, int32_t P, int64_t *start)
{
    __shared__ long long warpSum[32];
    __shared__ long long carry;
    if (threadIdx.x == 0) {
        carry = 0;
    }
    __syncthreads();
    for (int base = 0; base < P; base += blockDim.x) {
        const int p = base + threadIdx.x;
        long long t = 0;
        if (p < P) {
            for (int c = 0; c < nChunks; ++c) {
                t += hist[static_cast<int64_t>(c) * P + p];
            }
        }
        // block-wide exclusive scan of t
        const int lane = threadIdx.x & 31;
        const int warp = threadIdx.x >> 5;
        long long inc = t;
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) {
                inc += y;
            }
        }
        if (lane == 31) {
            warpSum[warp] = inc;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            long long run = 0;
            for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
                const long long v = warpSum[w];
                warpSum[w] = run;
                run += v;
            }
        }
        __syncthreads();
        if (p < P) {
            start[p] = carry + warpSum[warp] + inc - t;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) {
            carry += warpSum[warp] + inc;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        start[P] = carry;
    }
}

// Placement of each (chunk, partition): place[c * P + p] = start[p] + rows of partition p in
// chunks before c.  One thread per partition.
__global__ void PlaceKernel(const uint32_t *hist, int32_t nChunks, int32_t P, const int64_t *start, int64_t *place)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) {
        return;
    }
    int64_t run = start[p];
    for (int c = 0; c < nChunks; ++c) {
        place[static_cast<int64_t>(c) * P + p] = run;
        run += hist[static_cast<int64_t>(c) * P + p];
    }
}

__device__ __forceinline__ void CopyBytes(uint8_t *dst, const uint8_t *src, int bytes)
{
    if (bytes == 16) {
        *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(src);
    } else if (bytes == 8) {
        *reinterpret_cast<uint64_t *>(dst) = *reinterpret_cast<const uint64_t *>(src);
    } else {
        for (int i = 0; i < bytes; ++i) {
            dst[i] = src[i];
        }
    }
}

// Scatter of a chunk's non-NULL rows to their partitions: key, and (build side) the packed
// payload bytes of the row's output columns.
__global__ void __launch_bounds__(kPartThreads) KeyScatterKernel(const int64_t *keys, const uint8_t *nulls, int64_t n,
    const __grid_constant__ JoinPartFn f, int32_t nChunks, const int64_t *place, int64_t *outKeys,
    const __grid_constant__ PayloadCols pay, uint8_t *outPay)
{
    extern __shared__ unsigned char smem[];
    unsigned long long *cur = reinterpret_cast<unsigned long long *>(smem + kRangeSmem);
    const int P = 1 << f.bits;
    const RangeLut rl = StageSplits(f, smem);
    for (int c = blockIdx.x; c < nChunks; c += gridDim.x) {
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            cur[i] = static_cast<unsigned long long>(place[static_cast<int64_t>(c) * P + i]);
        }
        __syncthreads();
        int64_t b, e;
        ChunkRange(n, nChunks, c, &b, &e);
        for (int64_t r0 = b + threadIdx.x; r0 < e; r0 += 4 * static_cast<int64_t>(blockDim.x)) {
            int64_t k4[4];
            bool ok[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int64_t r = r0 + j * static_cast<int64_t>(blockDim.x);
                ok[j] = r < e && !NullRO(nulls, r);
                k4[j] = r < e ? __ldg(keys + r) : 0;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (!ok[j]) {
                    continue;
                }
                const int64_t r = r0 + j * static_cast<int64_t>(blockDim.x);
                const int p = PartOfKey(k4[j], f.kind, f.bits, rl);
                const unsigned long long pos = atomicAdd(&cur[p], 1ull);
                outKeys[pos] = k4[j];
                if (outPay != nullptr) {
                    int off = 0;
                    for (int k = 0; k < pay.nCols; ++k) {
                        const int w = pay.width[k];
                        CopyBytes(outPay + pos * pay.rowBytes + off, static_cast<const uint8_t *>(pay.cols[k]) + r * w,
                            w);
                        off += w;
                    }
                }
            }
        }
        __syncthreads();
    }
}

// Per partition p: an open-addressing table of capacity tabCap[p] (a power of two) at slab
// offset tabStart[p], keys (kEmptyKey = free) and the row index into the partitioned build.
// One CTA per partition.
__global__ void __launch_bounds__(256) PartTableBuildKernel(const int64_t *pkeys, const int64_t *start, int32_t P,
    const int64_t *tabStart, uint64_t *tabKeys, int32_t *tabRow, int32_t *error)
{
    for (int p = blockIdx.x; p < P; p += gridDim.x) {
        const int64_t b = start[p];
        const int64_t e = start[p + 1];
        const int64_t t0 = tabStart[p];
        const uint64_t mask = static_cast<uint64_t>(tabStart[p + 1] - t0) - 1;
        for (int64_t r = b + threadIdx.x; r < e; r += blockDim.x) {
            const uint64_t key = static_cast<uint64_t>(pkeys[r]);
            if (key == kEmptyKey) {
                SetError(error, 5);  // the EMPTY sentinel as a build key: the direct path handles it
                continue;
            }
            uint64_t i = Mix64(key) & mask;
            bool done = false;
            for (uint64_t probe = 0; probe <= mask; ++probe) {
                const unsigned long long prev = atomicCAS(reinterpret_cast<unsigned long long *>(tabKeys + t0 + i),
                    kEmptyKey, static_cast<unsigned long long>(key));
                if (prev == kEmptyKey) {
                    tabRow[t0 + i] = static_cast<int32_t>(r - b);
                    done = true;
                    break;
                }
                if (prev == key) {
                    SetError(error, 3);  // duplicate build key: not a unique build
                    done = true;
                    break;
                }
                i = (i + 1) & mask;
            }
            if (!done) {
                SetError(error, 4);
            }
        }
    }
}

__global__ void FillEmptyKernel(uint64_t *k, int64_t n)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        k[i] = kEmptyKey;
    }
}

// Probe of the partitioned probe keys: warp segments of 128 rows (4 rounds of 32), the row's
// partition recomputed from its key, lookups in that partition's table, matches compacted per
// warp into output regions (one counter per region).
constexpr int kProbeRounds = 4;

__global__ void __launch_bounds__(256) PartProbeKernel(const __grid_constant__ PartProbeLaunch q)
{
    extern __shared__ unsigned char smem[];
    const JoinPartFn &f = q.fn;
    const RangeLut rl = StageSplits(f, smem);
    const int lane = threadIdx.x & 31;
    const unsigned int lanesBelow = (1u << lane) - 1u;
    constexpr int kSegRows = kProbeRounds * 32;
    const int64_t nSegs = (q.n + kSegRows - 1) / kSegRows;
    const int64_t warpsTotal = static_cast<int64_t>(gridDim.x) * (blockDim.x / 32);
    for (int64_t seg = static_cast<int64_t>(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5); seg < nSegs;
         seg += warpsTotal) {
        const int64_t base = seg * kSegRows;
        int64_t key[kProbeRounds];
        int32_t hitRow[kProbeRounds];
        int32_t hitPart[kProbeRounds];
        uint32_t hit = 0;
#pragma unroll
        for (int i = 0; i < kProbeRounds; ++i) {
            const int64_t r = base + i * 32 + lane;
            key[i] = r < q.n ? __ldg(q.keys + r) : 0;
        }
#pragma unroll
        for (int i = 0; i < kProbeRounds; ++i) {
            const int64_t r = base + i * 32 + lane;
            hitRow[i] = -1;
            hitPart[i] = 0;
            if (r < q.n && static_cast<uint64_t>(key[i]) != kEmptyKey) {
                const int p = PartOfKey(key[i], f.kind, f.bits, rl);
                const int64_t t0 = __ldg(q.tabStart + p);
                const uint64_t mask = static_cast<uint64_t>(__ldg(q.tabStart + p + 1) - t0) - 1;
                uint64_t s = Mix64(static_cast<uint64_t>(key[i])) & mask;
                for (uint64_t probe = 0; probe <= mask; ++probe) {
                    const uint64_t k = __ldg(reinterpret_cast<const unsigned long long *>(q.tabKeys) + t0 + s);
                    if (k == static_cast<uint64_t>(key[i])) {
                        hitRow[i] = __ldg(q.tabRow + t0 + s);
                        hitPart[i] = p;
                        break;
                    }
                    if (k == kEmptyKey) {
                        break;
                    }
                    s = (s + 1) & mask;
                }
                hit |= (hitRow[i] >= 0 ? 1u : 0u) << i;
            }
        }
        uint32_t total = 0;
#pragma unroll
        for (int i = 0; i < kProbeRounds; ++i) {
            total += __popc(__ballot_sync(0xffffffffu, (hit >> i) & 1u));
        }
        const int region = static_cast<int>(seg % q.nRegions);
        unsigned long long pos = 0;
        if (lane == 0 && total != 0) {
            pos = atomicAdd(q.outCount + region * kRegionStride, static_cast<unsigned long long>(total));
        }
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (total == 0) {
            continue;
        }
        const uint64_t regionBase = static_cast<uint64_t>(region) * q.regionCap;
#pragma unroll
        for (int i = 0; i < kProbeRounds; ++i) {
            const unsigned int m = __ballot_sync(0xffffffffu, (hit >> i) & 1u);
            if ((hit >> i) & 1u) {
                const uint64_t rat = pos + __popc(m & lanesBelow);
                if (rat < q.regionCap) {
                    const uint64_t at = regionBase + rat;
                    if (q.keyOut != nullptr) {
                        q.keyOut[at] = key[i];
                    }
                    const uint8_t *src = q.pay + (__ldg(q.start + hitPart[i]) + hitRow[i]) * q.payBytes;
                    int off = 0;
                    for (int k = 0; k < q.nPayOut; ++k) {
                        const int w = q.payWidth[k];
                        CopyBytes(static_cast<uint8_t *>(q.payOut[k]) + at * w, src + off, w);
                        off += w;
                    }
                }
            }
            pos += __popc(m);
        }
    }
}

size_t SplitsSmem(const JoinPartFn &f) { return f.kind == JOIN_PART_RANGE ? kRangeSmem : 0; }

}  // namespace

cudaError_t LaunchKeyPartition(const int64_t *keys, const uint8_t *nulls, int64_t n, const JoinPartFn &f,
    int32_t nChunks, uint32_t *hist, int64_t *start, int64_t *place, int64_t *outKeys, const PayloadCols &pay,
    uint8_t *outPay, cudaStream_t stream)
{
    const int P = 1 << f.bits;
    const size_t smemHist = kRangeSmem + sizeof(unsigned int) * P;
    const size_t smemScatter = kRangeSmem + sizeof(unsigned long long) * P;
    cudaError_t err = EnsureDynamicSmem(reinterpret_cast<const void *>(KeyHistKernel), smemHist);
    if (err == cudaSuccess) {
        err = EnsureDynamicSmem(reinterpret_cast<const void *>(KeyScatterKernel), smemScatter);
    }
    if (err != cudaSuccess) {
        return err;
    }
    const int grid = nChunks < SMs() * 4 ? nChunks : SMs() * 4;
    KeyHistKernel<<<grid, kPartThreads, smemHist, stream>>>(keys, nulls, n, f, nChunks, hist);
    PartTotalsKernel<<<1, 1024, 0, stream>>>(hist, nChunks, P, start);
    PlaceKernel<<<(P + 255) / 256, 256, 0, stream>>>(hist, nChunks, P, start, place);
    KeyScatterKernel<<<grid, kPartThreads, smemScatter, stream>>>(keys, nulls, n, f, nChunks, place, outKeys, pay,
        outPay);
    return cudaGetLastError();
}

cudaError_t LaunchPartTableBuild(const int64_t *pkeys, const int64_t *start, int32_t P, const int64_t *tabStart,
    int64_t tabSlots, uint64_t *tabKeys, int32_t *tabRow, int32_t *error, cudaStream_t stream)
{
    FillEmptyKernel<<<SMs() * 4, 256, 0, stream>>>(tabKeys, tabSlots);
    PartTableBuildKernel<<<P < SMs() * 8 ? P : SMs() * 8, 256, 0, stream>>>(pkeys, start, P, tabStart, tabKeys, tabRow,
        error);
    return cudaGetLastError();
}

cudaError_t LaunchPartProbe(const PartProbeLaunch &q, cudaStream_t stream)
{
    if (q.n <= 0) {
        return cudaSuccess;
    }
    cudaError_t err = EnsureDynamicSmem(reinterpret_cast<const void *>(PartProbeKernel), kRangeSmem);
    if (err != cudaSuccess) {
        return err;
    }
    const int perSM = BlocksPerSM(reinterpret_cast<const void *>(PartProbeKernel), 256, SplitsSmem(q.fn));
    const int64_t segs = (q.n + kProbeRounds * 32 - 1) / (kProbeRounds * 32);
    const int64_t want = (segs + 7) / 8;
    const int64_t cap = static_cast<int64_t>(SMs()) * perSM;
    PartProbeKernel<<<static_cast<unsigned>(want < cap ? want : cap), 256, SplitsSmem(q.fn), stream>>>(q);
    return cudaGetLastError();
}

}  // namespace omg
