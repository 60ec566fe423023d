// Order-independent fingerprint of the rows of a batch list (for checking that two operator
// runs produced the same row multiset without copying the rows out).
#include <cstdint>
#include <cuda_runtime.h>
#include <map>
#include <mutex>
#include <tuple>

#include "device_common.cuh"
#include "launch.h"
#include "plan.h"

namespace omg {
namespace {

// Per row: h = Mix64 chain over the columns (value bits, NULL as a tag); out[0] += 1,
// out[1] += Mix64(h), out[2] += Mix64(h ^ c) — sums, so the row order does not matter.
__global__ void FingerprintKernel(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles, int32_t nCols,
    const int32_t *widths, unsigned long long *out)
{
    unsigned long long cnt = 0, f1 = 0, f2 = 0;
    for (int t = blockIdx.x; t < nTiles; t += gridDim.x) {
        const TileDesc tile = tiles[t];
        const BatchDesc &b = batches[tile.batch];
        for (int r = threadIdx.x; r < tile.rows; r += blockDim.x) {
            const int64_t row = static_cast<int64_t>(tile.row0) + r;
            uint64_t h = 0x243f6a8885a308d3ull;
            for (int c = 0; c < nCols; ++c) {
                const int w = widths[c];
                if (NullRO(b.nulls[c], row)) {
                    h = Mix64(h ^ 0x9e3779b97f4a7c15ull ^ static_cast<uint64_t>(c));
                    continue;
                }
                if (w == 16) {
                    const uint64_t *v = static_cast<const uint64_t *>(b.cols[c]) + 2 * row;
                    h = Mix64(h ^ v[0]);
                    h = Mix64(h ^ v[1]);
                } else {
                    h = Mix64(h ^ LoadBitsRO(b.cols[c], row, w));
                }
            }
            ++cnt;
            f1 += Mix64(h);
            f2 += Mix64(h ^ 0xc2b2ae3d27d4eb4full);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
        f1 += __shfl_down_sync(0xffffffffu, f1, o);
        f2 += __shfl_down_sync(0xffffffffu, f2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], cnt);
        atomicAdd(&out[1], f1);
        atomicAdd(&out[2], f2);
    }
}

// One warp per 32-row word of one job: lane l decides row 32w + l, the ballot is the word.
__global__ void MaskNullsKernel(const MaskJob *jobs, int32_t nJobs)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.y) * blockDim.x + threadIdx.x) >> 5;
    const int64_t warps = (static_cast<int64_t>(gridDim.y) * blockDim.x) >> 5;
    for (int j = blockIdx.x; j < nJobs; j += gridDim.x) {
        const MaskJob job = jobs[j];
        const int64_t words = (job.rows + 31) >> 5;
        for (int64_t w = warp; w < words; w += warps) {
            const int64_t row = (w << 5) + lane;
            bool skip = false;
            if (row < job.rows) {
                bool drop;
                if (job.mode == 2) {
                    drop = NullRO(job.maskNulls, row);
                } else {
                    const uint8_t m = __ldg(job.maskValues + row);
                    drop = job.mode == 1 ? m != 0 : (m == 0 || NullRO(job.maskNulls, row));
                }
                skip = drop || NullRO(job.valueNulls, row);
            }
            const unsigned bits = __ballot_sync(0xffffffffu, skip);
            if (lane == 0) {
                job.out[w] = bits;
            }
        }
    }
}

std::mutex g_attrMutex;
// (device, kernel) -> dynamic shared-memory limit set so far.
std::map<std::tuple<int, const void *>, size_t> g_smemSet;
// (device, kernel, threads, bytes) -> CTAs per SM.
std::map<std::tuple<int, const void *, int, size_t>, int> g_blocksPerSM;
std::map<int, int> g_smCount;

int CurrentDevice()
{
    int dev = 0;
    cudaGetDevice(&dev);
    return dev;
}

}  // namespace

int DeviceSMCount()
{
    const int dev = CurrentDevice();
    std::lock_guard<std::mutex> lock(g_attrMutex);
    auto it = g_smCount.find(dev);
    if (it != g_smCount.end()) {
        return it->second;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 1;
    }
    g_smCount[dev] = n;
    return n;
}

cudaError_t EnsureDynamicSmem(const void *kernel, size_t bytes)
{
    if (bytes <= 48 * 1024) {
        return cudaSuccess;
    }
    const auto key = std::make_tuple(CurrentDevice(), kernel);
    std::lock_guard<std::mutex> lock(g_attrMutex);
    auto it = g_smemSet.find(key);
    if (it != g_smemSet.end() && it->second >= bytes) {
        return cudaSuccess;
    }
    const cudaError_t err =
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
    if (err == cudaSuccess) {
        g_smemSet[key] = bytes;
    }
    return err;
}

int BlocksPerSM(const void *kernel, int threads, size_t smemBytes)
{
    const auto key = std::make_tuple(CurrentDevice(), kernel, threads, smemBytes);
    {
        std::lock_guard<std::mutex> lock(g_attrMutex);
        auto it = g_blocksPerSM.find(key);
        if (it != g_blocksPerSM.end()) {
            return it->second;
        }
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smemBytes) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    n = n > 0 ? n : 1;
    std::lock_guard<std::mutex> lock(g_attrMutex);
    g_blocksPerSM[key] = n;
    return n;
}

cudaError_t LaunchMaskNulls(const MaskJob *jobs, int32_t nJobs, cudaStream_t stream)
{
    if (nJobs <= 0) {
        return cudaSuccess;
    }
    const dim3 grid(static_cast<unsigned>(nJobs < 65535 ? nJobs : 65535), 8);
    MaskNullsKernel<<<grid, 256, 0, stream>>>(jobs, nJobs);
    return cudaGetLastError();
}

cudaError_t LaunchFingerprint(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles, int32_t nCols,
    const int32_t *widths, unsigned long long *out, cudaStream_t stream)
{
    cudaError_t err = cudaMemsetAsync(out, 0, 3 * sizeof(unsigned long long), stream);
    if (err != cudaSuccess || nTiles <= 0) {
        return err;
    }
    const int grid = nTiles < DeviceSMCount() * 8 ? nTiles : DeviceSMCount() * 8;
    FingerprintKernel<<<grid, 256, 0, stream>>>(batches, tiles, nTiles, nCols, widths, out);
    return cudaGetLastError();
}

}  // namespace omg
