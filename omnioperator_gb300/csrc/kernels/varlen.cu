// VARCHAR / CHAR columns (the LargeStringContainer layout: n + 1 int32 offsets into a character
// buffer, vector/vector.h) in the join: build columns gathered into one contiguous column with
// 64-bit offsets, and output columns materialised from per-row handles in two passes (lengths,
// then a scan and the byte copy).  Strings are moved with one thread per row: they are short
// next to a tile, and the rows of a warp copy to adjacent output bytes.
#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "launch.h"
#include "plan.h"

namespace omg {
namespace {

unsigned Grid(int64_t n, int threads)
{
    int64_t blocks = (n + threads - 1) / threads;
    const int64_t cap = static_cast<int64_t>(DeviceSMCount()) * 8;
    if (blocks > cap) {
        blocks = cap;
    }
    return static_cast<unsigned>(blocks < 1 ? 1 : blocks);
}

__device__ __forceinline__ void CopyBytes(uint8_t *dst, const uint8_t *src, int64_t len)
{
    for (int64_t i = 0; i < len; ++i) {
        dst[i] = src[i];
    }
}

// Lengths of a batch VARCHAR input, in tile output order.
__global__ void VarlenTileLensKernel(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, int32_t input, uint32_t *lens)
{
    for (int t = blockIdx.x; t < nTiles; t += gridDim.x) {
        const TileDesc tile = tiles[t];
        const BatchDesc &b = batches[tile.batch];
        const int32_t *offs = b.offs[input];
        for (int r = threadIdx.x; r < tile.rows; r += blockDim.x) {
            const int64_t row = static_cast<int64_t>(tile.row0) + r;
            lens[tileOutRow[t] + r] = static_cast<uint32_t>(offs[row + 1] - offs[row]);
        }
    }
}

// Characters of a batch VARCHAR input to positions `dstOffs` (tile output order).
__global__ void VarlenTileCopyKernel(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, int32_t input, const int64_t *dstOffs, uint8_t *dst)
{
    for (int t = blockIdx.x; t < nTiles; t += gridDim.x) {
        const TileDesc tile = tiles[t];
        const BatchDesc &b = batches[tile.batch];
        const int32_t *offs = b.offs[input];
        const uint8_t *chars = static_cast<const uint8_t *>(b.cols[input]);
        for (int r = threadIdx.x; r < tile.rows; r += blockDim.x) {
            const int64_t row = static_cast<int64_t>(tile.row0) + r;
            const int64_t o = tileOutRow[t] + r;
            CopyBytes(dst + dstOffs[o], chars + offs[row], offs[row + 1] - offs[row]);
        }
    }
}

// Source string of output position i: a probe-row handle (batch << 32 | row), a build row, or
// -1 (NULL, no characters).
__device__ __forceinline__ void HandleSource(const int64_t *handles, int64_t i, int side, const BatchDesc *batches,
    int32_t input, const int64_t *buildOffs, const uint8_t *buildChars, const uint8_t *&src, int64_t &len)
{
    const int64_t h = handles[i];
    src = nullptr;
    len = 0;
    if (h < 0) {
        return;
    }
    if (side == 0) {
        const BatchDesc &b = batches[h >> 32];
        const int64_t row = h & 0xffffffffll;
        const int32_t *offs = b.offs[input];
        src = static_cast<const uint8_t *>(b.cols[input]) + offs[row];
        len = offs[row + 1] - offs[row];
    } else {
        src = buildChars + buildOffs[h];
        len = buildOffs[h + 1] - buildOffs[h];
    }
}

// Output positions are regions of `regionCap` rows; only the first regionCounts[r] rows of
// region r are rows (the rest contribute no characters).
__global__ void VarlenOutLensKernel(const int64_t *handles, int64_t nPos, uint64_t regionCap,
    const unsigned long long *regionCounts, int side, const BatchDesc *batches, int32_t input,
    const int64_t *buildOffs, uint32_t *lens)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nPos;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const uint64_t r = static_cast<uint64_t>(i) / regionCap;
        const uint64_t k = static_cast<uint64_t>(i) % regionCap;
        uint32_t len = 0;
        if (k < regionCounts[r * kRegionStride]) {
            const uint8_t *src;
            int64_t l;
            HandleSource(handles, i, side, batches, input, buildOffs, nullptr, src, l);
            len = static_cast<uint32_t>(l);
        }
        lens[i] = len;
    }
}

__global__ void VarlenOutCopyKernel(const int64_t *handles, int64_t nPos, uint64_t regionCap,
    const unsigned long long *regionCounts, int side, const BatchDesc *batches, int32_t input,
    const int64_t *buildOffs, const uint8_t *buildChars, const int64_t *offs64, uint8_t *chars, int32_t *offs32,
    long long total)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nPos;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const uint64_t r = static_cast<uint64_t>(i) / regionCap;
        const uint64_t k = static_cast<uint64_t>(i) % regionCap;
        offs32[i] = static_cast<int32_t>(offs64[i]);
        if (k < regionCounts[r * kRegionStride]) {
            const uint8_t *src;
            int64_t len;
            HandleSource(handles, i, side, batches, input, buildOffs, buildChars, src, len);
            if (len > 0) {
                CopyBytes(chars + offs64[i], src, len);
            }
        }
        if (i == nPos - 1) {
            offs32[nPos] = static_cast<int32_t>(total);
        }
    }
}

// Rows `rows[i]` of a contiguous build VARCHAR column (64-bit offsets).
__global__ void VarlenRowsLensKernel(const int32_t *rows, int64_t n, const int64_t *srcOffs, uint32_t *lens)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t r = rows[i];
        lens[i] = static_cast<uint32_t>(srcOffs[r + 1] - srcOffs[r]);
    }
}

__global__ void VarlenRowsCopyKernel(const int32_t *rows, int64_t n, const int64_t *srcOffs, const uint8_t *srcChars,
    const int64_t *offs64, uint8_t *chars, int32_t *offs32, long long total)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t r = rows[i];
        offs32[i] = static_cast<int32_t>(offs64[i]);
        CopyBytes(chars + offs64[i], srcChars + srcOffs[r], srcOffs[r + 1] - srcOffs[r]);
        if (i == n - 1) {
            offs32[n] = static_cast<int32_t>(total);
        }
    }
}

// Exclusive offsets (n + 1 entries, the last the total) of 64-bit lengths given as u32.
__global__ void OffsetsTailKernel(int64_t *offs, int64_t n, const long long *total)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        offs[n] = *total;
    }
}

}  // namespace

cudaError_t LaunchVarlenTileLens(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, int32_t input, uint32_t *lens, cudaStream_t stream)
{
    if (nTiles <= 0) {
        return cudaSuccess;
    }
    VarlenTileLensKernel<<<Grid(static_cast<int64_t>(nTiles) * 256, 256), 256, 0, stream>>>(batches, tiles, nTiles,
        tileOutRow, input, lens);
    return cudaGetLastError();
}

cudaError_t LaunchVarlenTileCopy(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, int32_t input, const int64_t *dstOffs, uint8_t *dst, cudaStream_t stream)
{
    if (nTiles <= 0) {
        return cudaSuccess;
    }
    VarlenTileCopyKernel<<<Grid(static_cast<int64_t>(nTiles) * 256, 256), 256, 0, stream>>>(batches, tiles, nTiles,
        tileOutRow, input, dstOffs, dst);
    return cudaGetLastError();
}

cudaError_t LaunchVarlenOutLens(const int64_t *handles, int64_t nPos, uint64_t regionCap,
    const unsigned long long *regionCounts, int side, const BatchDesc *batches, int32_t input,
    const int64_t *buildOffs, uint32_t *lens, cudaStream_t stream)
{
    if (nPos <= 0) {
        return cudaSuccess;
    }
    VarlenOutLensKernel<<<Grid(nPos, 256), 256, 0, stream>>>(handles, nPos, regionCap, regionCounts, side, batches,
        input, buildOffs, lens);
    return cudaGetLastError();
}

cudaError_t LaunchVarlenOutCopy(const int64_t *handles, int64_t nPos, uint64_t regionCap,
    const unsigned long long *regionCounts, int side, const BatchDesc *batches, int32_t input,
    const int64_t *buildOffs, const uint8_t *buildChars, const int64_t *offs64, uint8_t *chars, int32_t *offs32,
    long long total, cudaStream_t stream)
{
    if (nPos <= 0) {
        return cudaSuccess;
    }
    VarlenOutCopyKernel<<<Grid(nPos, 256), 256, 0, stream>>>(handles, nPos, regionCap, regionCounts, side, batches,
        input, buildOffs, buildChars, offs64, chars, offs32, total);
    return cudaGetLastError();
}

cudaError_t LaunchVarlenRowsLens(const int32_t *rows, int64_t n, const int64_t *srcOffs, uint32_t *lens,
    cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    VarlenRowsLensKernel<<<Grid(n, 256), 256, 0, stream>>>(rows, n, srcOffs, lens);
    return cudaGetLastError();
}

cudaError_t LaunchVarlenRowsCopy(const int32_t *rows, int64_t n, const int64_t *srcOffs, const uint8_t *srcChars,
    const int64_t *offs64, uint8_t *chars, int32_t *offs32, long long total, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    VarlenRowsCopyKernel<<<Grid(n, 256), 256, 0, stream>>>(rows, n, srcOffs, srcChars, offs64, chars, offs32, total);
    return cudaGetLastError();
}

cudaError_t LaunchOffsetsTail(int64_t *offs, int64_t n, const long long *total, cudaStream_t stream)
{
    OffsetsTailKernel<<<1, 32, 0, stream>>>(offs, n, total);
    return cudaGetLastError();
}

}  // namespace omg
