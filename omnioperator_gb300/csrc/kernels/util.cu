// Order-independent fingerprint of the rows of a batch list (for checking that two operator
// runs produced the same row multiset without copying the rows out).
#include <cstdint>
#include <cuda_runtime.h>

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

}  // namespace

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
