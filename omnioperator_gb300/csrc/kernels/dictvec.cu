// Dictionary-encoded input vectors (row i = row ids[i] of a flat dictionary vector,
// vector/dictionary_container.h) flattened on the device before an operator uses them: fixed-
// width values are gathered in one pass, VARCHAR/CHAR values in two (lengths, then a scan and the
// byte copy).  A row is NULL when its dictionary row is.  Every id is bounds-checked: an id
// outside [0, dictSize) sets the error word and its row becomes NULL (or empty), so a bad id
// never reads outside the dictionary.  Null bits are written a 32-bit word per warp (ballot), so
// the output bitmap needs no atomics.
#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "launch.h"

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

// The dictionary row of output row i, or -1 when the row is NULL (a NULL dictionary row, or an
// id out of range, which also sets *error).
__device__ __forceinline__ int64_t DictRow(const int32_t *ids, int64_t i, const uint8_t *dictNulls, int32_t dictSize,
    int32_t *error)
{
    const int32_t id = ids[i];
    if (id < 0 || id >= dictSize) {
        atomicExch(error, 1);
        return -1;
    }
    return RowIsNull(dictNulls, id) ? -1 : id;
}

// Rows are walked a warp (32 consecutive, aligned rows) at a time so that lane 0 can store the
// warp's null bits as one word.
__global__ void DictGatherFixedKernel(const int32_t *ids, int64_t n, const uint8_t *dictValues,
    const uint8_t *dictNulls, int32_t dictSize, int width, uint8_t *out, uint32_t *outNulls, int32_t *error)
{
    const int lane = threadIdx.x & 31;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); base < n;
         base += stride) {
        const int64_t i = base + lane;
        int64_t r = -1;
        if (i < n) {
            r = DictRow(ids, i, dictNulls, dictSize, error);
            const int64_t src = r < 0 ? 0 : r;
            switch (width) {
                case 1:
                    out[i] = r < 0 ? 0 : dictValues[src];
                    break;
                case 2:
                    reinterpret_cast<uint16_t *>(out)[i] = r < 0 ? 0 : reinterpret_cast<const uint16_t *>(dictValues)[src];
                    break;
                case 4:
                    reinterpret_cast<uint32_t *>(out)[i] = r < 0 ? 0 : reinterpret_cast<const uint32_t *>(dictValues)[src];
                    break;
                case 8:
                    reinterpret_cast<uint64_t *>(out)[i] = r < 0 ? 0 : reinterpret_cast<const uint64_t *>(dictValues)[src];
                    break;
                default: {
                    ulonglong2 v = make_ulonglong2(0, 0);
                    if (r >= 0) {
                        v = reinterpret_cast<const ulonglong2 *>(dictValues)[src];
                    }
                    reinterpret_cast<ulonglong2 *>(out)[i] = v;
                    break;
                }
            }
        }
        const unsigned int nullBits = __ballot_sync(0xffffffffu, i < n && r < 0);
        if (lane == 0) {
            outNulls[base >> 5] = nullBits;
        }
    }
}

__global__ void DictGatherLensKernel(const int32_t *ids, int64_t n, const int32_t *dictOffs, const uint8_t *dictNulls,
    int32_t dictSize, uint32_t *lens, uint32_t *outNulls, int32_t *error)
{
    const int lane = threadIdx.x & 31;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); base < n;
         base += stride) {
        const int64_t i = base + lane;
        int64_t r = -1;
        if (i < n) {
            r = DictRow(ids, i, dictNulls, dictSize, error);
            lens[i] = r < 0 ? 0u : static_cast<uint32_t>(dictOffs[r + 1] - dictOffs[r]);
        }
        const unsigned int nullBits = __ballot_sync(0xffffffffu, i < n && r < 0);
        if (lane == 0) {
            outNulls[base >> 5] = nullBits;
        }
    }
}

__global__ void DictGatherCharsKernel(const int32_t *ids, int64_t n, const int32_t *dictOffs,
    const uint8_t *dictChars, const uint8_t *dictNulls, int32_t dictSize, const int64_t *offs64, uint8_t *chars,
    int32_t *offs32, long long total)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        offs32[i] = static_cast<int32_t>(offs64[i]);
        const int32_t id = ids[i];
        if (id >= 0 && id < dictSize && !RowIsNull(dictNulls, id)) {
            const uint8_t *src = dictChars + dictOffs[id];
            const int64_t len = dictOffs[id + 1] - dictOffs[id];
            uint8_t *dst = chars + offs64[i];
            for (int64_t j = 0; j < len; ++j) {
                dst[j] = src[j];
            }
        }
        if (i == n - 1) {
            offs32[n] = static_cast<int32_t>(total);
        }
    }
}

}  // namespace

cudaError_t LaunchDictGatherFixed(const int32_t *ids, int64_t n, const uint8_t *dictValues, const uint8_t *dictNulls,
    int32_t dictSize, int width, uint8_t *out, uint32_t *outNulls, int32_t *error, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    DictGatherFixedKernel<<<Grid(n, 256), 256, 0, stream>>>(ids, n, dictValues, dictNulls, dictSize, width, out,
        outNulls, error);
    return cudaGetLastError();
}

cudaError_t LaunchDictGatherLens(const int32_t *ids, int64_t n, const int32_t *dictOffs, const uint8_t *dictNulls,
    int32_t dictSize, uint32_t *lens, uint32_t *outNulls, int32_t *error, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    DictGatherLensKernel<<<Grid(n, 256), 256, 0, stream>>>(ids, n, dictOffs, dictNulls, dictSize, lens, outNulls,
        error);
    return cudaGetLastError();
}

cudaError_t LaunchDictGatherChars(const int32_t *ids, int64_t n, const int32_t *dictOffs, const uint8_t *dictChars,
    const uint8_t *dictNulls, int32_t dictSize, const int64_t *offs64, uint8_t *chars, int32_t *offs32,
    long long total, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    DictGatherCharsKernel<<<Grid(n, 256), 256, 0, stream>>>(ids, n, dictOffs, dictChars, dictNulls, dictSize, offs64,
        chars, offs32, total);
    return cudaGetLastError();
}

}  // namespace omg
