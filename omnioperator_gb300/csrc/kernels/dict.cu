// String dictionary for VARCHAR group-by keys: every distinct string of a column gets a dense
// int32 id that stays the same for the life of the operator, so the aggregation runs on ids
// and the strings come back at output time.
//
// The dictionary is an open-addressing table of (hash, id) slots plus an arena holding each
// id's characters.  Insertion needs no waiting: a row claims a free slot by CAS on the hash
// word, and the first row to reach a slot of the current batch set becomes its representative
// by CAS on the slot's representative word; every other row with that hash compares its bytes
// with the representative's (or, for a slot from an earlier batch set, with the arena copy)
// and moves on along the probe sequence when they differ.  With linear probing and no
// deletions, equal strings always stop at the same slot.  New slots get ids and their
// characters are appended to the arena by the host after the insert kernel.
#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "launch.h"
#include "plan.h"

namespace omg {
namespace {

constexpr uint64_t kDictEmpty = ~0ull;
constexpr unsigned long long kNoRep = ~0ull;

unsigned Grid(int64_t n, int threads)
{
    int64_t blocks = (n + threads - 1) / threads;
    const int64_t cap = static_cast<int64_t>(DeviceSMCount()) * 8;
    if (blocks > cap) {
        blocks = cap;
    }
    return static_cast<unsigned>(blocks < 1 ? 1 : blocks);
}

__device__ __forceinline__ uint64_t StringHash(const uint8_t *p, int64_t len)
{
    const uint64_t h = KeyTupleBytes(1, p, len);
    return h == kDictEmpty ? kDictEmpty - 1 : h;
}

__device__ __forceinline__ bool SameBytes(const uint8_t *a, int64_t la, const uint8_t *b, int64_t lb)
{
    if (la != lb) {
        return false;
    }
    for (int64_t i = 0; i < la; ++i) {
        if (a[i] != b[i]) {
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void RowString(const BatchDesc *batches, int32_t input, unsigned long long handle,
    const uint8_t *&p, int64_t &len)
{
    const BatchDesc &b = batches[handle >> 32];
    const int64_t row = static_cast<int64_t>(handle & 0xffffffffull);
    const int32_t *offs = b.offs[input];
    p = static_cast<const uint8_t *>(b.cols[input]) + offs[row];
    len = offs[row + 1] - offs[row];
}

__global__ void DictInsertKernel(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, int32_t input, unsigned long long *hash, const int32_t *id, unsigned long long *rep,
    uint64_t cap, const int64_t *arenaOff, const uint8_t *arena, int32_t *rowSlot, int32_t *error)
{
    const uint64_t mask = cap - 1;
    for (int t = blockIdx.x; t < nTiles; t += gridDim.x) {
        const TileDesc tile = tiles[t];
        const BatchDesc &b = batches[tile.batch];
        for (int r = threadIdx.x; r < tile.rows; r += blockDim.x) {
            const int64_t row = static_cast<int64_t>(tile.row0) + r;
            const int64_t out = tileOutRow[t] + r;
            if (RowIsNull(b.nulls[input], row)) {
                rowSlot[out] = -1;
                continue;
            }
            const unsigned long long mine = (static_cast<unsigned long long>(tile.batch) << 32) |
                static_cast<unsigned long long>(row);
            const int32_t *offs = b.offs[input];
            const uint8_t *p = static_cast<const uint8_t *>(b.cols[input]) + offs[row];
            const int64_t len = offs[row + 1] - offs[row];
            const uint64_t h = StringHash(p, len);
            uint64_t i = Mix64(h) & mask;
            int64_t found = -1;
            for (uint64_t n = 0; n < cap; ++n, i = (i + 1) & mask) {
                unsigned long long s = hash[i];
                if (s == kDictEmpty) {
                    s = atomicCAS(hash + i, kDictEmpty, static_cast<unsigned long long>(h));
                    if (s == kDictEmpty) {
                        s = h;
                    }
                }
                if (s != h) {
                    continue;
                }
                const int32_t sid = id[i];
                if (sid >= 0) {  // a string of an earlier batch set: compare with its arena copy
                    if (SameBytes(p, len, arena + arenaOff[sid], arenaOff[sid + 1] - arenaOff[sid])) {
                        found = static_cast<int64_t>(i);
                        break;
                    }
                    continue;
                }
                const unsigned long long prev = atomicCAS(rep + i, kNoRep, mine);
                const unsigned long long other = prev == kNoRep ? mine : prev;
                if (other != mine) {
                    const uint8_t *q;
                    int64_t lq;
                    RowString(batches, input, other, q, lq);
                    if (!SameBytes(p, len, q, lq)) {
                        continue;
                    }
                }
                found = static_cast<int64_t>(i);
                break;
            }
            if (found < 0) {
                atomicExch(error, 1);  // the table is sized so that this cannot happen
            }
            rowSlot[out] = static_cast<int32_t>(found);
        }
    }
}

// Slots claimed in this batch set: new ids, their representatives and string lengths.
__global__ void DictMaterializeKernel(const unsigned long long *hash, int32_t *id, const unsigned long long *rep,
    uint64_t cap, int32_t firstId, unsigned int *counter, unsigned long long *newRep, uint32_t *newLen,
    const BatchDesc *batches, int32_t input)
{
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < cap;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        if (hash[i] == kDictEmpty || id[i] >= 0 || rep[i] == kNoRep) {
            continue;
        }
        const unsigned int k = atomicAdd(counter, 1u);
        id[i] = firstId + static_cast<int32_t>(k);
        newRep[k] = rep[i];
        const uint8_t *q;
        int64_t lq;
        RowString(batches, input, rep[i], q, lq);
        newLen[k] = static_cast<uint32_t>(lq);
    }
}

// Characters of the new ids into the arena at offsets arenaOff[firstId + k].
__global__ void DictAppendKernel(const unsigned long long *newRep, int64_t nNew, int32_t firstId,
    const int64_t *arenaOff, uint8_t *arena, const BatchDesc *batches, int32_t input)
{
    for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < nNew;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const uint8_t *q;
        int64_t lq;
        RowString(batches, input, newRep[k], q, lq);
        uint8_t *d = arena + arenaOff[firstId + k];
        for (int64_t j = 0; j < lq; ++j) {
            d[j] = q[j];
        }
    }
}

// Move every slot of a smaller table (all materialised) into a larger empty one.
__global__ void DictRehashKernel(const unsigned long long *oldHash, const int32_t *oldId, uint64_t oldCap,
    unsigned long long *hash, int32_t *id, uint64_t cap, int32_t *error)
{
    const uint64_t mask = cap - 1;
    for (uint64_t j = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; j < oldCap;
         j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const unsigned long long h = oldHash[j];
        if (h == kDictEmpty) {
            continue;
        }
        uint64_t i = Mix64(h) & mask;
        bool placed = false;
        for (uint64_t n = 0; n < cap; ++n, i = (i + 1) & mask) {
            if (atomicCAS(hash + i, kDictEmpty, h) == kDictEmpty) {
                id[i] = oldId[j];
                placed = true;
                break;
            }
        }
        if (!placed) {
            atomicExch(error, 1);
        }
    }
}

// offs[k] (k = 0..nNew, exclusive offsets of the new strings) shifted by the arena's size.
__global__ void DictShiftOffsetsKernel(const int64_t *offs, int64_t nNew, int64_t base, int64_t *arenaOff)
{
    for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k <= nNew;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        arenaOff[k] = base + offs[k];
    }
}

__global__ void DictRowIdsKernel(const int32_t *rowSlot, int64_t n, const int32_t *id, int32_t *ids)
{
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t s = rowSlot[r];
        ids[r] = s >= 0 ? id[s] : 0;
    }
}

__global__ void DictDecodeLensKernel(const int32_t *ids, const uint8_t *nulls, int64_t n, const int64_t *arenaOff,
    uint32_t *lens)
{
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t k = ids[r];
        lens[r] = RowIsNull(nulls, r) ? 0u : static_cast<uint32_t>(arenaOff[k + 1] - arenaOff[k]);
    }
}

__global__ void DictDecodeCopyKernel(const int32_t *ids, const uint8_t *nulls, int64_t n, const int64_t *arenaOff,
    const uint8_t *arena, const int64_t *offs64, uint8_t *chars, int32_t *offs32, long long total)
{
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        offs32[r] = static_cast<int32_t>(offs64[r]);
        if (!RowIsNull(nulls, r)) {
            const int32_t k = ids[r];
            const int64_t len = arenaOff[k + 1] - arenaOff[k];
            for (int64_t j = 0; j < len; ++j) {
                chars[offs64[r] + j] = arena[arenaOff[k] + j];
            }
        }
        if (r == n - 1) {
            offs32[n] = static_cast<int32_t>(total);
        }
    }
}

}  // namespace

cudaError_t LaunchDictInsert(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles, const int64_t *tileOutRow,
    int32_t input, unsigned long long *hash, const int32_t *id, unsigned long long *rep, uint64_t cap,
    const int64_t *arenaOff, const uint8_t *arena, int32_t *rowSlot, int32_t *error, cudaStream_t stream)
{
    if (nTiles <= 0) {
        return cudaSuccess;
    }
    DictInsertKernel<<<Grid(static_cast<int64_t>(nTiles) * 256, 256), 256, 0, stream>>>(batches, tiles, nTiles,
        tileOutRow, input, hash, id, rep, cap, arenaOff, arena, rowSlot, error);
    return cudaGetLastError();
}

cudaError_t LaunchDictMaterialize(const unsigned long long *hash, int32_t *id, const unsigned long long *rep,
    uint64_t cap, int32_t firstId, unsigned int *counter, unsigned long long *newRep, uint32_t *newLen,
    const BatchDesc *batches, int32_t input, cudaStream_t stream)
{
    DictMaterializeKernel<<<Grid(static_cast<int64_t>(cap), 256), 256, 0, stream>>>(hash, id, rep, cap, firstId,
        counter, newRep, newLen, batches, input);
    return cudaGetLastError();
}

cudaError_t LaunchDictAppend(const unsigned long long *newRep, int64_t nNew, int32_t firstId, const int64_t *arenaOff,
    uint8_t *arena, const BatchDesc *batches, int32_t input, cudaStream_t stream)
{
    if (nNew <= 0) {
        return cudaSuccess;
    }
    DictAppendKernel<<<Grid(nNew, 256), 256, 0, stream>>>(newRep, nNew, firstId, arenaOff, arena, batches, input);
    return cudaGetLastError();
}

cudaError_t LaunchDictRehash(const unsigned long long *oldHash, const int32_t *oldId, uint64_t oldCap,
    unsigned long long *hash, int32_t *id, uint64_t cap, int32_t *error, cudaStream_t stream)
{
    if (oldCap == 0) {
        return cudaSuccess;
    }
    DictRehashKernel<<<Grid(static_cast<int64_t>(oldCap), 256), 256, 0, stream>>>(oldHash, oldId, oldCap, hash, id,
        cap, error);
    return cudaGetLastError();
}

cudaError_t LaunchDictShiftOffsets(const int64_t *offs, int64_t nNew, int64_t base, int64_t *arenaOff,
    cudaStream_t stream)
{
    DictShiftOffsetsKernel<<<Grid(nNew + 1, 256), 256, 0, stream>>>(offs, nNew, base, arenaOff);
    return cudaGetLastError();
}

cudaError_t LaunchDictRowIds(const int32_t *rowSlot, int64_t n, const int32_t *id, int32_t *ids, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    DictRowIdsKernel<<<Grid(n, 256), 256, 0, stream>>>(rowSlot, n, id, ids);
    return cudaGetLastError();
}

cudaError_t LaunchDictDecodeLens(const int32_t *ids, const uint8_t *nulls, int64_t n, const int64_t *arenaOff,
    uint32_t *lens, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    DictDecodeLensKernel<<<Grid(n, 256), 256, 0, stream>>>(ids, nulls, n, arenaOff, lens);
    return cudaGetLastError();
}

cudaError_t LaunchDictDecodeCopy(const int32_t *ids, const uint8_t *nulls, int64_t n, const int64_t *arenaOff,
    const uint8_t *arena, const int64_t *offs64, uint8_t *chars, int32_t *offs32, long long total,
    cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    DictDecodeCopyKernel<<<Grid(n, 256), 256, 0, stream>>>(ids, nulls, n, arenaOff, arena, offs64, chars, offs32,
        total);
    return cudaGetLastError();
}

}  // namespace omg
