// Device helpers shared by the aggregation and join kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "plan.h"

namespace omg {

// 64-bit finaliser of MurmurHash3 (public domain, Austin Appleby): a bijective mix, so
// distinct keys never collide in the 64-bit hash, only in the slot index.
__device__ __forceinline__ uint64_t Mix64(uint64_t k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

__device__ __forceinline__ bool RowIsNull(const uint8_t *nulls, int64_t row)
{
    return nulls != nullptr && ((nulls[row >> 3] >> (row & 7)) & 1u);
}

// Load an integer-like value of `width` bytes, sign-extended to int64.
__device__ __forceinline__ int64_t LoadInt(const void *col, int64_t row, int width)
{
    switch (width) {
        case 1:
            return static_cast<const int8_t *>(col)[row];
        case 2:
            return static_cast<const int16_t *>(col)[row];
        case 4:
            return static_cast<const int32_t *>(col)[row];
        default:
            return static_cast<const int64_t *>(col)[row];
    }
}

// Unsigned bit pattern of a value of `width` bytes (no sign extension), for packed keys.
__device__ __forceinline__ uint64_t LoadBits(const void *col, int64_t row, int width)
{
    switch (width) {
        case 1:
            return static_cast<const uint8_t *>(col)[row];
        case 2:
            return static_cast<const uint16_t *>(col)[row];
        case 4:
            return static_cast<const uint32_t *>(col)[row];
        default:
            return static_cast<const uint64_t *>(col)[row];
    }
}

// Read-only (non-coherent path) loads of input columns the kernels never write.
__device__ __forceinline__ uint64_t LoadBitsRO(const void *col, int64_t row, int width)
{
    switch (width) {
        case 1:
            return static_cast<uint8_t>(__ldg(static_cast<const char *>(col) + row));
        case 2:
            return static_cast<uint16_t>(__ldg(static_cast<const short *>(col) + row));
        case 4:
            return static_cast<uint32_t>(__ldg(static_cast<const int *>(col) + row));
        default:
            return static_cast<uint64_t>(__ldg(static_cast<const long long *>(col) + row));
    }
}

__device__ __forceinline__ bool NullRO(const uint8_t *nulls, int64_t row)
{
    return nulls != nullptr && ((__ldg(reinterpret_cast<const unsigned char *>(nulls) + (row >> 3)) >> (row & 7)) & 1u);
}

__device__ __forceinline__ int64_t SignExtend(uint64_t bits, int width)
{
    switch (width) {
        case 1:
            return static_cast<int8_t>(bits);
        case 2:
            return static_cast<int16_t>(bits);
        case 4:
            return static_cast<int32_t>(bits);
        default:
            return static_cast<int64_t>(bits);
    }
}

__device__ __forceinline__ double LoadAsDouble(const void *col, int64_t row, int inKind, int width)
{
    if (inKind == IN_DOUBLE) {
        return static_cast<const double *>(col)[row];
    }
    if (inKind == IN_FLOAT) {
        return static_cast<double>(static_cast<const float *>(col)[row]);
    }
    return static_cast<double>(LoadInt(col, row, width));
}

__device__ __forceinline__ double LoadAsDoubleRO(const void *col, int64_t row, int inKind, int width)
{
    if (inKind == IN_DOUBLE) {
        return __ldg(static_cast<const double *>(col) + row);
    }
    if (inKind == IN_FLOAT) {
        return static_cast<double>(__ldg(static_cast<const float *>(col) + row));
    }
    return static_cast<double>(SignExtend(LoadBitsRO(col, row, width), width));
}

// One step of the hash of a join key tuple; build and probe sides feed the same value bits
// (zero-extended, 16-byte values as two words) in key-column order.
__device__ __forceinline__ uint64_t KeyTupleStep(uint64_t h, uint64_t v)
{
    return Mix64(h ^ (v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2)));
}

// A VARCHAR value in a key tuple hash: its length, then its bytes as little-endian 8-byte words
// (the last zero-padded).
__device__ __forceinline__ uint64_t KeyTupleBytes(uint64_t h, const uint8_t *p, int64_t len)
{
    h = KeyTupleStep(h, static_cast<uint64_t>(len));
    for (int64_t i = 0; i < len; i += 8) {
        uint64_t v = 0;
        const int64_t m = len - i < 8 ? len - i : 8;
        for (int64_t j = 0; j < m; ++j) {
            v |= static_cast<uint64_t>(p[i + j]) << (8 * j);
        }
        h = KeyTupleStep(h, v);
    }
    return h;
}

// Order-preserving map of a non-NaN double onto int64 (-0.0 sorts just below +0.0).
__device__ __forceinline__ int64_t OrderedFromDouble(double x)
{
    int64_t b = __double_as_longlong(x);
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}
__device__ __forceinline__ double DoubleFromOrdered(int64_t k)
{
    return __longlong_as_double(k >= 0 ? k : (k ^ 0x7fffffffffffffffll));
}

// Exact multi-word unsigned accumulation by 64-bit atomics.  Each atomicAdd returns the
// word's previous value, so the adding thread knows whether its own addition carried and
// forwards exactly that carry: the final words equal the exact sum whatever the order.
__device__ __forceinline__ void AtomicAddU128(uint64_t *w, uint64_t lo, uint64_t hi)
{
    unsigned long long *a = reinterpret_cast<unsigned long long *>(w);
    if (lo != 0) {
        unsigned long long old = atomicAdd(a, static_cast<unsigned long long>(lo));
        hi += (old + lo < old) ? 1u : 0u;
    }
    if (hi != 0) {
        atomicAdd(a + 1, static_cast<unsigned long long>(hi));
    }
}

__device__ __forceinline__ void AtomicAddU192(uint64_t *w, uint64_t lo, uint64_t mid, uint64_t hi)
{
    unsigned long long *a = reinterpret_cast<unsigned long long *>(w);
    if (lo != 0) {
        unsigned long long old = atomicAdd(a, static_cast<unsigned long long>(lo));
        if (old + lo < old) {
            mid += 1;
            hi += (mid == 0) ? 1u : 0u;
        }
    }
    if (mid != 0) {
        unsigned long long old = atomicAdd(a + 1, static_cast<unsigned long long>(mid));
        hi += (old + mid < old) ? 1u : 0u;
    }
    if (hi != 0) {
        atomicAdd(a + 2, static_cast<unsigned long long>(hi));
    }
}

// Compensated atomic double sum.  atomicAdd(double) stores fl(old + x) (round to nearest
// even) and returns `old`, so the adding thread can form the exact rounding error of its own
// addition with Knuth's TwoSum and push it into the companion word.  s + c then carries the
// sum to about twice the working precision regardless of the order of the additions.
__device__ __forceinline__ void AtomicAddCompensated(uint64_t *w, double x, double extraErr)
{
    double *s = reinterpret_cast<double *>(w);
    double old = atomicAdd(s, x);
    double sum = __dadd_rn(old, x);
    double err = extraErr;
    if (isfinite(sum)) {
        double bv = __dsub_rn(sum, old);
        double av = __dsub_rn(sum, bv);
        err = __dadd_rn(err, __dadd_rn(__dsub_rn(old, av), __dsub_rn(x, bv)));
    }
    if (err != 0.0) {
        atomicAdd(s + 1, err);
    }
}

__device__ __forceinline__ void AtomicMinI64(uint64_t *w, int64_t v)
{
    long long *a = reinterpret_cast<long long *>(w);
    if (v < *reinterpret_cast<volatile long long *>(a)) {
        atomicMin(a, static_cast<long long>(v));
    }
}
__device__ __forceinline__ void AtomicMaxI64(uint64_t *w, int64_t v)
{
    long long *a = reinterpret_cast<long long *>(w);
    if (v > *reinterpret_cast<volatile long long *>(a)) {
        atomicMax(a, static_cast<long long>(v));
    }
}

__device__ __forceinline__ uint64_t LoadAcquire(const uint64_t *p)
{
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void StoreRelease(uint64_t *p, uint64_t v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void SetError(int32_t *error, int32_t code)
{
    if (error != nullptr) {
        atomicCAS(error, 0, code);
    }
}

}  // namespace omg
