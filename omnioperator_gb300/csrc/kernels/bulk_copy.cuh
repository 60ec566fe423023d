// Bulk-copy (TMA) engine and mbarrier primitives for sm_103a, as inline PTX.
//
// A one-dimensional `cp.async.bulk` moves a contiguous run between global and shared memory
// without the L1 request path: one instruction per run, issued by one thread.  Global to shared
// copies complete on an mbarrier in shared memory (the issuing thread arms it with the byte
// count, the copy engine counts the bytes down); shared to global copies are tracked in per-
// thread bulk async-groups.  Both ends of a copy start on a 16-byte boundary and its size is a
// multiple of 16 bytes.
#pragma once

#include <cstdint>

namespace omg {

__device__ __forceinline__ uint32_t SmemAddr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// One arrival (the arming thread's) completes a phase once the armed bytes have landed.
__device__ __forceinline__ void MbarInit(uint64_t *bar, uint32_t arrivals)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(bar)), "r"(arrivals) : "memory");
}

// Makes initialised mbarriers visible to the copy engine (the async proxy).
__device__ __forceinline__ void MbarInitFence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before later copy-engine
// accesses of the same bytes.
__device__ __forceinline__ void FenceProxyAsyncShared()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void MbarArmTx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     SmemAddr(bar)),
        "r"(bytes)
        : "memory");
}

// Global -> shared, `bytes` (a multiple of 16) from a 16-byte aligned source into a 16-byte
// aligned destination of this CTA, counted down on `bar`.
__device__ __forceinline__ void BulkLoad(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     SmemAddr(dst)),
        "l"(src), "r"(bytes), "r"(SmemAddr(bar))
        : "memory");
}

// Shared -> global, same alignment rules; joins this thread's open bulk async-group.
__device__ __forceinline__ void BulkStore(void *dst, const void *src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(SmemAddr(src)),
        "r"(bytes)
        : "memory");
}

__device__ __forceinline__ void BulkCommit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Waits until at most kPending of this thread's committed bulk groups still read shared memory.
template <int kPending>
__device__ __forceinline__ void BulkWaitRead()
{
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(kPending) : "memory");
}

// Waits until all of this thread's committed bulk groups are complete (writes performed).
__device__ __forceinline__ void BulkWaitAll() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ bool MbarTryWait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(SmemAddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase of `bar` with parity `parity` to complete, for at most `budget` clock64
// ticks; false when the budget ran out first.
__device__ __forceinline__ bool MbarWaitBounded(uint64_t *bar, uint32_t parity, long long budget)
{
    if (MbarTryWait(bar, parity)) {
        return true;
    }
    const long long t0 = clock64();
    while (!MbarTryWait(bar, parity)) {
        if (clock64() - t0 > budget) {
            return false;
        }
    }
    return true;
}

}  // namespace omg
