// Pinned-host and device memory for the GB300 operators (see omniop/memory.h).
#include "omniop/memory.h"

#include <cuda_runtime.h>

#include <atomic>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "omniop/types.h"

namespace omg {
namespace {

std::atomic<int32_t> g_failNext{0};

// Size classes: powers of two from 4 KiB; larger than 1 GiB is exact-size.
size_t RoundClass(size_t bytes)
{
    size_t c = 4096;
    while (c < bytes && c < (size_t(1) << 30)) {
        c <<= 1;
    }
    return c < bytes ? bytes : c;
}

class PinnedCache {
public:
    void *Get(size_t bytes)
    {
        const size_t cls = RoundClass(bytes);
        {
            std::lock_guard<std::mutex> g(mu_);
            auto it = free_.find(cls);
            if (it != free_.end() && !it->second.empty()) {
                void *p = it->second.back();
                it->second.pop_back();
                cached_ -= cls;
                return p;
            }
        }
        void *p = nullptr;
        if (DeviceAvailable()) {
            if (cudaHostAlloc(&p, cls, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
        } else {
            if (posix_memalign(&p, 256, cls) != 0) {
                return nullptr;
            }
        }
        return p;
    }
    void Put(void *p, size_t bytes)
    {
        const size_t cls = RoundClass(bytes);
        std::lock_guard<std::mutex> g(mu_);
        // Keep up to 8 GiB of freed pinned memory for reuse; release the rest.
        if (cached_ + cls > (size_t(8) << 30)) {
            Release(p);
            return;
        }
        free_[cls].push_back(p);
        cached_ += cls;
    }

private:
    static void Release(void *p)
    {
        if (DeviceAvailable()) {
            cudaFreeHost(p);
        } else {
            free(p);
        }
    }
    std::mutex mu_;
    std::map<size_t, std::vector<void *>> free_;
    size_t cached_ = 0;
};

PinnedCache &Pinned()
{
    static PinnedCache *cache = new PinnedCache();  // intentionally leaked: outlives static buffers
    return *cache;
}

void ConfigurePool()
{
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t threshold = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        }
        cudaGetLastError();
    });
}

}  // namespace

bool DeviceAvailable()
{
    static int available = -1;
    if (available < 0) {
        int n = 0;
        available = (cudaGetDeviceCount(&n) == cudaSuccess && n > 0) ? 1 : 0;
        cudaGetLastError();
    }
    return available == 1;
}

void *HostAlloc(size_t bytes, bool zero)
{
    if (bytes == 0) {
        bytes = 1;
    }
    void *p = Pinned().Get(bytes);
    if (p != nullptr && zero) {
        std::memset(p, 0, bytes);
    }
    return p;
}

void HostFree(void *p, size_t bytes)
{
    if (p != nullptr) {
        Pinned().Put(p, bytes == 0 ? 1 : bytes);
    }
}

void SetFailNextDeviceAllocs(int32_t n) { g_failNext.store(n); }

void *DeviceAlloc(size_t bytes, void *stream)
{
    using omniruntime::exception::OmniException;
    if (!DeviceAvailable()) {
        throw OmniException("CUDA_ERROR", "no CUDA device available", -8);
    }
    int32_t f = g_failNext.load();
    while (f > 0) {
        if (g_failNext.compare_exchange_weak(f, f - 1)) {
            throw OmniException("MEM_CAP_EXCEEDED", "injected device allocation failure", -4);
        }
    }
    ConfigurePool();
    void *p = nullptr;
    cudaError_t err = cudaMallocAsync(&p, bytes == 0 ? 256 : bytes, static_cast<cudaStream_t>(stream));
    if (err != cudaSuccess) {
        cudaGetLastError();
        throw OmniException("MEM_CAP_EXCEEDED",
            "device allocation of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(err), -4);
    }
    return p;
}

void DeviceFree(void *p, void *stream)
{
    if (p != nullptr) {
        cudaFreeAsync(p, static_cast<cudaStream_t>(stream));
    }
}

Buffer::~Buffer()
{
    switch (kind_) {
        case Kind::HOST:
            HostFree(ptr_, bytes_);
            break;
        case Kind::DEVICE:
            // Stream-ordered free: every use of this buffer was issued on its stream before
            // the buffer's last reference went away.
            DeviceFree(ptr_, stream_);
            break;
        default:
            break;
    }
}

std::shared_ptr<Buffer> Buffer::NewHost(size_t bytes, bool zero)
{
    void *p = HostAlloc(bytes, zero);
    if (p == nullptr) {
        throw omniruntime::exception::OmniException("MEM_CAP_EXCEEDED",
            "host allocation of " + std::to_string(bytes) + " bytes failed", -4);
    }
    return std::make_shared<Buffer>(Kind::HOST, p, bytes);
}

std::shared_ptr<Buffer> Buffer::NewDevice(size_t bytes, void *stream, bool zero)
{
    void *p = DeviceAlloc(bytes, stream);
    if (zero) {
        cudaMemsetAsync(p, 0, bytes, static_cast<cudaStream_t>(stream));
    }
    return std::make_shared<Buffer>(Kind::DEVICE, p, bytes, stream);
}

}  // namespace omg
