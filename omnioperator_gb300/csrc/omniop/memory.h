// Memory for the GB300 operators.
//
// Host side: OmniVec buffers live in page-locked ("pinned") host memory that the GPU can
// read and write directly over NVLink-C2C / PCIe, so an AddInput of a host batch needs no
// staging copy.  Pinned allocations are expensive, so blocks are cached in size classes and
// reused.  Without a CUDA device (CPU-only hosts) plain aligned host memory is used; compute
// entry points then refuse to run.
//
// Device side: stream-ordered allocations from the device's default memory pool
// (cudaMallocAsync), with the pool's release threshold raised so freed blocks stay cached.
//
// The reference's equivalents are mem::Allocator over jemalloc (memory/allocator.h:14-32)
// and the per-operator arena (memory/simple_arena_allocator.h:15-225).
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <memory>

namespace omg {

// True if a CUDA device is present and usable (checked once).
bool DeviceAvailable();

// Pinned host memory (cached).  Returns nullptr on failure.  `zero` clears the block.
void *HostAlloc(size_t bytes, bool zero);
void HostFree(void *p, size_t bytes);

// Device memory, stream-ordered.  Throws OmniException(OMG_ERR_OOM) on failure.
void *DeviceAlloc(size_t bytes, void *stream);
void DeviceFree(void *p, void *stream);

// Host-side fault injection: the next n DeviceAlloc calls fail.
void SetFailNextDeviceAllocs(int32_t n);

// A reference-counted memory block: host (pinned) or device, owned or borrowed.
class Buffer {
public:
    enum class Kind : int8_t { HOST, DEVICE, DEVICE_VIEW, HOST_VIEW };
    Buffer(Kind kind, void *ptr, size_t bytes, void *stream = nullptr)
        : kind_(kind), ptr_(ptr), bytes_(bytes), stream_(stream)
    {}
    ~Buffer();
    Buffer(const Buffer &) = delete;
    Buffer &operator=(const Buffer &) = delete;

    static std::shared_ptr<Buffer> NewHost(size_t bytes, bool zero);
    static std::shared_ptr<Buffer> NewDevice(size_t bytes, void *stream, bool zero);
    static std::shared_ptr<Buffer> DeviceView(void *ptr, size_t bytes)
    {
        return std::make_shared<Buffer>(Kind::DEVICE_VIEW, ptr, bytes);
    }

    void *Data() const { return ptr_; }
    size_t Bytes() const { return bytes_; }
    bool IsDevice() const { return kind_ == Kind::DEVICE || kind_ == Kind::DEVICE_VIEW; }
    Kind GetKind() const { return kind_; }

private:
    Kind kind_;
    void *ptr_;
    size_t bytes_;
    void *stream_;  // device buffers are freed in order on the stream they were allocated on
};
using BufferPtr = std::shared_ptr<Buffer>;

}  // namespace omg
