// OmniVec vectors and batches (see omniop/vector.h).
#include "omniop/vector.h"

#include <cuda_runtime.h>

#include "host/gpu_runtime.h"
#include "omniop/types.h"

namespace omniruntime {
namespace vec {

namespace {
size_t ValuesBytes(int32_t width, int32_t size)
{
    // Round up to 16 bytes so vectorised device loads never cross the allocation.
    size_t b = static_cast<size_t>(width) * static_cast<size_t>(size < 1 ? 1 : size);
    return (b + 15) & ~size_t(15);
}
size_t NullsBytes(int32_t size)
{
    // Whole 32-bit words plus the reference's 8 spare bytes: device kernels set null bits
    // with 32-bit atomicOr.
    return static_cast<size_t>(((size + 31) / 32) * 4 + 8);
}
}  // namespace

BaseVector::BaseVector(DataTypeId type, int32_t width, int32_t size, bool device, void *stream)
    : type_(type), width_(width), size_(size)
{
    if (width <= 0) {
        throw exception::OmniException("UNSUPPORTED_ERROR", "unsupported vector type " + std::to_string(type), -2);
    }
    if (device) {
        values_ = omg::Buffer::NewDevice(ValuesBytes(width, size), stream, true);
        nulls_ = omg::Buffer::NewDevice(NullsBytes(size), stream, true);
    } else {
        values_ = omg::Buffer::NewHost(ValuesBytes(width, size), true);
        nulls_ = omg::Buffer::NewHost(NullsBytes(size), true);
    }
}

BaseVector::BaseVector(DataTypeId type, int32_t width, int32_t size, omg::BufferPtr values, size_t valuesOffset,
    omg::BufferPtr nulls, size_t nullsOffset, bool hasNull)
    : type_(type), width_(width), size_(size), hasNull_(hasNull), values_(std::move(values)),
      valuesOffset_(valuesOffset), nulls_(std::move(nulls)), nullsOffset_(nullsOffset)
{}

BaseVector::BaseVector(DataTypeId type, int32_t size, int64_t dataBytes, bool device, void *stream)
    : type_(type), width_(0), size_(size), dataBytes_(dataBytes)
{
    if (!IsVarlen() || dataBytes < 0) {
        throw exception::OmniException("UNSUPPORTED_ERROR", "not a variable-length vector type", -2);
    }
    const size_t cb = static_cast<size_t>(dataBytes) + 16;
    const size_t ob = (static_cast<size_t>(size) + 1) * sizeof(int32_t);
    if (device) {
        values_ = omg::Buffer::NewDevice(cb, stream, false);
        offsets_ = omg::Buffer::NewDevice(ob, stream, true);
        nulls_ = omg::Buffer::NewDevice(NullsBytes(size), stream, true);
    } else {
        values_ = omg::Buffer::NewHost(cb, false);
        offsets_ = omg::Buffer::NewHost(ob, true);
        nulls_ = omg::Buffer::NewHost(NullsBytes(size), true);
    }
}

BaseVector::BaseVector(DataTypeId type, int32_t size, omg::BufferPtr chars, int64_t dataBytes, omg::BufferPtr offsets,
    size_t offsetsOffset, omg::BufferPtr nulls, size_t nullsOffset, bool hasNull)
    : type_(type), width_(0), size_(size), hasNull_(hasNull), values_(std::move(chars)), valuesOffset_(0),
      nulls_(std::move(nulls)), nullsOffset_(nullsOffset), offsets_(std::move(offsets)),
      offsetsOffset_(offsetsOffset), dataBytes_(dataBytes)
{}

BaseVector::BaseVector(omg::BufferPtr ids, int32_t size, const BaseVector &dictionary)
    : type_(dictionary.type_), width_(dictionary.width_), size_(size), hasNull_(dictionary.hasNull_),
      values_(std::move(ids)), dataBytes_(dictionary.dataBytes_)
{
    if (dictionary.dictionary_) {
        throw exception::OmniException("UNSUPPORTED_ERROR", "a dictionary of a dictionary vector", -2);
    }
    if (dictionary.IsVarlen()) {
        dictionary_ = std::make_shared<BaseVector>(dictionary.type_, dictionary.size_, dictionary.values_,
            dictionary.dataBytes_, dictionary.offsets_, dictionary.offsetsOffset_, dictionary.nulls_,
            dictionary.nullsOffset_, dictionary.hasNull_);
    } else {
        dictionary_ = std::make_shared<BaseVector>(dictionary.type_, dictionary.width_, dictionary.size_,
            dictionary.values_, dictionary.valuesOffset_, dictionary.nulls_, dictionary.nullsOffset_,
            dictionary.hasNull_);
    }
}

BaseVector *VectorHelper::CreateDictionaryVector(const int32_t *values, int32_t valueSize, const BaseVector &vector)
{
    if (valueSize < 0 || (valueSize > 0 && values == nullptr)) {
        throw exception::OmniException("INVALID_ARGUMENT", "invalid dictionary ids", -1);
    }
    if (vector.GetEncoding() != OMNI_FLAT) {
        throw exception::OmniException("UNSUPPORTED_ERROR", "a dictionary of a dictionary vector", -2);
    }
    for (int32_t i = 0; i < valueSize; ++i) {
        if (values[i] < 0 || values[i] >= vector.GetSize()) {
            throw exception::OmniException("INVALID_ARGUMENT",
                "dictionary id " + std::to_string(values[i]) + " out of range", -1);
        }
    }
    auto ids = omg::Buffer::NewHost(ValuesBytes(sizeof(int32_t), valueSize), false);
    if (valueSize > 0) {
        std::memcpy(ids->Data(), values, sizeof(int32_t) * static_cast<size_t>(valueSize));
    }
    return new BaseVector(ids, valueSize, vector);
}

bool BaseVector::HasNull()
{
    if (hasNull_) {
        return true;
    }
    if (dictionary_) {
        return false;  // takes the dictionary's flag
    }
    if (nulls_ == nullptr || IsDevice()) {
        return false;  // device vectors rely on the writer's flag
    }
    const uint8_t *n = RawNulls();
    const int32_t fullBytes = size_ >> 3;
    for (int32_t i = 0; i < fullBytes; ++i) {
        if (n[i] != 0) {
            hasNull_ = true;
            return true;
        }
    }
    for (int32_t i = fullBytes * 8; i < size_; ++i) {
        if (IsNull(i)) {
            hasNull_ = true;
            return true;
        }
    }
    return false;
}

int32_t BaseVector::GetNullCount()
{
    if (IsDevice() || nulls_ == nullptr) {
        return 0;
    }
    int32_t c = 0;
    for (int32_t i = 0; i < size_; ++i) {
        c += IsNull(i) ? 1 : 0;
    }
    return c;
}

VectorBatch::~VectorBatch() = default;

void VectorBatch::FreeAllVectors()
{
    for (auto *v : vectors_) {
        delete v;
    }
    vectors_.clear();
}

bool VectorBatch::IsDevice() const
{
    for (auto *v : vectors_) {
        if (v->IsDevice()) {
            return true;
        }
    }
    return false;
}

BaseVector::BaseVector(std::vector<BaseVector *> fields) : type_(OMNI_CONTAINER), width_(0), size_(0)
{
    if (fields.empty()) {
        throw exception::OmniException("INVALID_ARGUMENT", "a container vector needs fields", -1);
    }
    for (auto *f : fields) {
        fields_.emplace_back(f);  // owned from here on
    }
    size_ = fields[0]->GetSize();
    for (auto *f : fields) {
        if (f->GetSize() != size_ || f->GetEncoding() != OMNI_FLAT) {
            throw exception::OmniException("INVALID_ARGUMENT", "container fields are flat vectors of one length", -1);
        }
    }
    // Values and residency are the first field's; no row is NULL unless every field has NULLs,
    // which the operators' container outputs never have.
    values_ = fields[0]->ValuesBuffer();
    valuesOffset_ = fields[0]->ValuesOffset();
    bool allNullable = true;
    for (auto *f : fields) {
        allNullable = allNullable && f->RawNulls() != nullptr && f->NullFlag();
    }
    if (allNullable) {
        throw exception::OmniException("UNSUPPORTED_ERROR", "container vectors whose every field has NULLs", -2);
    }
}

VectorBatch *VectorHelper::CopyBatch(VectorBatch *batch, bool toDevice, void *stream)
{
    auto *out = new VectorBatch(batch->GetRowCount());
    try {
        for (int32_t i = 0; i < batch->GetVectorCount(); ++i) {
            BaseVector *src = batch->Get(i);
            if (src->GetEncoding() == OMNI_ENCODING_CONTAINER) {
                // Each field copied as a one-vector batch, then wrapped again.
                std::vector<BaseVector *> fields;
                for (int32_t f = 0; f < src->NumFields(); ++f) {
                    VectorBatch one(batch->GetRowCount());
                    one.Append(src->Field(f));
                    VectorBatch *c = CopyBatch(&one, toDevice, stream);
                    one.ClearVectors();  // the field stays the container's
                    fields.push_back(c->Get(0));
                    c->ClearVectors();
                    delete c;
                }
                out->Append(new BaseVector(fields));
                continue;
            }
            std::unique_ptr<BaseVector> flat;
            if (src->GetEncoding() == OMNI_DICTIONARY) {
                flat.reset(omg::FlattenDictionary(*src, static_cast<cudaStream_t>(stream)));
                src = flat.get();
            }
            cudaMemcpyKind kind = cudaMemcpyDefault;
            BaseVector *dst;
            size_t vb;
            if (src->IsVarlen()) {
                dst = new BaseVector(src->GetTypeId(), src->GetSize(), src->DataBytes(), toDevice, stream);
                vb = static_cast<size_t>(src->DataBytes());
                const size_t ob = (static_cast<size_t>(src->GetSize()) + 1) * sizeof(int32_t);
                if (cudaMemcpyAsync(dst->RawOffsets(), src->RawOffsets(), ob, kind,
                        static_cast<cudaStream_t>(stream)) != cudaSuccess) {
                    delete dst;
                    throw exception::OmniException("CUDA_ERROR", "batch copy failed", -3);
                }
            } else {
                dst = new BaseVector(src->GetTypeId(), src->GetWidth(), src->GetSize(), toDevice, stream);
                vb = static_cast<size_t>(src->GetWidth()) * src->GetSize();
            }
            out->Append(dst);
            if (vb > 0 && cudaMemcpyAsync(dst->RawValues(), src->RawValues(), vb, kind,
                              static_cast<cudaStream_t>(stream)) != cudaSuccess) {
                throw exception::OmniException("CUDA_ERROR", "batch copy failed", -3);
            }
            if (src->RawNulls() != nullptr) {
                const size_t nb = static_cast<size_t>((src->GetSize() + 7) / 8);
                if (nb > 0 && cudaMemcpyAsync(dst->RawNulls(), src->RawNulls(), nb, kind,
                                  static_cast<cudaStream_t>(stream)) != cudaSuccess) {
                    throw exception::OmniException("CUDA_ERROR", "batch copy failed", -3);
                }
            }
            dst->SetNullFlag(src->HasNull());
        }
        if (cudaStreamSynchronize(static_cast<cudaStream_t>(stream)) != cudaSuccess) {
            throw exception::OmniException("CUDA_ERROR", "batch copy failed", -3);
        }
    } catch (...) {
        VectorHelper::FreeVecBatch(out);
        throw;
    }
    return out;
}

}  // namespace vec

namespace op {
namespace {
SupportContainerVecRule g_rule = SupportContainerVecRule::NOT_SUPPORT;
NegativeStartIndexOutOfBoundsRule g_negativeStart = NegativeStartIndexOutOfBoundsRule::INTERCEPT_FROM_BEYOND;
ZeroStartIndexSupportRule g_zeroStart = ZeroStartIndexSupportRule::IS_SUPPORT;
}  // namespace
SupportContainerVecRule GetSupportContainerVecRule() { return g_rule; }
void SetSupportContainerVecRule(SupportContainerVecRule rule) { g_rule = rule; }
NegativeStartIndexOutOfBoundsRule GetNegativeStartIndexOutOfBoundsRule() { return g_negativeStart; }
void SetNegativeStartIndexOutOfBoundsRule(NegativeStartIndexOutOfBoundsRule rule) { g_negativeStart = rule; }
ZeroStartIndexSupportRule GetZeroStartIndexSupportRule() { return g_zeroStart; }
void SetZeroStartIndexSupportRule(ZeroStartIndexSupportRule rule) { g_zeroStart = rule; }
}  // namespace op
}  // namespace omniruntime
