// OmniVec columnar format for the GB300 operators.
//
// Layout follows the reference (vector/vector.h:45-404, vector/nulls_buffer.h:16-114):
//  - flat values, one fixed-width element per row;
//  - VARCHAR / CHAR: n + 1 int32 offsets into a character buffer (value i is bytes
//    [offsets[i], offsets[i + 1])), the LargeStringContainer layout of vector/vector.h;
//  - a null bitmap, LSB-first, bit set = NULL, of NullsBuffer::CalculateNbytes(n) =
//    ceil(n/8) + 8 bytes (the 8 spare bytes let 64-bit word loads run past the end).
// Both live in one Buffer each, host-pinned or in HBM (Residency).  A vector may be a
// view into a larger buffer (offset), which is how GetOutput carves many output batches
// out of one device->host copy without per-batch allocations.
#pragma once

#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "memory.h"
#include "types.h"

namespace omniruntime {
namespace vec {
using namespace omniruntime::type;

enum Encoding { OMNI_FLAT = 0, OMNI_DICTIONARY = 1, OMNI_ENCODING_CONTAINER = 2 };

class NullsBuffer {
public:
    static constexpr int32_t CalculateNbytes(int32_t bits) { return (bits + 7) / 8 + 8; }
};

class BaseVector {
public:
    // New owned flat vector, host or device.  Values and nulls are zeroed.
    BaseVector(DataTypeId type, int32_t width, int32_t size, bool device, void *stream = nullptr);
    // View over existing buffers (values at byte offset `valuesOffset`, nulls at byte offset
    // `nullsOffset`; nulls may be null).
    BaseVector(DataTypeId type, int32_t width, int32_t size, omg::BufferPtr values, size_t valuesOffset,
        omg::BufferPtr nulls, size_t nullsOffset, bool hasNull);
    // New owned VARCHAR/CHAR vector with `dataBytes` bytes of character storage; offsets and
    // nulls zeroed.
    BaseVector(DataTypeId type, int32_t size, int64_t dataBytes, bool device, void *stream = nullptr);
    // VARCHAR/CHAR view: offsets at byte offset `offsetsOffset` of `offsets` (absolute positions
    // in `chars`).
    BaseVector(DataTypeId type, int32_t size, omg::BufferPtr chars, int64_t dataBytes, omg::BufferPtr offsets,
        size_t offsetsOffset, omg::BufferPtr nulls, size_t nullsOffset, bool hasNull);
    // Dictionary-encoded vector (VectorHelper::CreateDictionaryVector, vector/vector_helper.h:
    // 70-82,381-420): row i is row ids[i] of `dictionary`, whose buffers this vector shares, and
    // is NULL when that dictionary row is.  `ids` holds `size` int32 values in
    // [0, dictionary.GetSize()).  The operators flatten such vectors on the device when they
    // take a batch (omg::FlattenDictionaries).
    BaseVector(omg::BufferPtr ids, int32_t size, const BaseVector &dictionary);
    // Container vector (operator/aggregation/container_vector.h:20-80): each row holds the values
    // of several equally long field vectors, owned by this vector (a partial AVG's double sum and
    // long count under the container-vector policy).  A row is NULL when it is NULL in every
    // field; the fields the operators produce are never NULL.
    explicit BaseVector(std::vector<BaseVector *> fields);
    virtual ~BaseVector() = default;

    bool IsVarlen() const { return type_ == OMNI_VARCHAR || type_ == OMNI_CHAR; }
    // VARCHAR/CHAR: n + 1 offsets (nullptr for fixed-width vectors) and the character buffer's size.
    int32_t *RawOffsets() const
    {
        return offsets_ ? reinterpret_cast<int32_t *>(static_cast<uint8_t *>(offsets_->Data()) + offsetsOffset_)
                        : nullptr;
    }
    int64_t DataBytes() const { return dataBytes_; }
    const omg::BufferPtr &OffsetsBuffer() const { return offsets_; }

    int32_t GetSize() const { return size_; }
    DataTypeId GetTypeId() const { return type_; }
    int32_t GetWidth() const { return width_; }
    Encoding GetEncoding() const
    {
        return dictionary_ ? OMNI_DICTIONARY : (fields_.empty() ? OMNI_FLAT : OMNI_ENCODING_CONTAINER);
    }
    // Container encoding: the field vectors.
    int32_t NumFields() const { return static_cast<int32_t>(fields_.size()); }
    BaseVector *Field(int32_t i) const { return fields_.at(i).get(); }
    // Dictionary encoding: the row ids (int32) and the dictionary (a flat view).
    const int32_t *RawIds() const { return dictionary_ ? reinterpret_cast<const int32_t *>(RawValues()) : nullptr; }
    const BaseVector *Dictionary() const { return dictionary_.get(); }
    bool IsDevice() const { return values_->IsDevice(); }

    uint8_t *RawValues() const { return static_cast<uint8_t *>(values_->Data()) + valuesOffset_; }
    // Null bitmap (nullptr for a device view created without nulls).
    uint8_t *RawNulls() const
    {
        return nulls_ ? static_cast<uint8_t *>(nulls_->Data()) + nullsOffset_ : nullptr;
    }

    // Host-only accessors (vector/vector.h SetNull/IsNull/HasNull).
    void SetNull(int32_t i)
    {
        RawNulls()[i >> 3] |= static_cast<uint8_t>(1u << (i & 7));
        hasNull_ = true;
    }
    void SetNotNull(int32_t i) { RawNulls()[i >> 3] &= static_cast<uint8_t>(~(1u << (i & 7))); }
    bool IsNull(int32_t i) const
    {
        if (dictionary_) {
            return dictionary_->IsNull(RawIds()[i]);
        }
        const uint8_t *n = RawNulls();
        return n != nullptr && ((n[i >> 3] >> (i & 7)) & 1u);
    }
    // hasNull is a hint kept by the writer (NullsBuffer::SetNullFlag); HasNull() scans the
    // bitmap of a host vector when the hint is false, as NullsBuffer::HasNull does.
    bool HasNull();
    void SetNullFlag(bool hasNull) { hasNull_ = hasNull; }
    bool NullFlag() const { return hasNull_; }
    int32_t GetNullCount();

    const omg::BufferPtr &ValuesBuffer() const { return values_; }
    const omg::BufferPtr &NullsBufferPtr() const { return nulls_; }
    size_t ValuesOffset() const { return valuesOffset_; }
    size_t NullsOffset() const { return nullsOffset_; }

protected:
    DataTypeId type_;
    int32_t width_;
    int32_t size_;
    bool hasNull_ = false;
    omg::BufferPtr values_;
    size_t valuesOffset_ = 0;
    omg::BufferPtr nulls_;
    size_t nullsOffset_ = 0;
    omg::BufferPtr offsets_;  // VARCHAR/CHAR only
    size_t offsetsOffset_ = 0;
    int64_t dataBytes_ = 0;
    std::shared_ptr<BaseVector> dictionary_;  // dictionary encoding only (values_ = the ids)
    std::vector<std::shared_ptr<BaseVector>> fields_;  // container encoding only
};

// Typed host accessor (vector/vector.h Vector<T>::GetValue/SetValue).
template <typename T> class Vector : public BaseVector {
public:
    using BaseVector::BaseVector;
    T GetValue(int32_t i) const
    {
        T v;
        std::memcpy(&v, RawValues() + static_cast<size_t>(i) * sizeof(T), sizeof(T));
        return v;
    }
    void SetValue(int32_t i, T v) { std::memcpy(RawValues() + static_cast<size_t>(i) * sizeof(T), &v, sizeof(T)); }
};

class VectorBatch {
public:
    explicit VectorBatch(size_t rowCnt) : rowCnt_(rowCnt) {}
    ~VectorBatch();
    VectorBatch(const VectorBatch &) = delete;
    VectorBatch &operator=(const VectorBatch &) = delete;

    void Append(BaseVector *vector) { vectors_.push_back(vector); }
    // Replace vector `index` (the old one is deleted).
    void Set(int32_t index, BaseVector *vector)
    {
        delete vectors_.at(index);
        vectors_.at(index) = vector;
    }
    BaseVector *Get(int32_t index) const { return vectors_.at(index); }
    int32_t GetRowCount() const { return static_cast<int32_t>(rowCnt_); }
    int32_t GetVectorCount() const { return static_cast<int32_t>(vectors_.size()); }
    void Resize(size_t rowCount) { rowCnt_ = rowCount; }
    void FreeAllVectors();
    void ClearVectors() { vectors_.clear(); }
    bool IsDevice() const;

private:
    size_t rowCnt_;
    std::vector<BaseVector *> vectors_;
};

class VectorHelper {
public:
    // VectorHelper::FreeVecBatch: delete the batch and its vectors.
    static void FreeVecBatch(VectorBatch *batch)
    {
        if (batch != nullptr) {
            batch->FreeAllVectors();
            delete batch;
        }
    }
    static BaseVector *CreateFlatVector(DataTypeId type, int32_t size, int32_t width = 0)
    {
        return new BaseVector(type, TypeWidth(type, width), size, false);
    }
    // VectorHelper::CreateDictionaryVector (vector/vector_helper.h:381-420): a host vector of
    // `valueSize` rows selecting rows `values` of `vector`; ids out of range are refused.
    static BaseVector *CreateDictionaryVector(const int32_t *values, int32_t valueSize, const BaseVector &vector);
    // Deep copy of a batch into host or device residency.
    static VectorBatch *CopyBatch(VectorBatch *batch, bool toDevice, void *stream);
};

}  // namespace vec
}  // namespace omniruntime
