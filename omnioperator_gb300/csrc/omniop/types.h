// Core enums and the DataType description used by the GB300 operators.
//
// The numbering of DataTypeId, FunctionType, JoinType and OmniStatus is the reference's
// (type/data_type.h:40-74, operator/util/function_type.h:11-27, plannode/planNode.h:406-414,
// operator/status.h:9-13) so that plans written against OmniOperator keep their meaning.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

enum OmniStatus {
    OMNI_STATUS_NORMAL = 0,
    OMNI_STATUS_FINISHED = 1,
    OMNI_STATUS_ERROR = -1,
};

namespace omniruntime {
namespace type {

enum DataTypeId {
    OMNI_NONE = 0,
    OMNI_INT = 1,
    OMNI_LONG = 2,
    OMNI_DOUBLE = 3,
    OMNI_BOOLEAN = 4,
    OMNI_SHORT = 5,
    OMNI_DECIMAL64 = 6,
    OMNI_DECIMAL128 = 7,
    OMNI_DATE32 = 8,
    OMNI_DATE64 = 9,
    OMNI_TIME32 = 10,
    OMNI_TIME64 = 11,
    OMNI_TIMESTAMP = 12,
    OMNI_VARCHAR = 15,
    OMNI_CHAR = 16,
    OMNI_CONTAINER = 17,
    OMNI_BYTE = 18,
    OMNI_FLOAT = 19,
    // Fixed-width byte strings (e.g. a 16-byte join payload).  No reference id exists for
    // this encoding; it stands in for a fixed-width varchar payload.
    OMNI_FIXEDBINARY = 40,
    OMNI_INVALID
};

// Size in bytes of one value of a fixed-width type (0 for unsupported types).
inline int32_t TypeWidth(DataTypeId id, int32_t width = 0)
{
    switch (id) {
        case OMNI_BYTE:
        case OMNI_BOOLEAN:
            return 1;
        case OMNI_SHORT:
            return 2;
        case OMNI_INT:
        case OMNI_DATE32:
        case OMNI_FLOAT:
            return 4;
        case OMNI_LONG:
        case OMNI_DOUBLE:
        case OMNI_DECIMAL64:
        case OMNI_DATE64:
        case OMNI_TIMESTAMP:
        case OMNI_TIME64:
            return 8;
        case OMNI_DECIMAL128:
            return 16;
        case OMNI_FIXEDBINARY:
            return width;
        default:
            return 0;
    }
}

class DataType {
public:
    DataType(DataTypeId id, int32_t precision = 0, int32_t scale = 0, int32_t width = 0)
        : id_(id), precision_(precision), scale_(scale), width_(width)
    {}
    DataTypeId GetId() const { return id_; }
    int32_t GetPrecision() const { return precision_; }
    int32_t GetScale() const { return scale_; }
    int32_t GetWidth() const { return width_; }
    int32_t ByteWidth() const { return TypeWidth(id_, width_); }

private:
    DataTypeId id_;
    int32_t precision_;
    int32_t scale_;
    int32_t width_;
};
using DataTypePtr = std::shared_ptr<DataType>;

inline DataTypePtr IntType() { return std::make_shared<DataType>(OMNI_INT); }
inline DataTypePtr LongType() { return std::make_shared<DataType>(OMNI_LONG); }
inline DataTypePtr ShortType() { return std::make_shared<DataType>(OMNI_SHORT); }
inline DataTypePtr DoubleType() { return std::make_shared<DataType>(OMNI_DOUBLE); }
inline DataTypePtr BooleanType() { return std::make_shared<DataType>(OMNI_BOOLEAN); }
inline DataTypePtr Decimal64Type(int32_t p = 18, int32_t s = 0)
{
    return std::make_shared<DataType>(OMNI_DECIMAL64, p, s);
}
inline DataTypePtr Decimal128Type(int32_t p = 38, int32_t s = 0)
{
    return std::make_shared<DataType>(OMNI_DECIMAL128, p, s);
}
inline DataTypePtr FixedBinaryType(int32_t width) { return std::make_shared<DataType>(OMNI_FIXEDBINARY, 0, 0, width); }

// An ordered list of column types (type/data_types.h DataTypes).
class DataTypes {
public:
    DataTypes() = default;
    explicit DataTypes(std::vector<DataTypePtr> types) : types_(std::move(types)) {}
    const std::vector<DataTypePtr> &Get() const { return types_; }
    int32_t GetSize() const { return static_cast<int32_t>(types_.size()); }
    const DataTypePtr &GetType(int32_t i) const { return types_.at(i); }
    std::vector<int32_t> GetIds() const
    {
        std::vector<int32_t> ids;
        for (auto &t : types_) {
            ids.push_back(t->GetId());
        }
        return ids;
    }

private:
    std::vector<DataTypePtr> types_;
};

// 128-bit decimal value, two's complement, little-endian words (type/decimal128.h:21-).
struct Decimal128 {
    uint64_t lowBits;
    int64_t highBits;
};

}  // namespace type

namespace exception {
// Error raised by the operators; `code` uses the reference's error-code strings
// ("OPERATOR_RUNTIME_ERROR", "UNSUPPORTED_ERROR", ...) and `status` the C ABI code.
class OmniException : public std::runtime_error {
public:
    OmniException(const std::string &code, const std::string &msg, int32_t status = -9)
        : std::runtime_error(code + ": " + msg), code_(code), status_(status)
    {}
    const std::string &GetCode() const { return code_; }
    int32_t GetStatus() const { return status_; }

private:
    std::string code_;
    int32_t status_;
};
}  // namespace exception

namespace op {
enum FunctionType {
    OMNI_AGGREGATION_TYPE_SUM = 0,
    OMNI_AGGREGATION_TYPE_COUNT_COLUMN,
    OMNI_AGGREGATION_TYPE_COUNT_ALL,
    OMNI_AGGREGATION_TYPE_AVG,
    OMNI_AGGREGATION_TYPE_SAMP,
    OMNI_AGGREGATION_TYPE_MAX,
    OMNI_AGGREGATION_TYPE_MIN,
};

enum JoinType {
    OMNI_JOIN_TYPE_INNER = 0,
    OMNI_JOIN_TYPE_LEFT,
    OMNI_JOIN_TYPE_RIGHT,
    OMNI_JOIN_TYPE_FULL,
    OMNI_JOIN_TYPE_LEFT_SEMI,
    OMNI_JOIN_TYPE_LEFT_ANTI,
    OMNI_JOIN_TYPE_EXISTENCE
};

// Which input of the join was built (plannode/planNode.h:29-33).  With OMNI_BUILD_LEFT the
// output vectors are rotated so that the build columns come first (lookup_join.cpp:1959-1962).
enum BuildSide { OMNI_BUILD_UNKNOWN = 0, OMNI_BUILD_LEFT, OMNI_BUILD_RIGHT };

// SupportContainerVecRule (util/policy.h:160-167): NOT_SUPPORT is the Spark policy.
enum class SupportContainerVecRule { NOT_SUPPORT = 0, SUPPORT = 1 };

// Global policy, the analogue of ConfigUtil::GetSupportContainerVecRule (util/config_util.h).
SupportContainerVecRule GetSupportContainerVecRule();
void SetSupportContainerVecRule(SupportContainerVecRule rule);

// substr policies (util/policy.h:70-100); the Spark defaults are INTERCEPT_FROM_BEYOND and
// IS_SUPPORT.  A join filter reads them when its factory compiles it.
enum class NegativeStartIndexOutOfBoundsRule { EMPTY_STRING = 0, INTERCEPT_FROM_BEYOND = 1 };
enum class ZeroStartIndexSupportRule { IS_NOT_SUPPORT = 0, IS_SUPPORT = 1 };
NegativeStartIndexOutOfBoundsRule GetNegativeStartIndexOutOfBoundsRule();
void SetNegativeStartIndexOutOfBoundsRule(NegativeStartIndexOutOfBoundsRule rule);
ZeroStartIndexSupportRule GetZeroStartIndexSupportRule();
void SetZeroStartIndexSupportRule(ZeroStartIndexSupportRule rule);

// Rows per output VectorBatch: ceil(1 MiB / rowSize) (operator/util/operator_util.h:33,111-115).
inline int32_t GetMaxRowCount(int32_t rowSize)
{
    constexpr int32_t kMaxBatchBytes = 1024 * 1024;
    return rowSize <= 0 ? kMaxBatchBytes : (kMaxBatchBytes + rowSize - 1) / rowSize;
}
}  // namespace op
}  // namespace omniruntime
