// HashBuilder / LookupJoin operators (see omniop/hash_join.h).
#include "omniop/hash_join.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "host/gpu_runtime.h"
#include "omniop/expressions.h"
#include "kernels/join_part.h"
#include "kernels/launch.h"

namespace omniruntime {
namespace op {

using exception::OmniException;
using omg::CudaCheck;
using omg::DevArray;
using namespace type;

namespace {

uint64_t NextPow2(uint64_t v)
{
    uint64_t p = 1;
    while (p < v) {
        p <<= 1;
    }
    return p;
}

bool JoinKeyType(DataTypeId id)
{
    switch (id) {
        case OMNI_BYTE:
        case OMNI_SHORT:
        case OMNI_INT:
        case OMNI_LONG:
        case OMNI_DATE32:
        case OMNI_DATE64:
        case OMNI_TIMESTAMP:
        case OMNI_DECIMAL64:
        case OMNI_DECIMAL128:
        case OMNI_VARCHAR:
        case OMNI_CHAR:
            return true;
        default:
            return false;
    }
}

bool Varlen(const DataTypePtr &t) { return t->GetId() == OMNI_VARCHAR || t->GetId() == OMNI_CHAR; }

}  // namespace

// Device-side build: contiguous build columns plus the ARRAY or HASH table.
struct JoinBuildState {
    JoinType joinType;
    BuildSide buildSide = OMNI_BUILD_UNKNOWN;
    int32_t kind = omg::JOIN_KIND_INNER;  // what the probes emit (omg::JoinKind)
    DataTypes buildTypes;
    std::vector<int32_t> hashCols;
    int32_t operatorCount;
    int32_t operatorIndex = 0;
    int32_t finished = 0;
    bool built = false;
    std::mutex mu;
    std::vector<vec::VectorBatch *> batches;  // retained until the factory is destroyed
    omg::OpStream stream;
    int64_t rows = 0;
    std::vector<DevArray<uint8_t>> colValues;
    std::vector<DevArray<uint8_t>> colNulls;
    std::vector<bool> colHasNull;
    std::vector<DevArray<int64_t>> colOffs;  // VARCHAR/CHAR columns: rows + 1 offsets into colValues
    DevArray<int64_t> entries;
    DevArray<uint64_t> hashKeys;
    DevArray<int32_t> csr;
    omg::JoinTable table{};
    uint32_t maxDup = 0;
    DevArray<uint8_t> visited;  // BUILD_OUTER / FULL: one byte per build row, set by the probes
    // Several key columns (or one 16-byte key): the table is keyed by the tuple hash of each row,
    // unless the key columns are fixed widths of 1-8 bytes whose build value ranges multiply to at
    // most 2^62: then each row's parts are packed into one 64-bit key (`packed`, multiKey false)
    // and the table is a single-key ARRAY or HASH table over the packed keys.
    bool multiKey = false;
    bool packed = false;
    omg::JoinKeyPack pack{};
    DevArray<uint64_t> keyHash;
    DevArray<uint8_t> keyHashNulls;

    bool TracksVisits() const { return kind == omg::JOIN_KIND_BUILD_OUTER || kind == omg::JOIN_KIND_FULL; }

    ~JoinBuildState()
    {
        for (auto *b : batches) {
            vec::VectorHelper::FreeVecBatch(b);
        }
    }

    void Build();
    bool TryPackKeys();
};

// Packs the key parts of every build row into keyHash (see `packed`) when they qualify.
bool JoinBuildState::TryPackKeys()
{
    cudaStream_t s = stream.Get();
    const int n = static_cast<int>(hashCols.size());
    omg::JoinKeyPack kp{};
    kp.nParts = n;
    omg::JoinKeyCols kc{};
    kc.nKeys = n;
    bool anyNull = false;
    for (int k = 0; k < n; ++k) {
        const int32_t c = hashCols[k];
        const auto &t = buildTypes.GetType(c);
        const int w = t->ByteWidth();
        if (Varlen(t) || (w != 1 && w != 2 && w != 4 && w != 8)) {
            return false;
        }
        kc.widths[k] = w;
        kc.cols[k] = colValues[c].Get();
        kc.nulls[k] = colHasNull[c] ? colNulls[c].Get() : nullptr;
        anyNull = anyNull || colHasNull[c];
        kp.width[k] = w;
    }
    // Per-part value ranges over the part's non-NULL build rows.
    DevArray<long long> stats(8, s, true);
    unsigned __int128 product = 1;
    for (int k = 0; k < n; ++k) {
        CudaCheck(cudaMemsetAsync(stats.Get(), 0, 8 * sizeof(long long), s), "reset");
        CudaCheck(omg::LaunchKeyStats(kc.cols[k], kc.nulls[k], rows, kc.widths[k], stats.Get(), s), "key part stats");
        long long h[3];
        CudaCheck(cudaMemcpyAsync(h, stats.Get(), sizeof(h), cudaMemcpyDeviceToHost, s), "read key part stats");
        stream.Sync();
        if (h[2] == 0) {
            return false;  // a part that is always NULL: no build row can match
        }
        const uint64_t span = static_cast<uint64_t>(h[1]) - static_cast<uint64_t>(h[0]) + 1;
        if (span == 0) {
            return false;
        }
        product *= span;
        if (product > (static_cast<unsigned __int128>(1) << 62)) {
            return false;
        }
        kp.minv[k] = h[0];
        kp.span[k] = span;
    }
    uint64_t stride = 1;
    for (int k = n - 1; k >= 0; --k) {
        kp.stride[k] = stride;
        stride *= kp.span[k];
    }
    keyHash.Reset(static_cast<size_t>(rows), s);
    if (anyNull) {
        keyHashNulls.Reset(omg::NullBitmapBytes(rows), s, true);
    }
    CudaCheck(omg::LaunchPackBuildKeys(kc, kp, rows, reinterpret_cast<int64_t *>(keyHash.Get()),
                  anyNull ? keyHashNulls.Get() : nullptr, s),
        "pack build keys");
    pack = kp;
    packed = true;
    multiKey = false;
    return true;
}

void JoinBuildState::Build()
{
    omg::RequireDevice();
    cudaStream_t s = stream.Get();
    std::memset(&table, 0, sizeof(table));
    table.mode = omg::JOIN_ARRAY;
    table.unique = 1;
    table.sentinelEntry = -1;
    rows = 0;
    for (auto *b : batches) {
        rows += b->GetRowCount();
    }
    const int nCols = buildTypes.GetSize();
    colValues.assign(nCols, DevArray<uint8_t>());
    colNulls.assign(nCols, DevArray<uint8_t>());
    colHasNull.assign(nCols, false);
    colOffs.assign(nCols, DevArray<int64_t>());
    const int32_t keyCol = hashCols[0];
    const int32_t keyWidth = multiKey ? 8 : buildTypes.GetType(keyCol)->ByteWidth();
    table.keyWidth = keyWidth;
    // Gather every build column into one contiguous HBM array (reading host-pinned or
    // device batches directly).
    for (int c = 0; c < nCols; ++c) {
        const bool varlen = Varlen(buildTypes.GetType(c));
        const int w = buildTypes.GetType(c)->ByteWidth();
        if (w <= 0 && !varlen) {
            throw OmniException("UNSUPPORTED_ERROR", "unsupported build column type", -2);
        }
        if (varlen) {
            colOffs[c].Reset(static_cast<size_t>(rows) + 1, s, true);
            colValues[c].Reset(16, s);
        } else {
            colValues[c].Reset(static_cast<size_t>(rows) * w + 16, s);
        }
        if (rows == 0) {
            continue;
        }
        omg::BatchTable bt;
        bt.Build(batches, {c});
        bt.Upload(s);
        if (bt.AnyNulls(0)) {
            colHasNull[c] = true;
            colNulls[c].Reset(omg::NullBitmapBytes(rows), s, true);
        }
        if (varlen) {
            // Lengths, their scan, then the characters: one contiguous column with 64-bit offsets.
            DevArray<uint32_t> lens(static_cast<size_t>(rows), s);
            CudaCheck(omg::LaunchVarlenTileLens(bt.DeviceBatches(), bt.DeviceTiles(), bt.NumTiles(),
                          bt.DeviceTileOutRows(), 0, lens.Get(), s),
                "build column lengths");
            const int64_t bytes = omg::ScanLengths(lens.Get(), rows, colOffs[c], s);
            colValues[c].Reset(static_cast<size_t>(bytes) + 16, s);
            CudaCheck(omg::LaunchVarlenTileCopy(bt.DeviceBatches(), bt.DeviceTiles(), bt.NumTiles(),
                          bt.DeviceTileOutRows(), 0, colOffs[c].Get(), colValues[c].Get(), s),
                "build column characters");
        }
        CudaCheck(omg::LaunchGatherColumn(bt.DeviceBatches(), bt.DeviceTiles(), bt.NumTiles(), bt.DeviceTileOutRows(),
                      0, w, colValues[c].Get(), colHasNull[c] ? colNulls[c].Get() : nullptr, s),
            "gather build column");
        stream.Sync();  // the batch table's staging must outlive the copy
    }
    if (rows == 0) {
        built = true;
        return;
    }
    if (TracksVisits()) {
        visited.Reset(static_cast<size_t>(rows), s, true);
    }
    const void *keys = colValues[keyCol].Get();
    const uint8_t *keyNulls = colHasNull[keyCol] ? colNulls[keyCol].Get() : nullptr;
    if (multiKey && TryPackKeys()) {
        keys = keyHash.Get();
        keyNulls = keyHashNulls.Get();
    } else if (multiKey) {
        omg::JoinKeyCols kc{};
        kc.nKeys = static_cast<int32_t>(hashCols.size());
        bool anyNull = false;
        for (int k = 0; k < kc.nKeys; ++k) {
            const int32_t c = hashCols[k];
            kc.widths[k] = buildTypes.GetType(c)->ByteWidth();
            kc.cols[k] = colValues[c].Get();
            kc.nulls[k] = colHasNull[c] ? colNulls[c].Get() : nullptr;
            kc.offs[k] = colOffs[c].Get();
            anyNull = anyNull || colHasNull[c];
        }
        keyHash.Reset(static_cast<size_t>(rows), s);
        if (anyNull) {
            keyHashNulls.Reset(omg::NullBitmapBytes(rows), s, true);
        }
        CudaCheck(omg::LaunchJoinKeyHash(kc, rows, keyHash.Get(), anyNull ? keyHashNulls.Get() : nullptr, s),
            "hash key tuples");
        keys = keyHash.Get();
        keyNulls = anyNull ? keyHashNulls.Get() : nullptr;
    }
    DevArray<long long> stats(8, s, true);
    CudaCheck(omg::LaunchKeyStats(keys, keyNulls, rows, keyWidth, stats.Get(), s), "key stats");
    long long h[3];
    CudaCheck(cudaMemcpyAsync(h, stats.Get(), sizeof(h), cudaMemcpyDeviceToHost, s), "read key stats");
    stream.Sync();
    const int64_t nonNull = h[2];
    if (nonNull == 0) {
        built = true;
        return;
    }
    table.minKey = h[0];
    const uint64_t range = static_cast<uint64_t>(h[1]) - static_cast<uint64_t>(h[0]) + 1;
    const bool arrayMode = range != 0 && range <= std::max<uint64_t>(2 * NextPow2(nonNull), 1024) &&
        range <= (uint64_t(1) << 31);
    DevArray<int32_t> err(4, s, true);
    unsigned int *maxCount = reinterpret_cast<unsigned int *>(stats.Get() + 3);
    uint32_t *sentinelCount = reinterpret_cast<uint32_t *>(stats.Get() + 4);
    unsigned int *sentinelCursor = reinterpret_cast<unsigned int *>(stats.Get() + 5);
    int64_t *sentinelEntry = reinterpret_cast<int64_t *>(stats.Get() + 6);
    CudaCheck(cudaMemsetAsync(stats.Get() + 3, 0, 3 * sizeof(long long), s), "reset");
    CudaCheck(omg::LaunchFillI64(sentinelEntry, -1, 1, s), "reset");
    uint64_t n;
    if (arrayMode) {
        table.mode = omg::JOIN_ARRAY;
        table.range = range;
        n = range;
    } else {
        table.mode = omg::JOIN_HASH;
        table.capacity = std::max<uint64_t>(NextPow2(2 * static_cast<uint64_t>(nonNull)), 1024);
        n = table.capacity;
        hashKeys.Reset(n, s);
        CudaCheck(omg::LaunchFillU64(hashKeys.Get(), omg::kEmptyKey, static_cast<int64_t>(n), s), "init hash keys");
    }
    DevArray<uint32_t> counts(n, s, true);
    CudaCheck(omg::LaunchBuildCount(table, keys, keyNulls, rows, keyWidth, hashKeys.Get(), counts.Get(), sentinelCount,
                  maxCount, err.Get(), s),
        "build count");
    long long h2[3];
    CudaCheck(cudaMemcpyAsync(h2, stats.Get() + 3, sizeof(h2), cudaMemcpyDeviceToHost, s), "read build stats");
    int32_t herr = 0;
    CudaCheck(cudaMemcpyAsync(&herr, err.Get(), sizeof(herr), cudaMemcpyDeviceToHost, s), "read error");
    stream.Sync();
    if (herr != 0) {
        throw OmniException("OPERATOR_RUNTIME_ERROR", "join build failed", -9);
    }
    maxDup = static_cast<uint32_t>(h2[0] & 0xffffffffll);
    const uint32_t nSentinel = static_cast<uint32_t>(h2[1] & 0xffffffffll);
    table.unique = (maxDup <= 1 && nSentinel <= 1) ? 1 : 0;
    entries.Reset(n, s);
    CudaCheck(omg::LaunchFillI64(entries.Get(), -1, static_cast<int64_t>(n), s), "init entries");
    DevArray<int64_t> offsets;
    DevArray<uint32_t> cursor;
    int64_t total = 0;
    if (!table.unique) {
        offsets.Reset(n, s);
        DevArray<int64_t> blockSums((n + 1023) / 1024 + 1, s);
        DevArray<long long> tot(1, s, true);
        CudaCheck(omg::LaunchScanCounts(counts.Get(), static_cast<int64_t>(n), offsets.Get(), blockSums.Get(), tot.Get(), s),
            "scan counts");
        long long ht = 0;
        CudaCheck(cudaMemcpyAsync(&ht, tot.Get(), sizeof(ht), cudaMemcpyDeviceToHost, s), "read total");
        stream.Sync();
        total = ht;
        csr.Reset(static_cast<size_t>(total + nSentinel + 1), s);
        cursor.Reset(n, s, true);
    }
    table.arrayEntries = entries.Get();
    table.hashEntries = entries.Get();
    table.hashKeys = hashKeys.Get();
    CudaCheck(omg::LaunchBuildFill(table, keys, keyNulls, rows, keyWidth, counts.Get(), offsets.Get(), cursor.Get(),
                  entries.Get(), csr.Get(), nSentinel, total, sentinelCursor, sentinelEntry, err.Get(), s),
        "build fill");
    int64_t hs = -1;
    CudaCheck(cudaMemcpyAsync(&hs, sentinelEntry, sizeof(hs), cudaMemcpyDeviceToHost, s), "read sentinel");
    CudaCheck(cudaMemcpyAsync(&herr, err.Get(), sizeof(herr), cudaMemcpyDeviceToHost, s), "read error");
    stream.Sync();
    if (herr != 0) {
        throw OmniException("OPERATOR_RUNTIME_ERROR", "join build failed", -9);
    }
    if (table.unique) {
        table.sentinelEntry = hs;
    } else {
        table.sentinelEntry = nSentinel > 0 ? ((total << 32) | static_cast<int64_t>(nSentinel)) : -1;
    }
    table.csrRows = csr.Get();
    built = true;
}

// ------------------------------------------------------------------------------ builder
HashBuilderOperatorFactory::HashBuilderOperatorFactory(JoinType joinType, const DataTypes &buildTypes,
    const int32_t *buildHashCols, int32_t buildHashColsCount, int32_t operatorCount)
    : HashBuilderOperatorFactory(joinType, OMNI_BUILD_UNKNOWN, buildTypes, buildHashCols, buildHashColsCount,
          operatorCount)
{}

HashBuilderOperatorFactory::HashBuilderOperatorFactory(JoinType joinType, BuildSide buildSide,
    const DataTypes &buildTypes, const int32_t *buildHashCols, int32_t buildHashColsCount, int32_t operatorCount)
    : state_(new JoinBuildState())
{
    // The probe a join type selects (lookup_join.cpp:330-411): a LEFT (RIGHT) join whose build is
    // the left (right) input keeps the unmatched build rows (same-side outer join), otherwise the
    // unmatched probe rows (opposite-side outer join).
    int32_t kind;
    switch (joinType) {
        case OMNI_JOIN_TYPE_INNER:
            kind = omg::JOIN_KIND_INNER;
            break;
        case OMNI_JOIN_TYPE_LEFT:
        case OMNI_JOIN_TYPE_RIGHT:
            kind = buildSide == (joinType == OMNI_JOIN_TYPE_LEFT ? OMNI_BUILD_LEFT : OMNI_BUILD_RIGHT)
                ? omg::JOIN_KIND_BUILD_OUTER
                : omg::JOIN_KIND_PROBE_OUTER;
            break;
        case OMNI_JOIN_TYPE_FULL:
            kind = omg::JOIN_KIND_FULL;
            break;
        case OMNI_JOIN_TYPE_LEFT_SEMI:
            kind = omg::JOIN_KIND_SEMI;
            break;
        case OMNI_JOIN_TYPE_LEFT_ANTI:
            kind = omg::JOIN_KIND_ANTI;
            break;
        case OMNI_JOIN_TYPE_EXISTENCE:
            kind = omg::JOIN_KIND_EXISTENCE;
            break;
        default:
            throw OmniException("UNSUPPORTED_ERROR", "unknown join type " + std::to_string(joinType), -2);
    }
    if (buildSide != OMNI_BUILD_UNKNOWN && buildSide != OMNI_BUILD_LEFT && buildSide != OMNI_BUILD_RIGHT) {
        throw OmniException("INVALID_ARGUMENT", "unknown build side", -1);
    }
    if (buildHashColsCount < 1 || buildHashColsCount > omg::kMaxJoinKeys || buildHashCols == nullptr) {
        throw OmniException("UNSUPPORTED_ERROR", "join keys have 1 to 4 columns", -2);
    }
    if (operatorCount < 1) {
        throw OmniException("INVALID_ARGUMENT", "operatorCount must be positive", -1);
    }
    for (int32_t i = 0; i < buildHashColsCount; ++i) {
        const int32_t k = buildHashCols[i];
        if (k < 0 || k >= buildTypes.GetSize() || !JoinKeyType(buildTypes.GetType(k)->GetId())) {
            throw OmniException("UNSUPPORTED_ERROR", "unsupported join key column", -2);
        }
    }
    state_->joinType = joinType;
    state_->buildSide = buildSide;
    state_->kind = kind;
    state_->buildTypes = buildTypes;
    state_->hashCols.assign(buildHashCols, buildHashCols + buildHashColsCount);
    state_->multiKey = buildHashColsCount > 1 || buildTypes.GetType(buildHashCols[0])->ByteWidth() == 16 ||
        Varlen(buildTypes.GetType(buildHashCols[0]));
    state_->operatorCount = operatorCount;
}

HashBuilderOperatorFactory::~HashBuilderOperatorFactory() = default;

HashBuilderOperatorFactory *HashBuilderOperatorFactory::CreateHashBuilderOperatorFactory(JoinType joinType,
    const DataTypes &buildTypes, const int32_t *buildHashCols, int32_t buildHashColsCount, int32_t operatorCount)
{
    return new HashBuilderOperatorFactory(joinType, buildTypes, buildHashCols, buildHashColsCount, operatorCount);
}

HashBuilderOperatorFactory *HashBuilderOperatorFactory::CreateHashBuilderOperatorFactory(JoinType joinType,
    BuildSide buildSide, const DataTypes &buildTypes, const int32_t *buildHashCols, int32_t buildHashColsCount,
    int32_t operatorCount)
{
    return new HashBuilderOperatorFactory(joinType, buildSide, buildTypes, buildHashCols, buildHashColsCount,
        operatorCount);
}

Operator *HashBuilderOperatorFactory::CreateOperator()
{
    std::lock_guard<std::mutex> g(state_->mu);
    ++state_->operatorIndex;
    return new HashBuilderOperator(state_.get());
}

int32_t HashBuilderOperator::AddInput(VectorBatch *vecBatch)
{
    if (vecBatch == nullptr) {
        throw OmniException("INVALID_ARGUMENT", "AddInput of a null batch", -1);
    }
    if (vecBatch->GetRowCount() <= 0) {
        vec::VectorHelper::FreeVecBatch(vecBatch);
        return 0;
    }
    if (vecBatch->GetVectorCount() < state_->buildTypes.GetSize()) {
        vec::VectorHelper::FreeVecBatch(vecBatch);
        throw OmniException("OPERATOR_RUNTIME_ERROR", "build batch has fewer vectors than build types", -1);
    }
    omg::FlattenTaken(vecBatch);  // dictionary-encoded vectors -> flat device vectors
    std::lock_guard<std::mutex> g(state_->mu);
    if (state_->built) {
        vec::VectorHelper::FreeVecBatch(vecBatch);
        throw OmniException("OPERATOR_RUNTIME_ERROR", "AddInput after the hash table was built", -6);
    }
    state_->batches.push_back(vecBatch);
    return 0;
}

int32_t HashBuilderOperator::GetOutput(VectorBatch **outputVecBatch)
{
    if (outputVecBatch != nullptr) {
        *outputVecBatch = nullptr;
    }
    if (!noMoreInput_) {
        SetStatus(OMNI_STATUS_NORMAL);
        return 0;
    }
    if (isFinished()) {
        return 0;
    }
    std::lock_guard<std::mutex> g(state_->mu);
    if (!counted_) {
        counted_ = true;
        ++state_->finished;
    }
    // The single GPU table is built once every builder of the factory has finished (the
    // reference builds one partition per builder and unblocks probes when all are built).
    if (!state_->built && state_->finished >= state_->operatorCount) {
        if (userStreamSet_) {
            state_->stream.SetUser(userStream_);
        }
        state_->Build();
    }
    SetStatus(OMNI_STATUS_FINISHED);
    return 0;
}

// ------------------------------------------------------------------------------ probe
LookupJoinOperatorFactory::LookupJoinOperatorFactory(const DataTypes &probeTypes_, const int32_t *probeOutputCols_,
    int32_t probeOutputColsCount, const int32_t *probeHashCols_, int32_t probeHashColsCount,
    const int32_t *buildOutputCols_, int32_t buildOutputColsCount, const DataTypes &buildOutputTypes_,
    HashBuilderOperatorFactory *builder)
    : probeTypes(probeTypes_), buildOutputTypes(buildOutputTypes_), build(builder->GetBuildState())
{
    if (probeHashColsCount != static_cast<int32_t>(build->hashCols.size())) {
        throw OmniException("INVALID_ARGUMENT", "probe and build key column counts differ", -1);
    }
    probeOutputCols.assign(probeOutputCols_, probeOutputCols_ + probeOutputColsCount);
    probeHashCols.assign(probeHashCols_, probeHashCols_ + probeHashColsCount);
    buildOutputCols.assign(buildOutputCols_, buildOutputCols_ + buildOutputColsCount);
    for (int32_t i = 0; i < probeHashColsCount; ++i) {
        const int32_t k = probeHashCols[i];
        if (k < 0 || k >= probeTypes.GetSize() || !JoinKeyType(probeTypes.GetType(k)->GetId())) {
            throw OmniException("UNSUPPORTED_ERROR", "unsupported probe key column", -2);
        }
        // A hashed key tuple compares value bytes, so each probe key column has its build
        // column's width.
        if (build->multiKey &&
            probeTypes.GetType(k)->ByteWidth() != build->buildTypes.GetType(build->hashCols[i])->ByteWidth()) {
            throw OmniException("INVALID_ARGUMENT", "probe and build key columns differ in width", -1);
        }
    }
    if (buildOutputTypes.GetSize() != buildOutputColsCount) {
        throw OmniException("INVALID_ARGUMENT", "build output types and columns disagree", -1);
    }
    const bool existence = build->kind == omg::JOIN_KIND_EXISTENCE;
    if (build->kind == omg::JOIN_KIND_SEMI && buildOutputColsCount != 0) {
        // The reference's plan path passes none (lookup_join.cpp:117-121); which build row a
        // semi join would pair with a probe row is not part of its contract.
        throw OmniException("UNSUPPORTED_ERROR", "a left semi join has no build output columns", -2);
    }
    if (existence) {
        // The output is the probe columns and one BOOLEAN existence column; build output columns
        // are not read (lookup_join.cpp:1934-1938).
        buildOutputCols.clear();
        buildOutputTypes = DataTypes(std::vector<DataTypePtr>{BooleanType()});
    }
    if (probeOutputColsCount + static_cast<int32_t>(buildOutputCols.size()) + (existence ? 1 : 0) >
        omg::kMaxOutCols) {
        throw OmniException("UNSUPPORTED_ERROR", "too many join output columns", -2);
    }
    int32_t rowSize = 0;
    for (int32_t c : probeOutputCols) {
        if (c < 0 || c >= probeTypes.GetSize()) {
            throw OmniException("INVALID_ARGUMENT", "probe output column out of range", -1);
        }
        rowSize += probeTypes.GetType(c)->ByteWidth();
    }
    for (size_t i = 0; i < buildOutputCols.size(); ++i) {
        const int32_t c = buildOutputCols[i];
        if (c < 0 || c >= build->buildTypes.GetSize()) {
            throw OmniException("INVALID_ARGUMENT", "build output column out of range", -1);
        }
        rowSize += buildOutputTypes.GetType(static_cast<int32_t>(i))->ByteWidth();
    }
    if (existence) {
        rowSize += 1;
    }
    rowsPerBatch = GetMaxRowCount(rowSize);
}

namespace {
using omniruntime::expressions::Expr;
using omniruntime::expressions::ExprType;
using ExprOp = omniruntime::expressions::Operator;

// Value kind of a filter operand type: 0 integer-like (compared as int64), 1 double, 2 string
// (VARCHAR/CHAR), -1 none.
constexpr int kFilterInt = 0;
constexpr int kFilterDouble = 1;
constexpr int kFilterString = 2;

int FilterKind(const DataTypePtr &t)
{
    switch (t->GetId()) {
        case OMNI_BYTE:
        case OMNI_BOOLEAN:
        case OMNI_SHORT:
        case OMNI_INT:
        case OMNI_DATE32:
        case OMNI_LONG:
        case OMNI_DATE64:
        case OMNI_TIMESTAMP:
            return kFilterInt;
        case OMNI_DOUBLE:
            return kFilterDouble;
        case OMNI_VARCHAR:
        case OMNI_CHAR:
            return kFilterString;
        default:
            return -1;
    }
}

[[noreturn]] void FilterUnsupported(const std::string &what)
{
    throw OmniException("EXPRESSION_NOT_SUPPORT", "The expression is not supported yet: " + what, -2);
}

// The postfix program being compiled, with the factory's literal bytes.
struct FilterCode {
    const DataTypes &probeTypes;
    const DataTypes &buildTypes;
    std::vector<omg::FilterInstr> &code;
    std::vector<int32_t> &cols;
    std::string &text;
};

// Postfix code of `e`; `depth` is the evaluation stack depth before it.  Returns the kind of
// the value it leaves (FilterKind's codes).
int CompileFilter(const Expr *e, FilterCode &fc, int depth)
{
    if (e == nullptr) {
        FilterUnsupported("null node");
    }
    omg::FilterInstr in;
    std::memset(&in, 0, sizeof(in));
    auto push = [&](int32_t col) {
        if (depth + 1 > omg::kMaxFilterDepth || fc.code.size() >= static_cast<size_t>(omg::kMaxFilterInstrs)) {
            FilterUnsupported("filter too large");
        }
        fc.code.push_back(in);
        fc.cols.push_back(col);
    };
    auto emit = [&](int16_t op) {
        if (fc.code.size() >= static_cast<size_t>(omg::kMaxFilterInstrs)) {
            FilterUnsupported("filter too large");
        }
        in.op = op;
        fc.code.push_back(in);
        fc.cols.push_back(-1);
    };
    switch (e->GetType()) {
        case ExprType::FIELD_E: {
            const auto *f = static_cast<const omniruntime::expressions::FieldExpr *>(e);
            const int32_t nProbe = fc.probeTypes.GetSize();
            const bool probe = f->colVal < nProbe;
            const int32_t c = probe ? f->colVal : f->colVal - nProbe;
            if (f->colVal < 0 || (!probe && c >= fc.buildTypes.GetSize())) {
                throw OmniException("INVALID_ARGUMENT", "filter column out of range", -1);
            }
            const DataTypePtr &t = probe ? fc.probeTypes.GetType(c) : fc.buildTypes.GetType(c);
            const int kind = FilterKind(t);
            if (kind < 0) {
                FilterUnsupported("column of type " + std::to_string(t->GetId()));
            }
            if (kind == kFilterString) {
                in.op = probe ? omg::FOP_PROBE_STR : omg::FOP_BUILD_STR;
            } else {
                in.op = probe ? omg::FOP_PROBE_COL : omg::FOP_BUILD_COL;
                in.width = static_cast<int16_t>(t->ByteWidth());
                in.dbl = static_cast<int16_t>(kind);
            }
            push(c);
            return kind;
        }
        case ExprType::LITERAL_E: {
            const auto *l = static_cast<const omniruntime::expressions::LiteralExpr *>(e);
            const int kind = FilterKind(l->dataType);
            if (kind < 0) {
                FilterUnsupported("literal of type " + std::to_string(l->dataType->GetId()));
            }
            in.isNull = l->isNull ? 1 : 0;
            if (kind == kFilterString) {
                const std::string *v = l->isNull ? nullptr : l->stringVal;
                if (v != nullptr && v->size() > static_cast<size_t>(INT32_MAX - 16)) {
                    FilterUnsupported("string literal too long");
                }
                in.op = omg::FOP_STR_LITERAL;
                in.input = v == nullptr ? 0 : static_cast<int32_t>(v->size());
                in.imm = static_cast<int64_t>(fc.text.size());
                if (v != nullptr) {
                    fc.text += *v;
                }
                push(-1);
                return kind;
            }
            in.op = omg::FOP_LITERAL;
            in.dbl = static_cast<int16_t>(kind);
            if (kind == kFilterDouble) {
                std::memcpy(&in.imm, &l->doubleVal, sizeof(double));
            } else {
                in.imm = l->longVal;
            }
            push(-1);
            return kind;
        }
        case ExprType::BINARY_E: {
            const auto *b = static_cast<const omniruntime::expressions::BinaryExpr *>(e);
            int16_t op;
            switch (b->op) {
                case ExprOp::EQ: op = omg::FOP_EQ; break;
                case ExprOp::NEQ: op = omg::FOP_NEQ; break;
                case ExprOp::LT: op = omg::FOP_LT; break;
                case ExprOp::LTE: op = omg::FOP_LTE; break;
                case ExprOp::GT: op = omg::FOP_GT; break;
                case ExprOp::GTE: op = omg::FOP_GTE; break;
                case ExprOp::AND: op = omg::FOP_AND; break;
                case ExprOp::OR: op = omg::FOP_OR; break;
                case ExprOp::ADD: op = omg::FOP_ADD; break;
                case ExprOp::SUB: op = omg::FOP_SUB; break;
                case ExprOp::MUL: op = omg::FOP_MUL; break;
                case ExprOp::DIV: op = omg::FOP_DIV; break;
                case ExprOp::MOD: op = omg::FOP_MOD; break;
                case ExprOp::TRY_ADD: op = omg::FOP_TRY_ADD; break;
                case ExprOp::TRY_SUB: op = omg::FOP_TRY_SUB; break;
                case ExprOp::TRY_MUL: op = omg::FOP_TRY_MUL; break;
                case ExprOp::TRY_DIV: op = omg::FOP_TRY_DIV; break;
                default: FilterUnsupported("binary operator " + std::to_string(static_cast<int>(b->op)));
            }
            const int lk = CompileFilter(b->left, fc, depth);
            const int rk = CompileFilter(b->right, fc, depth + 1);
            const bool compare = op >= omg::FOP_EQ && op <= omg::FOP_GTE;
            if ((lk == kFilterString || rk == kFilterString) && !(compare && lk == rk)) {
                FilterUnsupported("string operand of binary operator " + std::to_string(static_cast<int>(b->op)));
            }
            if (op >= omg::FOP_ADD) {
                // Arithmetic (the reference's math functions): the node's return type sets the
                // result width (int32 or int64, which wrap) or double.
                const DataTypePtr &rt = b->GetReturnType();
                const int kind = rt ? FilterKind(rt) : -1;
                const int w = kind == kFilterInt ? rt->ByteWidth() : 8;
                if ((kind != kFilterInt && kind != kFilterDouble) || (kind == kFilterInt && w != 4 && w != 8)) {
                    FilterUnsupported("arithmetic result of type " + std::to_string(rt ? rt->GetId() : -1));
                }
                in.width = static_cast<int16_t>(w);
                in.dbl = static_cast<int16_t>(kind);
                emit(op);
                return kind;
            }
            emit(op);
            return kFilterInt;
        }
        case ExprType::UNARY_E: {
            const auto *u = static_cast<const omniruntime::expressions::UnaryExpr *>(e);
            if (u->op != ExprOp::NOT) {
                FilterUnsupported("unary operator " + std::to_string(static_cast<int>(u->op)));
            }
            if (CompileFilter(u->exp, fc, depth) == kFilterString) {
                FilterUnsupported("NOT of a string");
            }
            emit(omg::FOP_NOT);
            return kFilterInt;
        }
        case ExprType::IS_NULL_E: {
            const auto *n = static_cast<const omniruntime::expressions::IsNullExpr *>(e);
            CompileFilter(n->value, fc, depth);
            emit(omg::FOP_IS_NULL);
            return kFilterInt;
        }
        case ExprType::FUNC_E: {
            // substr(str, start[, length]) with INT or LONG positions (func_registry_string.cpp:
            // 440-466), under the substr policies in force when the factory is created.
            const auto *fn = static_cast<const omniruntime::expressions::FuncExpr *>(e);
            const size_t n = fn->arguments.size();
            // Buffer-free string functions (func_registry_string.cpp:286-380): their registered
            // argument types, NULL in, NULL out except Greatest / Least.
            static const std::map<std::string, std::pair<int16_t, int>> kStrFns = {
                {"length", {omg::SFN_LENGTH, 1}}, {"char_length", {omg::SFN_LENGTH, 1}},
                {"instr", {omg::SFN_INSTR, 2}}, {"StartsWith", {omg::SFN_STARTS_WITH, 2}},
                {"EndsWith", {omg::SFN_ENDS_WITH, 2}}, {"Contains", {omg::SFN_CONTAINS, 2}},
                {"Greatest", {omg::SFN_GREATEST, 2}}, {"Least", {omg::SFN_LEAST, 2}}};
            if (fn->funcName == "CAST" && n == 1) {
                // Numeric CAST (func_registry_math.cpp:172-194,355-366): integer-like to integer-
                // like or DOUBLE, DOUBLE to LONG / INT (RoundingRule::DOWN, the default).
                const DataTypePtr &rt = fn->GetReturnType();
                const Expr *arg = fn->arguments[0];
                const DataTypePtr at = arg == nullptr ? nullptr : arg->GetReturnType();
                const int rk = rt ? FilterKind(rt) : -1;
                const int ak = CompileFilter(arg, fc, depth);
                const int rw = rk == kFilterInt ? rt->ByteWidth() : 8;
                const bool intTarget = rk == kFilterInt && (rw == 1 || rw == 2 || rw == 4 || rw == 8);
                if (ak == kFilterString || (rk != kFilterDouble && !intTarget) ||
                    (ak == kFilterDouble && rk == kFilterInt && rw != 4 && rw != 8) || at == nullptr) {
                    FilterUnsupported("CAST from type " + std::to_string(at ? at->GetId() : -1) + " to " +
                        std::to_string(rt ? rt->GetId() : -1));
                }
                in.width = static_cast<int16_t>(rw);
                in.dbl = static_cast<int16_t>(rk == kFilterDouble ? 1 : 0);
                emit(omg::FOP_CAST);
                return rk;
            }
            const auto sf = kStrFns.find(fn->funcName);
            if (sf != kStrFns.end()) {
                if (n != static_cast<size_t>(sf->second.second)) {
                    FilterUnsupported("function " + fn->funcName + " with " + std::to_string(n) + " arguments");
                }
                in.imm = -1;
                for (size_t a = 0; a < n; ++a) {
                    const Expr *arg = fn->arguments[a];
                    const DataTypePtr &t = arg == nullptr ? nullptr : arg->GetReturnType();
                    const int32_t id = t ? t->GetId() : -1;
                    // length / char_length also take CHAR (LengthChar: the declared width)
                    const bool ok = id == OMNI_VARCHAR || (id == OMNI_CHAR && sf->second.first == omg::SFN_LENGTH);
                    if (CompileFilter(arg, fc, depth + static_cast<int>(a)) != kFilterString || !ok) {
                        FilterUnsupported(fn->funcName + " of type " + std::to_string(id));
                    }
                    if (id == OMNI_CHAR) {
                        in.imm = t->GetWidth();
                    }
                }
                in.width = sf->second.first;
                emit(omg::FOP_STRFN);
                const bool str = sf->second.first == omg::SFN_GREATEST || sf->second.first == omg::SFN_LEAST;
                return str ? kFilterString : kFilterInt;
            }
            if (fn->funcName != "substr" || (n != 2 && n != 3)) {
                FilterUnsupported("function " + fn->funcName + " with " + std::to_string(n) + " arguments");
            }
            if (CompileFilter(fn->arguments[0], fc, depth) != kFilterString) {
                FilterUnsupported("substr of a non-string");
            }
            for (size_t a = 1; a < n; ++a) {
                const Expr *arg = fn->arguments[a];
                const DataTypePtr &t = arg->GetReturnType();
                if (CompileFilter(arg, fc, depth + static_cast<int>(a)) != kFilterInt || t == nullptr ||
                    (t->GetId() != OMNI_INT && t->GetId() != OMNI_LONG)) {
                    FilterUnsupported("substr position of type " + std::to_string(t ? t->GetId() : -1));
                }
            }
            in.width = static_cast<int16_t>(n);
            const bool negative =
                GetNegativeStartIndexOutOfBoundsRule() == NegativeStartIndexOutOfBoundsRule::INTERCEPT_FROM_BEYOND;
            const bool zero = GetZeroStartIndexSupportRule() == ZeroStartIndexSupportRule::IS_SUPPORT;
            in.input = (negative ? omg::kFilterSubstrNegative : 0) | (zero ? omg::kFilterSubstrZero : 0);
            emit(omg::FOP_SUBSTR);
            return kFilterString;
        }
        case ExprType::IF_E: {
            const auto *x = static_cast<const omniruntime::expressions::IfExpr *>(e);
            if (CompileFilter(x->condition, fc, depth) == kFilterString) {
                FilterUnsupported("IF on a string condition");
            }
            const int tk = CompileFilter(x->trueExpr, fc, depth + 1);
            if (CompileFilter(x->falseExpr, fc, depth + 2) != tk) {
                FilterUnsupported("IF branches of different kinds");
            }
            emit(omg::FOP_IF);
            return tk;
        }
        case ExprType::SWITCH_E: {
            // CASE WHEN c1 THEN r1 ... ELSE e END as IF(c1, r1, IF(c2, r2, ... e)): the clauses'
            // conditions and results, the ELSE value, then one IF per clause.
            const auto *x = static_cast<const omniruntime::expressions::SwitchExpr *>(e);
            if (x->whenClause.empty()) {
                FilterUnsupported("CASE without WHEN");
            }
            int d = depth;
            int kind = -2;
            for (const auto &w : x->whenClause) {
                if (CompileFilter(w.first, fc, d++) == kFilterString) {
                    FilterUnsupported("CASE on a string condition");
                }
                const int rk = CompileFilter(w.second, fc, d++);
                if (kind != -2 && rk != kind) {
                    FilterUnsupported("CASE results of different kinds");
                }
                kind = rk;
            }
            if (CompileFilter(x->falseExpr, fc, d) != kind) {
                FilterUnsupported("CASE results of different kinds");
            }
            for (size_t i = 0; i < x->whenClause.size(); ++i) {
                emit(omg::FOP_IF);
            }
            return kind;
        }
        case ExprType::COALESCE_E: {
            const auto *x = static_cast<const omniruntime::expressions::CoalesceExpr *>(e);
            const int k = CompileFilter(x->value1, fc, depth);
            if (CompileFilter(x->value2, fc, depth + 1) != k) {
                FilterUnsupported("COALESCE of different kinds");
            }
            emit(omg::FOP_COALESCE);
            return k;
        }
        case ExprType::BETWEEN_E:
        case ExprType::IN_E: {
            // The value's type must be one the reference's IN / BETWEEN code handles
            // (expression_codegen.cpp:599-640, :2119-2160), and every operand of its kind.
            const bool between = e->GetType() == ExprType::BETWEEN_E;
            std::vector<const Expr *> args;
            if (between) {
                const auto *x = static_cast<const omniruntime::expressions::BetweenExpr *>(e);
                args = {x->value, x->lowerBound, x->upperBound};
            } else {
                const auto *x = static_cast<const omniruntime::expressions::InExpr *>(e);
                args.assign(x->arguments.begin(), x->arguments.end());
                if (args.size() < 2) {
                    FilterUnsupported("IN without a list");
                }
            }
            const DataTypePtr vt = args[0] == nullptr ? nullptr : args[0]->GetReturnType();
            const int32_t id = vt ? vt->GetId() : -1;
            if (id != OMNI_INT && id != OMNI_LONG && id != OMNI_DATE32 && id != OMNI_TIMESTAMP && id != OMNI_DOUBLE &&
                id != OMNI_VARCHAR && id != OMNI_CHAR) {
                FilterUnsupported(std::string(between ? "BETWEEN" : "IN") + " of type " + std::to_string(id));
            }
            if (!between) {
                in.op = omg::FOP_IN_BEGIN;
                push(-1);
            }
            const int base = between ? depth : depth + 1;
            const int k = CompileFilter(args[0], fc, base);
            auto isString = [](int32_t t) { return t == OMNI_VARCHAR || t == OMNI_CHAR; };
            for (size_t a = 1; a < args.size(); ++a) {
                // ExprVerifier::AreInvalidDataTypes (expr_verifier.cpp:25-29): the same type, or both
                // strings.
                const DataTypePtr at = args[a] == nullptr ? nullptr : args[a]->GetReturnType();
                const int32_t aid = at ? at->GetId() : -1;
                if (CompileFilter(args[a], fc, between ? base + static_cast<int>(a) : base + 1) != k ||
                    (aid != id && !(isString(aid) && isString(id)))) {
                    FilterUnsupported(std::string(between ? "BETWEEN" : "IN") + " operands of different types");
                }
                if (!between) {
                    emit(omg::FOP_IN_STEP);
                }
            }
            emit(between ? omg::FOP_BETWEEN : omg::FOP_IN_END);
            return kFilterInt;
        }
        default:
            FilterUnsupported("expression kind " + std::to_string(static_cast<int>(e->GetType())));
    }
}
}  // namespace

LookupJoinOperatorFactory *LookupJoinOperatorFactory::CreateLookupJoinOperatorFactory(const DataTypes &probeTypes,
    int32_t *probeOutputCols, int32_t probeOutputColsCount, int32_t *probeHashCols, int32_t probeHashColsCount,
    int32_t *buildOutputCols, int32_t buildOutputColsCount, const DataTypes &buildOutputTypes,
    int64_t hashBuilderFactoryAddr, const void *filterExpr, bool isShuffleExchangeBuildPlan, const void *overflowConfig)
{
    (void)isShuffleExchangeBuildPlan;
    (void)overflowConfig;
    auto *builder = reinterpret_cast<HashBuilderOperatorFactory *>(hashBuilderFactoryAddr);
    if (builder == nullptr) {
        throw OmniException("INVALID_ARGUMENT", "null hash builder factory", -1);
    }
    std::unique_ptr<LookupJoinOperatorFactory> f(new LookupJoinOperatorFactory(probeTypes, probeOutputCols,
        probeOutputColsCount, probeHashCols, probeHashColsCount, buildOutputCols, buildOutputColsCount,
        buildOutputTypes, builder));
    if (filterExpr != nullptr) {
        // JoinFilterCodeGen (lookup_join.cpp:175-187): compiled once per factory.
        // The filter returns BOOLEAN (SimpleFilter::Initialize, filter_and_project.cpp:51-54).
        const auto *root = static_cast<const Expr *>(filterExpr);
        if (root->GetReturnType() == nullptr || root->GetReturnType()->GetId() != OMNI_BOOLEAN) {
            FilterUnsupported("a filter that does not return BOOLEAN");
        }
        FilterCode fc{probeTypes, f->build->buildTypes, f->filter, f->filterCols, f->filterText};
        CompileFilter(root, fc, 0);
        if (f->filter.empty()) {
            FilterUnsupported("empty filter");
        }
    }
    return f.release();
}

Operator *LookupJoinOperatorFactory::CreateOperator() { return new LookupJoinOperator(*this); }

// One direct probe call between its launch and its completion: the batches it reads, its
// kernel parameters and outputs, and the event that marks its kernel and count copy done.
struct LookupJoinOperator::ProbeCall {
    std::vector<VectorBatch *> batches;
    omg::BatchTable bt;
    omg::ProbeLaunch p;
    std::vector<omg::OutColumn> cols;
    size_t nOut = 0;
    size_t nProbeOut = 0;
    int32_t nRegions = 0;
    uint64_t regionCap = 0;
    bool hostDirect = false;
    DevArray<unsigned long long> count;
    omg::PinnedArray<unsigned long long> hostCount;
    DevArray<int64_t> packKeys;   // packed multi-column probe keys (scratch input)
    DevArray<uint8_t> packNulls;
    omg::KernelTimer timer;
    cudaEvent_t done = nullptr;
    cudaStream_t s = nullptr;
    ~ProbeCall()
    {
        if (done != nullptr) {
            cudaEventSynchronize(done);  // the kernel may still read `batches`
            cudaEventDestroy(done);
            cudaGetLastError();
        }
        for (auto *b : batches) {
            vec::VectorHelper::FreeVecBatch(b);
        }
    }
};

struct LookupJoinOperator::Impl {
    omg::OpStream stream;
    omg::KernelTimer timer;
    // Probe calls launched and not yet finished, oldest first (the worker's once it runs).
    std::deque<std::unique_ptr<ProbeCall>> inflight;
    // Worker pipeline (pipelined callers).  The caller hands over full chunks of batches; the
    // worker launches each chunk's probe, finishes the oldest call once another is queued behind
    // it (or its kernel is done, or a flush was asked for) and moves its output batches to
    // `ready`.  `busy` counts chunks handed over and not finished.
    std::thread worker;
    std::mutex mu;
    std::condition_variable wake;      // to the worker: a chunk, a flush or stop
    std::condition_variable progress;  // to the caller: a chunk finished, or an error
    std::deque<std::vector<VectorBatch *>> chunks;
    std::deque<VectorBatch *> ready;
    int32_t busy = 0;
    bool flush = false;
    bool stop = false;
    std::exception_ptr error;
    int device = 0;
    omg::DevArray<uint8_t> filterText;  // the filter's string literals in HBM
};

namespace {
constexpr int32_t kMaxChunksAhead = 3;  // chunks handed to the worker before AddInput waits
}

LookupJoinOperator::LookupJoinOperator(const LookupJoinOperatorFactory &f) : f_(f), impl_(new Impl()) {}

LookupJoinOperator::~LookupJoinOperator() { Close(); }

void LookupJoinOperator::StopWorker()
{
    Impl &im = *impl_;
    if (!im.worker.joinable()) {
        return;
    }
    {
        std::lock_guard<std::mutex> g(im.mu);
        im.stop = true;
    }
    im.wake.notify_all();
    im.worker.join();
    for (auto &c : im.chunks) {
        for (auto *b : c) {
            vec::VectorHelper::FreeVecBatch(b);
        }
    }
    im.chunks.clear();
    for (auto *b : im.ready) {
        vec::VectorHelper::FreeVecBatch(b);
    }
    im.ready.clear();
    im.busy = 0;
}

OmniStatus LookupJoinOperator::Close()
{
    StopWorker();
    impl_->inflight.clear();  // waits for their kernels, frees their batches
    for (auto *b : pending_) {
        vec::VectorHelper::FreeVecBatch(b);
    }
    pending_.clear();
    pendingRows_ = 0;
    for (auto *b : outputs_) {
        vec::VectorHelper::FreeVecBatch(b);
    }
    outputs_.clear();
    return OMNI_STATUS_NORMAL;
}

BlockingReason LookupJoinOperator::IsBlocked()
{
    std::lock_guard<std::mutex> g(f_.build->mu);
    return f_.build->built ? BlockingReason::kNotBlocked : BlockingReason::kWaitForJoinBuild;
}

int32_t LookupJoinOperator::AddInput(VectorBatch *vecBatch)
{
    if (vecBatch == nullptr) {
        throw OmniException("INVALID_ARGUMENT", "AddInput of a null batch", -1);
    }
    if (vecBatch->GetRowCount() <= 0) {
        vec::VectorHelper::FreeVecBatch(vecBatch);
        SetStatus(OMNI_STATUS_NORMAL);
        return 0;
    }
    if (vecBatch->GetVectorCount() < f_.probeTypes.GetSize()) {
        vec::VectorHelper::FreeVecBatch(vecBatch);
        throw OmniException("OPERATOR_RUNTIME_ERROR", "probe batch has fewer vectors than probe types", -1);
    }
    omg::FlattenTaken(vecBatch);  // dictionary-encoded vectors -> flat device vectors
    pending_.push_back(vecBatch);
    pendingRows_ += vecBatch->GetRowCount();
    SetStatus(OMNI_STATUS_NORMAL);
    // Pipelined callers: a full chunk goes to the worker thread, which launches it at once, so
    // that its kernel runs while the caller queues the next chunk.
    if (!noMoreInput_ && pendingRows_ >= omg::ProbeChunkRows() &&
        (impl_->worker.joinable() || (strategy_ == kJoinDirect && f_.build->built))) {
        HandOff();
    }
    return 0;
}

void LookupJoinOperator::HandOff()
{
    Impl &im = *impl_;
    if (!im.worker.joinable()) {
        omg::RequireDevice();
        CudaCheck(cudaGetDevice(&im.device), "cudaGetDevice");
        im.worker = std::thread([this] { RunWorker(); });
    }
    std::unique_lock<std::mutex> lk(im.mu);
    im.progress.wait(lk, [&] { return im.busy < kMaxChunksAhead || im.error; });
    if (im.error) {
        std::exception_ptr e = im.error;
        lk.unlock();
        std::rethrow_exception(e);
    }
    im.chunks.push_back(std::move(pending_));
    pending_.clear();
    pendingRows_ = 0;
    ++im.busy;
    lk.unlock();
    im.wake.notify_one();
}

void LookupJoinOperator::RunWorker()
{
    Impl &im = *impl_;
    cudaSetDevice(im.device);
    auto &fl = im.inflight;
    for (;;) {
        std::vector<VectorBatch *> chunk;
        bool finish = false;
        {
            std::unique_lock<std::mutex> lk(im.mu);
            for (;;) {
                if (im.stop) {
                    return;
                }
                if (!im.chunks.empty() && !im.error) {
                    chunk = std::move(im.chunks.front());
                    im.chunks.pop_front();
                    break;
                }
                if (!fl.empty()) {
                    finish = im.flush || fl.size() > 1;
                    if (!finish) {
                        const cudaError_t q = cudaEventQuery(fl.front()->done);
                        cudaGetLastError();  // "not ready" is not an error
                        finish = q != cudaErrorNotReady;
                    }
                    if (finish) {
                        break;
                    }
                    im.wake.wait_for(lk, std::chrono::microseconds(50));  // poll the kernel
                    continue;
                }
                im.wake.wait(lk);
            }
        }
        try {
            if (!chunk.empty()) {
                const auto t0 = std::chrono::steady_clock::now();
                fl.push_back(LaunchBatches(std::move(chunk)));
                counters_[8] +=
                    std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
            } else if (finish) {
                std::unique_ptr<ProbeCall> pc = std::move(fl.front());
                fl.pop_front();
                std::deque<VectorBatch *> out;
                FinishProbe(*pc, out);
                pc.reset();
                {
                    std::lock_guard<std::mutex> g(im.mu);
                    for (auto *b : out) {
                        im.ready.push_back(b);
                    }
                    --im.busy;
                }
                im.progress.notify_all();
            }
        } catch (...) {
            fl.clear();  // waits for their kernels, frees their batches
            {
                std::lock_guard<std::mutex> g(im.mu);
                im.error = std::current_exception();
                for (auto &c : im.chunks) {
                    for (auto *b : c) {
                        vec::VectorHelper::FreeVecBatch(b);
                    }
                }
                im.chunks.clear();
                im.busy = 0;
            }
            im.progress.notify_all();
        }
    }
}

int32_t LookupJoinOperator::GetOutputFromWorker(VectorBatch **outputVecBatch)
{
    Impl &im = *impl_;
    std::unique_lock<std::mutex> lk(im.mu);
    if (noMoreInput_) {
        // The last, partial chunk, then wait for an output batch or the end of the work.
        if (!pending_.empty() && !im.error) {
            im.chunks.push_back(std::move(pending_));
            pending_.clear();
            pendingRows_ = 0;
            ++im.busy;
        }
        im.flush = true;
        im.wake.notify_one();
        im.progress.wait(lk, [&] { return !im.ready.empty() || im.busy == 0 || im.error; });
    }
    if (im.error) {
        std::exception_ptr e = im.error;
        lk.unlock();
        std::rethrow_exception(e);
    }
    if (!im.ready.empty()) {
        *outputVecBatch = im.ready.front();
        im.ready.pop_front();
    }
    if (noMoreInput_ && im.busy == 0 && im.ready.empty() && pending_.empty()) {
        SetStatus(OMNI_STATUS_FINISHED);
    }
    return 0;
}

void LookupJoinOperator::ProcessPending()
{
    if (strategy_ != kJoinDirect && ProcessPartitioned()) {
        return;
    }
    std::unique_ptr<ProbeCall> pc = LaunchPending();
    FinishProbe(*pc, outputs_);
}

// Take the queued batches, set up the probe and launch it; FinishProbe completes it.
std::unique_ptr<LookupJoinOperator::ProbeCall> LookupJoinOperator::LaunchPending()
{
    std::vector<VectorBatch *> batches;
    batches.swap(pending_);
    pendingRows_ = 0;
    return LaunchBatches(std::move(batches));
}

std::unique_ptr<LookupJoinOperator::ProbeCall> LookupJoinOperator::LaunchBatches(std::vector<VectorBatch *> &&batches)
{
    std::unique_ptr<ProbeCall> call(new ProbeCall());
    ProbeCall &pc = *call;
    pc.batches = std::move(batches);
    JoinBuildState &b = *f_.build;
    omg::RequireDevice();
    if (userStreamSet_) {
        impl_->stream.SetUser(userStream_);
    }
    cudaStream_t s = impl_->stream.Get();
    // Kernel inputs: probe key first, then the probe output columns.
    // Kernel inputs: the probe key column(s) first, then the probe output columns.
    std::vector<int32_t> inputCols;
    std::map<int32_t, int32_t> inputOf;
    for (int32_t c : f_.probeHashCols) {
        if (inputOf.count(c) == 0) {
            inputOf[c] = static_cast<int32_t>(inputCols.size());
            inputCols.push_back(c);
        }
    }
    for (int32_t c : f_.probeOutputCols) {
        if (inputOf.count(c) == 0) {
            inputOf[c] = static_cast<int32_t>(inputCols.size());
            inputCols.push_back(c);
        }
    }
    for (size_t i = 0; i < f_.filter.size(); ++i) {
        const int32_t c = f_.filterCols[i];
        const int16_t op = f_.filter[i].op;
        if ((op == omg::FOP_PROBE_COL || op == omg::FOP_PROBE_STR) && inputOf.count(c) == 0) {
            if (inputCols.size() >= static_cast<size_t>(omg::kMaxInputs)) {
                throw OmniException("UNSUPPORTED_ERROR", "too many probe columns for the join kernels", -2);
            }
            inputOf[c] = static_cast<int32_t>(inputCols.size());
            inputCols.push_back(c);
        }
    }
    // Packed multi-column keys: one more kernel input, a scratch column per batch (64-row aligned,
    // so that each batch's NULL bitmap starts on a word) that a packing pass fills before the probe.
    int32_t packInput = -1;
    if (b.packed) {
        if (inputCols.size() >= static_cast<size_t>(omg::kMaxInputs)) {
            throw OmniException("UNSUPPORTED_ERROR", "too many probe columns for the join kernels", -2);
        }
        packInput = static_cast<int32_t>(inputCols.size());
        inputCols.push_back(f_.probeHashCols[0]);  // placeholder, repointed below
    }
    omg::BatchTable &bt = pc.bt;
    bt.Build(pc.batches, inputCols);
    const int64_t probeRows = bt.TotalRows();
    const size_t nProbeOut = f_.probeOutputCols.size();
    const size_t nOut = nProbeOut + (b.kind == omg::JOIN_KIND_EXISTENCE ? 1 : f_.buildOutputCols.size());
    pc.cols.assign(nOut, omg::OutColumn{});
    std::vector<omg::OutColumn> &cols = pc.cols;
    omg::ProbeLaunch &p = pc.p;
    std::memset(&p, 0, sizeof(p));
    p.nTiles = bt.NumTiles();
    p.keyInput = b.multiKey ? -1 : (b.packed ? packInput : 0);
    p.keyWidth = b.packed ? 8 : f_.probeTypes.GetType(f_.probeHashCols[0])->ByteWidth();
    if (b.packed) {
        // The bitmap kernel packs the parts as it reads them; for the other kernels LaunchProbe
        // fills the scratch input first.
        p.pack = b.pack;
        p.pack.outInput = packInput;
        for (int k = 0; k < p.pack.nParts; ++k) {
            p.pack.input[k] = inputOf[f_.probeHashCols[k]];
            p.pack.width[k] = f_.probeTypes.GetType(f_.probeHashCols[k])->ByteWidth();
        }
    }
    if (b.multiKey) {
        p.nKeyCols = static_cast<int32_t>(f_.probeHashCols.size());
        for (int32_t k = 0; k < p.nKeyCols; ++k) {
            p.keyCols[k].input = static_cast<int16_t>(inputOf[f_.probeHashCols[k]]);
            p.keyCols[k].width = static_cast<int16_t>(f_.probeTypes.GetType(f_.probeHashCols[k])->ByteWidth());
            p.keyCols[k].buildValues = b.colValues[b.hashCols[k]].Get();
            p.keyCols[k].buildOffs = b.colOffs[b.hashCols[k]].Get();
        }
    }
    p.table = b.table;
    p.joinKind = b.kind;
    p.visited = b.TracksVisits() ? b.visited.Get() : nullptr;
    // Join filter: bind probe operands to kernel inputs and build operands to the build columns.
    p.nFilter = static_cast<int32_t>(f_.filter.size());
    if (!f_.filterText.empty() && impl_->filterText.Get() == nullptr) {
        // The string literals' bytes, once per operator (the factory's copy outlives the copy).
        impl_->filterText.Reset(f_.filterText.size(), s);
        CudaCheck(cudaMemcpyAsync(impl_->filterText.Get(), f_.filterText.data(), f_.filterText.size(),
                      cudaMemcpyHostToDevice, s),
            "filter literals");
    }
    for (size_t i = 0; i < f_.filter.size(); ++i) {
        omg::FilterInstr in = f_.filter[i];
        in.payloadShift = 0;  // set below when the column is a slot-payload field
        const int32_t c = f_.filterCols[i];
        if (in.op == omg::FOP_PROBE_COL || in.op == omg::FOP_PROBE_STR) {
            in.input = inputOf[c];
        } else if (in.op == omg::FOP_BUILD_COL || in.op == omg::FOP_BUILD_STR) {
            in.values = b.colValues[c].Get();
            in.nulls = b.colHasNull[c] ? b.colNulls[c].Get() : nullptr;
            in.offs = in.op == omg::FOP_BUILD_STR ? b.colOffs[c].Get() : nullptr;
        } else if (in.op == omg::FOP_STR_LITERAL) {
            in.values = impl_->filterText.Get() + in.imm;
        }
        p.filter[i] = in;
    }
    const bool nullBuild = b.kind == omg::JOIN_KIND_PROBE_OUTER || b.kind == omg::JOIN_KIND_FULL ||
        b.kind == omg::JOIN_KIND_ANTI;  // rows without a match carry NULL build columns
    p.nOut = static_cast<int32_t>(nOut);
    for (size_t o = 0; o < nOut; ++o) {
        omg::JoinOutCol &oc = p.out[o];
        if (o < nProbeOut) {
            const int32_t c = f_.probeOutputCols[o];
            const auto &t = f_.probeTypes.GetType(c);
            oc.side = 0;
            oc.src = static_cast<int16_t>(inputOf[c]);
            oc.width = static_cast<int16_t>(t->ByteWidth());
            cols[o].type = t->GetId();
            cols[o].hasNull = bt.AnyNulls(oc.src);
        } else if (b.kind == omg::JOIN_KIND_EXISTENCE) {
            oc.side = 2;
            oc.src = 0;
            oc.width = 1;
            cols[o].type = OMNI_BOOLEAN;
            cols[o].hasNull = false;
        } else {
            const size_t j = o - nProbeOut;
            const int32_t c = f_.buildOutputCols[j];
            const auto &t = f_.buildOutputTypes.GetType(static_cast<int32_t>(j));
            oc.side = 1;
            oc.src = static_cast<int16_t>(c);
            oc.width = static_cast<int16_t>(b.buildTypes.GetType(c)->ByteWidth());
            oc.buildValues = b.colValues[c].Get();
            oc.buildNulls = b.colHasNull[c] ? b.colNulls[c].Get() : nullptr;
            cols[o].type = t->GetId();
            cols[o].hasNull = b.colHasNull[c] || nullBuild;
        }
        cols[o].width = oc.width;
    }
    // Unique build keys and <= 8 bytes of NULL-free build output per row: fetch the build
    // values with the table entry from a per-slot packed copy (built once per factory).
    {
        bool eligible = b.table.unique && nOut > nProbeOut && b.kind != omg::JOIN_KIND_EXISTENCE && !b.multiKey;
        int shift = 0;
        for (size_t o = nProbeOut; o < nOut && eligible; ++o) {
            const int w = p.out[o].width;
            eligible = (w == 1 || w == 2 || w == 4 || w == 8) && !b.colHasNull[p.out[o].src] && shift + 8 * w <= 64;
            p.out[o].shift = static_cast<int16_t>(shift);
            shift += 8 * w;
        }
        std::lock_guard<std::mutex> g(f_.payloadMu);
        if (eligible && !f_.payloadDecided) {
            const uint64_t nSlots = b.table.mode == omg::JOIN_ARRAY ? b.table.range : b.table.capacity;
            f_.slotPayload = omg::Buffer::NewDevice((nSlots + 1) * sizeof(uint64_t), s, false);
            CudaCheck(omg::LaunchBuildSlotPayload(p, nSlots, static_cast<uint64_t *>(f_.slotPayload->Data()), s),
                "build slot payload");
            impl_->stream.Sync();
            f_.payloadDecided = true;
        }
        // Occupancy bitmap of a unique ARRAY table, for the bitmap probe (kinds that mark no
        // build rows; with or without a slot payload).
        const bool wantBits = b.table.unique && b.table.mode == omg::JOIN_ARRAY && !b.multiKey;
        if (wantBits && !f_.slotBits) {
            f_.slotBits = omg::Buffer::NewDevice(omg::SlotBitsBytes(b.table.range), s, false);
            CudaCheck(omg::LaunchBuildSlotBits(b.table.arrayEntries, b.table.range,
                          static_cast<uint32_t *>(f_.slotBits->Data()), s),
                "build slot bitmap");
            impl_->stream.Sync();
        }
        if (eligible && f_.slotPayload) {
            p.table.slotPayload = static_cast<const uint64_t *>(f_.slotPayload->Data());
            // Filter operands that are build output columns packed into the payload.
            for (int32_t i = 0; i < p.nFilter; ++i) {
                omg::FilterInstr &in = p.filter[i];
                in.payloadShift = 0;
                for (size_t o = nProbeOut; in.op == omg::FOP_BUILD_COL && o < nOut; ++o) {
                    if (p.out[o].src == f_.filterCols[i] && p.out[o].width == in.width) {
                        in.payloadShift = p.out[o].shift + 1;
                    }
                }
            }
        }
        if (wantBits && f_.slotBits) {
            p.table.slotBits = static_cast<const uint32_t *>(f_.slotBits->Data());
        }
    }
    // Output regions: tile t writes into region t % nRegions (see ProbeLaunch).  A region's
    // capacity starts at its probe rows (times up to 2 for duplicate build keys), rounded to 64
    // rows so that every region starts on a byte of the null bitmaps.
    const int32_t nRegions = std::max(1, std::min<int32_t>(omg::kMaxRegions, bt.NumTiles()));
    const std::vector<int64_t> regionRows = bt.RegionRows(nRegions);
    uint64_t regionCap = 1;
    for (int64_t r : regionRows) {
        regionCap = std::max<uint64_t>(regionCap, static_cast<uint64_t>(r));
    }
    if (!b.table.unique) {
        regionCap *= std::min<uint32_t>(b.maxDup, 2);
    }
    regionCap = (regionCap + 63) / 64 * 64;
    // The region counters, then one more 128-byte line whose first word is the kernel's error.
    pc.count.Reset(static_cast<size_t>(nRegions + 1) * omg::kRegionStride, s, true);
    pc.hostCount.Reset(static_cast<size_t>(nRegions + 1) * omg::kRegionStride);
    p.outCount = pc.count.Get();
    p.error = reinterpret_cast<int32_t *>(pc.count.Get() + static_cast<size_t>(nRegions) * omg::kRegionStride);
    p.waitBudget = omg::WaitBudget();
    p.nRegions = nRegions;
    p.singleBatch = pc.batches.size() == 1 ? 1 : 0;
    // Host output without VARCHAR columns: the kernel writes the rows straight into pinned host
    // memory over the CPU-GPU link, so no device-to-host copy follows the probe.
    bool hostDirect = !deviceOutput_;
    for (size_t o = 0; o < nOut; ++o) {
        hostDirect = hostDirect && cols[o].width != 0;
    }
    pc.hostDirect = hostDirect;
    p.hostOutput = hostDirect ? 1 : 0;
    p.deviceKeys = b.packed || (!b.multiKey && bt.AllOnDevice(p.keyInput)) ? 1 : 0;
    pc.regionCap = regionCap;
    pc.nRegions = nRegions;
    pc.nOut = nOut;
    pc.nProbeOut = nProbeOut;
    pc.s = s;
    if (b.packed && !omg::ProbePacksKeys(p)) {
        // A packing pass fills the scratch key input before the probe (see LaunchProbe).
        bool anyNull = false;
        for (int32_t c : f_.probeHashCols) {
            anyNull = anyNull || bt.AnyNulls(inputOf[c]);
        }
        std::vector<int64_t> base(pc.batches.size() + 1, 0);
        for (size_t i = 0; i < pc.batches.size(); ++i) {
            base[i + 1] = base[i] + (bt.BatchRows(i) + 63) / 64 * 64;
        }
        pc.packKeys.Reset(static_cast<size_t>(std::max<int64_t>(base.back(), 1)), s);
        if (anyNull) {
            pc.packNulls.Reset(static_cast<size_t>(std::max<int64_t>(base.back() / 8, 8)), s, false);
        }
        for (size_t i = 0; i < pc.batches.size(); ++i) {
            bt.SetInput(i, packInput, pc.packKeys.Get() + base[i]);
            bt.SetInputNulls(i, packInput, anyNull ? pc.packNulls.Get() + base[i] / 8 : nullptr);
        }
    }
    bt.Upload(s);
    p.batches = bt.DeviceBatches();
    p.tiles = bt.DeviceTiles();
    LaunchAttempt(pc);
    return call;
}

// Output buffers for the call's region capacity, the kernel, and the asynchronous copy of the
// region counts; the call's event marks the end.
void LookupJoinOperator::LaunchAttempt(ProbeCall &pc)
{
    cudaStream_t s = pc.s;
    omg::ProbeLaunch &p = pc.p;
    const uint64_t capacity = pc.regionCap * static_cast<uint64_t>(pc.nRegions);
    for (size_t o = 0; o < pc.nOut; ++o) {
        omg::OutColumn &c = pc.cols[o];
        // VARCHAR columns hold an 8-byte row handle per output row until the second pass.
        const size_t vw = c.width == 0 ? 8 : static_cast<size_t>(c.width);
        const size_t nb = omg::NullBitmapBytes(static_cast<int64_t>(capacity));
        c.values = pc.hostDirect ? omg::Buffer::NewHost(capacity * vw + 16, false)
                                 : omg::Buffer::NewDevice(capacity * vw + 16, s, false);
        c.nulls = !c.hasNull ? nullptr
                             : (pc.hostDirect ? omg::Buffer::NewHost(nb, true) : omg::Buffer::NewDevice(nb, s, true));
        p.out[o].values = c.values->Data();
        p.out[o].nulls = c.nulls ? static_cast<uint8_t *>(c.nulls->Data()) : nullptr;
    }
    p.regionCap = pc.regionCap;
    CudaCheck(cudaMemsetAsync(pc.count.Get(), 0, sizeof(unsigned long long) * pc.count.Size(), s), "reset counts");
    pc.timer.Start(s);
    CudaCheck(omg::LaunchProbe(p, s), "probe kernel");
    pc.timer.Stop(s);
    ++counters_[0];
    CudaCheck(cudaMemcpyAsync(pc.hostCount.Get(), pc.count.Get(), sizeof(unsigned long long) * pc.count.Size(),
                  cudaMemcpyDeviceToHost, s),
        "read counts");
    if (pc.done == nullptr) {
        CudaCheck(cudaEventCreateWithFlags(&pc.done, cudaEventDisableTiming), "cudaEventCreate");
    }
    CudaCheck(cudaEventRecord(pc.done, s), "cudaEventRecord");
}

// Wait for a launched probe, run it once more at the exact size if a region overflowed, then
// build VARCHAR outputs, carve the output batches and free the probe batches.
void LookupJoinOperator::FinishProbe(ProbeCall &pc, std::deque<VectorBatch *> &out)
{
    JoinBuildState &b = *f_.build;
    cudaStream_t s = pc.s;
    omg::ProbeLaunch &p = pc.p;
    omg::BatchTable &bt = pc.bt;
    std::vector<omg::OutColumn> &cols = pc.cols;
    const size_t nOut = pc.nOut;
    const size_t nProbeOut = pc.nProbeOut;
    const int32_t nRegions = pc.nRegions;
    const bool hostDirect = pc.hostDirect;
    std::vector<int64_t> regionCount(nRegions, 0);
    for (int attempt = 0; attempt < 2; ++attempt) {
        const auto tw = std::chrono::steady_clock::now();
        CudaCheck(cudaEventSynchronize(pc.done), "probe kernel");
        counters_[9] += std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - tw).count();
        counters_[6] += pc.timer.ElapsedNs();
        ++counters_[7];
        const int32_t kerr = static_cast<int32_t>(pc.hostCount[static_cast<size_t>(nRegions) * omg::kRegionStride]);
        if (kerr != 0) {
            throw OmniException("OPERATOR_RUNTIME_ERROR",
                kerr == 7 ? "probe kernel: a bounded wait for a bulk copy ran out" : "probe kernel error " + std::to_string(kerr),
                kerr == 7 ? -7 : -9);
        }
        uint64_t most = 0;
        for (int32_t r = 0; r < nRegions; ++r) {
            regionCount[r] = static_cast<int64_t>(pc.hostCount[static_cast<size_t>(r) * omg::kRegionStride]);
            most = std::max<uint64_t>(most, static_cast<uint64_t>(regionCount[r]));
        }
        if (most <= pc.regionCap) {
            break;
        }
        pc.regionCap = (most + 63) / 64 * 64;  // exact size known now: run once more
        ++counters_[1];
        LaunchAttempt(pc);
    }
    const uint64_t regionCap = pc.regionCap;
    // VARCHAR outputs: row handles -> lengths -> offsets -> characters, over all regions at once
    // (positions past a region's count contribute nothing).
    for (size_t o = 0; o < nOut; ++o) {
        if (cols[o].width != 0) {
            continue;
        }
        const omg::JoinOutCol &oc = p.out[o];
        const int64_t nPos = static_cast<int64_t>(regionCap) * nRegions;
        const int64_t *handles = static_cast<const int64_t *>(cols[o].values->Data());
        const int64_t *bOffs = oc.side == 1 ? b.colOffs[oc.src].Get() : nullptr;
        const uint8_t *bChars = oc.side == 1 ? b.colValues[oc.src].Get() : nullptr;
        DevArray<uint32_t> lens(static_cast<size_t>(nPos), s);
        CudaCheck(omg::LaunchVarlenOutLens(handles, nPos, regionCap, pc.count.Get(), oc.side, bt.DeviceBatches(), oc.src,
                      bOffs, lens.Get(), s),
            "output string lengths");
        DevArray<int64_t> offs64;
        const int64_t total = omg::ScanLengths(lens.Get(), nPos, offs64, s);
        if (total >= (int64_t(1) << 31)) {
            throw OmniException("UNSUPPORTED_ERROR", "more than 2 GiB of VARCHAR output in one probe call", -2);
        }
        auto chars = omg::Buffer::NewDevice(static_cast<size_t>(total) + 16, s, false);
        auto offs32 = omg::Buffer::NewDevice((static_cast<size_t>(nPos) + 1) * sizeof(int32_t), s, false);
        CudaCheck(omg::LaunchVarlenOutCopy(handles, nPos, regionCap, pc.count.Get(), oc.side, bt.DeviceBatches(), oc.src,
                      bOffs, bChars, offs64.Get(), static_cast<uint8_t *>(chars->Data()),
                      static_cast<int32_t *>(offs32->Data()), total, s),
            "output strings");
        impl_->stream.Sync();  // the scratch arrays above are freed on return
        cols[o].values = chars;
        cols[o].offsets = offs32;
        cols[o].dataBytes = total;
    }
    int64_t rows = 0;
    const auto tc = std::chrono::steady_clock::now();
    for (int32_t r = 0; r < nRegions; ++r) {
        const int64_t n = regionCount[r];
        if (n == 0) {
            continue;
        }
        const int64_t first = static_cast<int64_t>(r) * static_cast<int64_t>(regionCap);
        std::vector<omg::OutColumn> outCols = cols;
        int64_t firstRow = first;
        if (!deviceOutput_ && !hostDirect) {
            outCols = omg::CopyColumnsToHost(cols, n, s, first);
            firstRow = 0;
        }
        if (!deviceOutput_) {
            for (auto &c : outCols) {
                c.hasNull = false;  // host vectors: HasNull() scans the bitmap
            }
        }
        if (b.buildSide == OMNI_BUILD_LEFT) {
            std::rotate(outCols.begin(), outCols.begin() + static_cast<std::ptrdiff_t>(nProbeOut), outCols.end());
        }
        for (auto *ob : omg::CarveBatches(outCols, n, f_.rowsPerBatch, firstRow)) {
            out.push_back(ob);
        }
        rows += n;
    }
    if (!deviceOutput_ && !hostDirect) {
        impl_->stream.Sync();  // the copies to host batches (direct host output was complete at the event)
    }
    counters_[5] += rows;
    const auto tf = std::chrono::steady_clock::now();
    counters_[10] += std::chrono::duration_cast<std::chrono::nanoseconds>(tf - tc).count();
    omg::FreeBatchesLater(std::move(pc.batches));  // the probe kernel is done with them
    pc.batches.clear();
    counters_[11] += std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - tf).count();
}


// ---------------------------------------------------------------------------------- partitioned
struct JoinPartBuild {
    int32_t kind = 0;
    int32_t bits = 0;
    std::vector<int64_t> hostSplits;
    DevArray<int64_t> splits;
    DevArray<uint16_t> lut;  // RANGE: first split index per key bucket
    int64_t lutBase = 0;
    int32_t lutShift = 0;
    DevArray<int64_t> start;     // [P + 1] partitioned build rows
    DevArray<int64_t> tabStart;  // [P + 1] table slab offsets
    DevArray<uint64_t> tabKeys;
    DevArray<int32_t> tabRow;
    DevArray<uint8_t> pay;
    int32_t payBytes = 0;
    bool ok = false;  // false: this build cannot be partitioned (the direct probe is used)

    omg::JoinPartFn Fn() const
    {
        omg::JoinPartFn f;
        f.kind = kind;
        f.bits = bits;
        f.splits = kind == omg::JOIN_PART_RANGE ? splits.Get() : nullptr;
        f.nSplits = kind == omg::JOIN_PART_RANGE ? static_cast<int32_t>(hostSplits.size()) : 0;
        f.lutShift = lutShift;
        f.lutBase = lutBase;
        f.lut = kind == omg::JOIN_PART_RANGE ? lut.Get() : nullptr;
        return f;
    }
};

namespace {
// Chunks of the radix passes: about 16K rows each, at least one per SM (so small inputs still fill
// the GPU) and at most 1024 (the histogram matrix stays small).
int32_t PartChunks(int64_t n)
{
    const int64_t want = std::max<int64_t>(n / 16384, omg::DeviceSMCount());
    return static_cast<int32_t>(std::max<int64_t>(1, std::min<int64_t>({1024, want, std::max<int64_t>(n, 1)})));
}

std::shared_ptr<JoinPartBuild> MakePartBuild(JoinBuildState &b, const std::vector<int32_t> &buildOutputCols,
    int32_t kind, int32_t bits, const std::vector<int64_t> &splits, cudaStream_t s)
{
    auto pb = std::make_shared<JoinPartBuild>();
    pb->kind = kind;
    pb->bits = bits;
    pb->hostSplits = splits;
    const int32_t P = 1 << bits;
    const int32_t keyCol = b.hashCols[0];
    omg::PayloadCols pay;
    std::memset(&pay, 0, sizeof(pay));
    pay.nCols = static_cast<int32_t>(buildOutputCols.size());
    for (int32_t k = 0; k < pay.nCols; ++k) {
        const int32_t c = buildOutputCols[k];
        const int32_t w = b.buildTypes.GetType(c)->ByteWidth();
        if (b.colHasNull[c] || (w != 1 && w != 2 && w != 4 && w != 8 && w != 16)) {
            return pb;  // not eligible
        }
        pay.width[k] = w;
        pay.cols[k] = b.colValues[c].Get();
        pay.rowBytes += w;
    }
    pb->payBytes = pay.rowBytes;
    std::vector<uint16_t> lut;
    if (kind == omg::JOIN_PART_RANGE) {
        pb->splits.Reset(splits.size(), s);
        CudaCheck(cudaMemcpyAsync(pb->splits.Get(), splits.data(), sizeof(int64_t) * splits.size(),
                      cudaMemcpyHostToDevice, s),
            "upload splits");
        // Buckets of width 2^shift from the first split cover every split; lut[bb] = the number of
        // splits below bucket bb's first key.
        pb->lutBase = splits.front();
        const uint64_t span = static_cast<uint64_t>(splits.back()) - static_cast<uint64_t>(splits.front());
        while ((span >> pb->lutShift) >= static_cast<uint64_t>(omg::kJoinLutBuckets)) {
            ++pb->lutShift;
        }
        lut.resize(omg::kJoinLutBuckets + 1);
        size_t i = 0;
        for (int bb = 0; bb <= omg::kJoinLutBuckets; ++bb) {
            // offsets from the first split, unsigned (splits are sorted, so they are >= it)
            const uint64_t first = static_cast<uint64_t>(bb) << pb->lutShift;
            while (i < splits.size() &&
                static_cast<uint64_t>(splits[i]) - static_cast<uint64_t>(pb->lutBase) < first) {
                ++i;
            }
            lut[bb] = static_cast<uint16_t>(i);
        }
        pb->lut.Reset(lut.size(), s);
        CudaCheck(cudaMemcpyAsync(pb->lut.Get(), lut.data(), sizeof(uint16_t) * lut.size(), cudaMemcpyHostToDevice, s),
            "upload range table");
    }
    const int64_t n = b.rows;
    const int32_t chunks = PartChunks(n);
    DevArray<uint32_t> hist(static_cast<size_t>(chunks) * P, s);
    DevArray<int64_t> place(static_cast<size_t>(chunks) * P, s);
    DevArray<int64_t> pkeys(std::max<int64_t>(n, 1), s);
    pb->start.Reset(P + 1, s);
    pb->pay.Reset(static_cast<size_t>(std::max<int64_t>(n, 1)) * std::max(pay.rowBytes, 1) + 16, s);
    const uint8_t *keyNulls = b.colHasNull[keyCol] ? b.colNulls[keyCol].Get() : nullptr;
    CudaCheck(omg::LaunchKeyPartition(reinterpret_cast<const int64_t *>(b.colValues[keyCol].Get()), keyNulls, n,
                  pb->Fn(), chunks, hist.Get(), pb->start.Get(), place.Get(), pkeys.Get(), pay, pb->pay.Get(), s),
        "partition build keys");
    std::vector<int64_t> start(P + 1);
    CudaCheck(cudaMemcpyAsync(start.data(), pb->start.Get(), sizeof(int64_t) * (P + 1), cudaMemcpyDeviceToHost, s),
        "read partition sizes");
    CudaCheck(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    std::vector<int64_t> tabStart(P + 1, 0);
    for (int32_t p = 0; p < P; ++p) {
        const uint64_t rows = static_cast<uint64_t>(start[p + 1] - start[p]);
        tabStart[p + 1] = tabStart[p] + static_cast<int64_t>(std::max<uint64_t>(16, NextPow2(2 * rows)));
    }
    pb->tabStart.Reset(P + 1, s);
    CudaCheck(cudaMemcpyAsync(pb->tabStart.Get(), tabStart.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, s),
        "upload table offsets");
    pb->tabKeys.Reset(static_cast<size_t>(tabStart[P]), s);
    pb->tabRow.Reset(static_cast<size_t>(tabStart[P]), s);
    DevArray<int32_t> err(1, s, true);
    CudaCheck(omg::LaunchPartTableBuild(pkeys.Get(), pb->start.Get(), P, pb->tabStart.Get(), tabStart[P],
                  pb->tabKeys.Get(), pb->tabRow.Get(), err.Get(), s),
        "partition tables");
    int32_t herr = 0;
    CudaCheck(cudaMemcpyAsync(&herr, err.Get(), sizeof(herr), cudaMemcpyDeviceToHost, s), "read build error");
    CudaCheck(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    pb->ok = herr == 0;
    return pb;
}
}  // namespace

void LookupJoinOperator::SetJoinStrategy(int32_t strategy, int32_t bits, const int64_t *splits, int32_t nSplits)
{
    if (strategy == kJoinDirect) {
        strategy_ = kJoinDirect;
        return;
    }
    if ((strategy != kJoinHashPartitioned && strategy != kJoinRangePartitioned && strategy != kJoinLearned &&
            strategy != kJoinQuantile) ||
        bits < 1 || (1 << bits) > omg::kMaxJoinParts) {
        throw OmniException("INVALID_ARGUMENT", "join strategy: unknown strategy or bits outside [1, 12]", -1);
    }
    if (strategy == kJoinRangePartitioned || strategy == kJoinLearned || strategy == kJoinQuantile) {
        if (splits == nullptr || nSplits != (1 << bits) - 1) {
            throw OmniException("INVALID_ARGUMENT", "range partitioning needs 2^bits - 1 splits", -1);
        }
        for (int32_t i = 1; i < nSplits; ++i) {
            if (splits[i] < splits[i - 1]) {
                throw OmniException("INVALID_ARGUMENT", "range splits must be sorted", -1);
            }
        }
        splits_.assign(splits, splits + nSplits);
    } else {
        splits_.clear();
    }
    strategy_ = strategy;
    partBits_ = bits;
    if (strategy == kJoinLearned || strategy == kJoinQuantile) {
        // Splits are (learned or exact) quantiles of the probe keys: a hot key repeats as a run of
        // equal splits.
        int32_t run = 1;
        int32_t longest = 1;
        for (int32_t i = 1; i < nSplits; ++i) {
            run = splits[i] == splits[i - 1] ? run + 1 : 1;
            longest = std::max(longest, run);
        }
        const double runShare = static_cast<double>(longest) / static_cast<double>(1 << bits);
        const double threshold = strategy == kJoinLearned ? kLearnedDirectRun : kQuantileDirectRun;
        strategy_ = runShare > threshold ? kJoinDirect : kJoinHashPartitioned;
    }
}

bool LookupJoinOperator::ProcessPartitioned()
{
    JoinBuildState &b = *f_.build;
    const int32_t keyCol = f_.probeHashCols[0];
    if (!f_.filter.empty() || !b.table.unique || b.table.keyWidth != 8 || f_.probeTypes.GetType(keyCol)->ByteWidth() != 8 ||
        b.kind != omg::JOIN_KIND_INNER || b.buildSide == OMNI_BUILD_LEFT || b.multiKey || b.packed) {
        return false;
    }
    for (int32_t c : f_.probeOutputCols) {
        if (c != keyCol) {
            return false;
        }
    }
    omg::RequireDevice();
    if (userStreamSet_) {
        impl_->stream.SetUser(userStream_);
    }
    cudaStream_t s = impl_->stream.Get();
    const int32_t kind = strategy_ == kJoinRangePartitioned ? omg::JOIN_PART_RANGE : omg::JOIN_PART_HASH;
    std::shared_ptr<JoinPartBuild> pb;
    {
        std::lock_guard<std::mutex> g(f_.partMu);
        for (auto &x : f_.partBuilds) {
            if (x->kind == kind && x->bits == partBits_ && x->hostSplits == splits_) {
                pb = x;
            }
        }
        if (!pb) {
            pb = MakePartBuild(b, f_.buildOutputCols, kind, partBits_, splits_, s);
            ++counters_[0];
            f_.partBuilds.push_back(pb);
        }
    }
    if (!pb->ok) {
        return false;
    }
    // The probe key column, contiguous on the device.
    const int64_t *keys = nullptr;
    const uint8_t *keyNulls = nullptr;
    int64_t n = 0;
    DevArray<uint8_t> gathered, gatheredNulls;
    if (pending_.size() == 1 && pending_[0]->Get(keyCol)->IsDevice()) {
        vec::BaseVector *v = pending_[0]->Get(keyCol);
        keys = reinterpret_cast<const int64_t *>(v->RawValues());
        keyNulls = v->HasNull() ? v->RawNulls() : nullptr;
        n = pending_[0]->GetRowCount();
    } else {
        omg::BatchTable bt;
        bt.Build(pending_, {keyCol});
        bt.Upload(s);
        n = bt.TotalRows();
        gathered.Reset(static_cast<size_t>(n) * 8 + 16, s);
        if (bt.AnyNulls(0)) {
            gatheredNulls.Reset(omg::NullBitmapBytes(n), s, true);
        }
        CudaCheck(omg::LaunchGatherColumn(bt.DeviceBatches(), bt.DeviceTiles(), bt.NumTiles(), bt.DeviceTileOutRows(), 0,
                      8, gathered.Get(), bt.AnyNulls(0) ? gatheredNulls.Get() : nullptr, s),
            "gather probe keys");
        impl_->stream.Sync();  // the batch table's staging must outlive the copy
        keys = reinterpret_cast<const int64_t *>(gathered.Get());
        keyNulls = bt.AnyNulls(0) ? gatheredNulls.Get() : nullptr;
    }
    const int32_t P = 1 << partBits_;
    const int32_t chunks = PartChunks(n);
    DevArray<uint32_t> hist(static_cast<size_t>(chunks) * P, s);
    DevArray<int64_t> place(static_cast<size_t>(chunks) * P, s);
    DevArray<int64_t> start(P + 1, s);
    DevArray<int64_t> pkeys(std::max<int64_t>(n, 1), s);
    omg::PayloadCols none;
    std::memset(&none, 0, sizeof(none));
    impl_->timer.Start(s);
    CudaCheck(omg::LaunchKeyPartition(keys, keyNulls, n, pb->Fn(), chunks, hist.Get(), start.Get(), place.Get(),
                  pkeys.Get(), none, nullptr, s),
        "partition probe keys");
    int64_t live = 0;
    CudaCheck(cudaMemcpyAsync(&live, start.Get() + P, sizeof(live), cudaMemcpyDeviceToHost, s), "read probe rows");
    impl_->stream.Sync();
    // Output: the probe key (if requested) and the build output columns, in regions.
    const size_t nProbeOut = f_.probeOutputCols.size();
    const size_t nOut = nProbeOut + f_.buildOutputCols.size();
    constexpr int64_t kSeg = 128;
    const int64_t segs = (live + kSeg - 1) / kSeg;
    const int32_t nRegions = static_cast<int32_t>(std::max<int64_t>(1, std::min<int64_t>(omg::kMaxRegions, segs)));
    const uint64_t regionCap = static_cast<uint64_t>((segs + nRegions - 1) / nRegions * kSeg);
    std::vector<omg::OutColumn> cols(nOut);
    omg::PartProbeLaunch q;
    std::memset(&q, 0, sizeof(q));
    q.fn = pb->Fn();
    q.keys = pkeys.Get();
    q.n = live;
    q.tabStart = pb->tabStart.Get();
    q.tabKeys = pb->tabKeys.Get();
    q.tabRow = pb->tabRow.Get();
    q.start = pb->start.Get();
    q.pay = pb->pay.Get();
    q.payBytes = pb->payBytes;
    const uint64_t capacity = regionCap * static_cast<uint64_t>(nRegions);
    for (size_t o = 0; o < nOut; ++o) {
        const bool probeSide = o < nProbeOut;
        const int32_t c = probeSide ? f_.probeOutputCols[o] : f_.buildOutputCols[o - nProbeOut];
        const auto &t = probeSide ? f_.probeTypes.GetType(c) : f_.buildOutputTypes.GetType(static_cast<int32_t>(o - nProbeOut));
        cols[o].type = t->GetId();
        cols[o].width = probeSide ? 8 : b.buildTypes.GetType(c)->ByteWidth();
        cols[o].values = omg::Buffer::NewDevice(capacity * cols[o].width + 16, s, false);
        cols[o].nulls = nullptr;
        cols[o].hasNull = false;
        if (probeSide) {
            q.keyOut = static_cast<int64_t *>(cols[o].values->Data());
        } else {
            q.payWidth[q.nPayOut] = cols[o].width;
            q.payOut[q.nPayOut] = cols[o].values->Data();
            ++q.nPayOut;
        }
    }
    DevArray<unsigned long long> count(static_cast<size_t>(nRegions) * omg::kRegionStride, s, true);
    omg::PinnedArray<unsigned long long> hostCount(static_cast<size_t>(nRegions) * omg::kRegionStride);
    q.outCount = count.Get();
    q.nRegions = nRegions;
    q.regionCap = regionCap;
    CudaCheck(omg::LaunchPartProbe(q, s), "partitioned probe");
    impl_->timer.Stop(s);
    counters_[0] += 5;
    CudaCheck(cudaMemcpyAsync(hostCount.Get(), count.Get(), sizeof(unsigned long long) * count.Size(),
                  cudaMemcpyDeviceToHost, s),
        "read counts");
    impl_->stream.Sync();
    counters_[6] += impl_->timer.ElapsedNs();
    ++counters_[7];
    int64_t rows = 0;
    for (int32_t r = 0; r < nRegions; ++r) {
        const int64_t cnt = static_cast<int64_t>(hostCount[static_cast<size_t>(r) * omg::kRegionStride]);
        if (cnt == 0) {
            continue;
        }
        const int64_t first = static_cast<int64_t>(r) * static_cast<int64_t>(regionCap);
        std::vector<omg::OutColumn> outCols = cols;
        int64_t firstRow = first;
        if (!deviceOutput_) {
            outCols = omg::CopyColumnsToHost(cols, cnt, s, first);
            firstRow = 0;
        }
        for (auto *ob : omg::CarveBatches(outCols, cnt, f_.rowsPerBatch, firstRow)) {
            outputs_.push_back(ob);
        }
        rows += cnt;
    }
    if (!deviceOutput_) {
        impl_->stream.Sync();
    }
    counters_[5] += rows;
    for (auto *pbatch : pending_) {
        vec::VectorHelper::FreeVecBatch(pbatch);
    }
    pending_.clear();
    pendingRows_ = 0;
    return true;
}

int32_t LookupJoinOperator::GetOutput(VectorBatch **outputVecBatch)
{
    *outputVecBatch = nullptr;
    if (impl_->worker.joinable()) {
        return GetOutputFromWorker(outputVecBatch);
    }
    // Launched probe calls finish oldest first: when another is queued behind it, when its kernel
    // is done, or when no more input will come.
    auto &fl = impl_->inflight;
    while (outputs_.empty() && !fl.empty()) {
        bool ready = fl.size() > 1 || noMoreInput_;
        if (!ready) {
            const cudaError_t q = cudaEventQuery(fl.front()->done);
            cudaGetLastError();  // "not ready" is not an error of this operator
            ready = q != cudaErrorNotReady;
        }
        if (!ready) {
            break;
        }
        std::unique_ptr<ProbeCall> pc = std::move(fl.front());
        fl.pop_front();
        FinishProbe(*pc, outputs_);
    }
    if (outputs_.empty() && fl.empty() && !pending_.empty() && f_.build->built &&
        (noMoreInput_ || pendingRows_ >= omg::ProbeChunkRows())) {
        ProcessPending();
    }
    if (!outputs_.empty()) {
        *outputVecBatch = outputs_.front();
        outputs_.pop_front();
    }
    if (outputs_.empty() && pending_.empty() && fl.empty() && noMoreInput_) {
        SetStatus(OMNI_STATUS_FINISHED);
    }
    return 0;
}

// ------------------------------------------------------------------------------ outer join
LookupOuterJoinOperatorFactory::LookupOuterJoinOperatorFactory(const DataTypes &probeTypes,
    const int32_t *probeOutputCols, int32_t probeOutputColsCount, const int32_t *buildOutputCols_,
    const DataTypes &buildOutputTypes_, HashBuilderOperatorFactory *builder, BuildSide buildSide_)
    : buildOutputTypes(buildOutputTypes_), build(builder->GetBuildState()), buildSide(buildSide_)
{
    if (!build->TracksVisits()) {
        throw OmniException("UNSUPPORTED_ERROR",
            "the outer-join operator follows a full join or a build-side outer join", -2);
    }
    std::vector<DataTypePtr> pt;
    int32_t rowSize = 0;
    for (int32_t i = 0; i < probeOutputColsCount; ++i) {
        const int32_t c = probeOutputCols[i];
        if (c < 0 || c >= probeTypes.GetSize()) {
            throw OmniException("INVALID_ARGUMENT", "probe output column out of range", -1);
        }
        pt.push_back(probeTypes.GetType(c));
        rowSize += probeTypes.GetType(c)->ByteWidth();
    }
    probeOutputTypes = DataTypes(pt);
    const int32_t nBuild = buildOutputTypes.GetSize();
    buildOutputCols.assign(buildOutputCols_, buildOutputCols_ + nBuild);
    for (int32_t i = 0; i < nBuild; ++i) {
        const int32_t c = buildOutputCols[i];
        if (c < 0 || c >= build->buildTypes.GetSize() ||
            build->buildTypes.GetType(c)->ByteWidth() != buildOutputTypes.GetType(i)->ByteWidth()) {
            throw OmniException("INVALID_ARGUMENT", "build output column out of range", -1);
        }
        rowSize += buildOutputTypes.GetType(i)->ByteWidth();
    }
    // lookup_outer_join.cpp:111-118: a row of no columns counts as DEFAULT_ROW_SIZE (4 bytes).
    rowsPerBatch = GetMaxRowCount(probeOutputColsCount + nBuild == 0 ? 4 : rowSize);
}

LookupOuterJoinOperatorFactory *LookupOuterJoinOperatorFactory::CreateLookupOuterJoinOperatorFactory(
    const DataTypes &probeTypes, int32_t *probeOutputCols, int32_t probeOutputColsCount, int32_t *buildOutputCols,
    const DataTypes &buildOutputTypes, int64_t hashBuilderFactoryAddr)
{
    return CreateLookupOuterJoinOperatorFactory(probeTypes, probeOutputCols, probeOutputColsCount, buildOutputCols,
        buildOutputTypes, hashBuilderFactoryAddr, OMNI_BUILD_UNKNOWN);
}

LookupOuterJoinOperatorFactory *LookupOuterJoinOperatorFactory::CreateLookupOuterJoinOperatorFactory(
    const DataTypes &probeTypes, int32_t *probeOutputCols, int32_t probeOutputColsCount, int32_t *buildOutputCols,
    const DataTypes &buildOutputTypes, int64_t hashBuilderFactoryAddr, BuildSide buildSide)
{
    auto *builder = reinterpret_cast<HashBuilderOperatorFactory *>(hashBuilderFactoryAddr);
    if (builder == nullptr) {
        throw OmniException("INVALID_ARGUMENT", "null hash builder factory", -1);
    }
    return new LookupOuterJoinOperatorFactory(probeTypes, probeOutputCols, probeOutputColsCount, buildOutputCols,
        buildOutputTypes, builder, buildSide);
}

Operator *LookupOuterJoinOperatorFactory::CreateOperator() { return new LookupOuterJoinOperator(*this); }

struct LookupOuterJoinOperator::Impl {
    omg::OpStream stream;
};

LookupOuterJoinOperator::LookupOuterJoinOperator(const LookupOuterJoinOperatorFactory &f) : f_(f), impl_(new Impl()) {}

LookupOuterJoinOperator::~LookupOuterJoinOperator() { Close(); }

OmniStatus LookupOuterJoinOperator::Close()
{
    for (auto *b : outputs_) {
        vec::VectorHelper::FreeVecBatch(b);
    }
    outputs_.clear();
    return OMNI_STATUS_NORMAL;
}

int32_t LookupOuterJoinOperator::AddInput(VectorBatch *vecBatch)
{
    if (vecBatch != nullptr) {
        vec::VectorHelper::FreeVecBatch(vecBatch);
    }
    return 0;
}

// Every build row no probe marked, in build-row order, as output batches: probe columns NULL,
// build columns gathered on the device.
void LookupOuterJoinOperator::Prepare()
{
    JoinBuildState &b = *f_.build;
    {
        std::lock_guard<std::mutex> g(b.mu);
        if (!b.built) {
            throw OmniException("OPERATOR_RUNTIME_ERROR", "the outer-join rows are read before the build finished", -6);
        }
    }
    prepared_ = true;
    if (b.rows == 0) {
        return;
    }
    omg::RequireDevice();
    if (userStreamSet_) {
        impl_->stream.SetUser(userStream_);
    }
    cudaStream_t s = impl_->stream.Get();
    const int64_t n = b.rows;
    DevArray<uint32_t> flags(static_cast<size_t>(n), s);
    DevArray<int64_t> offsets(static_cast<size_t>(n), s);
    DevArray<int64_t> blockSums(static_cast<size_t>((n + 1023) / 1024 + 1), s);
    DevArray<long long> total(1, s, true);
    CudaCheck(omg::LaunchUnvisitedFlags(b.visited.Get(), n, flags.Get(), s), "unvisited flags");
    CudaCheck(omg::LaunchScanCounts(flags.Get(), n, offsets.Get(), blockSums.Get(), total.Get(), s), "scan flags");
    long long m = 0;
    CudaCheck(cudaMemcpyAsync(&m, total.Get(), sizeof(m), cudaMemcpyDeviceToHost, s), "read unvisited count");
    impl_->stream.Sync();
    ++counters_[0];
    if (m == 0) {
        return;
    }
    DevArray<int32_t> rows(static_cast<size_t>(m), s);
    CudaCheck(omg::LaunchUnvisitedRows(b.visited.Get(), offsets.Get(), n, rows.Get(), s), "unvisited rows");
    const int32_t nProbe = f_.probeOutputTypes.GetSize();
    const int32_t nBuild = f_.buildOutputTypes.GetSize();
    std::vector<omg::OutColumn> cols(static_cast<size_t>(nProbe + nBuild));
    for (int32_t o = 0; o < nProbe + nBuild; ++o) {
        omg::OutColumn &c = cols[o];
        const bool probe = o < nProbe;
        const auto &t = probe ? f_.probeOutputTypes.GetType(o) : f_.buildOutputTypes.GetType(o - nProbe);
        c.type = t->GetId();
        c.width = t->ByteWidth();
        const bool varlen = Varlen(t);
        c.values = omg::Buffer::NewDevice(static_cast<size_t>(m) * c.width + 16, s, probe);
        if (varlen) {
            c.offsets = omg::Buffer::NewDevice((static_cast<size_t>(m) + 1) * sizeof(int32_t), s, true);
        }
        if (probe) {
            c.hasNull = true;
            c.nulls = omg::Buffer::NewDevice(omg::NullBitmapBytes(m), s, false);
            CudaCheck(cudaMemsetAsync(c.nulls->Data(), 0xff, omg::NullBitmapBytes(m), s), "NULL probe columns");
        } else if (varlen) {
            const int32_t bc = f_.buildOutputCols[o - nProbe];
            c.hasNull = b.colHasNull[bc];
            c.nulls = c.hasNull ? omg::Buffer::NewDevice(omg::NullBitmapBytes(m), s, true) : nullptr;
            DevArray<uint32_t> lens(static_cast<size_t>(m), s);
            CudaCheck(omg::LaunchVarlenRowsLens(rows.Get(), m, b.colOffs[bc].Get(), lens.Get(), s), "string lengths");
            DevArray<int64_t> offs64;
            const int64_t total = omg::ScanLengths(lens.Get(), m, offs64, s);
            if (total >= (int64_t(1) << 31)) {
                throw OmniException("UNSUPPORTED_ERROR", "more than 2 GiB of VARCHAR output in one batch set", -2);
            }
            c.values = omg::Buffer::NewDevice(static_cast<size_t>(total) + 16, s, false);
            c.dataBytes = total;
            CudaCheck(omg::LaunchVarlenRowsCopy(rows.Get(), m, b.colOffs[bc].Get(), b.colValues[bc].Get(),
                          offs64.Get(), static_cast<uint8_t *>(c.values->Data()),
                          static_cast<int32_t *>(c.offsets->Data()), total, s),
                "gather unvisited build strings");
            if (c.hasNull) {
                CudaCheck(omg::LaunchGatherRows(b.colValues[bc].Get(), b.colNulls[bc].Get(), rows.Get(), m, 0,
                              c.values->Data(), static_cast<uint8_t *>(c.nulls->Data()), s),
                    "gather unvisited build NULLs");
            }
            impl_->stream.Sync();
        } else {
            const int32_t bc = f_.buildOutputCols[o - nProbe];
            c.hasNull = b.colHasNull[bc];
            c.nulls = c.hasNull ? omg::Buffer::NewDevice(omg::NullBitmapBytes(m), s, true) : nullptr;
            CudaCheck(omg::LaunchGatherRows(b.colValues[bc].Get(), c.hasNull ? b.colNulls[bc].Get() : nullptr,
                          rows.Get(), m, c.width, c.values->Data(),
                          c.hasNull ? static_cast<uint8_t *>(c.nulls->Data()) : nullptr, s),
                "gather unvisited build rows");
        }
    }
    std::vector<omg::OutColumn> outCols = cols;
    if (!deviceOutput_) {
        outCols = omg::CopyColumnsToHost(cols, m, s, 0);
        for (auto &c : outCols) {
            c.hasNull = false;  // host vectors: HasNull() scans the bitmap
        }
    }
    impl_->stream.Sync();
    if (f_.buildSide == OMNI_BUILD_LEFT) {
        std::rotate(outCols.begin(), outCols.begin() + nProbe, outCols.end());
    }
    for (auto *ob : omg::CarveBatches(outCols, m, f_.rowsPerBatch, 0)) {
        outputs_.push_back(ob);
    }
    counters_[5] += m;
}

int32_t LookupOuterJoinOperator::GetOutput(VectorBatch **outputVecBatch)
{
    if (outputVecBatch != nullptr) {
        *outputVecBatch = nullptr;
    }
    if (!prepared_) {
        Prepare();
    }
    if (outputs_.empty()) {
        SetStatus(OMNI_STATUS_FINISHED);
        return 0;
    }
    if (outputVecBatch != nullptr) {
        *outputVecBatch = outputs_.front();
    } else {
        vec::VectorHelper::FreeVecBatch(outputs_.front());
    }
    outputs_.pop_front();
    if (outputs_.empty()) {
        SetStatus(OMNI_STATUS_FINISHED);
    }
    return 0;
}

}  // namespace op
}  // namespace omniruntime
