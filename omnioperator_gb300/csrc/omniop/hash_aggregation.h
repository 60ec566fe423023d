// HashAggregationOperatorFactory / HashAggregationOperator for GB300.
//
// Same constructor and call surface as the reference
// (operator/aggregation/group_aggregation.h:203-301): the factory takes the group-by
// columns and types, per-aggregator input columns, input and output types and function
// ids, mask columns, the inputRaw/outputPartial flags and overflowAsNull.  The operator
// takes ownership of each AddInput batch, aggregates on the GPU, and GetOutput returns the
// groups in batches of ceil(1 MiB / rowBytes) rows, returning 1 per produced batch and
// setting OMNI_STATUS_FINISHED after the last (group_aggregation.cpp:454-474,1486-1538).
#pragma once

#include <cstdint>
#include <deque>
#include <memory>
#include <vector>

#include <cuda_runtime_api.h>

#include "kernels/plan.h"
#include "operator.h"

namespace omg {
class BatchTable;
class SizingModel;
}

namespace omg {
class OpStream;
template <typename T> class DevArray;
struct OutColumn;
}

namespace omniruntime {
namespace op {

// The compiled form of a factory's aggregation: kernel inputs, key packing, accumulators
// and output columns.
struct AggPlan {
    std::vector<int32_t> inputCols;        // batch column of each kernel input
    std::vector<int32_t> inputWidths;      // value bytes of each kernel input
    std::vector<int32_t> inputMasks;       // mask column of each kernel input (-1: none): the
                                           // rows whose mask is NULL or FALSE read as NULL
    omg::KeySpec key{};
    std::vector<omg::AccSpec> accs;
    std::vector<int16_t> regInput;         // kernel inputs cached in registers per row
    std::vector<int16_t> regWidth;
    int32_t stateWords = 0;
    int32_t keyWords = 0;                  // words before the state in a table slot
    int32_t slotWords = 0;
    std::vector<omg::OutSpec> outs;        // pointers filled at extraction
    std::vector<type::DataTypePtr> outTypes;
    int32_t rowsPerBatch = 0;
    int32_t smemSlots = 0;                 // per-CTA shared pre-aggregation slots
    bool overflowAsNull = false;
    bool orderDependent = false;           // has an OUT_SUM_EXACT column (sticky overflow)
    // Per output: > 0 when it starts a container output of that many fields (a partial AVG under
    // the container-vector policy), 0 otherwise.
    std::vector<int32_t> outContainer;
    std::vector<omg::AlignCol> align;      // AlignSchema columns; empty unless every aggregator
                                           // reads raw input and emits partials
    std::vector<int32_t> dictInputs;       // kernel inputs of VARCHAR/CHAR group-by columns: the
                                           // kernels read per-row string dictionary ids (int32)
    std::vector<int32_t> varlenInputs;     // other VARCHAR/CHAR inputs (COUNT reads their NULLs)
};

// Kernel launch parameters of a plan (table fields as given; stats: [groups, retry count,
// spill count, error] words, may be null).
omg::AggLaunch MakeAggLaunch(const AggPlan &plan, uint64_t *slots, uint64_t capacity, uint32_t *special,
    unsigned long long *stats);

class HashAggregationOperatorFactory : public OperatorFactory {
public:
    HashAggregationOperatorFactory(std::vector<uint32_t> &groupByCol, const type::DataTypes &groupInputTypes,
        std::vector<std::vector<uint32_t>> &aggsCols, std::vector<type::DataTypes> &aggInputTypes,
        std::vector<type::DataTypes> &aggOutputTypes, std::vector<uint32_t> &aggFuncTypes,
        std::vector<uint32_t> &maskColsVector, std::vector<bool> inputRaws, std::vector<bool> outputPartials,
        bool overflowAsNull = false);
    ~HashAggregationOperatorFactory() override = default;

    // Compiles and validates the plan; throws OmniException on unsupported shapes.
    OmniStatus Init();
    Operator *CreateOperator() override;
    const AggPlan &Plan() const { return plan_; }
    // Learned sizing model consulted by the operators created afterwards (nullptr: the plain
    // estimate).  The model must outlive those operators.
    void SetSizer(omg::SizingModel *sizer) { sizer_ = sizer; }

private:
    std::vector<uint32_t> groupByCols_;
    type::DataTypes groupTypes_;
    std::vector<std::vector<uint32_t>> aggCols_;
    std::vector<type::DataTypes> aggInputTypes_;
    std::vector<type::DataTypes> aggOutputTypes_;
    std::vector<uint32_t> aggFuncTypes_;
    std::vector<uint32_t> maskCols_;
    std::vector<bool> inputRaws_;
    std::vector<bool> outputPartials_;
    bool overflowAsNull_;
    SupportContainerVecRule policy_;
    AggPlan plan_;
    bool inited_ = false;
    omg::SizingModel *sizer_ = nullptr;
};

class HashAggregationOperator : public Operator {
public:
    explicit HashAggregationOperator(const AggPlan &plan, omg::SizingModel *sizer = nullptr);
    ~HashAggregationOperator() override;

    int32_t AddInput(VectorBatch *vecBatch) override;
    int32_t GetOutput(VectorBatch **outputVecBatch) override;
    OmniStatus Close() override;
    uint64_t GetHashMapUniqueKeys() override { return uniqueKeys_; }
    // Adaptive partial aggregation (group_aggregation.cpp:1182-1218): the input batch as
    // one-row partial results in the partial output schema, computed on the device; the input
    // is freed.  Only for plans whose aggregators all read raw input and emit partials.
    VectorBatch *AlignSchema(VectorBatch *inputVecBatch) override;

    // Spill (the reference's SpillConfig, operator/config/operator_config.h:28-100, and its spill
    // path, group_aggregation.cpp:1034-1475): with spill enabled the operator keeps its input
    // staged until GetOutput and, when the estimated group table would exceed `deviceBudgetBytes`
    // of device memory, hash-partitions the rows into pinned host memory and aggregates one
    // partition at a time (partitions hold disjoint groups).  Plans with VARCHAR/CHAR columns or
    // order-dependent sticky-overflow sums are refused (UNSUPPORTED).
    void SetSpill(bool enabled, uint64_t deviceBudgetBytes);
    uint64_t GetSpilledBytes() override { return spilledBytes_; }

    // Strategy hint (OMG_AGG_STRATEGY_*) and initial capacity in groups (0 = default).
    void SetStrategy(int32_t strategy, int64_t capacityHint)
    {
        strategy_ = strategy;
        capacityHint_ = capacityHint;
    }
    // How the group count is estimated when no capacity hint is given: 0 = the key sketch of a row
    // sample (and the factory's sizing model, if any); 1 = a HyperLogLog sketch of every row's key.
    void SetSizing(int32_t mode) { sizing_ = mode; }

    // Sizing record of the first flush: [0] rows flushed, [1..kSketchStats] the key sketch of a
    // row sample, then the group estimate used, the partition bits (-1 = global table), the
    // group count so far, the plain (sketch) estimate and whether a sizing model made the
    // estimate used.  Returns the number of values written.
    int32_t GetSizingLog(int64_t *out, int32_t n) const;

private:
    struct Impl;
    struct PartBuffers;
    void Decide(omg::BatchTable &bt, cudaStream_t s);
    void Partition(omg::BatchTable &bt, omg::AggLaunch &p, PartBuffers &pb, cudaStream_t s);
    void Flush();
    void EncodeStrings(omg::BatchTable &bt, cudaStream_t s);
    void BindStrings(omg::AggLaunch &p) const;
    void DecodeStrings(std::vector<omg::OutColumn> &cols, int64_t rows, cudaStream_t s);
    VectorBatch *DecodeKeyIds(VectorBatch *batch, const std::vector<size_t> &outs, cudaStream_t s);
    void Extract();
    bool ExtractSpilled();
    void ReleasePending();

    AggPlan plan_;
    std::unique_ptr<Impl> impl_;
    std::vector<VectorBatch *> pending_;
    int64_t pendingRows_ = 0;
    std::deque<VectorBatch *> outputs_;
    bool hasInputedData_ = false;
    bool extracted_ = false;
    uint64_t uniqueKeys_ = 0;
    int32_t strategy_ = 0;
    int64_t capacityHint_ = 0;
    int32_t sizing_ = 0;
    bool spillEnabled_ = false;
    uint64_t spillBudget_ = 0;
    uint64_t spilledBytes_ = 0;
    omg::SizingModel *sizer_ = nullptr;
};

}  // namespace op
}  // namespace omniruntime
