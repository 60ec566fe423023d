// HashBuilderOperator(Factory), LookupJoinOperator(Factory) and LookupOuterJoinOperator(Factory)
// for GB300: equi-joins on one key column, of every join type the reference probes
// (inner, left/right/full outer, left semi, left anti, existence).
//
// Call surface as in the reference (operator/join/hash_builder.h:18-80,
// operator/join/lookup_join.h:136-200): builder operators retain their batches and build the
// table when GetOutput runs after noMoreInput (hash_builder.cpp:169-213); probe operators
// report kWaitForJoinBuild until every builder finished (lookup_join.cpp:270-277), take
// ownership of probe batches and emit (probe output columns, build output columns) rows in
// batches of at most ceil(1 MiB / rowSize) rows (lookup_join.cpp:419-480,1628-1640).
//
// GB300 specifics: the build table and build columns live in HBM; the probe of one or many
// queued batches is one kernel launch.  With noMoreInput left true (per-batch callers) each
// AddInput batch is probed at the next GetOutput; pipelined callers that set it false get
// their batches probed in large chunks.
#pragma once

#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "kernels/plan.h"
#include "operator.h"

namespace omniruntime {
namespace op {

struct JoinBuildState;
struct JoinPartBuild;

// Probe strategies of a LookupJoin operator (no reference counterpart).
constexpr int32_t kJoinDirect = 0;           // one table for the whole build (default)
constexpr int32_t kJoinHashPartitioned = 1;  // 2^bits hash partitions per side
constexpr int32_t kJoinRangePartitioned = 2; // 2^bits key ranges per side, from 2^bits - 1 splits
// Learned: the splits learned from the probe keys decide.  A run of equal splits longer than
// kLearnedDirectRun of the partitions marks a hot key of about twice that probe share (the leaf
// models put a repeated key's CDF at its mid rank, so a key holding a share q of the rows repeats
// as about q/2 * 2^bits splits); such a key makes the direct probe, which keeps it in cache, the
// choice.  Otherwise the probe is hash-partitioned: on the skewed join workload hash partitions,
// with equal build keys each, probe faster than range partitions balanced by probe rows, whose
// cold partitions hold most build keys.
constexpr int32_t kJoinLearned = 3;
constexpr double kLearnedDirectRun = 0.075;
// Quantile: the same choice from exact sample quantiles (no network), where a key holding a share
// q of the rows repeats as about q * 2^bits splits: a run longer than kQuantileDirectRun (a key
// with about 15% of the probe rows, as for the learned rule) selects the direct probe.
constexpr int32_t kJoinQuantile = 4;
constexpr double kQuantileDirectRun = 0.15;

class HashBuilderOperatorFactory : public OperatorFactory {
public:
    HashBuilderOperatorFactory(JoinType joinType, const type::DataTypes &buildTypes, const int32_t *buildHashCols,
        int32_t buildHashColsCount, int32_t operatorCount);
    HashBuilderOperatorFactory(JoinType joinType, BuildSide buildSide, const type::DataTypes &buildTypes,
        const int32_t *buildHashCols, int32_t buildHashColsCount, int32_t operatorCount);
    ~HashBuilderOperatorFactory() override;
    static HashBuilderOperatorFactory *CreateHashBuilderOperatorFactory(JoinType joinType,
        const type::DataTypes &buildTypes, const int32_t *buildHashCols, int32_t buildHashColsCount,
        int32_t operatorCount);
    static HashBuilderOperatorFactory *CreateHashBuilderOperatorFactory(JoinType joinType, BuildSide buildSide,
        const type::DataTypes &buildTypes, const int32_t *buildHashCols, int32_t buildHashColsCount,
        int32_t operatorCount);
    Operator *CreateOperator() override;
    JoinBuildState *GetBuildState() { return state_.get(); }

private:
    std::unique_ptr<JoinBuildState> state_;
};

class HashBuilderOperator : public Operator {
public:
    explicit HashBuilderOperator(JoinBuildState *state) : state_(state) {}
    int32_t AddInput(VectorBatch *vecBatch) override;
    int32_t GetOutput(VectorBatch **outputVecBatch) override;
    OmniStatus Close() override { return OMNI_STATUS_NORMAL; }

private:
    JoinBuildState *state_;
    bool counted_ = false;
};

class LookupJoinOperatorFactory : public OperatorFactory {
public:
    LookupJoinOperatorFactory(const type::DataTypes &probeTypes, const int32_t *probeOutputCols,
        int32_t probeOutputColsCount, const int32_t *probeHashCols, int32_t probeHashColsCount,
        const int32_t *buildOutputCols, int32_t buildOutputColsCount, const type::DataTypes &buildOutputTypes,
        HashBuilderOperatorFactory *builder);
    static LookupJoinOperatorFactory *CreateLookupJoinOperatorFactory(const type::DataTypes &probeTypes,
        int32_t *probeOutputCols, int32_t probeOutputColsCount, int32_t *probeHashCols, int32_t probeHashColsCount,
        int32_t *buildOutputCols, int32_t buildOutputColsCount, const type::DataTypes &buildOutputTypes,
        int64_t hashBuilderFactoryAddr, const void *filterExpr, bool isShuffleExchangeBuildPlan,
        const void *overflowConfig);
    Operator *CreateOperator() override;

    type::DataTypes probeTypes;
    std::vector<int32_t> probeOutputCols;
    std::vector<int32_t> probeHashCols;
    std::vector<int32_t> buildOutputCols;
    type::DataTypes buildOutputTypes;
    JoinBuildState *build;
    int32_t rowsPerBatch;
    // Join filter compiled to a postfix program (empty: none).  Column operands are bound per
    // probe call: filterCols[i] is the probe column (side 0) or build column (side 1) of
    // instruction i, -1 for the others.
    std::vector<omg::FilterInstr> filter;
    std::vector<int32_t> filterCols;
    // Bytes of the filter's string literals (FOP_STR_LITERAL: imm is the offset of its bytes).
    std::string filterText;
    // Build output values packed per table slot, built by the first probe that can use it.
    mutable std::mutex payloadMu;
    mutable omg::BufferPtr slotPayload;
    mutable omg::BufferPtr slotBits;  // ARRAY tables: occupancy bitmap of the slots
    mutable bool payloadDecided = false;
    // Partitioned builds, one per partition function (kind, bits, splits), made by the first
    // partitioned probe that uses it.
    mutable std::mutex partMu;
    mutable std::vector<std::shared_ptr<JoinPartBuild>> partBuilds;
};

class LookupJoinOperator : public Operator {
public:
    explicit LookupJoinOperator(const LookupJoinOperatorFactory &f);
    ~LookupJoinOperator() override;
    int32_t AddInput(VectorBatch *vecBatch) override;
    int32_t GetOutput(VectorBatch **outputVecBatch) override;
    OmniStatus Close() override;
    BlockingReason IsBlocked() override;
    // Probe strategy for the batches processed afterwards (kJoin*; `splits` for the range
    // strategy: 2^bits - 1 sorted keys).  A partitioned strategy applies to unique builds with
    // 8-byte keys, NULL-free build output columns and the probe key as the only probe output;
    // other shapes keep the direct probe.  Results do not depend on the strategy.
    void SetJoinStrategy(int32_t strategy, int32_t bits, const int64_t *splits, int32_t nSplits);
    // The strategy the batches processed afterwards use (kJoinLearned resolved).
    int32_t JoinStrategy() const { return strategy_; }

private:
    struct Impl;
    struct ProbeCall;
    void ProcessPending();
    std::unique_ptr<ProbeCall> LaunchPending();
    std::unique_ptr<ProbeCall> LaunchBatches(std::vector<VectorBatch *> &&batches);
    void LaunchAttempt(ProbeCall &pc);
    void FinishProbe(ProbeCall &pc, std::deque<VectorBatch *> &out);
    // Pipelined callers: full chunks go to a worker thread that launches and finishes the probe
    // calls (RunWorker), so the caller's AddInput / GetOutput overlap with the launches.
    void HandOff();
    void RunWorker();
    void StopWorker();
    int32_t GetOutputFromWorker(VectorBatch **outputVecBatch);
    bool ProcessPartitioned();
    int32_t strategy_ = kJoinDirect;
    int32_t partBits_ = 0;
    std::vector<int64_t> splits_;
    const LookupJoinOperatorFactory &f_;
    std::unique_ptr<Impl> impl_;
    std::vector<VectorBatch *> pending_;
    int64_t pendingRows_ = 0;
    std::deque<VectorBatch *> outputs_;
};

// Emits the build rows no probe matched, with NULL probe columns, after every probe operator of
// a build-side outer or full join finished (operator/join/lookup_outer_join.h:19-100).
class LookupOuterJoinOperatorFactory : public OperatorFactory {
public:
    LookupOuterJoinOperatorFactory(const type::DataTypes &probeTypes, const int32_t *probeOutputCols,
        int32_t probeOutputColsCount, const int32_t *buildOutputCols, const type::DataTypes &buildOutputTypes,
        HashBuilderOperatorFactory *builder, BuildSide buildSide);
    static LookupOuterJoinOperatorFactory *CreateLookupOuterJoinOperatorFactory(const type::DataTypes &probeTypes,
        int32_t *probeOutputCols, int32_t probeOutputColsCount, int32_t *buildOutputCols,
        const type::DataTypes &buildOutputTypes, int64_t hashBuilderFactoryAddr);
    static LookupOuterJoinOperatorFactory *CreateLookupOuterJoinOperatorFactory(const type::DataTypes &probeTypes,
        int32_t *probeOutputCols, int32_t probeOutputColsCount, int32_t *buildOutputCols,
        const type::DataTypes &buildOutputTypes, int64_t hashBuilderFactoryAddr, BuildSide buildSide);
    Operator *CreateOperator() override;

    type::DataTypes probeOutputTypes;  // types of the probe output columns (all NULL here)
    std::vector<int32_t> buildOutputCols;
    type::DataTypes buildOutputTypes;
    JoinBuildState *build;
    BuildSide buildSide;
    int32_t rowsPerBatch;
};

class LookupOuterJoinOperator : public Operator {
public:
    explicit LookupOuterJoinOperator(const LookupOuterJoinOperatorFactory &f);
    ~LookupOuterJoinOperator() override;
    // Nothing to do: the rows come from the build (lookup_outer_join.cpp:167-171).
    int32_t AddInput(VectorBatch *vecBatch) override;
    // One batch of unmatched build rows per call; FINISHED after the last (or at once when there
    // are none), lookup_outer_join.cpp:173-203.
    int32_t GetOutput(VectorBatch **outputVecBatch) override;
    OmniStatus Close() override;

private:
    struct Impl;
    void Prepare();
    const LookupOuterJoinOperatorFactory &f_;
    std::unique_ptr<Impl> impl_;
    bool prepared_ = false;
    std::deque<VectorBatch *> outputs_;
};

}  // namespace op
}  // namespace omniruntime
