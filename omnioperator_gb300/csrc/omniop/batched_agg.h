// Many independent HashAggregation tasks in one launch (no reference counterpart: the reference
// runs one operator instance per task, operator/aggregation/group_aggregation.cpp:320-406).
//
// Each task is one VectorBatch aggregated by the factory's plan into its own table.  The tables
// live in one slab sized per task from a batched key sketch (or a learned sizing model); one
// persistent kernel walks the tiles of every task, and per-task count and extraction kernels
// write all tasks' groups into shared output columns.  The launch sequence is captured once as a
// CUDA graph and replayed on every Run; the persistent kernel's launch shape is chosen by timing
// the candidates on the first Run (cached per plan and workload size).  A task whose groups
// outgrow its table is re-run through a regular operator, so results are always exact.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "hash_aggregation.h"

namespace omniruntime {
namespace op {

constexpr int32_t kBatchDeviceOutput = 1;  // outputs stay in HBM
constexpr int32_t kBatchNoGraph = 2;       // launch the sequence directly instead of a CUDA graph
constexpr int32_t kBatchNoTune = 4;        // default launch shape, no autotuning
constexpr int32_t kBatchTinyTables = 8;    // test hook: 64-slot tables, overflowing tasks re-run by operators
constexpr int32_t kBatchTinyGrow = 16;     // test hook: 64-slot tables, overflowing tasks take the grow pass

class BatchedAggregation {
public:
    // The task batches stay owned by the caller and must outlive this object.
    BatchedAggregation(HashAggregationOperatorFactory &factory, std::vector<vec::VectorBatch *> tasks,
        omg::SizingModel *sizer, int32_t flags);
    ~BatchedAggregation();
    BatchedAggregation(const BatchedAggregation &) = delete;
    BatchedAggregation &operator=(const BatchedAggregation &) = delete;

    // Aggregate every task (on `stream` when not null).  The first call sizes the tables, tunes
    // the launch shape and captures the graph; later calls replay it.
    void Run(void *stream);
    // New output batches of the last Run (caller frees them) and the task of each, task order.
    void Outputs(std::vector<vec::VectorBatch *> &batches, std::vector<int32_t> &taskOf);
    // [0] tasks, [1] input rows, [2] table slots, [3] tasks re-run exactly, [4] threads per CTA,
    // [5] CTAs per SM, [6] runs, [7] groups, [8] tuning us, [9] preparation us, [10] last run's
    // device time us, [11] 1 if a sizing model sized the tables, [12] 1 if the runs replay a
    // CUDA graph.
    std::vector<int64_t> Info() const;
    // Per task, the sizing record layout of HashAggregationOperator::GetSizingLog (23 values).
    std::vector<int64_t> SizingLogs() const;

private:
    struct Impl;
    std::unique_ptr<Impl> impl_;
};

}  // namespace op
}  // namespace omniruntime
