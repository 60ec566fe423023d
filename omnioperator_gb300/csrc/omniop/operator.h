// Operator / OperatorFactory base classes with the reference's method names and state
// machine (operator/operator.h:22-266, operator/operator_factory.h:13-29).
#pragma once

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include "types.h"
#include "vector.h"

namespace omniruntime {
namespace op {
using vec::VectorBatch;

enum class BlockingReason { kNotBlocked = 0, kWaitForJoinBuild = 1 };

class Operator {
public:
    Operator() = default;
    virtual ~Operator() = default;

    virtual int32_t AddInput(VectorBatch *vecBatch) = 0;
    virtual int32_t GetOutput(VectorBatch **result) = 0;

    static void DeleteOperator(Operator *op)
    {
        op->Close();
        delete op;
    }

    OmniStatus GetStatus() const { return status_; }
    void SetStatus(OmniStatus s) { status_ = s; }
    virtual OmniStatus Init() { return OMNI_STATUS_NORMAL; }
    virtual OmniStatus Close() { return OMNI_STATUS_NORMAL; }
    virtual uint64_t GetHashMapUniqueKeys() { return 0; }
    // Bytes this operator moved out of device memory (Operator::GetSpilledBytes, operator.h:66).
    virtual uint64_t GetSpilledBytes() { return 0; }
    // Operators without a partial schema return the batch itself (operator.h:92-95).
    virtual VectorBatch *AlignSchema(VectorBatch *inputVecBatch) { return inputVecBatch; }
    virtual BlockingReason IsBlocked() { return BlockingReason::kNotBlocked; }

    // noMoreInput_ defaults to true, as in the reference (operator.h:204): a caller that
    // feeds one batch and drains it needs no further call.  Pipelined callers (the
    // reference's LocalPlanner, compute/local_planner.cpp:34) set it false and call
    // noMoreInput() at the end, which lets the GB300 operators batch many VectorBatches
    // into one kernel launch.
    virtual void noMoreInput() { noMoreInput_ = true; }
    virtual void setNoMoreInput(bool v) { noMoreInput_ = v; }
    virtual bool needsInput() { return status_ != OMNI_STATUS_FINISHED && !noMoreInput_; }
    bool isFinished() const { return status_ == OMNI_STATUS_FINISHED; }

    // GB300 controls.
    // Run on the caller's stream (the legacy default stream when `stream` is null).
    void SetStream(void *stream)
    {
        userStream_ = stream;
        userStreamSet_ = true;
    }
    void SetDeviceOutput(bool on) { deviceOutput_ = on; }
    std::vector<int64_t> Counters() const
    {
        std::vector<int64_t> v(kCounters);
        for (int i = 0; i < kCounters; ++i) {
            v[i] = counters_[i].load(std::memory_order_relaxed);
        }
        return v;
    }
    static constexpr int kCounters = 12;

protected:
    bool noMoreInput_ = true;
    void *userStream_ = nullptr;
    bool userStreamSet_ = false;
    bool deviceOutput_ = false;
    // [0] launches, [1] resizes / re-runs, [2] retried rows, [3] groups, [4] ordered groups,
    // [5] output rows, [6] kernel ns, [7] timed kernel launches, and host time of the probe
    // pipeline: [8] ns setting up and launching probe calls, [9] ns waiting for their kernels,
    // [10] ns carving output batches, [11] ns freeing the probe input batches.
    // Atomic: a probe operator's worker thread updates them while the caller may read them.
    std::atomic<int64_t> counters_[kCounters]{};

private:
    OmniStatus status_ = OMNI_STATUS_NORMAL;
};

class OperatorFactory {
public:
    OperatorFactory() = default;
    virtual ~OperatorFactory() = default;
    virtual Operator *CreateOperator() { return nullptr; }
};

}  // namespace op
}  // namespace omniruntime
