// Allocation-free hash aggregation of one device-resident batch (see agg_noalloc.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "kernels/plan.h"

namespace omg {

// Size of the file-scope device scratch array: 64 MiB.  It bounds the group table
// ((2 * max_groups rounded up to a power of two, plus 2) slots of the plan's slot size) plus the
// tile descriptors of the rows.
constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;

// The compiled aggregation a call runs (copied from a HashAggregationOperatorFactory plan into
// fixed-size arrays, so a call needs no heap memory either).
struct NoAllocPlan {
    int32_t nInputs = 0;
    int32_t inputCols[kMaxInputs] = {};
    KeySpec key{};
    int32_t nAccs = 0;
    AccSpec accs[kMaxAccs] = {};
    int32_t nRegInputs = 0;
    int16_t regInput[kRegInputs] = {};
    int16_t regWidth[kRegInputs] = {};
    int32_t stateWords = 0;
    int32_t keyWords = 0;
    int32_t slotWords = 0;
    int32_t nOut = 0;
    OutSpec outs[kMaxOutCols] = {};
    bool overflowAsNull = false;
    int32_t smemSlots = 0;
    long long waitBudget = kDefaultWaitBudget;  // clock64 ticks of a bounded device-side wait
};

struct NoAllocStatus {
    int32_t code = 0;        // 0 or an OMG_ERR_* value
    char message[192] = {};  // set when code != 0
};

// Aggregates `nRows` rows of device columns `cols[]` / null bitmaps `nulls[]` (indexed by batch
// column; `nulls` may be null or hold null entries) into the caller's device output columns:
// `nOut` value arrays and null bitmaps with room for `maxGroups` rows (the bitmaps are cleared
// here).  Synchronises `stream` and stores the number of groups in *numGroups.  Allocates no
// device or host memory.
NoAllocStatus RunAggNoAlloc(const NoAllocPlan &plan, const void *const *cols, const uint8_t *const *nulls,
    int32_t nCols, int64_t nRows, void *const *outValues, uint8_t *const *outNulls, int32_t nOut, int64_t maxGroups,
    int64_t *numGroups, cudaStream_t stream);

}  // namespace omg
