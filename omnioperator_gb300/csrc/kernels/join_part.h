// Partitioned inner hash join for unique 8-byte build keys (join_part.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "plan.h"

namespace omg {

enum JoinPartKind : int32_t { JOIN_PART_HASH = 0, JOIN_PART_RANGE = 1 };
constexpr int kMaxJoinParts = 4096;
constexpr int kMaxJoinSplits = kMaxJoinParts - 1;

// Partition function: HASH = top `bits` bits of the key's 64-bit mix; RANGE = the number of
// splits <= key (splits sorted, nSplits = 2^bits - 1).  1 <= bits <= 12.
struct JoinPartFn {
    int32_t kind;
    int32_t bits;
    const int64_t *splits;
    int32_t nSplits;
    int32_t lutShift;        // RANGE: bucket of a key = (key - lutBase) >> lutShift (clamped)
    int64_t lutBase;
    const uint16_t *lut;     // RANGE: [kJoinLutBuckets + 1] first split index of each bucket
};

// Range lookup table: kJoinLutBuckets buckets over [min split, max split]; a key's partition
// is found by a binary search over the splits of its bucket only.
constexpr int kJoinLutBuckets = 1 << 14;

// Build output columns copied with the key into partition order, packed per row.
struct PayloadCols {
    int32_t nCols;
    int32_t rowBytes;
    int32_t width[kMaxOutCols];
    const void *cols[kMaxOutCols];
};

struct PartProbeLaunch {
    JoinPartFn fn;
    const int64_t *keys;       // partitioned probe keys (NULLs already dropped)
    int64_t n;
    const int64_t *tabStart;   // [P + 1] slab offsets of the partitions' tables
    const uint64_t *tabKeys;
    const int32_t *tabRow;     // row within the partition's build rows
    const int64_t *start;      // [P + 1] first partitioned build row of each partition
    const uint8_t *pay;        // partitioned build payload, payBytes per row
    int32_t payBytes;
    int32_t nPayOut;
    int32_t payWidth[kMaxOutCols];
    void *payOut[kMaxOutCols];  // build output columns
    int64_t *keyOut;            // probe key output column (nullptr: not an output)
    unsigned long long *outCount;  // nRegions counters, kRegionStride apart
    int32_t nRegions;
    int32_t pad;
    uint64_t regionCap;
};

// Radix partition of a key column (NULL rows dropped) into 2^f.bits partitions in nChunks
// chunks: hist [nChunks * P] u32, start [P + 1], place [nChunks * P] i64 scratch, outKeys (and,
// when outPay is not null, the packed payload of each row) in partition order.
cudaError_t LaunchKeyPartition(const int64_t *keys, const uint8_t *nulls, int64_t n, const JoinPartFn &f,
    int32_t nChunks, uint32_t *hist, int64_t *start, int64_t *place, int64_t *outKeys, const PayloadCols &pay,
    uint8_t *outPay, cudaStream_t stream);
// Per-partition tables of the partitioned build keys (error: 3 duplicate key, 4 table full,
// 5 a key equal to the EMPTY sentinel).
cudaError_t LaunchPartTableBuild(const int64_t *pkeys, const int64_t *start, int32_t P, const int64_t *tabStart,
    int64_t tabSlots, uint64_t *tabKeys, int32_t *tabRow, int32_t *error, cudaStream_t stream);
cudaError_t LaunchPartProbe(const PartProbeLaunch &q, cudaStream_t stream);

}  // namespace omg
