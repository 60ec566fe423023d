// Host-callable launchers of the operator kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "plan.h"

namespace omg {

// SM count of the current device (cached per device).
int DeviceSMCount();
// Raises `kernel`'s dynamic shared-memory limit on the current device to at least `bytes`.
// The attribute belongs to one device, so the record of what was set is kept per device (and
// guarded by a mutex: operators launch from several host threads).
cudaError_t EnsureDynamicSmem(const void *kernel, size_t bytes);
// CTAs of `kernel` resident per SM at (threads, dynamic shared memory) on the current device,
// at least 1; cached per (device, kernel, threads, bytes).
int BlocksPerSM(const void *kernel, int threads, size_t smemBytes);

// ---- aggregation (agg.cu)
cudaError_t LaunchAggInitTable(const AggLaunch &p, cudaStream_t stream);
cudaError_t LaunchAggRehash(const AggLaunch &p, const AggTable &from, const AggTable &to, cudaStream_t stream);
cudaError_t LaunchAgg(const AggLaunch &p, uint64_t *spill, unsigned int *nSpill, uint32_t spillCap,
    const uint64_t *spillIn, uint32_t nSpillIn, int gridBlocks, cudaStream_t stream);
// Partitioned aggregation: shared slots per CTA of a partitioned launch, and the partition pass
// (histogram, layout, scatter) over p's batches into a's buffers; a.hist must be zero.
int32_t AggPartSmemSlots(int32_t slotWords);
cudaError_t LaunchAggPartition(const AggLaunch &p, const PartArgs &a, cudaStream_t stream);
// Key sketch of nSample rows stratified over p's tiles; stats as described at kSketchStats.
// tabKeys / tabCounts hold kSketchCap entries.
cudaError_t LaunchAggSketch(const AggLaunch &p, int32_t nSample, unsigned long long *tabKeys,
    unsigned int *tabCounts, unsigned long long *stats, cudaStream_t stream);
// HyperLogLog registers over every row of p's tiles into regs[kHllRegs + 2] (zeroed here).
cudaError_t LaunchAggHll(const AggLaunch &p, unsigned int *regs, cudaStream_t stream);
// Batched tasks: per-task sketch (kSketchStats per task), the persistent aggregation over all
// tasks' tiles (autotuned threads per CTA and grid), per-task group counts and extraction at
// per-task output offsets.
cudaError_t LaunchAggTaskSketch(const AggLaunch &p, int32_t nTasks, unsigned long long *stats, cudaStream_t stream);
int32_t AggTasksVariants();
void AggTasksVariantShape(int32_t variant, int32_t *threads, int32_t *blocksPerSM);
cudaError_t LaunchAggTasks(const AggLaunch &p, int32_t variant, cudaStream_t stream);
cudaError_t LaunchAggTaskCount(const AggTable *tables, int32_t nTasks, int32_t keyKind, uint32_t *counts,
    cudaStream_t stream);
cudaError_t LaunchAggTaskPad(const uint32_t *groups, int32_t nTasks, uint32_t *padded, cudaStream_t stream);
cudaError_t LaunchAggTaskExtract(const AggExtract &e, const AggTable *tables, int32_t nTasks, const int64_t *offsets,
    cudaStream_t stream);
cudaError_t LaunchAggCount(const AggTable &t, int keyKind, unsigned long long *out, cudaStream_t stream);
cudaError_t LaunchAggExtract(const AggExtract &e, cudaStream_t stream);
// Ordered replay of order-dependent sticky-overflow groups; sets forced[slot] bit k when
// exact-SUM output k of that group overflowed on some row-ordered prefix.
cudaError_t LaunchAggOrdered(const AggLaunch &p, int32_t nBatches, const AggExtract &e,
    const unsigned long long *ambSlots, uint32_t nAmb, uint8_t *forced, cudaStream_t stream);

// Inner probes on a bitmap ARRAY table use the group-staged kernel when it fits (default on);
// off selects the per-warp bitmap kernel.  Process-wide; for tests and measurements.
void SetStagedProbe(bool on);
// Bulk-copy inner probe for HBM output: 0 off (default), 1 keys by cp.async.bulk, 2 keys and
// output runs by cp.async.bulk.
void SetBulkProbe(int mode);
// Which probe kernel the latest LaunchProbe in this process started.
enum ProbeKernelId {
    PROBE_KERNEL_NONE = 0,
    PROBE_KERNEL_KIND = 1,     // ProbeKindKernel: multi-column keys, filters
    PROBE_KERNEL_GENERAL = 2,  // ProbeKernel
    PROBE_KERNEL_FAST = 3,     // ProbeFastKernel
    PROBE_KERNEL_BITS = 4,     // ProbeBitsKernel: bitmap in shared memory, per-lane loads and stores
    PROBE_KERNEL_GROUP = 5,    // ProbeGroupKernel: group-staged output runs (pinned host output)
    PROBE_KERNEL_BULK = 6,     // ProbeBulkKernel: keys and output runs by cp.async.bulk
};
int LastProbeKernel();

// ---- utilities (util.cu)
// Masked-input NULL bitmaps, one per job (see MaskJob).
cudaError_t LaunchMaskNulls(const MaskJob *jobs, int32_t nJobs, cudaStream_t stream);
// [0] rows, [1] and [2] two order-independent 64-bit sums of per-row column hashes.
cudaError_t LaunchFingerprint(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles, int32_t nCols,
    const int32_t *widths, unsigned long long *out, cudaStream_t stream);

// ---- join (join.cu)
// Copy column `input` of every batch into one contiguous device array (values) and, if
// `nullsOut` is given, one contiguous null bitmap (zeroed by the caller).
cudaError_t LaunchGatherColumn(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, int32_t input, int32_t width, void *valuesOut, uint8_t *nullsOut,
    cudaStream_t stream);
// Min / max / count of the non-null keys of a contiguous key column.
// stats[0] = min, stats[1] = max, stats[2] = count (initialised by the launcher).
cudaError_t LaunchKeyStats(const void *keys, const uint8_t *nulls, int64_t n, int32_t width,
    long long *stats, cudaStream_t stream);
// ARRAY mode: counts[key - min] += 1; HASH mode: insert keys, counts per slot.
cudaError_t LaunchBuildCount(JoinTable t, const void *keys, const uint8_t *nulls, int64_t n, int32_t width,
    uint64_t *hashKeysMutable, uint32_t *counts, uint32_t *sentinelCount, unsigned int *maxCount,
    int32_t *error, cudaStream_t stream);
// Exclusive scan of uint32 counts into int64 offsets; total written to *total.
cudaError_t LaunchScanCounts(const uint32_t *counts, int64_t n, int64_t *offsets, int64_t *blockSums,
    long long *total, cudaStream_t stream);
// Fill entries: unique -> row, else (offset << 32 | count), and the CSR row lists.
cudaError_t LaunchBuildFill(JoinTable t, const void *keys, const uint8_t *nulls, int64_t n, int32_t width,
    const uint32_t *counts, const int64_t *offsets, uint32_t *cursor, int64_t *entriesMutable,
    int32_t *csrRowsMutable, uint32_t sentinelCount, int64_t sentinelOffset, unsigned int *sentinelCursor,
    int64_t *sentinelEntryOut, int32_t *error, cudaStream_t stream);
cudaError_t LaunchProbe(const ProbeLaunch &p, cudaStream_t stream);
// One output column of AlignSchema (adaptive partial aggregation) for every input row.
cudaError_t LaunchAlignColumn(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, const AlignCol &c, void *out, uint8_t *outNulls, cudaStream_t stream);
// VARCHAR columns: lengths / characters of a batch input in tile output order; output columns
// from per-row handles over regions (see JoinOutCol); rows of a contiguous column.  Offsets
// passed in are exclusive scans of the lengths (LaunchScanCounts) with the total at [n]
// (LaunchOffsetsTail).
cudaError_t LaunchVarlenTileLens(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, int32_t input, uint32_t *lens, cudaStream_t stream);
cudaError_t LaunchVarlenTileCopy(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, int32_t input, const int64_t *dstOffs, uint8_t *dst, cudaStream_t stream);
cudaError_t LaunchVarlenOutLens(const int64_t *handles, int64_t nPos, uint64_t regionCap,
    const unsigned long long *regionCounts, int side, const BatchDesc *batches, int32_t input,
    const int64_t *buildOffs, uint32_t *lens, cudaStream_t stream);
cudaError_t LaunchVarlenOutCopy(const int64_t *handles, int64_t nPos, uint64_t regionCap,
    const unsigned long long *regionCounts, int side, const BatchDesc *batches, int32_t input,
    const int64_t *buildOffs, const uint8_t *buildChars, const int64_t *offs64, uint8_t *chars, int32_t *offs32,
    long long total, cudaStream_t stream);
cudaError_t LaunchVarlenRowsLens(const int32_t *rows, int64_t n, const int64_t *srcOffs, uint32_t *lens,
    cudaStream_t stream);
cudaError_t LaunchVarlenRowsCopy(const int32_t *rows, int64_t n, const int64_t *srcOffs, const uint8_t *srcChars,
    const int64_t *offs64, uint8_t *chars, int32_t *offs32, long long total, cudaStream_t stream);
cudaError_t LaunchOffsetsTail(int64_t *offs, int64_t n, const long long *total, cudaStream_t stream);
// String dictionary of VARCHAR group-by columns (kernels/dict.cu): insert a batch set's strings
// (rowSlot per row in tile output order, -1 for NULL), give new slots ids, append their
// characters to the arena, grow the table, map rows to ids, and turn ids back into strings.
cudaError_t LaunchDictInsert(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles, const int64_t *tileOutRow,
    int32_t input, unsigned long long *hash, const int32_t *id, unsigned long long *rep, uint64_t cap,
    const int64_t *arenaOff, const uint8_t *arena, int32_t *rowSlot, int32_t *error, cudaStream_t stream);
cudaError_t LaunchDictMaterialize(const unsigned long long *hash, int32_t *id, const unsigned long long *rep,
    uint64_t cap, int32_t firstId, unsigned int *counter, unsigned long long *newRep, uint32_t *newLen,
    const BatchDesc *batches, int32_t input, cudaStream_t stream);
cudaError_t LaunchDictAppend(const unsigned long long *newRep, int64_t nNew, int32_t firstId, const int64_t *arenaOff,
    uint8_t *arena, const BatchDesc *batches, int32_t input, cudaStream_t stream);
cudaError_t LaunchDictRehash(const unsigned long long *oldHash, const int32_t *oldId, uint64_t oldCap,
    unsigned long long *hash, int32_t *id, uint64_t cap, int32_t *error, cudaStream_t stream);
cudaError_t LaunchDictShiftOffsets(const int64_t *offs, int64_t nNew, int64_t base, int64_t *arenaOff,
    cudaStream_t stream);
cudaError_t LaunchDictRowIds(const int32_t *rowSlot, int64_t n, const int32_t *id, int32_t *ids, cudaStream_t stream);
cudaError_t LaunchDictDecodeLens(const int32_t *ids, const uint8_t *nulls, int64_t n, const int64_t *arenaOff,
    uint32_t *lens, cudaStream_t stream);
cudaError_t LaunchDictDecodeCopy(const int32_t *ids, const uint8_t *nulls, int64_t n, const int64_t *arenaOff,
    const uint8_t *arena, const int64_t *offs64, uint8_t *chars, int32_t *offs32, long long total,
    cudaStream_t stream);
// Dictionary-encoded input vectors (kernels/dictvec.cu): fixed-width values and null bits
// gathered through the ids; VARCHAR lengths (with null bits), then characters.  Out-of-range ids
// set *error and give NULL rows.
cudaError_t LaunchDictGatherFixed(const int32_t *ids, int64_t n, const uint8_t *dictValues, const uint8_t *dictNulls,
    int32_t dictSize, int width, uint8_t *out, uint32_t *outNulls, int32_t *error, cudaStream_t stream);
cudaError_t LaunchDictGatherLens(const int32_t *ids, int64_t n, const int32_t *dictOffs, const uint8_t *dictNulls,
    int32_t dictSize, uint32_t *lens, uint32_t *outNulls, int32_t *error, cudaStream_t stream);
cudaError_t LaunchDictGatherChars(const int32_t *ids, int64_t n, const int32_t *dictOffs, const uint8_t *dictChars,
    const uint8_t *dictNulls, int32_t dictSize, const int64_t *offs64, uint8_t *chars, int32_t *offs32,
    long long total, cudaStream_t stream);
// Multi-column join keys: the tuple hash of each build row (NULL if a key column is NULL).
// Packed multi-column join keys (JoinKeyPack): of the build's contiguous key columns into `out`
// (+ NULL bitmap), and of the probe batches' key parts into input kp.outInput of each batch.
cudaError_t LaunchPackBuildKeys(const JoinKeyCols &kc, const JoinKeyPack &kp, int64_t n, int64_t *out,
    uint8_t *outNulls, cudaStream_t stream);
// True when LaunchProbe's kernel for `p` packs the key parts (p.pack) itself; otherwise it runs
// the packing pass into the scratch input p.pack.outInput first.
bool ProbePacksKeys(const ProbeLaunch &p);
cudaError_t LaunchPackProbeKeys(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles, const JoinKeyPack &kp,
    cudaStream_t stream);
cudaError_t LaunchJoinKeyHash(const JoinKeyCols &kc, int64_t n, uint64_t *out, uint8_t *outNulls, cudaStream_t stream);
// Outer joins: flags[i] = 1 for build rows never matched; their row numbers in order (offsets =
// exclusive scan of the flags); dst[i] = src[rows[i]] with NULL bits.
cudaError_t LaunchUnvisitedFlags(const uint8_t *visited, int64_t n, uint32_t *flags, cudaStream_t stream);
cudaError_t LaunchUnvisitedRows(const uint8_t *visited, const int64_t *offsets, int64_t n, int32_t *rows,
    cudaStream_t stream);
cudaError_t LaunchGatherRows(const void *src, const uint8_t *srcNulls, const int32_t *rows, int64_t n, int32_t width,
    void *dst, uint8_t *dstNulls, cudaStream_t stream);
// Packs the build output columns named by p.out (side 1, with shifts set) per table slot into
// payload[nSlots + 1] (the last slot holds the EMPTY-key row of a HASH table).
cudaError_t LaunchBuildSlotPayload(const ProbeLaunch &p, uint64_t nSlots, uint64_t *payload, cudaStream_t stream);
// Occupancy bitmap of an ARRAY table (bit d set iff arrayEntries[d] >= 0) into a buffer of
// SlotBitsBytes(range) bytes.
uint64_t SlotBitsBytes(uint64_t range);
cudaError_t LaunchBuildSlotBits(const int64_t *arrayEntries, uint64_t range, uint32_t *bits, cudaStream_t stream);
cudaError_t LaunchFillI64(int64_t *p, int64_t v, int64_t n, cudaStream_t stream);
cudaError_t LaunchFillU64(uint64_t *p, uint64_t v, int64_t n, cudaStream_t stream);

}  // namespace omg
