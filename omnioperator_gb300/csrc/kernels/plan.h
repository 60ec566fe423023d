// Launch descriptors shared by the host operators and the CUDA kernels.
//
// A kernel reads its input as a list of VectorBatch descriptors (one per OmniVec batch, host
// pinned or HBM) cut into tiles of at most kTileRows rows, so one launch covers any number of
// batches of uneven sizes.
#pragma once

#include <cstdint>

namespace omg {

constexpr int kMaxInputs = 12;   // distinct input columns a kernel reads
constexpr int kMaxAccs = 24;     // accumulators per group
constexpr int kMaxKeyCols = 4;   // composite group-by / join key columns
constexpr int kMaxOutCols = 16;  // output columns of an aggregation or join
constexpr int kTileRows = 4096;  // rows per tile

// One VectorBatch as the kernels see it.  cols[i] / nulls[i] are the values and the null
// bitmap (LSB-first, set bit = NULL) of kernel input i; nulls[i] == nullptr means the
// column has no nulls in this batch.
struct BatchDesc {
    const void *cols[kMaxInputs];       // values (VARCHAR/CHAR: the character buffer)
    const uint8_t *nulls[kMaxInputs];
    const int32_t *offs[kMaxInputs];    // VARCHAR/CHAR: n + 1 offsets into cols[i]; else nullptr
    int64_t rows;
    int64_t rowBase;  // index of the batch's first row in arrival order
};

// An aggregation input whose rows are filtered by a mask column
// (MaskColAggregator::ProcessGroup, mask_column_assistant_aggregator.h:44-53): `out` receives
// the input's NULL bitmap with every row whose mask value is NULL or FALSE added to it, so
// every accumulator skips those rows as it skips NULL values.
struct MaskJob {
    const uint8_t *valueNulls;  // the value column's NULL bitmap (nullptr: none)
    const uint8_t *maskValues;  // BOOLEAN mask column, one byte per row
    const uint8_t *maskNulls;   // its NULL bitmap (nullptr: none)
    uint32_t *out;              // ceil(rows / 32) words
    int64_t rows;
    int32_t mode;               // 0: drop rows whose mask is NULL or FALSE; 1: drop rows whose mask
                                // byte is non-zero (its NULL flag not read); 2: drop rows whose mask
                                // column is NULL (its values not read)
    int32_t pad;
};

struct TileDesc {
    int32_t batch;
    int32_t row0;
    int32_t rows;
    int32_t pad;
};

// How kernel input values are widened.
enum InKind : int16_t { IN_INT = 0, IN_DOUBLE = 1, IN_FLOAT = 2, IN_DEC128 = 3, IN_NONE = 4 };

// ---- group-by key -------------------------------------------------------------------------
// KEY_SINGLE: one integer-like column widened to int64; the NULL key is its own group.
// KEY_PACKED: several fixed-width columns packed little-endian into `words` 64-bit words,
// followed by a null-mask byte (bit c set = column c is NULL; its value bytes are zero).
enum KeyKind : int32_t { KEY_SINGLE = 0, KEY_PACKED = 1 };

struct KeyCol {
    int16_t input;       // kernel input index
    int16_t width;       // bytes: 1, 2, 4, 8, 16
    int16_t byteOffset;  // offset inside the packed key
    int16_t pad;
};

struct KeySpec {
    int32_t kind;
    int32_t nCols;
    int32_t words;       // packed words (KEY_PACKED), 1 for KEY_SINGLE
    int32_t maskByte;    // byte offset of the null mask (KEY_PACKED)
    KeyCol cols[kMaxKeyCols];
};

// ---- accumulators -----------------------------------------------------------------------------
// Per-group state is a row of 64-bit words.  Every aggregate is computed from these:
//  COUNT_ALL  rows of the group                          1 word
//  NULLS      NULL rows of input column `input`          1 word   (COUNT(col) = COUNT_ALL - NULLS)
//  ISUM       wrapping int64 sum                         1 word
//  WSUM2      exact sum of int64 values                  4 words
//  WSUM3      exact sum of int128 (decimal128) values    8 words
//  DSUM       compensated double sum (s, c)              2 words
//  IMIN/IMAX  int64 min / max                            1 word
//  DMIN/DMAX  double min / max as order-preserving int64 1 word
//  SMIN/SMAX  VARCHAR min / max: the string dictionary id 1 word (-1: no value yet)
//  XMIN/XMAX  decimal128 min / max (low, high word)     2 words, 16-byte aligned in the slot
// WSUM keeps the positive and the negative values apart, each as sums of 32-bit chunks: word k
// of a side accumulates bits [32k, 32k+32) of every magnitude.  A word therefore never carries
// for fewer than 2^32 rows per group, every update is a fire-and-forget atomic add, the exact
// sum is pos - neg and sum|x| is pos + neg (the sticky-overflow rule needs both).
enum AccKind : int16_t {
    ACC_COUNT_ALL = 0,
    ACC_NULLS = 1,
    ACC_ISUM = 2,
    ACC_WSUM2 = 3,
    ACC_WSUM3 = 4,
    ACC_DSUM = 5,
    ACC_IMIN = 6,
    ACC_IMAX = 7,
    ACC_DMIN = 8,
    ACC_DMAX = 9,
    ACC_SMIN = 10,
    ACC_SMAX = 11,
    ACC_XMIN = 12,
    ACC_XMAX = 13,
};

struct AccSpec {
    int16_t kind;
    int16_t input;    // kernel input index (-1 for COUNT_ALL)
    int16_t inKind;   // InKind
    int16_t inWidth;  // bytes per input value
    int32_t word;     // first state word
    int32_t reg;      // slot of the input in the per-row register cache (-1: load directly)
    int64_t init;     // initial value of the first word
};

inline int AccWords(int kind)
{
    switch (kind) {
        case ACC_WSUM2:
            return 4;
        case ACC_WSUM3:
            return 8;
        case ACC_DSUM:
        case ACC_XMIN:
        case ACC_XMAX:
            return 2;
        default:
            return 1;
    }
}

// Global open-addressing group table.  Slot s occupies slotWords words at
// slots + s * slotWords: [key words][state words].  KEY_SINGLE: one key word, EMPTY marks a
// free slot (a real key equal to EMPTY lives in the special slot kSentinelSlot).  KEY_PACKED:
// a tag word (0 free, 1 being written, else published) and `words` key words.  Two special
// slots follow the `capacity` hashed slots: the NULL-key group and the EMPTY-key group.
constexpr uint64_t kEmptyKey = 0x8000000000000000ull;
constexpr int kNullSlotOffset = 0;      // slot capacity + 0
constexpr int kSentinelSlotOffset = 1;  // slot capacity + 1

struct AggTable {
    uint64_t *slots;
    uint64_t capacity;  // power of two
    int32_t slotWords;
    int32_t keyWords;   // words before the state
    uint32_t *specialUsed;            // [2] flags of the special slots
    unsigned long long *groupCount;   // groups inserted so far (block-aggregated)
};

constexpr int kRegInputs = 4;  // kernel inputs of <= 8 bytes loaded into registers per row

struct AggLaunch {
    const BatchDesc *batches;
    const TileDesc *tiles;
    int32_t nTiles;
    int32_t nAccs;
    int32_t nRegInputs;               // inputs cached in registers (<= kRegInputs)
    int16_t regInput[kRegInputs];     // their kernel input indices
    int16_t regWidth[kRegInputs];     // their widths in bytes
    KeySpec key;
    AccSpec accs[kMaxAccs];
    int32_t stateWords;
    int32_t maxProbe;
    AggTable table;
    // Rows whose group could not be placed (probe limit hit) are queued here as
    // (batch << 32 | row) and re-run after the table grows.
    unsigned long long *retry;
    unsigned int *nRetry;
    uint32_t retryCap;
    // When non-null the kernel processes these queued rows instead of the tiles.
    const unsigned long long *retryIn;
    uint32_t nRetryIn;
    int32_t smemSlots;  // per-CTA shared-memory pre-aggregation slots (0 = off)
    int32_t *error;     // sticky device error code (0 = none)
    long long waitBudget;  // clock64 ticks a thread may wait for another's slot publication
    // Partitioned launches (nParts > 0): the batches are hash partitions, tiles
    // [partTileStart[q], partTileStart[q + 1]) belong to partition q, and CTA c works on
    // partition c % nParts only, so its shared table sees only that partition's groups.
    int32_t nParts;
    const int32_t *partTileStart;
    // Batched tasks (AggTasksKernel): batch i is task i with its own table taskTables[i]; a
    // task whose group does not fit sets taskFailed[i] (the host re-runs it exactly).
    const AggTable *taskTables;
    uint32_t *taskFailed;
    // VARCHAR inputs aggregated by SMIN/SMAX: the input's string dictionary (id k's characters
    // are strChars[strOff[k], strOff[k + 1])), for comparing two ids' strings.
    const int64_t *strOff[kMaxInputs];
    const uint8_t *strChars[kMaxInputs];
};

constexpr int kTaskSketchRows = 1024;   // rows sampled per task by the batched sketch
constexpr int kTaskSketchSlots = 2048;

// ---- hash partitioning of aggregation input -------------------------------------------------
// Rows go to partition (hash >> kPartShift) & (nParts - 1); the shared tables index slots with
// the hash's top 32 bits and the global table with its low bits, so the three are independent.
constexpr int kPartShift = 24;
constexpr int kMaxParts = 64;

struct PartArgs {
    int32_t partBits;                  // nParts = 1 << partBits
    int32_t nInputs;                   // kernel inputs copied into the partitions
    int32_t width[kMaxInputs];         // bytes per value (1, 2, 4, 8, 16)
    void *cols[kMaxInputs];            // partitioned values, rows + kMaxParts * 64 rows each
    uint32_t *nulls[kMaxInputs];       // partitioned NULL bitmaps (zeroed) or nullptr
    unsigned long long *hist;          // [nParts] rows per partition
    unsigned long long *cursor;        // [nParts] next free row of each partition
    BatchDesc *partBatches;            // [nParts] one batch per partition
    TileDesc *partTiles;               // [maxTiles]
    int32_t *partTileStart;            // [nParts + 1]
    int32_t maxTiles;
    // stable: rows keep their input order within every partition (tiles in order, rows of a tile
    // in order), for plans whose results depend on row order; tileHist is then a [nTiles][nParts]
    // scratch of per-tile counts.
    int32_t stable;
    unsigned int *tileHist;
};

// ---- key sketch of a row sample (feeds the group-count estimate) ----------------------------
constexpr int kSketchCap = 1 << 17;  // sketch table slots (sample <= kSketchCap / 2 rows)
constexpr int kSketchStats = 16;
// stats: [0] sampled rows, [1] special-key rows (NULL / EMPTY key), [2] distinct hashes d,
// [3] f1 (hashes seen once), [4] f2, [5] f3, [6] hashes seen 4-7 times, [7] 8+ times,
// [8] largest count, [9] rows held by hashes seen 8+ times.

// HyperLogLog sketch of every row's key (the distinct-count sizing baseline): 2^kHllBits
// registers; register = top kHllBits bits of the key hash, value = the position of the first set
// bit of the remaining bits (1-based).  regs[kHllRegs] and regs[kHllRegs + 1] flag the NULL key and
// the EMPTY-sentinel key, which are groups of their own.
constexpr int kHllBits = 14;
constexpr int kHllRegs = 1 << kHllBits;

// Default bounded-wait budget (clock64 ticks, about two seconds at 2 GHz).
constexpr long long kDefaultWaitBudget = 1ll << 32;

// ---- aggregation output ---------------------------------------------------------------------
enum OutKind : int16_t {
    OUT_KEY = 0,         // group-by column `src`
    OUT_COUNT = 1,       // COUNT(col) / COUNT(*)
    OUT_SUM_WRAP = 2,    // Spark int SUM (wrapping)
    OUT_SUM_EXACT = 3,   // generic int SUM / decimal SUM from WSUM2/WSUM3
    OUT_SUM_DOUBLE = 4,  // double SUM
    OUT_AVG = 5,         // double AVG
    OUT_MIN_INT = 6,
    OUT_MAX_INT = 7,
    OUT_MIN_DOUBLE = 8,
    OUT_MAX_DOUBLE = 9,
    OUT_COUNT_MERGE = 10,      // final COUNT: the sum of partial counts (acc src, ISUM), never NULL
    OUT_AVG_PARTIAL_SUM = 11,  // partial AVG sum: the double sum, 0 for a group without values
                               // (count: COUNT_ALL - NULLS(countAcc), or the ISUM countAcc when
                               // boundKind == 1)
    OUT_AVG_MERGE = 12,        // final AVG: sum (acc src, DSUM) / count (acc countAcc, ISUM), NULL if 0
    OUT_STR_ID = 13,           // VARCHAR MIN/MAX: the dictionary id (int32) of acc src, NULL if none
    OUT_IS_EMPTY = 14,         // decimal SUM partial: BOOLEAN, 1 when no value reached the group's sum
                               // (count as for OUT_COUNT, and no partial sum overflowed: flagAcc)
    OUT_MINMAX_DEC128 = 15,    // decimal128 MIN / MAX: the two words of acc src
    OUT_AVG_DEC = 16,          // decimal AVG: the exact sum of acc src (sticky overflow as for
                               // OUT_SUM_EXACT) over the count, rescaled and rounded as Spark does
};

struct OutSpec {
    int16_t kind;
    int16_t src;        // key column (OUT_KEY) or main accumulator index
    int16_t countAcc;   // NULLS accumulator of the input column (-1 = COUNT(*))
    int16_t outWidth;   // bytes per output value
    int16_t outType;    // DataTypeId of the output
    int16_t boundKind;  // OUT_SUM_EXACT: 0 = int64 range, 1 = decimal(38) range
    int16_t rescalePow; // OUT_SUM_EXACT: multiply the sum by 10^rescalePow
    int16_t pad;        // OUT_SUM_EXACT: index of the exact sum (bit of the ordered-replay flags)
    int16_t flagAcc;    // OUT_SUM_EXACT / OUT_IS_EMPTY of a merging stage: NULLS accumulator of the
                        // partial sums; a NULL partial sum is an overflow of that partial (0: none)
    int16_t partial;    // OUT_SUM_EXACT: 1 = decimal SUM partial (overflow -> NULL without an
                        // error, empty -> 0, not NULL); 2 = decimal AVG partial sum (overflow ->
                        // NULL or an error, empty -> 0)
    int16_t sumPrec;    // OUT_AVG_DEC: precision and scale of the summed values' decimal type
    int16_t sumScale;
    int16_t countSummed;  // 1: countAcc is an ISUM of partial counts (else a NULLS accumulator)
    int16_t pad2[3];
    void *values;       // device output column
    uint8_t *nulls;     // device output null bitmap (zeroed by the host)
};

// Adaptive partial aggregation (HashAggregationOperator::AlignSchema,
// group_aggregation.cpp:1182-1218): every input row becomes a one-row partial result.  One
// descriptor per output column of the partial schema.
enum AlignOp : int16_t {
    ALIGN_COPY = 0,     // the input value and NULL bit (group-by columns)
    ALIGN_INT = 1,      // integer input cast to the output width, NULL bit kept (SUM/MIN/MAX partials)
    ALIGN_DOUBLE = 2,   // input converted to double (or float), NULL bit kept
    ALIGN_ONE = 3,      // 1 (COUNT(*) partial)
    ALIGN_VALID = 4,    // 1 for a non-NULL input, else 0 (COUNT(col) and AVG count partials)
    ALIGN_AVG_SUM = 5,  // the input as double, 0 for NULL, never NULL (AVG sum partial)
};

struct AlignCol {
    int16_t op;
    int16_t input;     // kernel input (-1 for ALIGN_ONE)
    int16_t inKind;    // IN_INT / IN_FLOAT / IN_DOUBLE
    int16_t inWidth;
    int16_t outWidth;
    int16_t pad[3];
};

struct AggExtract {
    AggTable table;
    KeySpec key;
    AccSpec accs[kMaxAccs];
    int32_t nAccs;
    int32_t nOut;
    OutSpec out[kMaxOutCols];
    unsigned long long *outCount;  // rows written
    int32_t overflowAsNull;
    int32_t *error;                // set to 1 on overflow when overflow is an error
    unsigned long long *nAmbiguous;    // groups whose sticky-overflow result is order dependent
    unsigned long long *ambiguousSlots;  // their slot ids (capacity ambiguousCap)
    uint32_t ambiguousCap;
    // Groups resolved by the ordered path: slot -> forced state (per OUT_SUM_EXACT column):
    // 0 = use the exact sum, 1 = overflowed.  nullptr when there are none.
    const uint8_t *forcedOverflow;
};

// ---- join ---------------------------------------------------------------------------------------
// Build side columns are gathered into contiguous HBM arrays.  ARRAY mode indexes a table by
// key - minKey; HASH mode is open addressing on the 64-bit key.  An entry holds either the
// build row (unique keys) or an offset/count pair into a CSR of build rows (duplicates).
enum JoinMode : int32_t { JOIN_ARRAY = 0, JOIN_HASH = 1 };

struct JoinTable {
    int32_t mode;
    int32_t unique;           // 1: entries are rows, 0: entries are (offset << 32 | count)
    int64_t minKey;
    uint64_t range;           // ARRAY: number of entries
    uint64_t capacity;        // HASH: power of two
    const int64_t *arrayEntries;   // ARRAY: entry per key - minKey, -1 = none
    const uint64_t *hashKeys;      // HASH: keys, kEmptyKey = free
    const int64_t *hashEntries;    // HASH: entry per slot
    int64_t sentinelEntry;         // entry of the key equal to kEmptyKey (-1 = none)
    const int32_t *csrRows;        // build rows grouped by key
    int32_t keyWidth;              // probe key width in bytes
    int32_t pad;
    // Unique tables whose build output values fit in 8 bytes and hold no NULLs: those values
    // packed per table slot (ARRAY: key - minKey; HASH: slot; the EMPTY-key row at `capacity`),
    // so the probe fetches them with the entry instead of gathering by build row afterwards.
    const uint64_t *slotPayload;
    // ARRAY tables with a slot payload: bit d set iff slot d holds a build row.
    const uint32_t *slotBits;
};

// What a probe emits per probe row (lookup_join.cpp:330-411 selects one of these from the join
// type and the build side).
enum JoinKind : int32_t {
    JOIN_KIND_INNER = 0,        // one row per match
    JOIN_KIND_PROBE_OUTER = 1,  // one row per match, else one row with NULL build columns
    JOIN_KIND_BUILD_OUTER = 2,  // one row per match, matched build rows marked visited
    JOIN_KIND_FULL = 3,         // PROBE_OUTER rows, matched build rows marked visited
    JOIN_KIND_SEMI = 4,         // the probe row once if it has a match
    JOIN_KIND_ANTI = 5,         // the probe row (NULL build columns) if it has no match
    JOIN_KIND_EXISTENCE = 6,    // every probe row with a BOOLEAN "has a match" column
};

struct JoinOutCol {
    int16_t side;    // 0 = probe column, 1 = build column, 2 = existence flag (1 byte)
    int16_t src;     // probe kernel input index / build column index
    int16_t width;   // bytes; 0 = VARCHAR: the probe writes an 8-byte row handle per output row
                     // (probe: batch << 32 | row, build: build row, -1: NULL) that a second
                     // pass turns into offsets and characters
    int16_t shift;   // side 1 with a slot payload: bit offset of the value in the packed payload
    const void *buildValues;     // side 1: contiguous build column in HBM
    const uint8_t *buildNulls;   // side 1: contiguous build null bitmap (nullptr = no nulls)
    void *values;                // output column
    uint8_t *nulls;              // output null bitmap (nullptr = output has no nulls)
};

// Multi-column (or 16-byte) join keys: the table is keyed by a 64-bit hash of the key tuple and
// every candidate build row is compared column by column before it counts as a match.
constexpr int kMaxJoinKeys = 4;

struct JoinKeyCol {
    int16_t input;             // probe kernel input index
    int16_t width;             // bytes (1, 2, 4, 8 or 16), 0 = VARCHAR; equal on both sides
    int32_t pad;
    const void *buildValues;   // contiguous build key column in HBM (VARCHAR: characters)
    const int64_t *buildOffs;  // VARCHAR: rows + 1 offsets into buildValues
};

// Key columns of one side, for hashing (build: contiguous columns).
struct JoinKeyCols {
    int32_t nKeys;
    int32_t widths[kMaxJoinKeys];       // 0 = VARCHAR
    const void *cols[kMaxJoinKeys];
    const uint8_t *nulls[kMaxJoinKeys];
    const int64_t *offs[kMaxJoinKeys];  // VARCHAR offsets
};

// Multi-column join keys of fixed widths (1-8 bytes each) packed into one 64-bit key: part k of
// a row, its value sign-extended from width[k] bytes, contributes (v - minv[k]) * stride[k].  The
// build's per-part value ranges [minv[k], minv[k] + span[k]) multiply to at most 2^62, so packed
// build keys are non-negative; a probe row with a part outside its range gets key -1, which no
// build row has.  NULL in any part makes the packed key NULL.
struct JoinKeyPack {
    int32_t nParts;
    int32_t outInput;  // probe side: the kernel input whose column the packed keys are written to
    int32_t input[kMaxJoinKeys];
    int32_t width[kMaxJoinKeys];
    int64_t minv[kMaxJoinKeys];
    uint64_t span[kMaxJoinKeys];
    uint64_t stride[kMaxJoinKeys];
};

// Join filter (the LookupJoin filter expression, lookup_join.cpp:175-187,1440-1466) compiled to a
// postfix program over one (probe row, build row) candidate pair.  Values are 64-bit integers or
// doubles with a NULL flag; comparisons and NOT/AND/OR follow SQL three-valued logic, and a pair
// passes when the program leaves TRUE (NULL fails).
enum FilterOp : int16_t {
    FOP_PROBE_COL = 0,  // push probe input `input` (width, dbl)
    FOP_BUILD_COL,      // push build column values/nulls (width, dbl)
    FOP_LITERAL,        // push imm (dbl: double bits), NULL when isNull
    FOP_EQ, FOP_NEQ, FOP_LT, FOP_LTE, FOP_GT, FOP_GTE,
    FOP_AND, FOP_OR, FOP_NOT,
    FOP_IS_NULL, FOP_IS_NOT_NULL,
    // Arithmetic (the reference's math functions, codegen/functions/mathfunctions.cpp): integers
    // wrap at the result width (width 4 or 8), DIV / MOD by zero give NULL, TRY_* give NULL on
    // overflow (TRY_DIV is DIV); doubles (dbl = 1) are IEEE, DIV / MOD by zero give NULL, MOD is
    // fmod.  A NULL operand gives NULL.
    FOP_ADD, FOP_SUB, FOP_MUL, FOP_DIV, FOP_MOD,
    FOP_TRY_ADD, FOP_TRY_SUB, FOP_TRY_MUL, FOP_TRY_DIV,
    // Strings (VARCHAR/CHAR): a string value is a (pointer, byte length) pair; the comparisons
    // above compare two strings byte-wise as unsigned, a proper prefix first
    // (codegen/functions/stringfunctions.cpp StrCompare / StrEquals).
    FOP_PROBE_STR,    // push probe input `input` (characters and int32 offsets of its batch)
    FOP_BUILD_STR,    // push build column: values = characters, offs = int64 offsets, nulls
    FOP_STR_LITERAL,  // push values (device bytes) of length `input`, NULL when isNull
    // substr(str, start[, length]) over UTF-8 code points (stringfunctions.h:215-318): width =
    // 2 or 3 arguments, input bit 0: a negative start before the string keeps the part inside it
    // (INTERCEPT_FROM_BEYOND), bit 1: start 0 means 1 (ZeroStartIndexSupportRule IS_SUPPORT).
    // A NULL argument gives NULL.
    FOP_SUBSTR,
    // Conditionals and sets (codegen/expression_codegen.cpp:352-760), over numbers or strings:
    FOP_IF,        // (cond, then, else): then when cond is TRUE, else otherwise (NULL included)
    FOP_COALESCE,  // (a, b): a unless it is NULL
    FOP_BETWEEN,   // (v, lo, hi): NULL if any is NULL, else lo <= v <= hi (doubles: unordered counts
                   // as <=, the reference's ULE)
    FOP_IN_BEGIN,  // push the IN accumulator (bit 0: a list item equalled the value, bit 1: an item
                   // was NULL) before the value
    FOP_IN_STEP,   // (acc, v, item) -> (acc, v): fold one list item in
    FOP_IN_END,    // (acc, v): TRUE if matched, else NULL if v or an item was NULL, else FALSE
    // String functions that need no result buffer (stringfunctions.cpp:2064-2092, 2801-2944),
    // function in `width` (FilterStrFn); NULL if an argument is NULL unless stated:
    FOP_STRFN,
    // CAST between numbers (codegen/functions/mathfunctions.cpp:24-113, the RoundingRule::DOWN
    // registry): to the width in `width` (wrapping, as static_cast) or to DOUBLE (dbl = 1); a
    // DOUBLE to LONG / INT truncates toward zero, saturating out of range, NaN to 0 (the
    // conversion of the Arm hosts the reference runs on).  NULL stays NULL.
    FOP_CAST,
};
enum FilterStrFn : int16_t {
    SFN_LENGTH = 0,  // (s): code points; imm >= 0: a CHAR column's declared width instead
    SFN_INSTR,       // (s, sub): 1-based code point position of the first occurrence, 0 if none
    SFN_STARTS_WITH, // (s, prefix)
    SFN_ENDS_WITH,   // (s, suffix)
    SFN_CONTAINS,    // (s, sub)
    SFN_GREATEST,    // (a, b): the greater string, NULL only when both are NULL
    SFN_LEAST,       // (a, b): the lesser string, NULL only when both are NULL
};
constexpr int kFilterSubstrNegative = 1;
constexpr int kFilterSubstrZero = 2;
constexpr int kMaxFilterInstrs = 32;
constexpr int kMaxFilterDepth = 8;

struct FilterInstr {
    int16_t op;
    int16_t width;    // column value bytes (1, 2, 4, 8)
    int16_t dbl;      // 1: the value is a double (columns: DOUBLE; literals: imm is double bits)
    int16_t isNull;   // literals: NULL
    int32_t input;    // FOP_PROBE_COL: probe kernel input index
    int32_t payloadShift;  // FOP_BUILD_COL: s + 1 when the column is also a slot-payload field at bit s
    const void *values;    // FOP_BUILD_COL / FOP_BUILD_STR: contiguous build column
    const uint8_t *nulls;  // FOP_BUILD_COL / FOP_BUILD_STR: its NULL bitmap (may be null)
    const int64_t *offs;   // FOP_BUILD_STR: the column's row offsets into values
    int64_t imm;
};

constexpr int kRegionStride = 16;  // counters 128 bytes apart
constexpr int kMaxRegions = 16;

struct ProbeLaunch {
    const BatchDesc *batches;
    const TileDesc *tiles;
    int32_t nTiles;
    int32_t keyInput;     // kernel input index of the probe key
    int32_t keyWidth;
    int32_t nOut;
    JoinTable table;
    JoinOutCol out[kMaxOutCols];
    // The output is cut into nRegions regions of regionCap rows; tile t writes its matches
    // compacted into region t % nRegions, counted by outCount[region * kRegionStride] (matches
    // past regionCap are counted but not written).  Regions spread the output-range atomics
    // over several addresses.
    unsigned long long *outCount;
    int32_t nRegions;
    int32_t singleBatch;  // 1: one batch, tiles t cover its rows [t * kTileRows, ...) in order
    int32_t hostOutput;   // 1: the output columns are pinned host memory (written over the link)
    int32_t deviceKeys;   // 1: every batch's probe key column (and its validity) is device memory
    uint64_t regionCap;
    int32_t countOnly;
    int32_t *error;     // nonzero after the kernel: 7 = a bounded wait for a bulk copy ran out
    long long waitBudget;  // clock64 ticks of a bounded device-side wait
    int32_t joinKind;   // JoinKind
    uint8_t *visited;   // BUILD_OUTER / FULL: one byte per build row, set to 1 when matched
    int32_t nKeyCols;   // > 0: hashed multi-column key (keyInput unused, -1)
    JoinKeyCol keyCols[kMaxJoinKeys];
    int32_t nFilter;    // > 0: candidate pairs must pass the filter program
    FilterInstr filter[kMaxFilterInstrs];
    // nParts > 0: the key is the packed multi-column key; keyInput (= pack.outInput) is a scratch
    // column that LaunchProbe fills with a packing pass unless the kernel packs the parts itself.
    JoinKeyPack pack;
};

}  // namespace omg
