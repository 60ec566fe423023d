// Hash aggregation kernels for sm_103a.
//
// Replaces the row loop of HashAggregationOperator::AddInput / Emplace
// (operator/aggregation/group_aggregation.cpp:320-406,811-890): find-or-insert the group of
// every row, then update its aggregate states (operations_hash_aggregator.h:16-76).
//
// Design:
//  * One persistent grid walks the tile list of many VectorBatches (host-pinned or HBM).
//  * Each CTA keeps a shared-memory pre-aggregation table; a row whose group is found or
//    placed there is updated with shared-memory atomics.  Rows that miss (table full) go to
//    the global open-addressing table with 64-bit atomicCAS insertion and global atomics.
//    At the end each CTA merges its shared table into the global one.
//  * States are exact or order-free: wrapping int64 sums, exact 128/192-bit sums kept as
//    separate positive and negative magnitudes (so Sum|x| is known for the sticky-overflow
//    rule), compensated double sums, and monotone min/max with a read-before-atomic filter.
//  * A row that cannot be placed within `maxProbe` probes is queued, never half-applied; the
//    host grows the table and re-runs the queue.  A shared-table entry that cannot be merged
//    is spilled as a partial record and merged after the growth.
#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "launch.h"
#include "plan.h"

namespace omg {
namespace {

constexpr int kSmemProbe = 8;
constexpr uint64_t kTagLocked = 1;
constexpr int kAggThreads = 512;

// ------------------------------------------------------------------ key handling
struct RowKey {
    uint64_t w[3];  // KEY_SINGLE: w[0] = key; KEY_PACKED: packed words
    uint64_t hash;
    int special;    // -1 normal, kNullSlotOffset / kSentinelSlotOffset for the special groups
};

__device__ __forceinline__ RowKey ReadKey(const KeySpec &ks, const BatchDesc &b, int64_t row, int kind)
{
    RowKey k;
    k.w[0] = k.w[1] = k.w[2] = 0;
    k.special = -1;
    if (kind == KEY_SINGLE) {
        const KeyCol &c = ks.cols[0];
        if (NullRO(b.nulls[c.input], row)) {
            k.special = kNullSlotOffset;
            k.hash = 0;
            return k;
        }
        uint64_t v = static_cast<uint64_t>(SignExtend(LoadBitsRO(b.cols[c.input], row, c.width), c.width));
        k.w[0] = v;
        if (v == kEmptyKey) {
            k.special = kSentinelSlotOffset;
        }
        k.hash = Mix64(v);
        return k;
    }
    uint32_t mask = 0;
    for (int ci = 0; ci < ks.nCols; ++ci) {
        const KeyCol &c = ks.cols[ci];
        if (NullRO(b.nulls[c.input], row)) {
            mask |= 1u << ci;
            continue;
        }
        const int wi = c.byteOffset >> 3;
        const int sh = (c.byteOffset & 7) * 8;
        if (c.width == 16) {
            const uint64_t *p = static_cast<const uint64_t *>(b.cols[c.input]) + 2 * row;
            k.w[wi] = p[0];
            k.w[wi + 1] = p[1];
        } else {
            k.w[wi] |= LoadBitsRO(b.cols[c.input], row, c.width) << sh;
        }
    }
    k.w[ks.maskByte >> 3] |= static_cast<uint64_t>(mask) << ((ks.maskByte & 7) * 8);
    uint64_t h = 0x9e3779b97f4a7c15ull;
    for (int i = 0; i < ks.words; ++i) {
        h = Mix64(h ^ k.w[i]);
    }
    k.hash = h;
    return k;
}

// Published tag of a packed slot: never 0 (free) or 1 (locked).
__device__ __forceinline__ uint64_t PublishedTag(uint64_t hash) { return (hash | 2ull) & ~1ull; }

// ------------------------------------------------------------------ row inputs
// A row's key plus the values and null bits of up to kRegInputs narrow inputs, all loaded up
// front through the read-only path so their latencies overlap.
struct RowIn {
    RowKey k;
    uint64_t v[kRegInputs];  // raw bits, zero-extended
    uint32_t nulls;          // bit i: register input i is NULL
};

template <int kKind>
__device__ __forceinline__ RowIn LoadRow(const AggLaunch &p, const BatchDesc &b, int64_t row)
{
    RowIn in;
    in.k = ReadKey(p.key, b, row, kKind);
    in.nulls = 0;
#pragma unroll
    for (int i = 0; i < kRegInputs; ++i) {
        in.v[i] = 0;
        if (i < p.nRegInputs) {
            const int c = p.regInput[i];
            in.v[i] = LoadBitsRO(b.cols[c], row, p.regWidth[i]);
            in.nulls |= (NullRO(b.nulls[c], row) ? 1u : 0u) << i;
        }
    }
    return in;
}

__device__ __forceinline__ uint64_t CachedBits(const AccSpec &s, const RowIn &in)
{
    uint64_t r = 0;
#pragma unroll
    for (int i = 0; i < kRegInputs; ++i) {
        r = (i == s.reg) ? in.v[i] : r;
    }
    return r;
}

__device__ __forceinline__ int64_t AccInt(const AccSpec &s, const BatchDesc &b, int64_t row, const RowIn &in)
{
    return s.reg >= 0 ? SignExtend(CachedBits(s, in), s.inWidth) : LoadInt(b.cols[s.input], row, s.inWidth);
}

__device__ __forceinline__ double AccDouble(const AccSpec &s, const BatchDesc &b, int64_t row, const RowIn &in)
{
    if (s.reg < 0) {
        return LoadAsDouble(b.cols[s.input], row, s.inKind, s.inWidth);
    }
    const uint64_t bits = CachedBits(s, in);
    if (s.inKind == IN_DOUBLE) {
        return __longlong_as_double(static_cast<long long>(bits));
    }
    if (s.inKind == IN_FLOAT) {
        return static_cast<double>(__int_as_float(static_cast<int>(bits)));
    }
    return static_cast<double>(SignExtend(bits, s.inWidth));
}

__device__ __forceinline__ bool AccNull(const AccSpec &s, const BatchDesc &b, int64_t row, const RowIn &in)
{
    return s.reg >= 0 ? ((in.nulls >> s.reg) & 1u) != 0 : RowIsNull(b.nulls[s.input], row);
}

__device__ __forceinline__ void Red(uint64_t *w, uint64_t v)
{
    if (v != 0) {
        atomicAdd(reinterpret_cast<unsigned long long *>(w), static_cast<unsigned long long>(v));
    }
}

// ------------------------------------------------------------------ VARCHAR min / max
// Order of the strings of dictionary ids a and b of input `input`: bytes compared as unsigned,
// a proper prefix first (std::string_view::compare, as the reference's MIN/MAX of VARCHAR).
__device__ __forceinline__ int CompareDictStrings(const AggLaunch &p, int input, int64_t a, int64_t b)
{
    const int64_t *off = p.strOff[input];
    const uint8_t *chars = p.strChars[input];
    const int64_t la = off[a + 1] - off[a];
    const int64_t lb = off[b + 1] - off[b];
    const uint8_t *x = chars + off[a];
    const uint8_t *y = chars + off[b];
    const int64_t n = la < lb ? la : lb;
    for (int64_t i = 0; i < n; ++i) {
        if (x[i] != y[i]) {
            return x[i] < y[i] ? -1 : 1;
        }
    }
    return la < lb ? -1 : (la > lb ? 1 : 0);
}

// Lock-free min / max of dictionary ids by their strings: a CAS succeeds only with a strictly
// better string, so every retry follows another thread's improvement and the loop ends.
__device__ __forceinline__ void AtomicStrMinMax(const AggLaunch &p, int input, uint64_t *w, int64_t id, bool isMin)
{
    unsigned long long *a = reinterpret_cast<unsigned long long *>(w);
    unsigned long long cur = *reinterpret_cast<volatile unsigned long long *>(a);
    while (true) {
        if (static_cast<int64_t>(cur) >= 0) {
            if (static_cast<int64_t>(cur) == id) {
                return;
            }
            const int c = CompareDictStrings(p, input, id, static_cast<int64_t>(cur));
            if (isMin ? c >= 0 : c <= 0) {
                return;
            }
        }
        const unsigned long long prev = atomicCAS(a, cur, static_cast<unsigned long long>(id));
        if (prev == cur) {
            return;
        }
        cur = prev;
    }
}

// Double sums: the first kPlainSumRows rows of a table slot (by their COUNT_ALL arrival order)
// are added with a plain atomic add, the later ones with the compensated add.  A slot of a
// shared table or of the global table therefore leaves at most kPlainSumRows additions
// uncompensated, whose rounding errors add up to at most kPlainSumRows * 2^-53 * sum|x| (the
// slots of one group hold disjoint rows, so the bound holds for the group too): 7.1e-15 of
// sum|x| for 64.  Shared-table partials are merged compensated.  (2048 plain rows, 2.3e-13,
// measured no faster on the uniform workload: 190.7 us against 182-192 us.)
constexpr unsigned long long kPlainSumRows = 64;

__device__ __forceinline__ void AddDoubleState(uint64_t *w, double x, unsigned long long arrival)
{
    if (arrival < kPlainSumRows) {
        atomicAdd(reinterpret_cast<double *>(w), x);  // result unused: a fire-and-forget add
    } else {
        AtomicAddCompensated(w, x, 0.0);
    }
}

// ------------------------------------------------------------------ decimal128 min / max
// The state is a 16-byte (low, high) word pair; its initial value is +-(10^38 - 1), the
// reference's GetMax<Decimal128> (min_aggregator.h:31-34).
constexpr uint64_t kDec38MaxLo = 687399551400673279ull;
constexpr uint64_t kDec38MaxHi = 5421010862427522170ull;
constexpr uint64_t kDec38MinLo = ~kDec38MaxLo + 1ull;  // two's complement of 10^38 - 1
constexpr uint64_t kDec38MinHi = ~kDec38MaxHi;          // the low word is not zero: no carry

struct alignas(16) Dec128Word {
    unsigned long long lo;
    unsigned long long hi;
};

__device__ __forceinline__ void InitMinMax128(int kind, uint64_t *w)
{
    w[0] = kind == ACC_XMIN ? kDec38MaxLo : kDec38MinLo;
    w[1] = kind == ACC_XMIN ? kDec38MaxHi : kDec38MinHi;
}

__device__ __forceinline__ bool IsInitMinMax128(int kind, const uint64_t *w)
{
    return kind == ACC_XMIN ? (w[0] == kDec38MaxLo && w[1] == kDec38MaxHi) : (w[0] == kDec38MinLo && w[1] == kDec38MinHi);
}

// Lock-free 128-bit min / max: the current value is read with a no-op compare-and-swap (one
// atomic 16-byte read), and a CAS installs the value only while it is strictly better, so every
// retry follows another thread's improvement and the loop ends.
__device__ __forceinline__ void AtomicMinMax128(uint64_t *w, uint64_t lo, uint64_t hi, bool isMin)
{
    Dec128Word *a = reinterpret_cast<Dec128Word *>(w);
    Dec128Word val;
    val.lo = lo;
    val.hi = hi;
    Dec128Word cur = atomicCAS(a, val, val);
    while (true) {
        const int64_t vh = static_cast<int64_t>(hi);
        const int64_t ch = static_cast<int64_t>(cur.hi);
        const bool less = vh < ch || (vh == ch && lo < cur.lo);
        const bool greater = vh > ch || (vh == ch && lo > cur.lo);
        if (isMin ? !less : !greater) {
            return;
        }
        const Dec128Word prev = atomicCAS(a, cur, val);
        if (prev.lo == cur.lo && prev.hi == cur.hi) {
            return;
        }
        cur = prev;
    }
}

// ------------------------------------------------------------------ state updates
// `st` points at the group's state words, in shared or global memory.
__device__ __forceinline__ void UpdateStates(const AggLaunch &p, const BatchDesc &b, int64_t row, const RowIn &in,
    uint64_t *st)
{
    unsigned long long arrival = kPlainSumRows;  // rows of the slot before this one (COUNT_ALL is accs[0])
    for (int a = 0; a < p.nAccs; ++a) {
        const AccSpec &s = p.accs[a];
        uint64_t *w = st + s.word;
        if (s.kind == ACC_COUNT_ALL) {
            arrival = atomicAdd(reinterpret_cast<unsigned long long *>(w), 1ull);
            continue;
        }
        const bool isNull = AccNull(s, b, row, in);
        if (s.kind == ACC_NULLS) {
            if (isNull) {
                atomicAdd(reinterpret_cast<unsigned long long *>(w), 1ull);
            }
            continue;
        }
        if (isNull) {
            continue;
        }
        switch (s.kind) {
            case ACC_ISUM:
                Red(w, static_cast<uint64_t>(AccInt(s, b, row, in)));
                break;
            case ACC_WSUM2: {
                const int64_t x = AccInt(s, b, row, in);
                const uint64_t m = x >= 0 ? static_cast<uint64_t>(x) : 0ull - static_cast<uint64_t>(x);
                uint64_t *side = x >= 0 ? w : w + 2;
                Red(side, m & 0xffffffffull);
                Red(side + 1, m >> 32);
                break;
            }
            case ACC_WSUM3: {
                const uint64_t *v = static_cast<const uint64_t *>(b.cols[s.input]) + 2 * row;
                uint64_t lo = v[0];
                uint64_t hi = v[1];
                uint64_t *side = w;
                if (static_cast<int64_t>(hi) < 0) {  // magnitude = -(hi:lo)
                    lo = ~lo + 1;
                    hi = ~hi + (lo == 0 ? 1u : 0u);
                    side = w + 4;
                }
                Red(side, lo & 0xffffffffull);
                Red(side + 1, lo >> 32);
                Red(side + 2, hi & 0xffffffffull);
                Red(side + 3, hi >> 32);
                break;
            }
            case ACC_DSUM:
                AddDoubleState(w, AccDouble(s, b, row, in), arrival);
                break;
            case ACC_IMIN:
                AtomicMinI64(w, AccInt(s, b, row, in));
                break;
            case ACC_IMAX:
                AtomicMaxI64(w, AccInt(s, b, row, in));
                break;
            case ACC_DMIN: {
                const double x = AccDouble(s, b, row, in);
                if (!isnan(x)) {
                    AtomicMinI64(w, OrderedFromDouble(x));
                }
                break;
            }
            case ACC_DMAX: {
                const double x = AccDouble(s, b, row, in);
                if (!isnan(x)) {
                    AtomicMaxI64(w, OrderedFromDouble(x));
                }
                break;
            }
            case ACC_SMIN:
            case ACC_SMAX:
                AtomicStrMinMax(p, s.input, w, AccInt(s, b, row, in), s.kind == ACC_SMIN);
                break;
            case ACC_XMIN:
            case ACC_XMAX: {
                const uint64_t *v = static_cast<const uint64_t *>(b.cols[s.input]) + 2 * row;
                AtomicMinMax128(w, v[0], v[1], s.kind == ACC_XMIN);
                break;
            }
            default:
                break;
        }
    }
}

// Merge a partial state (shared table entry or spilled record) into `dst`.
__device__ __forceinline__ void MergeStates(const AggLaunch &p, const AccSpec *accs, int nAccs, const uint64_t *src,
    uint64_t *dst)
{
    for (int a = 0; a < nAccs; ++a) {
        const AccSpec &s = accs[a];
        const uint64_t *v = src + s.word;
        uint64_t *w = dst + s.word;
        switch (s.kind) {
            case ACC_COUNT_ALL:
            case ACC_NULLS:
            case ACC_ISUM:
                if (v[0] != 0) {
                    atomicAdd(reinterpret_cast<unsigned long long *>(w), static_cast<unsigned long long>(v[0]));
                }
                break;
            case ACC_WSUM2:
            case ACC_WSUM3:
                // chunk sums add word by word
                for (int j = 0; j < (s.kind == ACC_WSUM2 ? 4 : 8); ++j) {
                    Red(w + j, v[j]);
                }
                break;
            case ACC_DSUM: {
                double s0 = __longlong_as_double(static_cast<long long>(v[0]));
                double c0 = __longlong_as_double(static_cast<long long>(v[1]));
                if (s0 != 0.0 || c0 != 0.0) {
                    AtomicAddCompensated(w, s0, c0);
                }
                break;
            }
            case ACC_IMIN:
            case ACC_DMIN:
                if (static_cast<int64_t>(v[0]) != s.init) {
                    AtomicMinI64(w, static_cast<int64_t>(v[0]));
                }
                break;
            case ACC_IMAX:
            case ACC_DMAX:
                if (static_cast<int64_t>(v[0]) != s.init) {
                    AtomicMaxI64(w, static_cast<int64_t>(v[0]));
                }
                break;
            case ACC_SMIN:
            case ACC_SMAX:
                if (static_cast<int64_t>(v[0]) >= 0) {
                    AtomicStrMinMax(p, s.input, w, static_cast<int64_t>(v[0]), s.kind == ACC_SMIN);
                }
                break;
            case ACC_XMIN:
            case ACC_XMAX:
                if (!IsInitMinMax128(s.kind, v)) {
                    AtomicMinMax128(w, v[0], v[1], s.kind == ACC_XMIN);
                }
                break;
            default:
                break;
        }
    }
}

__device__ __forceinline__ void InitStates(const AccSpec *accs, int nAccs, int stateWords, uint64_t *st)
{
    for (int i = 0; i < stateWords; ++i) {
        st[i] = 0;
    }
    for (int a = 0; a < nAccs; ++a) {
        st[accs[a].word] = static_cast<uint64_t>(accs[a].init);
        if (accs[a].kind == ACC_XMIN || accs[a].kind == ACC_XMAX) {
            InitMinMax128(accs[a].kind, st + accs[a].word);
        }
    }
}

// ------------------------------------------------------------------ global table
// Returns the slot index or -1 when no slot was found within maxProbe probes.
__device__ __forceinline__ int64_t GlobalFind(const AggTable &t, const KeySpec &ks, const RowKey &k, int maxProbe,
    int32_t *error, bool *inserted, long long waitBudget, int kind)
{
    *inserted = false;
    if (k.special >= 0) {
        const uint64_t slot = t.capacity + static_cast<uint64_t>(k.special);
        if (t.specialUsed[k.special] == 0) {
            atomicExch(&t.specialUsed[k.special], 1u);
        }
        return static_cast<int64_t>(slot);
    }
    const uint64_t mask = t.capacity - 1;
    uint64_t i = k.hash & mask;
    if (kind == KEY_SINGLE) {
        for (int probe = 0; probe < maxProbe; ++probe) {
            unsigned long long *kp = reinterpret_cast<unsigned long long *>(t.slots + i * t.slotWords);
            unsigned long long cur = *reinterpret_cast<volatile unsigned long long *>(kp);
            if (cur == k.w[0]) {
                return static_cast<int64_t>(i);
            }
            if (cur == kEmptyKey) {
                unsigned long long prev = atomicCAS(kp, kEmptyKey, k.w[0]);
                if (prev == kEmptyKey) {
                    *inserted = true;
                    return static_cast<int64_t>(i);
                }
                if (prev == k.w[0]) {
                    return static_cast<int64_t>(i);
                }
            }
            i = (i + 1) & mask;
        }
        return -1;
    }
    const uint64_t tag = PublishedTag(k.hash);
    for (int probe = 0; probe < maxProbe; ++probe) {
        uint64_t *slot = t.slots + i * t.slotWords;
        uint64_t cur = LoadAcquire(slot);
        if (cur == 0) {
            unsigned long long prev =
                atomicCAS(reinterpret_cast<unsigned long long *>(slot), 0ull, static_cast<unsigned long long>(kTagLocked));
            if (prev == 0) {
                for (int j = 0; j < ks.words; ++j) {
                    slot[1 + j] = k.w[j];
                }
                StoreRelease(slot, tag);
                *inserted = true;
                return static_cast<int64_t>(i);
            }
            cur = prev;
        }
        if (cur == kTagLocked) {
            // Another thread is publishing this slot's key: wait a bounded time.
            long long start = clock64();
            while ((cur = LoadAcquire(slot)) == kTagLocked) {
                if (clock64() - start > waitBudget) {
                    SetError(error, 7);
                    return -1;
                }
            }
        }
        if (cur == tag) {
            bool eq = true;
            for (int j = 0; j < ks.words; ++j) {
                eq = eq && (slot[1 + j] == k.w[j]);
            }
            if (eq) {
                return static_cast<int64_t>(i);
            }
        }
        i = (i + 1) & mask;
    }
    return -1;
}

// ------------------------------------------------------------------ shared-memory table
// Same layout as the global table (slotWords words per slot), nSlots slots, no special
// slots (those rows go straight to the global table).  Returns the slot or -1.
__device__ __forceinline__ int SmemFind(uint64_t *sm, int nSlots, int slotWords, const KeySpec &ks, const RowKey &k,
    int kind)
{
    int i = static_cast<int>((static_cast<uint64_t>(static_cast<uint32_t>(k.hash >> 32)) * nSlots) >> 32);
    if (kind == KEY_SINGLE) {
        for (int probe = 0; probe < kSmemProbe; ++probe) {
            unsigned long long *kp = reinterpret_cast<unsigned long long *>(sm + static_cast<int64_t>(i) * slotWords);
            unsigned long long cur = *reinterpret_cast<volatile unsigned long long *>(kp);
            if (cur == k.w[0]) {
                return i;
            }
            if (cur == kEmptyKey) {
                unsigned long long prev = atomicCAS(kp, kEmptyKey, k.w[0]);
                if (prev == kEmptyKey || prev == k.w[0]) {
                    return i;
                }
            }
            if (++i == nSlots) {
                i = 0;
            }
        }
        return -1;
    }
    const uint64_t tag = PublishedTag(k.hash);
    for (int probe = 0; probe < kSmemProbe; ++probe) {
        uint64_t *slot = sm + static_cast<int64_t>(i) * slotWords;
        volatile uint64_t *vs = slot;
        uint64_t cur = vs[0];
        if (cur == 0) {
            unsigned long long prev =
                atomicCAS(reinterpret_cast<unsigned long long *>(slot), 0ull, static_cast<unsigned long long>(kTagLocked));
            if (prev == 0) {
                for (int j = 0; j < ks.words; ++j) {
                    vs[1 + j] = k.w[j];
                }
                __threadfence_block();
                vs[0] = tag;
                return i;
            }
            cur = prev;
        }
        if (cur == kTagLocked) {
            int spins = 0;
            while ((cur = vs[0]) == kTagLocked) {
                if (++spins > (1 << 20)) {
                    return -1;  // give up on the shared table; the row goes global
                }
            }
        }
        if (cur == tag) {
            __threadfence_block();
            bool eq = true;
            for (int j = 0; j < ks.words; ++j) {
                eq = eq && (vs[1 + j] == k.w[j]);
            }
            if (eq) {
                return i;
            }
        }
        if (++i == nSlots) {
            i = 0;
        }
    }
    return -1;
}

__device__ __forceinline__ bool SlotOccupied(const KeySpec &ks, uint64_t firstWord)
{
    return ks.kind == KEY_SINGLE ? firstWord != kEmptyKey : (firstWord != 0 && firstWord != kTagLocked);
}

__device__ __forceinline__ void QueueRetry(const AggLaunch &p, int32_t batch, int64_t row)
{
    unsigned int pos = atomicAdd(p.nRetry, 1u);
    if (pos < p.retryCap) {
        p.retry[pos] = (static_cast<unsigned long long>(batch) << 32) | static_cast<unsigned long long>(row);
    } else {
        SetError(p.error, 4);  // queue overflow: the host sized it for every row, so this is a bug
    }
}

template <int kKind>
__device__ __forceinline__ void ProcessRow(const AggLaunch &p, int32_t batchIdx, const BatchDesc &b, int64_t row,
    const RowIn &in, uint64_t *sm, int smSlots, unsigned int *newGroups)
{
    const int sw = p.table.slotWords;
    const int kw = p.table.keyWords;
    if (smSlots > 0 && in.k.special < 0) {
        int i = SmemFind(sm, smSlots, sw, p.key, in.k, kKind);
        if (i >= 0) {
            UpdateStates(p, b, row, in, sm + static_cast<int64_t>(i) * sw + kw);
            return;
        }
    }
    bool inserted = false;
    int64_t g = GlobalFind(p.table, p.key, in.k, p.maxProbe, p.error, &inserted, p.waitBudget, kKind);
    if (g < 0) {
        QueueRetry(p, batchIdx, row);
        return;
    }
    if (inserted) {
        atomicAdd(newGroups, 1u);
    }
    UpdateStates(p, b, row, in, p.table.slots + g * sw + kw);
}

// Spill records: [key words (keyWords)][state words], slotWords words each.
struct SpillArgs {
    uint64_t *spill;
    unsigned int *nSpill;
    uint32_t spillCap;
    const uint64_t *spillIn;
    uint32_t nSpillIn;
};

template <int kKind>
__device__ __forceinline__ void MergeRecord(const AggLaunch &p, const SpillArgs &sp, const uint64_t *rec,
    unsigned int *newGroups)
{
    const int sw = p.table.slotWords;
    const int kw = p.table.keyWords;
    RowKey k;
    k.special = -1;
    k.w[0] = k.w[1] = k.w[2] = 0;
    if (kKind == KEY_SINGLE) {
        k.w[0] = rec[0];
        k.hash = Mix64(k.w[0]);
    } else {
        uint64_t h = 0x9e3779b97f4a7c15ull;
        for (int i = 0; i < p.key.words; ++i) {
            k.w[i] = rec[1 + i];
            h = Mix64(h ^ k.w[i]);
        }
        k.hash = h;
    }
    bool inserted = false;
    int64_t g = GlobalFind(p.table, p.key, k, p.maxProbe, p.error, &inserted, p.waitBudget, kKind);
    if (g < 0) {
        unsigned int pos = atomicAdd(sp.nSpill, 1u);
        if (pos < sp.spillCap) {
            uint64_t *dst = sp.spill + static_cast<int64_t>(pos) * sw;
            for (int i = 0; i < sw; ++i) {
                dst[i] = rec[i];
            }
        } else {
            SetError(p.error, 4);
        }
        return;
    }
    if (inserted) {
        atomicAdd(newGroups, 1u);
    }
    MergeStates(p, p.accs, p.nAccs, rec + kw, p.table.slots + g * sw + kw);
}

// ------------------------------------------------------------------ partitioned tiles
// Partitioned launches process a tile in two passes.  Pass 1 resolves each of the thread's rows
// to a slot of the CTA's shared table (a row whose group does not fit, or a NULL / EMPTY key,
// goes through the generic global path at once).  Pass 2 walks the accumulators once per tile:
// the accumulator's kind and input width are dispatched once, then applied to the thread's rows,
// so the per-row work is the value load and the shared-memory atomic.
constexpr int kPartRows = kTileRows / 1024;

template <int kW>
__device__ __forceinline__ int64_t LoadIntW(const void *col, int64_t row)
{
    if (kW == 8) {
        return __ldg(static_cast<const long long *>(col) + row);
    } else if (kW == 4) {
        return __ldg(static_cast<const int *>(col) + row);
    } else if (kW == 2) {
        return __ldg(static_cast<const short *>(col) + row);
    } else {
        return static_cast<int64_t>(static_cast<signed char>(__ldg(static_cast<const char *>(col) + row)));
    }
}

// The low 32 bits of a little-endian 64-bit state word.
__device__ __forceinline__ unsigned int *LowWord(uint64_t *w) { return reinterpret_cast<unsigned int *>(w); }

template <int kW>
__device__ __forceinline__ void ApplyIntAcc(const AccSpec &s, const void *col, const uint8_t *nulls, int64_t row0,
    const int (&slot)[kPartRows], uint64_t *sm, int sw)
{
    int64_t x[kPartRows];
    bool ok[kPartRows];
#pragma unroll
    for (int k = 0; k < kPartRows; ++k) {
        const int64_t row = row0 + k * 1024;
        ok[k] = slot[k] >= 0 && !NullRO(nulls, row);
        x[k] = ok[k] ? LoadIntW<kW>(col, row) : 0;
    }
#pragma unroll
    for (int k = 0; k < kPartRows; ++k) {
        if (!ok[k]) {
            continue;
        }
        uint64_t *w = sm + slot[k] * sw + s.word;
        if (s.kind == ACC_ISUM) {
            atomicAdd(reinterpret_cast<unsigned long long *>(w), static_cast<unsigned long long>(x[k]));
        } else if (s.kind == ACC_WSUM2) {
            const uint64_t m = x[k] >= 0 ? static_cast<uint64_t>(x[k]) : 0ull - static_cast<uint64_t>(x[k]);
            uint64_t *side = x[k] >= 0 ? w : w + 2;
            atomicAdd(reinterpret_cast<unsigned long long *>(side), m & 0xffffffffull);
            if ((m >> 32) != 0) {
                atomicAdd(reinterpret_cast<unsigned long long *>(side + 1), m >> 32);
            }
        } else if (s.kind == ACC_IMIN) {
            AtomicMinI64(w, x[k]);
        } else {
            AtomicMaxI64(w, x[k]);
        }
    }
}

template <int kKind>
__device__ __forceinline__ void ProcessPartTile(const AggLaunch &p, int32_t batchIdx, const BatchDesc &b,
    const TileDesc &tile, uint64_t *sm, int smSlots, unsigned int *newGroups)
{
    const int sw = p.table.slotWords;
    const int kw = p.table.keyWords;
    const int64_t row0 = static_cast<int64_t>(tile.row0) + threadIdx.x;
    int slot[kPartRows];  // >= 0: slot index in the shared table, -1: nothing to do in pass 2
    uint32_t arrival[kPartRows];  // the row's COUNT_ALL arrival order in its slot (capped)
#pragma unroll
    for (int k = 0; k < kPartRows; ++k) {
        slot[k] = -1;
        arrival[k] = static_cast<uint32_t>(kPlainSumRows);
        const int r = static_cast<int>(threadIdx.x) + k * 1024;
        if (r < tile.rows) {
            const RowKey key = ReadKey(p.key, b, row0 + k * 1024, kKind);
            const int i = key.special < 0 ? SmemFind(sm, smSlots, sw, p.key, key, kKind) : -1;
            slot[k] = i >= 0 ? i : -2;
        }
    }
    // Rows whose group is not in the shared table: the generic global path.
#pragma unroll 1
    for (int k = 0; k < kPartRows; ++k) {
        if (slot[k] == -2) {
            const int64_t row = row0 + k * 1024;
            ProcessRow<kKind>(p, batchIdx, b, row, LoadRow<kKind>(p, b, row), sm, 0, newGroups);
        }
    }
    uint64_t *st = sm + kw;  // state words of slot i start at st + i * sw
    for (int a = 0; a < p.nAccs; ++a) {
        const AccSpec s = p.accs[a];
        const void *col = s.input >= 0 ? b.cols[s.input] : nullptr;
        const uint8_t *nulls = s.input >= 0 ? b.nulls[s.input] : nullptr;
        switch (s.kind) {
            case ACC_COUNT_ALL:
#pragma unroll
                for (int k = 0; k < kPartRows; ++k) {
                    if (slot[k] >= 0) {
                        // A shared table counts the rows of one launch (< 2^32): a 32-bit add on the
                        // word's low half (little-endian) is exact and faster than a 64-bit one.
                        arrival[k] = static_cast<uint32_t>(min(
                            static_cast<unsigned long long>(atomicAdd(LowWord(st + slot[k] * sw + s.word), 1u)),
                            kPlainSumRows));
                    }
                }
                break;
            case ACC_NULLS:
                if (nulls != nullptr) {
#pragma unroll
                    for (int k = 0; k < kPartRows; ++k) {
                        if (slot[k] >= 0 && NullRO(nulls, row0 + k * 1024)) {
                            atomicAdd(LowWord(st + slot[k] * sw + s.word), 1u);
                        }
                    }
                }
                break;
            case ACC_ISUM:
            case ACC_WSUM2:
            case ACC_IMIN:
            case ACC_IMAX:
                if (s.inWidth == 8) {
                    ApplyIntAcc<8>(s, col, nulls, row0, slot, st, sw);
                } else if (s.inWidth == 4) {
                    ApplyIntAcc<4>(s, col, nulls, row0, slot, st, sw);
                } else if (s.inWidth == 2) {
                    ApplyIntAcc<2>(s, col, nulls, row0, slot, st, sw);
                } else {
                    ApplyIntAcc<1>(s, col, nulls, row0, slot, st, sw);
                }
                break;
            case ACC_DSUM:
            case ACC_DMIN:
            case ACC_DMAX: {
                double x[kPartRows];
                bool ok[kPartRows];
#pragma unroll
                for (int k = 0; k < kPartRows; ++k) {
                    const int64_t row = row0 + k * 1024;
                    ok[k] = slot[k] >= 0 && !NullRO(nulls, row);
                    x[k] = ok[k] ? LoadAsDoubleRO(col, row, s.inKind, s.inWidth) : 0.0;
                }
#pragma unroll
                for (int k = 0; k < kPartRows; ++k) {
                    if (!ok[k]) {
                        continue;
                    }
                    uint64_t *w = st + slot[k] * sw + s.word;
                    if (s.kind == ACC_DSUM) {
                        AddDoubleState(w, x[k], arrival[k]);
                    } else if (!isnan(x[k])) {
                        if (s.kind == ACC_DMIN) {
                            AtomicMinI64(w, OrderedFromDouble(x[k]));
                        } else {
                            AtomicMaxI64(w, OrderedFromDouble(x[k]));
                        }
                    }
                }
                break;
            }
            case ACC_WSUM3:
#pragma unroll
                for (int k = 0; k < kPartRows; ++k) {
                    const int64_t row = row0 + k * 1024;
                    if (slot[k] < 0 || NullRO(nulls, row)) {
                        continue;
                    }
                    const ulonglong2 v = __ldg(static_cast<const ulonglong2 *>(col) + row);
                    uint64_t lo = v.x;
                    uint64_t hi = v.y;
                    uint64_t *side = st + slot[k] * sw + s.word;
                    if (static_cast<int64_t>(hi) < 0) {  // magnitude = -(hi:lo)
                        lo = ~lo + 1;
                        hi = ~hi + (lo == 0 ? 1u : 0u);
                        side += 4;
                    }
                    Red(side, lo & 0xffffffffull);
                    Red(side + 1, lo >> 32);
                    Red(side + 2, hi & 0xffffffffull);
                    Red(side + 3, hi >> 32);
                }
                break;
            case ACC_SMIN:
            case ACC_SMAX:
#pragma unroll
                for (int k = 0; k < kPartRows; ++k) {
                    const int64_t row = row0 + k * 1024;
                    if (slot[k] < 0 || NullRO(nulls, row)) {
                        continue;
                    }
                    AtomicStrMinMax(p, s.input, st + slot[k] * sw + s.word, LoadIntW<4>(col, row), s.kind == ACC_SMIN);
                }
                break;
            case ACC_XMIN:
            case ACC_XMAX:
#pragma unroll
                for (int k = 0; k < kPartRows; ++k) {
                    const int64_t row = row0 + k * 1024;
                    if (slot[k] < 0 || NullRO(nulls, row)) {
                        continue;
                    }
                    const ulonglong2 v = __ldg(static_cast<const ulonglong2 *>(col) + row);
                    AtomicMinMax128(st + slot[k] * sw + s.word, v.x, v.y, s.kind == ACC_XMIN);
                }
                break;
            default:
                break;
        }
    }
}

template <int kKind, bool kPart>
__device__ __forceinline__ void AggBody(const AggLaunch &p, const SpillArgs &sp, uint64_t *smem,
    unsigned int &newGroups)
{
    const int sw = p.table.slotWords;
    const int kw = p.table.keyWords;
    const int smSlots = (p.retryIn == nullptr && sp.spillIn == nullptr) ? p.smemSlots : 0;
    if (threadIdx.x == 0) {
        newGroups = 0;
    }
    for (int i = threadIdx.x; i < smSlots; i += blockDim.x) {
        uint64_t *slot = smem + static_cast<int64_t>(i) * sw;
        slot[0] = (p.key.kind == KEY_SINGLE) ? kEmptyKey : 0ull;
        for (int j = 1; j < kw; ++j) {
            slot[j] = 0;
        }
        InitStates(p.accs, p.nAccs, p.stateWords, slot + kw);
    }
    __syncthreads();

    if (p.retryIn != nullptr || sp.spillIn != nullptr) {
        const int64_t gtid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
        const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
        for (int64_t i = gtid; i < p.nRetryIn; i += stride) {
            unsigned long long e = p.retryIn[i];
            const int32_t bi = static_cast<int32_t>(e >> 32);
            const int64_t row = static_cast<int64_t>(e & 0xffffffffull);
            const BatchDesc &b = p.batches[bi];
            ProcessRow<kKind>(p, bi, b, row, LoadRow<kKind>(p, b, row), smem, 0, &newGroups);
        }
        for (int64_t i = gtid; i < sp.nSpillIn; i += stride) {
            MergeRecord<kKind>(p, sp, sp.spillIn + i * sw, &newGroups);
        }
    } else {
        // Two rows per thread per step: both rows' loads are issued before either is processed.
        int tFirst = blockIdx.x;
        int tEnd = p.nTiles;
        int tStep = gridDim.x;
        if (p.nParts > 0) {  // gridDim.x is a multiple of nParts
            const int q = blockIdx.x % p.nParts;
            tFirst = p.partTileStart[q] + blockIdx.x / p.nParts;
            tEnd = p.partTileStart[q + 1];
            tStep = gridDim.x / p.nParts;
        }
        if (kPart && smSlots > 0) {
            for (int t = tFirst; t < tEnd; t += tStep) {
                const TileDesc tile = p.tiles[t];
                ProcessPartTile<kKind>(p, tile.batch, p.batches[tile.batch], tile, smem, smSlots, &newGroups);
            }
            tEnd = tFirst;  // done
        }
        for (int t = tFirst; t < tEnd; t += tStep) {
            const TileDesc tile = p.tiles[t];
            const BatchDesc &b = p.batches[tile.batch];
            for (int r = threadIdx.x; r < tile.rows; r += 2 * blockDim.x) {
                const int64_t row0 = static_cast<int64_t>(tile.row0) + r;
                const bool second = r + static_cast<int>(blockDim.x) < tile.rows;
                const RowIn a = LoadRow<kKind>(p, b, row0);
                RowIn c;
                if (second) {
                    c = LoadRow<kKind>(p, b, row0 + blockDim.x);
                }
                ProcessRow<kKind>(p, tile.batch, b, row0, a, smem, smSlots, &newGroups);
                if (second) {
                    ProcessRow<kKind>(p, tile.batch, b, row0 + blockDim.x, c, smem, smSlots, &newGroups);
                }
            }
        }
    }
    __syncthreads();

    // Merge the shared table into the global table.
    for (int i = threadIdx.x; i < smSlots; i += blockDim.x) {
        const uint64_t *slot = smem + static_cast<int64_t>(i) * sw;
        if (SlotOccupied(p.key, slot[0])) {
            MergeRecord<kKind>(p, sp, slot, &newGroups);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && newGroups != 0) {
        atomicAdd(p.table.groupCount, static_cast<unsigned long long>(newGroups));
    }
}

template <int kKind>
__global__ void __launch_bounds__(kAggThreads, 2) AggKernel(const __grid_constant__ AggLaunch p,
    const __grid_constant__ SpillArgs sp)
{
    extern __shared__ __align__(16) uint64_t smem[];
    __shared__ unsigned int newGroups;
    AggBody<kKind, false>(p, sp, smem, newGroups);
}

// Partitioned launches: one 1024-thread CTA per SM with a shared table of up to
// kPartSmemBytes (the partition's groups).
constexpr int kPartThreads = 1024;
constexpr size_t kPartSmemBytes = 200 * 1024;

template <int kKind>
__global__ void __launch_bounds__(kPartThreads, 1) AggPartKernel(const __grid_constant__ AggLaunch p,
    const __grid_constant__ SpillArgs sp)
{
    extern __shared__ __align__(16) uint64_t smem[];
    __shared__ unsigned int newGroups;
    AggBody<kKind, true>(p, sp, smem, newGroups);
}

// ------------------------------------------------------------------ table maintenance
__global__ void InitTableKernel(AggTable t, int keyKind, const __grid_constant__ AggLaunch p)
{
    const uint64_t n = t.capacity + 2;
    for (uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; s < n;
         s += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint64_t *slot = t.slots + s * t.slotWords;
        slot[0] = (keyKind == KEY_SINGLE) ? kEmptyKey : 0ull;
        for (int j = 1; j < t.keyWords; ++j) {
            slot[j] = 0;
        }
        InitStates(p.accs, p.nAccs, p.stateWords, slot + t.keyWords);
    }
    if (blockIdx.x == 0 && threadIdx.x < 2) {
        t.specialUsed[threadIdx.x] = 0;
    }
}

// Move every group of `from` into the (initialised, larger) table `to`.
__global__ void RehashKernel(AggTable from, AggTable to, const __grid_constant__ AggLaunch p)
{
    const uint64_t n = from.capacity + 2;
    for (uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; s < n;
         s += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t *src = from.slots + s * from.slotWords;
        uint64_t *dst = nullptr;
        if (s >= from.capacity) {
            const int sp = static_cast<int>(s - from.capacity);
            if (from.specialUsed[sp] == 0) {
                continue;
            }
            to.specialUsed[sp] = 1;
            dst = to.slots + (to.capacity + sp) * to.slotWords;
        } else {
            if (!SlotOccupied(p.key, src[0])) {
                continue;
            }
            RowKey k;
            k.special = -1;
            k.w[0] = k.w[1] = k.w[2] = 0;
            if (p.key.kind == KEY_SINGLE) {
                k.w[0] = src[0];
                k.hash = Mix64(k.w[0]);
            } else {
                uint64_t h = 0x9e3779b97f4a7c15ull;
                for (int i = 0; i < p.key.words; ++i) {
                    k.w[i] = src[1 + i];
                    h = Mix64(h ^ k.w[i]);
                }
                k.hash = h;
            }
            bool inserted = false;
            int64_t g = GlobalFind(to, p.key, k, static_cast<int>(to.capacity < (1ull << 30) ? to.capacity : (1ull << 30)),
                p.error, &inserted, p.waitBudget, p.key.kind);
            if (g < 0) {
                SetError(p.error, 4);
                continue;
            }
            dst = to.slots + g * to.slotWords;
        }
        for (int j = to.keyWords; j < to.slotWords; ++j) {
            dst[j] = src[j];
        }
    }
}

__global__ void CountGroupsKernel(AggTable t, int keyKind, unsigned long long *out)
{
    unsigned int local = 0;
    for (uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; s < t.capacity;
         s += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t w = t.slots[s * t.slotWords];
        local += (keyKind == KEY_SINGLE) ? (w != kEmptyKey) : (w != 0 && w != kTagLocked);
    }
    for (int o = 16; o > 0; o >>= 1) {
        local += __shfl_down_sync(0xffffffffu, local, o);
    }
    if ((threadIdx.x & 31) == 0 && local != 0) {
        atomicAdd(out, static_cast<unsigned long long>(local));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(out, static_cast<unsigned long long>(t.specialUsed[0] + t.specialUsed[1]));
    }
}

// ------------------------------------------------------------------ output extraction
__device__ __forceinline__ void SetOutNull(uint8_t *nulls, uint64_t pos)
{
    atomicOr(reinterpret_cast<unsigned int *>(nulls) + (pos >> 5), 1u << (pos & 31));
}

__device__ __forceinline__ void StoreWidth(void *col, uint64_t pos, int width, uint64_t bits)
{
    switch (width) {
        case 1:
            static_cast<uint8_t *>(col)[pos] = static_cast<uint8_t>(bits);
            break;
        case 2:
            static_cast<uint16_t *>(col)[pos] = static_cast<uint16_t>(bits);
            break;
        case 4:
            static_cast<uint32_t *>(col)[pos] = static_cast<uint32_t>(bits);
            break;
        default:
            static_cast<uint64_t *>(col)[pos] = bits;
            break;
    }
}

// One output column of AlignSchema over the tiles of the input batches (row order kept).
__global__ void AlignColumnKernel(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, const AlignCol c, void *out, uint8_t *outNulls)
{
    for (int t = blockIdx.x; t < nTiles; t += gridDim.x) {
        const TileDesc tile = tiles[t];
        const BatchDesc &b = batches[tile.batch];
        const int64_t out0 = tileOutRow[t];
        const void *col = c.input >= 0 ? b.cols[c.input] : nullptr;
        const uint8_t *nulls = c.input >= 0 ? b.nulls[c.input] : nullptr;
        for (int r = threadIdx.x; r < tile.rows; r += blockDim.x) {
            const int64_t row = static_cast<int64_t>(tile.row0) + r;
            const uint64_t pos = static_cast<uint64_t>(out0 + r);
            const bool isNull = NullRO(nulls, row);
            switch (c.op) {
                case ALIGN_COPY:
                    if (c.inWidth == 16) {
                        static_cast<longlong2 *>(out)[pos] = __ldg(static_cast<const longlong2 *>(col) + row);
                    } else {
                        StoreWidth(out, pos, c.outWidth, LoadBitsRO(col, row, c.inWidth));
                    }
                    break;
                case ALIGN_INT:
                    StoreWidth(out, pos, c.outWidth,
                        static_cast<uint64_t>(SignExtend(LoadBitsRO(col, row, c.inWidth), c.inWidth)));
                    break;
                case ALIGN_DOUBLE: {
                    const double v = LoadAsDoubleRO(col, row, c.inKind, c.inWidth);
                    if (c.outWidth == 4) {
                        static_cast<float *>(out)[pos] = static_cast<float>(v);
                    } else {
                        static_cast<double *>(out)[pos] = v;
                    }
                    break;
                }
                case ALIGN_ONE:
                    static_cast<int64_t *>(out)[pos] = 1;
                    break;
                case ALIGN_VALID:
                    static_cast<int64_t *>(out)[pos] = isNull ? 0 : 1;
                    break;
                default:  // ALIGN_AVG_SUM
                    static_cast<double *>(out)[pos] = isNull ? 0.0 : LoadAsDoubleRO(col, row, c.inKind, c.inWidth);
            }
            if (isNull && outNulls != nullptr) {
                SetOutNull(outNulls, pos);
            }
        }
    }
}

// 10^38 - 1 as a 128-bit unsigned value (type/base_operations.h:20-21).
__device__ __forceinline__ unsigned __int128 Dec38Max()
{
    return (static_cast<unsigned __int128>(5421010862427522170ull) << 64) | 687399551400673279ull;
}

// Decode a WSUM accumulator: exact signed sum (as sign + 192-bit magnitude) and Sum|x|.
struct WideSum {
    bool negative;
    uint64_t mag[3];   // |sum|
    uint64_t abs[3];   // Sum|x| (saturated bit set in abs[2] top bit if it overflowed 192 bits)
};

__device__ __forceinline__ int Cmp192(const uint64_t *a, const uint64_t *b)
{
    for (int i = 2; i >= 0; --i) {
        if (a[i] != b[i]) {
            return a[i] < b[i] ? -1 : 1;
        }
    }
    return 0;
}

__device__ __forceinline__ void Sub192(const uint64_t *a, const uint64_t *b, uint64_t *r)
{
    uint64_t borrow = 0;
    for (int i = 0; i < 3; ++i) {
        uint64_t d = a[i] - b[i];
        uint64_t b1 = a[i] < b[i];
        uint64_t d2 = d - borrow;
        uint64_t b2 = d < borrow;
        r[i] = d2;
        borrow = b1 | b2;
    }
}

__device__ __forceinline__ void Add192(const uint64_t *a, const uint64_t *b, uint64_t *r)
{
    uint64_t carry = 0;
    for (int i = 0; i < 3; ++i) {
        uint64_t s = a[i] + b[i];
        uint64_t c1 = s < a[i];
        uint64_t s2 = s + carry;
        uint64_t c2 = s2 < s;
        r[i] = s2;
        carry = c1 | c2;
    }
}

__device__ __forceinline__ WideSum DecodeWide(const AccSpec &s, const uint64_t *w)
{
    // Side value = sum over k of word_k * 2^(32k) (each word is a sum of 32-bit chunks).
    const int n = s.kind == ACC_WSUM2 ? 2 : 4;
    uint64_t pos[3] = {0, 0, 0};
    uint64_t neg[3] = {0, 0, 0};
    for (int k = 0; k < n; ++k) {
        uint64_t a[3] = {0, 0, 0};
        uint64_t b[3] = {0, 0, 0};
        const int sh = 32 * k;
        const int wi = sh >> 6;
        const int bi = sh & 63;
        a[wi] = w[k] << bi;
        b[wi] = w[n + k] << bi;
        if (bi != 0 && wi + 1 < 3) {
            a[wi + 1] = w[k] >> (64 - bi);
            b[wi + 1] = w[n + k] >> (64 - bi);
        }
        Add192(pos, a, pos);
        Add192(neg, b, neg);
    }
    WideSum r;
    if (Cmp192(pos, neg) >= 0) {
        r.negative = false;
        Sub192(pos, neg, r.mag);
    } else {
        r.negative = true;
        Sub192(neg, pos, r.mag);
    }
    Add192(pos, neg, r.abs);
    return r;
}

// True if magnitude `m` (192-bit) exceeds the bound of the output: int64 range (negative
// sums may reach 2^63) or 10^38 - 1.
__device__ __forceinline__ bool ExceedsBound(const uint64_t *m, bool negative, int boundKind)
{
    if (boundKind == 0) {
        if (m[2] != 0 || m[1] != 0) {
            return true;
        }
        return negative ? (m[0] > 0x8000000000000000ull) : (m[0] > 0x7fffffffffffffffull);
    }
    if (m[2] != 0) {
        return true;
    }
    const unsigned __int128 v = (static_cast<unsigned __int128>(m[1]) << 64) | m[0];
    return v > Dec38Max();
}

// Whether an exact sum's sticky-overflow outcome is an overflow: the total beyond the bound
// always is; a total within it whose sum of magnitudes exceeds the bound depends on the row
// order and is decided by the ordered replay (the slot is queued for it, or its answer read).
__device__ __forceinline__ bool ExactSumOverflowed(const AggExtract &e, const OutSpec &os, const WideSum &ws,
    uint64_t s)
{
    bool overflow = ExceedsBound(ws.mag, ws.negative, os.boundKind);
    if (!overflow && ExceedsBound(ws.abs, false, os.boundKind)) {
        if (e.forcedOverflow != nullptr) {
            overflow = ((e.forcedOverflow[s] >> os.pad) & 1u) != 0;
        } else {
            unsigned long long k = atomicAdd(e.nAmbiguous, 1ull);
            if (k < e.ambiguousCap) {
                e.ambiguousSlots[k] = s;
            }
        }
    }
    return overflow;
}

__device__ __forceinline__ unsigned __int128 Pow10U128(int n)
{
    unsigned __int128 p = 1;
    for (int i = 0; i < n; ++i) {
        p *= 10;
    }
    return p;
}

// Spark's decimal average of a checked sum (magnitude `sum`, the sign applied by the caller)
// over `count` rows (CalcAvg, average_spark_decimal_aggregator.h:477-546): the quotient's scale
// is max(6, sumScale + 21) at precision sumPrec - sumScale + scale, cut back to 38 digits
// keeping the integer digits and at least min(scale, 6) fractional ones; the sum is rescaled to
// it (checked against 10^38 - 1), divided by the count rounding half away from zero, and
// rescaled to the output scale (multiplied, checked, or divided, rounded again).  Magnitudes
// round the same way as the signed values.  False on overflow.
__device__ __forceinline__ bool DecimalAverage(unsigned __int128 sum, uint64_t count, int sumPrec, int sumScale,
    int outScale, unsigned __int128 *out)
{
    int scale = sumScale + 21 > 6 ? sumScale + 21 : 6;
    const int prec = sumPrec - sumScale + scale;
    if (prec > 38) {
        const int intDigits = prec - scale;
        const int minScale = scale < 6 ? scale : 6;
        scale = 38 - intDigits > minScale ? 38 - intDigits : minScale;
    }
    const unsigned __int128 f = Pow10U128(scale - sumScale);
    if (sum != 0 && sum > Dec38Max() / f) {
        return false;
    }
    const unsigned __int128 dividend = sum * f;
    const unsigned __int128 avg = (dividend + count / 2) / count;
    const int diff = outScale - scale;
    if (diff >= 0) {
        const unsigned __int128 g = Pow10U128(diff);
        if (avg != 0 && avg > Dec38Max() / g) {
            return false;
        }
        *out = avg * g;
    } else {
        const unsigned __int128 g = Pow10U128(-diff);
        *out = (avg + g / 2) / g;
    }
    return true;
}

// A zero value at output row `pos` (a 16-byte column holds two words per row).
__device__ __forceinline__ void StoreZero(const OutSpec &os, uint64_t pos)
{
    if (os.outWidth == 16) {
        uint64_t *dst = static_cast<uint64_t *>(os.values) + 2 * pos;
        dst[0] = 0;
        dst[1] = 0;
    } else {
        StoreWidth(os.values, pos, os.outWidth, 0);
    }
}

// Output row `pos` of the group in slot s (occupied) of table t: keys, counts and aggregates.
__device__ __forceinline__ void WriteGroup(const AggExtract &e, const AggTable &t, uint64_t s, const uint64_t *slot,
    uint64_t pos)
{
    const uint64_t *st = slot + t.keyWords;
    const bool nullSlot = (s == t.capacity + kNullSlotOffset);
    const bool sentinelSlot = (s == t.capacity + kSentinelSlotOffset);
    for (int o = 0; o < e.nOut; ++o) {
        const OutSpec &os = e.out[o];
        if (os.kind == OUT_KEY) {
            const KeyCol &kc = e.key.cols[os.src];
            if (e.key.kind == KEY_SINGLE) {
                if (nullSlot) {
                    SetOutNull(os.nulls, pos);
                    StoreWidth(os.values, pos, os.outWidth, 0);
                } else {
                    StoreWidth(os.values, pos, os.outWidth, sentinelSlot ? kEmptyKey : slot[0]);
                }
            } else {
                const uint64_t *kwds = slot + 1;
                const uint32_t mask = static_cast<uint32_t>(
                    (kwds[e.key.maskByte >> 3] >> ((e.key.maskByte & 7) * 8)) & 0xffu);
                const bool isNull = (mask >> os.src) & 1u;
                const int wi = kc.byteOffset >> 3;
                if (kc.width == 16) {
                    uint64_t *dst = static_cast<uint64_t *>(os.values) + 2 * pos;
                    dst[0] = isNull ? 0 : kwds[wi];
                    dst[1] = isNull ? 0 : kwds[wi + 1];
                } else {
                    const int sh = (kc.byteOffset & 7) * 8;
                    uint64_t bits = kwds[wi] >> sh;
                    StoreWidth(os.values, pos, os.outWidth, isNull ? 0 : bits);
                }
                if (isNull) {
                    SetOutNull(os.nulls, pos);
                }
            }
            continue;
        }
        if (os.kind == OUT_COUNT_MERGE) {
            StoreWidth(os.values, pos, 8, st[e.accs[os.src].word]);
            continue;
        }
        // A merging stage's decimal SUM saw a NULL partial sum: that partial overflowed, and the
        // overflow is sticky whatever the row order (sum_spark_decimal_aggregator.h, final stage).
        const bool flagged = os.flagAcc > 0 && st[e.accs[os.flagAcc].word] != 0;
        if (os.kind == OUT_IS_EMPTY) {
            const int64_t n = static_cast<int64_t>(st[e.accs[0].word]) -
                static_cast<int64_t>(st[e.accs[os.countAcc].word]);
            StoreWidth(os.values, pos, 1, (n == 0 && !flagged) ? 1u : 0u);
            continue;
        }
        if (os.kind == OUT_AVG_MERGE || os.kind == OUT_AVG_PARTIAL_SUM) {
            const uint64_t *w = st + e.accs[os.src].word;
            double sum = __dadd_rn(__longlong_as_double(static_cast<long long>(w[0])),
                __longlong_as_double(static_cast<long long>(w[1])));
            if (!isfinite(__longlong_as_double(static_cast<long long>(w[0])))) {
                sum = __longlong_as_double(static_cast<long long>(w[0]));
            }
            int64_t n;
            if (os.kind == OUT_AVG_MERGE || os.boundKind == 1) {
                n = static_cast<int64_t>(st[e.accs[os.countAcc].word]);  // summed partial counts
            } else {
                n = static_cast<int64_t>(st[e.accs[0].word]) - static_cast<int64_t>(st[e.accs[os.countAcc].word]);
            }
            if (n == 0) {
                if (os.kind == OUT_AVG_MERGE) {
                    SetOutNull(os.nulls, pos);
                }
                static_cast<double *>(os.values)[pos] = 0.0;
            } else {
                static_cast<double *>(os.values)[pos] = os.kind == OUT_AVG_MERGE ? sum / static_cast<double>(n) : sum;
            }
            continue;
        }
        int64_t cnt = static_cast<int64_t>(st[e.accs[0].word]);  // accs[0] is COUNT_ALL
        if (os.countAcc >= 0) {
            cnt = os.countSummed ? static_cast<int64_t>(st[e.accs[os.countAcc].word])
                                 : cnt - static_cast<int64_t>(st[e.accs[os.countAcc].word]);
        }
        if (os.kind == OUT_COUNT) {
            StoreWidth(os.values, pos, 8, static_cast<uint64_t>(cnt));
            continue;
        }
        if (flagged || (cnt == 0 && os.partial != 0)) {
            // An overflowed merge: NULL (an error unless overflow is NULL or the output is a
            // partial).  An empty partial sum: 0, not NULL.
            if (flagged) {
                SetOutNull(os.nulls, pos);
                if (!e.overflowAsNull && os.partial != 1) {
                    SetError(e.error, 5);
                }
            }
            StoreZero(os, pos);
            continue;
        }
        if (cnt == 0) {
            SetOutNull(os.nulls, pos);
            StoreZero(os, pos);
            continue;
        }
        const AccSpec &acc = e.accs[os.src];
        const uint64_t *w = st + acc.word;
        switch (os.kind) {
            case OUT_SUM_WRAP:
            case OUT_MIN_INT:
            case OUT_MAX_INT:
            case OUT_STR_ID:  // a dictionary id; the host turns it back into the string
                StoreWidth(os.values, pos, os.outWidth, w[0]);
                break;
            case OUT_MINMAX_DEC128: {
                uint64_t *dst = static_cast<uint64_t *>(os.values) + 2 * pos;
                dst[0] = w[0];
                dst[1] = w[1];
                break;
            }
            case OUT_SUM_DOUBLE:
            case OUT_AVG: {
                double sum = __dadd_rn(__longlong_as_double(static_cast<long long>(w[0])),
                    __longlong_as_double(static_cast<long long>(w[1])));
                if (!isfinite(__longlong_as_double(static_cast<long long>(w[0])))) {
                    sum = __longlong_as_double(static_cast<long long>(w[0]));
                }
                const double v = (os.kind == OUT_AVG) ? sum / static_cast<double>(cnt) : sum;
                static_cast<double *>(os.values)[pos] = v;
                break;
            }
            case OUT_MIN_DOUBLE:
            case OUT_MAX_DOUBLE: {
                const double v = DoubleFromOrdered(static_cast<int64_t>(w[0]));
                if (os.outWidth == 4) {
                    static_cast<float *>(os.values)[pos] = static_cast<float>(v);
                } else {
                    static_cast<double *>(os.values)[pos] = v;
                }
                break;
            }
            case OUT_AVG_DEC: {
                WideSum ws = DecodeWide(acc, w);
                bool overflow = ExactSumOverflowed(e, os, ws, s);
                unsigned __int128 mag = 0;
                if (!overflow) {
                    const unsigned __int128 sum = (static_cast<unsigned __int128>(ws.mag[1]) << 64) | ws.mag[0];
                    overflow = !DecimalAverage(sum, static_cast<uint64_t>(cnt), os.sumPrec, os.sumScale, os.rescalePow,
                        &mag);
                }
                if (overflow) {
                    SetOutNull(os.nulls, pos);
                    if (!e.overflowAsNull) {
                        SetError(e.error, 5);
                    }
                    StoreZero(os, pos);
                    break;
                }
                const unsigned __int128 v = ws.negative ? (~mag + 1) : mag;
                if (os.outWidth == 16) {
                    uint64_t *dst = static_cast<uint64_t *>(os.values) + 2 * pos;
                    dst[0] = static_cast<uint64_t>(v);
                    dst[1] = static_cast<uint64_t>(v >> 64);
                } else {
                    StoreWidth(os.values, pos, os.outWidth, static_cast<uint64_t>(v));  // cut to 64 bits
                }
                break;
            }
            case OUT_SUM_EXACT: {
                WideSum ws = DecodeWide(acc, w);
                bool overflow = ExactSumOverflowed(e, os, ws, s);
                unsigned __int128 mag = (static_cast<unsigned __int128>(ws.mag[1]) << 64) | ws.mag[0];
                if (!overflow && os.rescalePow > 0) {
                    unsigned __int128 f = 1;
                    for (int i = 0; i < os.rescalePow; ++i) {
                        f *= 10;
                    }
                    // |mag| <= 10^38 - 1 < 2^127 and f <= 10^38: check mag * f <= bound.
                    if (mag != 0 && mag > Dec38Max() / f) {
                        overflow = true;
                    } else {
                        mag *= f;
                    }
                }
                if (overflow) {
                    SetOutNull(os.nulls, pos);
                    if (!e.overflowAsNull && os.partial != 1) {
                        SetError(e.error, 5);
                    }
                    mag = 0;
                }
                unsigned __int128 v = ws.negative ? (~mag + 1) : mag;
                if (os.outWidth == 16) {
                    uint64_t *dst = static_cast<uint64_t *>(os.values) + 2 * pos;
                    dst[0] = static_cast<uint64_t>(v);
                    dst[1] = static_cast<uint64_t>(v >> 64);
                } else {
                    StoreWidth(os.values, pos, os.outWidth, static_cast<uint64_t>(v));
                }
                break;
            }
            default:
                break;
        }
    }
}

__global__ void ExtractKernel(const __grid_constant__ AggExtract e)
{
    __shared__ unsigned int warpCounts[32];
    __shared__ unsigned long long blockBase;
    const AggTable &t = e.table;
    const uint64_t nSlots = t.capacity + 2;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nWarps = blockDim.x >> 5;
    for (uint64_t base = static_cast<uint64_t>(blockIdx.x) * blockDim.x; base < nSlots;
         base += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t s = base + threadIdx.x;
        bool occ = false;
        const uint64_t *slot = nullptr;
        if (s < nSlots) {
            slot = t.slots + s * t.slotWords;
            occ = (s >= t.capacity) ? (t.specialUsed[s - t.capacity] != 0) : SlotOccupied(e.key, slot[0]);
        }
        const unsigned int ballot = __ballot_sync(0xffffffffu, occ);
        if (lane == 0) {
            warpCounts[warp] = __popc(ballot);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned int total = 0;
            for (int w = 0; w < nWarps; ++w) {
                unsigned int c = warpCounts[w];
                warpCounts[w] = total;
                total += c;
            }
            blockBase = total ? atomicAdd(e.outCount, static_cast<unsigned long long>(total)) : 0ull;
        }
        __syncthreads();
        if (occ) {
            const uint64_t pos = blockBase + warpCounts[warp] + __popc(ballot & ((1u << lane) - 1u));
            WriteGroup(e, t, s, slot, pos);
        }
        __syncthreads();
    }
}


// ------------------------------------------------------------------ batched tasks
// Many independent aggregations (tasks) in one launch: task i is batch i and owns table
// taskTables[i] inside one slab.  AggTasksKernel walks the tiles of all tasks (tiles of a task are
// adjacent); per-task sketch, count and extraction kernels run one CTA per task.

// Rows per thread per step: their loads and first probes are issued together.
constexpr int kTaskRows = 1;

template <int kKind, int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks) AggTasksKernel(const __grid_constant__ AggLaunch p)
{
    const int sw = p.table.slotWords;
    const int kw = p.table.keyWords;
    for (int t = blockIdx.x; t < p.nTiles; t += gridDim.x) {
        const TileDesc tile = p.tiles[t];
        // A task that already overflowed its table is re-run exactly by the host: skip its rows.
        if (*reinterpret_cast<volatile uint32_t *>(p.taskFailed + tile.batch) != 0u) {
            continue;
        }
        const BatchDesc &b = p.batches[tile.batch];
        const AggTable tab = p.taskTables[tile.batch];
        for (int r0 = threadIdx.x; r0 < tile.rows; r0 += kThreads * kTaskRows) {
            RowIn in[kTaskRows];
            int64_t g[kTaskRows];
#pragma unroll
            for (int k = 0; k < kTaskRows; ++k) {
                const int r = r0 + k * kThreads;
                if (r < tile.rows) {
                    in[k] = LoadRow<kKind>(p, b, static_cast<int64_t>(tile.row0) + r);
                }
            }
#pragma unroll
            for (int k = 0; k < kTaskRows; ++k) {
                g[k] = -2;
                if (r0 + k * kThreads < tile.rows) {
                    bool inserted = false;
                    g[k] = GlobalFind(tab, p.key, in[k].k, p.maxProbe, p.error, &inserted, p.waitBudget, kKind);
                }
            }
#pragma unroll
            for (int k = 0; k < kTaskRows; ++k) {
                if (g[k] == -1) {
                    p.taskFailed[tile.batch] = 1u;
                } else if (g[k] >= 0) {
                    UpdateStates(p, b, static_cast<int64_t>(tile.row0) + r0 + k * kThreads, in[k],
                        tab.slots + g[k] * sw + kw);
                }
            }
        }
    }
}

// Per task: a sketch of up to kTaskSketchRows rows (stratified over the task's rows) in a
// shared-memory table; stats laid out as the operator's sketch (kSketchStats per task).
template <int kKind>
__global__ void __launch_bounds__(256) TaskSketchKernel(const __grid_constant__ AggLaunch p, int32_t nTasks,
    unsigned long long *stats)
{
    __shared__ unsigned long long keys[kTaskSketchSlots];
    __shared__ unsigned int counts[kTaskSketchSlots];
    __shared__ unsigned long long acc[kSketchStats];
    for (int task = blockIdx.x; task < nTasks; task += gridDim.x) {
        for (int i = threadIdx.x; i < kTaskSketchSlots; i += blockDim.x) {
            keys[i] = kEmptyKey;
            counts[i] = 0;
        }
        for (int i = threadIdx.x; i < kSketchStats; i += blockDim.x) {
            acc[i] = 0;
        }
        __syncthreads();
        const BatchDesc &b = p.batches[task];
        const int64_t rows = b.rows;
        const int n = static_cast<int>(rows < kTaskSketchRows ? rows : kTaskSketchRows);
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int64_t row = (static_cast<int64_t>(i) * rows) / n;
            const RowKey k = ReadKey(p.key, b, row, kKind);
            atomicAdd(&acc[0], 1ull);
            if (k.special >= 0) {
                atomicAdd(&acc[1], 1ull);
                continue;
            }
            const unsigned long long h = k.hash == kEmptyKey ? (k.hash ^ 1ull) : k.hash;
            uint32_t j = static_cast<uint32_t>(h) & (kTaskSketchSlots - 1);
            for (int probe = 0; probe < kTaskSketchSlots; ++probe) {
                const unsigned long long prev = atomicCAS(&keys[j], kEmptyKey, h);
                if (prev == kEmptyKey || prev == h) {
                    atomicAdd(&counts[j], 1u);
                    break;
                }
                j = (j + 1) & (kTaskSketchSlots - 1);
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < kTaskSketchSlots; i += blockDim.x) {
            if (keys[i] == kEmptyKey) {
                continue;
            }
            const unsigned int c = counts[i];
            atomicAdd(&acc[2], 1ull);
            if (c == 1) {
                atomicAdd(&acc[3], 1ull);
            } else if (c == 2) {
                atomicAdd(&acc[4], 1ull);
            } else if (c == 3) {
                atomicAdd(&acc[5], 1ull);
            } else if (c < 8) {
                atomicAdd(&acc[6], 1ull);
            } else {
                atomicAdd(&acc[7], 1ull);
                atomicAdd(&acc[9], static_cast<unsigned long long>(c));
            }
            atomicMax(&acc[8], static_cast<unsigned long long>(c));
        }
        __syncthreads();
        for (int i = threadIdx.x; i < kSketchStats; i += blockDim.x) {
            stats[static_cast<int64_t>(task) * kSketchStats + i] = acc[i];
        }
        __syncthreads();
    }
}

// Per task: occupied slots (special slots included).
__global__ void __launch_bounds__(256) TaskCountKernel(const AggTable *tables, int32_t nTasks, int32_t keyKind,
    uint32_t *counts)
{
    __shared__ unsigned int total;
    KeySpec ks;
    ks.kind = keyKind;
    for (int task = blockIdx.x; task < nTasks; task += gridDim.x) {
        if (threadIdx.x == 0) {
            total = 0;
        }
        __syncthreads();
        const AggTable t = tables[task];
        unsigned int mine = 0;
        for (uint64_t s = threadIdx.x; s < t.capacity + 2; s += blockDim.x) {
            const uint64_t *slot = t.slots + s * t.slotWords;
            mine += (s >= t.capacity) ? (t.specialUsed[s - t.capacity] != 0) : SlotOccupied(ks, slot[0]);
        }
        mine = __reduce_add_sync(0xffffffffu, mine);
        if ((threadIdx.x & 31) == 0 && mine != 0) {
            atomicAdd(&total, mine);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            counts[task] = total;
        }
        __syncthreads();
    }
}

// Output region of each task: its group count rounded up to 64 rows, so that every region of the
// shared output columns starts on a byte of their null bitmaps.
__global__ void TaskPadKernel(const uint32_t *groups, int32_t nTasks, uint32_t *padded)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nTasks) {
        padded[t] = (groups[t] + 63u) / 64u * 64u;
    }
}

// Per task: the task's groups written at rows [offsets[task], offsets[task] + count) of the
// output columns, in slot order.
__global__ void __launch_bounds__(256) TaskExtractKernel(const __grid_constant__ AggExtract e, const AggTable *tables,
    int32_t nTasks, const int64_t *offsets)
{
    __shared__ unsigned int warpCounts[8];
    __shared__ unsigned long long running;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    for (int task = blockIdx.x; task < nTasks; task += gridDim.x) {
        const AggTable t = tables[task];
        if (threadIdx.x == 0) {
            running = static_cast<unsigned long long>(offsets[task]);
        }
        __syncthreads();
        const uint64_t nSlots = t.capacity + 2;
        for (uint64_t base = 0; base < nSlots; base += blockDim.x) {
            const uint64_t s = base + threadIdx.x;
            bool occ = false;
            const uint64_t *slot = nullptr;
            if (s < nSlots) {
                slot = t.slots + s * t.slotWords;
                occ = (s >= t.capacity) ? (t.specialUsed[s - t.capacity] != 0) : SlotOccupied(e.key, slot[0]);
            }
            const unsigned int ballot = __ballot_sync(0xffffffffu, occ);
            if (lane == 0) {
                warpCounts[warp] = __popc(ballot);
            }
            __syncthreads();
            unsigned int below = 0, total = 0;
            for (int w = 0; w < (static_cast<int>(blockDim.x) >> 5); ++w) {
                below += w < warp ? warpCounts[w] : 0u;
                total += warpCounts[w];
            }
            if (occ) {
                WriteGroup(e, t, s, slot, running + below + __popc(ballot & ((1u << lane) - 1u)));
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                running += total;
            }
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------------ ordered overflow replay
// For a group whose sticky-overflow outcome depends on row order (|exact sum| within the
// bound but Sum|x| beyond it), the reference marks the sum overflowed as soon as one
// row-ordered prefix leaves the bound (sum_aggregator.h:43-49, sum_spark_decimal_aggregator.h:
// 16-66).  This kernel replays those groups' rows in arrival order (batch, then row) on one
// thread and records, per group and exact-SUM column, whether a prefix left the bound.
// It only runs when such groups exist.
__device__ __forceinline__ int64_t FindSlot(const AggTable &t, const KeySpec &ks, const RowKey &k)
{
    if (k.special >= 0) {
        return static_cast<int64_t>(t.capacity) + k.special;
    }
    const uint64_t mask = t.capacity - 1;
    uint64_t i = k.hash & mask;
    const uint64_t tag = PublishedTag(k.hash);
    for (uint64_t probe = 0; probe < t.capacity; ++probe) {
        const uint64_t *slot = t.slots + i * t.slotWords;
        if (ks.kind == KEY_SINGLE) {
            if (slot[0] == k.w[0]) {
                return static_cast<int64_t>(i);
            }
            if (slot[0] == kEmptyKey) {
                return -1;
            }
        } else {
            if (slot[0] == 0) {
                return -1;
            }
            if (slot[0] == tag) {
                bool eq = true;
                for (int j = 0; j < ks.words; ++j) {
                    eq = eq && (slot[1 + j] == k.w[j]);
                }
                if (eq) {
                    return static_cast<int64_t>(i);
                }
            }
        }
        i = (i + 1) & mask;
    }
    return -1;
}

__global__ void OrderedOverflowKernel(const __grid_constant__ AggLaunch p, int32_t nBatches,
    const __grid_constant__ AggExtract e, const unsigned long long *ambSlots, uint32_t nAmb, int32_t *denseOf,
    uint64_t *prefix, uint8_t *forced)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) {
        return;
    }
    for (uint32_t i = 0; i < nAmb; ++i) {
        denseOf[ambSlots[i]] = static_cast<int32_t>(i);
    }
    for (int32_t bi = 0; bi < nBatches; ++bi) {
        const BatchDesc &b = p.batches[bi];
        for (int64_t row = 0; row < b.rows; ++row) {
            const RowKey k = ReadKey(p.key, b, row, p.key.kind);
            const int64_t slot = FindSlot(p.table, p.key, k);
            if (slot < 0 || denseOf[slot] < 0) {
                continue;
            }
            const int32_t d = denseOf[slot];
            for (int o = 0; o < e.nOut; ++o) {
                const OutSpec &os = e.out[o];
                if (os.kind != OUT_SUM_EXACT && os.kind != OUT_AVG_DEC) {
                    continue;
                }
                const uint8_t bit = static_cast<uint8_t>(1u << os.pad);
                if (forced[slot] & bit) {
                    continue;  // sticky: no further additions once overflowed
                }
                const AccSpec &acc = e.accs[os.src];
                if (RowIsNull(b.nulls[acc.input], row)) {
                    continue;
                }
                uint64_t x0, x1, x2;
                if (acc.kind == ACC_WSUM3) {
                    const uint64_t *v = static_cast<const uint64_t *>(b.cols[acc.input]) + 2 * row;
                    x0 = v[0];
                    x1 = v[1];
                    x2 = (static_cast<int64_t>(x1) < 0) ? ~0ull : 0ull;
                } else {
                    const int64_t v = LoadInt(b.cols[acc.input], row, acc.inWidth);
                    x0 = static_cast<uint64_t>(v);
                    x1 = x2 = (v < 0) ? ~0ull : 0ull;
                }
                uint64_t *pw = prefix + (static_cast<int64_t>(d) * 8 + os.pad) * 3;
                uint64_t a[3] = {pw[0], pw[1], pw[2]};
                uint64_t x[3] = {x0, x1, x2};
                uint64_t r[3];
                Add192(a, x, r);
                pw[0] = r[0];
                pw[1] = r[1];
                pw[2] = r[2];
                const bool neg = static_cast<int64_t>(r[2]) < 0;
                uint64_t mag[3];
                if (neg) {
                    const uint64_t zero[3] = {0, 0, 0};
                    Sub192(zero, r, mag);
                } else {
                    mag[0] = r[0];
                    mag[1] = r[1];
                    mag[2] = r[2];
                }
                if (ExceedsBound(mag, neg, os.boundKind)) {
                    forced[slot] |= bit;
                }
            }
        }
    }
}

// ------------------------------------------------------------------ hash partitioning
__device__ __forceinline__ int PartOf(uint64_t hash, int partBits)
{
    return static_cast<int>((hash >> kPartShift) & ((1u << partBits) - 1u));
}

// Warp-aggregated increment of counter[part]: lanes with the same part elect one leader that adds
// the group's size; returns this lane's rank within its group plus the counter's old value.
__device__ __forceinline__ unsigned int WarpAggAdd(unsigned int *counter, int part, unsigned int active)
{
    const unsigned int peers = __match_any_sync(active, part);
    const int leader = __ffs(peers) - 1;
    const int lane = threadIdx.x & 31;
    unsigned int base = 0;
    if (lane == leader) {
        base = atomicAdd(&counter[part], static_cast<unsigned int>(__popc(peers)));
    }
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

template <int kKind>
__global__ void __launch_bounds__(512) PartHistKernel(const __grid_constant__ AggLaunch p,
    const __grid_constant__ PartArgs a)
{
    __shared__ unsigned int h[kMaxParts];
    const int nParts = 1 << a.partBits;
    for (int i = threadIdx.x; i < nParts; i += blockDim.x) {
        h[i] = 0;
    }
    __syncthreads();
    for (int t = blockIdx.x; t < p.nTiles; t += gridDim.x) {
        const TileDesc tile = p.tiles[t];
        const BatchDesc &b = p.batches[tile.batch];
        // Four rows per thread per step: their key loads are in flight together.
        for (int r0 = 0; r0 < tile.rows; r0 += 4 * static_cast<int>(blockDim.x)) {
            int q[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int r = r0 + j * static_cast<int>(blockDim.x) + static_cast<int>(threadIdx.x);
                q[j] = r < tile.rows ? PartOf(ReadKey(p.key, b, static_cast<int64_t>(tile.row0) + r, kKind).hash,
                                              a.partBits)
                                     : -1;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const unsigned int active = __ballot_sync(0xffffffffu, q[j] >= 0);
                if (q[j] >= 0) {
                    WarpAggAdd(h, q[j], active);
                }
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nParts; i += blockDim.x) {
        if (h[i] != 0) {
            atomicAdd(&a.hist[i], static_cast<unsigned long long>(h[i]));
        }
    }
}

// One block: partition offsets (64-row aligned so every partition's NULL bitmap starts on a
// byte), the cursors, one batch descriptor per partition and the partitions' tiles.
__global__ void PartLayoutKernel(const __grid_constant__ PartArgs a)
{
    __shared__ unsigned long long offset[kMaxParts];
    const int nParts = 1 << a.partBits;
    if (threadIdx.x == 0) {
        unsigned long long off = 0;
        int tiles = 0;
        for (int q = 0; q < nParts; ++q) {
            offset[q] = off;
            a.cursor[q] = off;
            off += (a.hist[q] + 63) / 64 * 64;
            a.partTileStart[q] = tiles;
            tiles += static_cast<int>((a.hist[q] + kTileRows - 1) / kTileRows);
        }
        a.partTileStart[nParts] = tiles;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nParts; q += blockDim.x) {
        BatchDesc d;
        for (int i = 0; i < kMaxInputs; ++i) {
            d.cols[i] = nullptr;
            d.nulls[i] = nullptr;
            d.offs[i] = nullptr;
        }
        for (int i = 0; i < a.nInputs; ++i) {
            d.cols[i] = static_cast<char *>(a.cols[i]) + offset[q] * a.width[i];
            d.nulls[i] = a.nulls[i] != nullptr ? reinterpret_cast<const uint8_t *>(a.nulls[i]) + offset[q] / 8 : nullptr;
        }
        d.rows = static_cast<int64_t>(a.hist[q]);
        d.rowBase = static_cast<int64_t>(offset[q]);
        a.partBatches[q] = d;
        const int first = a.partTileStart[q];
        const int n = a.partTileStart[q + 1] - first;
        for (int k = 0; k < n && first + k < a.maxTiles; ++k) {
            TileDesc td;
            td.batch = q;
            td.row0 = k * kTileRows;
            td.rows = static_cast<int32_t>(min(static_cast<unsigned long long>(kTileRows), a.hist[q] - k * kTileRows));
            td.pad = 0;
            a.partTiles[first + k] = td;
        }
    }
}

__device__ __forceinline__ void CopyInput(const void *src, int64_t row, void *dst, uint64_t pos, int width)
{
    switch (width) {
        case 1:
            static_cast<uint8_t *>(dst)[pos] = static_cast<uint8_t>(__ldg(static_cast<const unsigned char *>(src) + row));
            break;
        case 2:
            static_cast<uint16_t *>(dst)[pos] = static_cast<uint16_t>(__ldg(static_cast<const unsigned short *>(src) + row));
            break;
        case 4:
            static_cast<uint32_t *>(dst)[pos] = __ldg(static_cast<const unsigned int *>(src) + row);
            break;
        case 8:
            static_cast<uint64_t *>(dst)[pos] = __ldg(static_cast<const unsigned long long *>(src) + row);
            break;
        default: {
            const ulonglong2 v = __ldg(static_cast<const ulonglong2 *>(src) + row);
            static_cast<ulonglong2 *>(dst)[pos] = v;
            break;
        }
    }
}

// Per tile: partition of every row, one cursor reservation per partition, then each row's
// inputs copied to its partition (rows of a partition from one warp land contiguously).
constexpr int kScatterThreads = 512;
constexpr int kScatterRows = kTileRows / kScatterThreads;

template <int kKind>
__global__ void __launch_bounds__(kScatterThreads) PartScatterKernel(const __grid_constant__ AggLaunch p,
    const __grid_constant__ PartArgs a)
{
    __shared__ unsigned int cnt[kMaxParts];
    __shared__ unsigned long long base[kMaxParts];
    const int nParts = 1 << a.partBits;
    for (int t = blockIdx.x; t < p.nTiles; t += gridDim.x) {
        const TileDesc tile = p.tiles[t];
        const BatchDesc &b = p.batches[tile.batch];
        for (int i = threadIdx.x; i < nParts; i += blockDim.x) {
            cnt[i] = 0;
        }
        __syncthreads();
        uint8_t part[kScatterRows];
#pragma unroll
        for (int j = 0; j < kScatterRows; ++j) {
            const int r = j * kScatterThreads + threadIdx.x;
            const unsigned int active = __ballot_sync(0xffffffffu, r < tile.rows);
            part[j] = 0;
            if (r < tile.rows) {
                const RowKey k = ReadKey(p.key, b, static_cast<int64_t>(tile.row0) + r, kKind);
                part[j] = static_cast<uint8_t>(PartOf(k.hash, a.partBits));
                WarpAggAdd(cnt, part[j], active);
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nParts; i += blockDim.x) {
            base[i] = cnt[i] != 0 ? atomicAdd(&a.cursor[i], static_cast<unsigned long long>(cnt[i])) : 0ull;
            cnt[i] = 0;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kScatterRows; ++j) {
            const int r = j * kScatterThreads + threadIdx.x;
            const unsigned int active = __ballot_sync(0xffffffffu, r < tile.rows);
            if (r < tile.rows) {
                const int q = part[j];
                const uint64_t pos = base[q] + WarpAggAdd(cnt, q, active);
                const int64_t row = static_cast<int64_t>(tile.row0) + r;
                for (int i = 0; i < a.nInputs; ++i) {
                    CopyInput(b.cols[i], row, a.cols[i], pos, a.width[i]);
                    if (a.nulls[i] != nullptr && RowIsNull(b.nulls[i], row)) {
                        atomicOr(&a.nulls[i][pos >> 5], 1u << (pos & 31));
                    }
                }
            }
        }
        __syncthreads();
    }
}

// ---- stable partitioning (order-dependent plans) ----
// Per tile: rows per partition.
template <int kKind>
__global__ void __launch_bounds__(512) PartTileHistKernel(const __grid_constant__ AggLaunch p,
    const __grid_constant__ PartArgs a)
{
    __shared__ unsigned int h[kMaxParts];
    const int nParts = 1 << a.partBits;
    for (int t = blockIdx.x; t < p.nTiles; t += gridDim.x) {
        for (int i = threadIdx.x; i < nParts; i += blockDim.x) {
            h[i] = 0;
        }
        __syncthreads();
        const TileDesc tile = p.tiles[t];
        const BatchDesc &b = p.batches[tile.batch];
        for (int r = threadIdx.x; r < tile.rows; r += blockDim.x) {
            atomicAdd(&h[PartOf(ReadKey(p.key, b, static_cast<int64_t>(tile.row0) + r, kKind).hash, a.partBits)], 1u);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nParts; i += blockDim.x) {
            a.tileHist[static_cast<int64_t>(t) * nParts + i] = h[i];
        }
        __syncthreads();
    }
}

// One block per partition: the exclusive prefix of its per-tile counts in tile order (in place)
// and its total rows.
__global__ void __launch_bounds__(1024) PartTileScanKernel(const __grid_constant__ PartArgs a, int32_t nTiles)
{
    __shared__ unsigned long long warpSum[32];
    __shared__ unsigned long long carry;
    const int q = blockIdx.x;
    const int nParts = 1 << a.partBits;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        carry = 0;
    }
    __syncthreads();
    for (int t0 = 0; t0 < nTiles; t0 += blockDim.x) {
        const int t = t0 + static_cast<int>(threadIdx.x);
        const unsigned long long v = t < nTiles ? a.tileHist[static_cast<int64_t>(t) * nParts + q] : 0ull;
        unsigned long long incl = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xffffffffu, incl, d);
            incl += lane >= d ? u : 0ull;
        }
        if (lane == 31) {
            warpSum[warp] = incl;
        }
        __syncthreads();
        if (warp == 0) {
            const unsigned long long w = lane < static_cast<int>(blockDim.x >> 5) ? warpSum[lane] : 0ull;
            unsigned long long wi = w;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned long long u = __shfl_up_sync(0xffffffffu, wi, d);
                wi += lane >= d ? u : 0ull;
            }
            warpSum[lane] = wi - w;  // exclusive prefix of the warps
        }
        __syncthreads();
        const unsigned long long excl = carry + warpSum[warp] + incl - v;
        if (t < nTiles) {
            a.tileHist[static_cast<int64_t>(t) * nParts + q] = static_cast<unsigned int>(excl);
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) {
            carry = excl + v;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.hist[q] = carry;
    }
}

// Per tile: each row to its partition at the tile's offset there plus its rank among the tile's
// earlier rows of that partition (rounds in order; within a round, warps in order, then lanes).
template <int kKind>
__global__ void __launch_bounds__(kScatterThreads) PartScatterStableKernel(const __grid_constant__ AggLaunch p,
    const __grid_constant__ PartArgs a)
{
    constexpr int kWarps = kScatterThreads / 32;
    __shared__ unsigned int warpCnt[kWarps][kMaxParts];  // counts, then exclusive prefixes over warps
    __shared__ unsigned int roundTotal[kMaxParts];
    __shared__ unsigned long long running[kMaxParts];
    const int nParts = 1 << a.partBits;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const unsigned int below = (1u << lane) - 1u;
    for (int t = blockIdx.x; t < p.nTiles; t += gridDim.x) {
        const TileDesc tile = p.tiles[t];
        const BatchDesc &b = p.batches[tile.batch];
        for (int i = threadIdx.x; i < nParts; i += blockDim.x) {
            running[i] = a.cursor[i] + a.tileHist[static_cast<int64_t>(t) * nParts + i];
        }
        for (int j = 0; j < kScatterRows; ++j) {
            for (int i = threadIdx.x; i < kWarps * kMaxParts; i += blockDim.x) {
                warpCnt[i / kMaxParts][i % kMaxParts] = 0;
            }
            __syncthreads();
            const int r = j * kScatterThreads + static_cast<int>(threadIdx.x);
            const bool live = r < tile.rows;
            const unsigned int active = __ballot_sync(0xffffffffu, live);
            int q = 0;
            unsigned int peers = 0;
            if (live) {
                q = PartOf(ReadKey(p.key, b, static_cast<int64_t>(tile.row0) + r, kKind).hash, a.partBits);
                peers = __match_any_sync(active, q);
                if ((peers & below) == 0) {
                    warpCnt[warp][q] = __popc(peers);  // written by the partition's first lane
                }
            }
            __syncthreads();
            for (int i = threadIdx.x; i < nParts; i += blockDim.x) {
                unsigned int acc = 0;
                for (int w = 0; w < kWarps; ++w) {
                    const unsigned int c = warpCnt[w][i];
                    warpCnt[w][i] = acc;
                    acc += c;
                }
                roundTotal[i] = acc;
            }
            __syncthreads();
            if (live) {
                const uint64_t pos = running[q] + warpCnt[warp][q] + __popc(peers & below);
                const int64_t row = static_cast<int64_t>(tile.row0) + r;
                for (int i = 0; i < a.nInputs; ++i) {
                    CopyInput(b.cols[i], row, a.cols[i], pos, a.width[i]);
                    if (a.nulls[i] != nullptr && RowIsNull(b.nulls[i], row)) {
                        atomicOr(&a.nulls[i][pos >> 5], 1u << (pos & 31));
                    }
                }
            }
            __syncthreads();
            for (int i = threadIdx.x; i < nParts; i += blockDim.x) {
                running[i] += roundTotal[i];
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ key sketch
// A sample of the rows, stratified over the tiles of the launch (sample s reads a hashed row of
// tile s * nTiles / nSample), is hashed into an open-addressing table of (hash, count);
// SketchStatsKernel then summarises the counts.
template <int kKind>
__global__ void SketchKernel(const __grid_constant__ AggLaunch p, int32_t nSample, unsigned long long *tabKeys,
    unsigned int *tabCounts, unsigned long long *stats)
{
    const uint32_t mask = kSketchCap - 1;
    unsigned long long seen = 0, special = 0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nSample; s += gridDim.x * blockDim.x) {
        const int t = static_cast<int>((static_cast<int64_t>(s) * p.nTiles) / nSample);
        const TileDesc tile = p.tiles[t];
        if (tile.rows <= 0) {
            continue;
        }
        const int off = static_cast<int>(Mix64(static_cast<uint64_t>(s)) % static_cast<uint64_t>(tile.rows));
        const RowKey k = ReadKey(p.key, p.batches[tile.batch], static_cast<int64_t>(tile.row0) + off, kKind);
        ++seen;
        if (k.special >= 0) {
            ++special;
            continue;
        }
        const unsigned long long h = k.hash == kEmptyKey ? (k.hash ^ 1ull) : k.hash;
        uint32_t i = static_cast<uint32_t>(h) & mask;
        for (int probe = 0; probe < kSketchCap; ++probe) {
            const unsigned long long prev = atomicCAS(&tabKeys[i], kEmptyKey, h);
            if (prev == kEmptyKey || prev == h) {
                atomicAdd(&tabCounts[i], 1u);
                break;
            }
            i = (i + 1) & mask;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        seen += __shfl_down_sync(0xffffffffu, seen, o);
        special += __shfl_down_sync(0xffffffffu, special, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&stats[0], seen);
        if (special != 0) {
            atomicAdd(&stats[1], special);
        }
    }
}

__global__ void SketchInitKernel(unsigned long long *tabKeys, unsigned int *tabCounts, unsigned long long *stats)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kSketchCap; i += gridDim.x * blockDim.x) {
        tabKeys[i] = kEmptyKey;
        tabCounts[i] = 0;
        if (i < kSketchStats) {
            stats[i] = 0;
        }
    }
}

__global__ void SketchStatsKernel(const unsigned long long *tabKeys, const unsigned int *tabCounts,
    unsigned long long *stats)
{
    unsigned long long v[7] = {0, 0, 0, 0, 0, 0, 0};  // d, f1, f2, f3, f4-7, f8+, heavy rows
    unsigned long long mx = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kSketchCap; i += gridDim.x * blockDim.x) {
        if (tabKeys[i] == kEmptyKey) {
            continue;
        }
        const unsigned int c = tabCounts[i];
        v[0] += 1;
        v[1] += c == 1;
        v[2] += c == 2;
        v[3] += c == 3;
        v[4] += (c >= 4 && c < 8);
        v[5] += c >= 8;
        v[6] += c >= 8 ? c : 0;
        mx = c > mx ? c : mx;
    }
#pragma unroll
    for (int j = 0; j < 7; ++j) {
        for (int o = 16; o > 0; o >>= 1) {
            v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long om = __shfl_down_sync(0xffffffffu, mx, o);
        mx = om > mx ? om : mx;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&stats[2], v[0]);
        atomicAdd(&stats[3], v[1]);
        atomicAdd(&stats[4], v[2]);
        atomicAdd(&stats[5], v[3]);
        atomicAdd(&stats[6], v[4]);
        atomicAdd(&stats[7], v[5]);
        atomicMax(&stats[8], mx);
        atomicAdd(&stats[9], v[6]);
    }
}

int NumSMs() { return DeviceSMCount(); }

}  // namespace

cudaError_t LaunchAggInitTable(const AggLaunch &p, cudaStream_t stream)
{
    const uint64_t n = p.table.capacity + 2;
    const int threads = 256;
    uint64_t blocks = (n + threads - 1) / threads;
    const uint64_t maxBlocks = static_cast<uint64_t>(NumSMs()) * 16;
    if (blocks > maxBlocks) {
        blocks = maxBlocks;
    }
    InitTableKernel<<<static_cast<unsigned>(blocks), threads, 0, stream>>>(p.table, p.key.kind, p);
    return cudaGetLastError();
}

cudaError_t LaunchAggRehash(const AggLaunch &p, const AggTable &from, const AggTable &to, cudaStream_t stream)
{
    const uint64_t n = from.capacity + 2;
    const int threads = 256;
    uint64_t blocks = (n + threads - 1) / threads;
    const uint64_t maxBlocks = static_cast<uint64_t>(NumSMs()) * 16;
    if (blocks > maxBlocks) {
        blocks = maxBlocks;
    }
    RehashKernel<<<static_cast<unsigned>(blocks), threads, 0, stream>>>(from, to, p);
    return cudaGetLastError();
}

cudaError_t LaunchAgg(const AggLaunch &p, uint64_t *spill, unsigned int *nSpill, uint32_t spillCap,
    const uint64_t *spillIn, uint32_t nSpillIn, int gridBlocks, cudaStream_t stream)
{
    SpillArgs sp{spill, nSpill, spillCap, spillIn, nSpillIn};
    const size_t smemBytes = static_cast<size_t>(p.smemSlots) * p.table.slotWords * sizeof(uint64_t);
    if (p.nParts > 0) {
        if (smemBytes > kPartSmemBytes) {
            return cudaErrorInvalidValue;
        }
        auto pk = p.key.kind == KEY_SINGLE ? AggPartKernel<KEY_SINGLE> : AggPartKernel<KEY_PACKED>;
        cudaError_t err = EnsureDynamicSmem(reinterpret_cast<const void *>(pk), kPartSmemBytes);
        if (err != cudaSuccess) {
            return err;
        }
        const int perPart = NumSMs() / p.nParts > 0 ? NumSMs() / p.nParts : 1;
        pk<<<perPart * p.nParts, kPartThreads, smemBytes, stream>>>(p, sp);
        return cudaGetLastError();
    }
    auto kernel = p.key.kind == KEY_SINGLE ? AggKernel<KEY_SINGLE> : AggKernel<KEY_PACKED>;
    cudaError_t err = EnsureDynamicSmem(reinterpret_cast<const void *>(kernel), smemBytes);
    if (err != cudaSuccess) {
        return err;
    }
    if (gridBlocks <= 0) {
        gridBlocks = NumSMs() * BlocksPerSM(reinterpret_cast<const void *>(kernel), kAggThreads, smemBytes);
    }
    kernel<<<gridBlocks, kAggThreads, smemBytes, stream>>>(p, sp);
    return cudaGetLastError();
}

cudaError_t LaunchAggCount(const AggTable &t, int keyKind, unsigned long long *out, cudaStream_t stream)
{
    const int threads = 256;
    uint64_t blocks = (t.capacity + threads - 1) / threads;
    const uint64_t maxBlocks = static_cast<uint64_t>(NumSMs()) * 8;
    if (blocks > maxBlocks) {
        blocks = maxBlocks;
    }
    if (blocks == 0) {
        blocks = 1;
    }
    CountGroupsKernel<<<static_cast<unsigned>(blocks), threads, 0, stream>>>(t, keyKind, out);
    return cudaGetLastError();
}

cudaError_t LaunchAggExtract(const AggExtract &e, cudaStream_t stream)
{
    const int threads = 256;
    const uint64_t n = e.table.capacity + 2;
    uint64_t blocks = (n + threads - 1) / threads;
    const uint64_t maxBlocks = static_cast<uint64_t>(NumSMs()) * 8;
    if (blocks > maxBlocks) {
        blocks = maxBlocks;
    }
    ExtractKernel<<<static_cast<unsigned>(blocks), threads, 0, stream>>>(e);
    return cudaGetLastError();
}

cudaError_t LaunchAggOrdered(const AggLaunch &p, int32_t nBatches, const AggExtract &e,
    const unsigned long long *ambSlots, uint32_t nAmb, uint8_t *forced, cudaStream_t stream)
{
    const uint64_t nSlots = p.table.capacity + 2;
    int32_t *denseOf = nullptr;
    uint64_t *prefix = nullptr;
    cudaError_t err = cudaMallocAsync(reinterpret_cast<void **>(&denseOf), nSlots * sizeof(int32_t), stream);
    if (err != cudaSuccess) {
        return err;
    }
    err = cudaMallocAsync(reinterpret_cast<void **>(&prefix), static_cast<size_t>(nAmb) * 8 * 3 * sizeof(uint64_t) + 8,
        stream);
    if (err != cudaSuccess) {
        cudaFreeAsync(denseOf, stream);
        return err;
    }
    cudaMemsetAsync(denseOf, 0xff, nSlots * sizeof(int32_t), stream);
    cudaMemsetAsync(prefix, 0, static_cast<size_t>(nAmb) * 8 * 3 * sizeof(uint64_t) + 8, stream);
    OrderedOverflowKernel<<<1, 1, 0, stream>>>(p, nBatches, e, ambSlots, nAmb, denseOf, prefix, forced);
    err = cudaGetLastError();
    cudaFreeAsync(denseOf, stream);
    cudaFreeAsync(prefix, stream);
    return err;
}

cudaError_t LaunchAggTaskSketch(const AggLaunch &p, int32_t nTasks, unsigned long long *stats, cudaStream_t stream)
{
    if (nTasks <= 0) {
        return cudaSuccess;
    }
    const int grid = nTasks < NumSMs() * 8 ? nTasks : NumSMs() * 8;
    if (p.key.kind == KEY_SINGLE) {
        TaskSketchKernel<KEY_SINGLE><<<grid, 256, 0, stream>>>(p, nTasks, stats);
    } else {
        TaskSketchKernel<KEY_PACKED><<<grid, 256, 0, stream>>>(p, nTasks, stats);
    }
    return cudaGetLastError();
}

namespace {
// Launch shapes the autotuner chooses from: threads per CTA and the CTAs per SM the kernel is
// compiled for (the persistent grid is that many CTAs on every SM).
using TasksKernelFn = void (*)(AggLaunch);
struct TasksVariant {
    int32_t threads;
    int32_t blocksPerSM;
    TasksKernelFn single;
    TasksKernelFn packed;
};
const TasksVariant kTasksVariants[] = {
    {128, 8, AggTasksKernel<KEY_SINGLE, 128, 8>, AggTasksKernel<KEY_PACKED, 128, 8>},
    {256, 4, AggTasksKernel<KEY_SINGLE, 256, 4>, AggTasksKernel<KEY_PACKED, 256, 4>},
    {512, 2, AggTasksKernel<KEY_SINGLE, 512, 2>, AggTasksKernel<KEY_PACKED, 512, 2>},
    {1024, 1, AggTasksKernel<KEY_SINGLE, 1024, 1>, AggTasksKernel<KEY_PACKED, 1024, 1>},
};
}  // namespace

int32_t AggTasksVariants() { return static_cast<int32_t>(sizeof(kTasksVariants) / sizeof(kTasksVariants[0])); }

void AggTasksVariantShape(int32_t v, int32_t *threads, int32_t *blocksPerSM)
{
    *threads = kTasksVariants[v].threads;
    *blocksPerSM = kTasksVariants[v].blocksPerSM;
}

cudaError_t LaunchAggTasks(const AggLaunch &p, int32_t variant, cudaStream_t stream)
{
    if (p.nTiles <= 0) {
        return cudaSuccess;
    }
    if (variant < 0 || variant >= AggTasksVariants()) {
        return cudaErrorInvalidValue;
    }
    const TasksVariant &v = kTasksVariants[variant];
    int perSM = BlocksPerSM(reinterpret_cast<const void *>(p.key.kind == KEY_SINGLE ? v.single : v.packed), v.threads, 0);
    perSM = perSM > v.blocksPerSM ? v.blocksPerSM : perSM;
    int grid = NumSMs() * perSM;
    if (grid > p.nTiles) {
        grid = p.nTiles;
    }
    (p.key.kind == KEY_SINGLE ? v.single : v.packed)<<<grid, v.threads, 0, stream>>>(p);
    return cudaGetLastError();
}

cudaError_t LaunchAggTaskCount(const AggTable *tables, int32_t nTasks, int32_t keyKind, uint32_t *counts,
    cudaStream_t stream)
{
    if (nTasks <= 0) {
        return cudaSuccess;
    }
    const int grid = nTasks < NumSMs() * 8 ? nTasks : NumSMs() * 8;
    TaskCountKernel<<<grid, 256, 0, stream>>>(tables, nTasks, keyKind, counts);
    return cudaGetLastError();
}

cudaError_t LaunchAggTaskPad(const uint32_t *groups, int32_t nTasks, uint32_t *padded, cudaStream_t stream)
{
    if (nTasks <= 0) {
        return cudaSuccess;
    }
    TaskPadKernel<<<(nTasks + 255) / 256, 256, 0, stream>>>(groups, nTasks, padded);
    return cudaGetLastError();
}

cudaError_t LaunchAggTaskExtract(const AggExtract &e, const AggTable *tables, int32_t nTasks, const int64_t *offsets,
    cudaStream_t stream)
{
    if (nTasks <= 0) {
        return cudaSuccess;
    }
    const int grid = nTasks < NumSMs() * 8 ? nTasks : NumSMs() * 8;
    TaskExtractKernel<<<grid, 256, 0, stream>>>(e, tables, nTasks, offsets);
    return cudaGetLastError();
}

int32_t AggPartSmemSlots(int32_t slotWords)
{
    return static_cast<int32_t>(kPartSmemBytes / (static_cast<size_t>(slotWords) * sizeof(uint64_t)));
}

cudaError_t LaunchAggPartition(const AggLaunch &p, const PartArgs &a, cudaStream_t stream)
{
    if (p.nTiles <= 0) {
        return cudaSuccess;
    }
    const int grid = p.nTiles < NumSMs() * 4 ? p.nTiles : NumSMs() * 4;
    if (a.stable) {
        // Per-tile counts, their prefixes in tile order, the layout, then the ordered scatter.
        if (p.key.kind == KEY_SINGLE) {
            PartTileHistKernel<KEY_SINGLE><<<grid, 512, 0, stream>>>(p, a);
        } else {
            PartTileHistKernel<KEY_PACKED><<<grid, 512, 0, stream>>>(p, a);
        }
        PartTileScanKernel<<<1 << a.partBits, 1024, 0, stream>>>(a, p.nTiles);
        PartLayoutKernel<<<1, kMaxParts, 0, stream>>>(a);
        if (p.key.kind == KEY_SINGLE) {
            PartScatterStableKernel<KEY_SINGLE><<<grid, kScatterThreads, 0, stream>>>(p, a);
        } else {
            PartScatterStableKernel<KEY_PACKED><<<grid, kScatterThreads, 0, stream>>>(p, a);
        }
        return cudaGetLastError();
    }
    if (p.key.kind == KEY_SINGLE) {
        PartHistKernel<KEY_SINGLE><<<grid, 512, 0, stream>>>(p, a);
    } else {
        PartHistKernel<KEY_PACKED><<<grid, 512, 0, stream>>>(p, a);
    }
    PartLayoutKernel<<<1, kMaxParts, 0, stream>>>(a);
    if (p.key.kind == KEY_SINGLE) {
        PartScatterKernel<KEY_SINGLE><<<grid, kScatterThreads, 0, stream>>>(p, a);
    } else {
        PartScatterKernel<KEY_PACKED><<<grid, kScatterThreads, 0, stream>>>(p, a);
    }
    return cudaGetLastError();
}

cudaError_t LaunchAggSketch(const AggLaunch &p, int32_t nSample, unsigned long long *tabKeys,
    unsigned int *tabCounts, unsigned long long *stats, cudaStream_t stream)
{
    if (p.nTiles <= 0 || nSample <= 0) {
        return cudaSuccess;
    }
    SketchInitKernel<<<64, 256, 0, stream>>>(tabKeys, tabCounts, stats);
    const int blocks = (nSample + 255) / 256;
    if (p.key.kind == KEY_SINGLE) {
        SketchKernel<KEY_SINGLE><<<blocks, 256, 0, stream>>>(p, nSample, tabKeys, tabCounts, stats);
    } else {
        SketchKernel<KEY_PACKED><<<blocks, 256, 0, stream>>>(p, nSample, tabKeys, tabCounts, stats);
    }
    SketchStatsKernel<<<64, 256, 0, stream>>>(tabKeys, tabCounts, stats);
    return cudaGetLastError();
}

// One CTA's registers in shared memory, merged into the global ones with atomicMax.
template <int kKind>
__global__ void __launch_bounds__(512) HllKernel(const __grid_constant__ AggLaunch p, unsigned int *regs)
{
    __shared__ unsigned int r[kHllRegs + 2];
    for (int i = threadIdx.x; i < kHllRegs + 2; i += blockDim.x) {
        r[i] = 0;
    }
    __syncthreads();
    for (int t = blockIdx.x; t < p.nTiles; t += gridDim.x) {
        const TileDesc tile = p.tiles[t];
        const BatchDesc &b = p.batches[tile.batch];
        for (int row = threadIdx.x; row < tile.rows; row += blockDim.x) {
            const RowKey k = ReadKey(p.key, b, static_cast<int64_t>(tile.row0) + row, kKind);
            if (k.special >= 0) {
                r[kHllRegs + k.special] = 1u;
                continue;
            }
            const uint64_t h = Mix64(k.hash ^ 0x5851f42d4c957f2dull);  // bits independent of the table's
            const unsigned int reg = static_cast<unsigned int>(h >> (64 - kHllBits));
            const uint64_t rest = (h << kHllBits) | (1ull << (kHllBits - 1));
            atomicMax(&r[reg], static_cast<unsigned int>(__clzll(static_cast<long long>(rest)) + 1));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kHllRegs + 2; i += blockDim.x) {
        if (r[i] != 0) {
            atomicMax(&regs[i], r[i]);
        }
    }
}

cudaError_t LaunchAggHll(const AggLaunch &p, unsigned int *regs, cudaStream_t stream)
{
    cudaError_t err = cudaMemsetAsync(regs, 0, (kHllRegs + 2) * sizeof(unsigned int), stream);
    if (err != cudaSuccess || p.nTiles <= 0) {
        return err;
    }
    const int grid = p.nTiles < DeviceSMCount() * 2 ? p.nTiles : DeviceSMCount() * 2;
    if (p.key.kind == KEY_SINGLE) {
        HllKernel<KEY_SINGLE><<<grid, 512, 0, stream>>>(p, regs);
    } else {
        HllKernel<KEY_PACKED><<<grid, 512, 0, stream>>>(p, regs);
    }
    return cudaGetLastError();
}

cudaError_t LaunchAlignColumn(const BatchDesc *batches, const TileDesc *tiles, int32_t nTiles,
    const int64_t *tileOutRow, const AlignCol &c, void *out, uint8_t *outNulls, cudaStream_t stream)
{
    if (nTiles <= 0) {
        return cudaSuccess;
    }
    const int grid = nTiles < DeviceSMCount() * 8 ? nTiles : DeviceSMCount() * 8;
    AlignColumnKernel<<<grid, 256, 0, stream>>>(batches, tiles, nTiles, tileOutRow, c, out, outNulls);
    return cudaGetLastError();
}

}  // namespace omg
