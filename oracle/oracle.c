/*
 * oracle.c -- CPU restatement of OmniOperator's hash aggregation and inner hash join,
 * used ONLY as test infrastructure: the parity checker of the GB300 kernels and the timed
 * CPU baseline.  Nothing in the product links or calls this file.
 *
 * It follows the reference's semantics, not its data structures:
 *  - aggregation states are updated row by row in arrival order, exactly as the reference's
 *    AddUseRowIndex / AddConditionalUseRowIndex loops do
 *    (operator/aggregation/aggregator/operations_hash_aggregator.h:16-76);
 *  - SUM of integers under the Spark policy wraps (sum_flatim_aggregator.h:33 with
 *    SumOp<..., CareOverFlow=false>, sum_aggregator.h:49-52); under the generic policy it is
 *    checked with __builtin_add_overflow and sticky (sum_aggregator.h:43-49, count = -1);
 *  - SUM of decimals adds in int128 with AddCheckedOverflow against +-(10^38-1)
 *    (type/base_operations.h:20-28) and is sticky (sum_spark_decimal_aggregator.h:16-66); a
 *    decimal64 result adds in int64 with __builtin_add_overflow; the result is rescaled by
 *    10^(outScale-inScale) with MulCheckedOverflow (sum_spark_decimal_aggregator.h:180-245);
 *  - SUM/AVG of doubles is the naive fold `value += x` (operations_hash_aggregator.h:28-30,
 *    average_flatim_aggregator.h:225-290); AVG of integers converts each value to double first;
 *  - MIN/MAX start at the type's max/lowest and apply std::min/std::max in row order
 *    (min_aggregator.h:16-45, max_aggregator.h:16-45), so NaN inputs never replace the state;
 *  - COUNT(col) counts non-null values, COUNT(*) all rows (count_*_aggregator.h);
 *  - a NULL group-by key is its own group (hashmap/base_hash_map.h:579-589); keys compare by
 *    value bytes (fixed-width handlers and the serialized composite key of
 *    hashmap/column_marshaller.h:27-287, where a NULL column differs from any value);
 *  - inner join: NULL keys never match; every (probe row, build row) pair with equal keys is
 *    emitted (operator/join/lookup_join.cpp:924-1035, join_hash_table_variants.cpp:695-863);
 *  - the other join types follow the probe loops of lookup_join.cpp:1037-1430 and the
 *    unmatched-build-row pass of lookup_outer_join.cpp:173-374 (see orc_join).
 * Output order is not part of the contract (the reference emits in hash-slot order), so the
 * tables here are plain open addressing.  Parity of this file is pinned by the reference's
 * own test vectors (tests/golden/).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef __int128 i128;

enum { T_INT = 1, T_LONG = 2, T_DOUBLE = 3, T_BOOLEAN = 4, T_SHORT = 5, T_DEC64 = 6, T_DEC128 = 7, T_DATE32 = 8,
    T_DATE64 = 9, T_TIMESTAMP = 12, T_BYTE = 18, T_FLOAT = 19 };
enum { F_SUM = 0, F_COUNT_COL = 1, F_COUNT_ALL = 2, F_AVG = 3, F_MAX = 5, F_MIN = 6 };
enum { ST_EMPTY = 0, ST_NORMAL = 1, ST_OVERFLOW = 2 };

static const i128 DEC38_MAX = (((i128)5421010862427522170LL) << 64) + (i128)687399551400673279ULL;

static int64_t load_int(const void *col, int64_t r, int w)
{
    switch (w) {
        case 1: return ((const int8_t *)col)[r];
        case 2: return ((const int16_t *)col)[r];
        case 4: return ((const int32_t *)col)[r];
        default: return ((const int64_t *)col)[r];
    }
}

static int is_int_type(int t)
{
    return t == T_INT || t == T_LONG || t == T_SHORT || t == T_BYTE || t == T_BOOLEAN || t == T_DATE32 ||
        t == T_DATE64 || t == T_TIMESTAMP || t == T_DEC64;
}

static double load_double(const void *col, int64_t r, int t, int w)
{
    if (t == T_DOUBLE) return ((const double *)col)[r];
    if (t == T_FLOAT) return (double)((const float *)col)[r];
    return (double)load_int(col, r, w);
}

/* ---------------------------------------------------------------- group table */
typedef struct {
    int nkey;
    int keybytes;        /* packed key: per column [null byte][width bytes] */
    uint64_t cap;
    uint8_t *keys;       /* cap * keybytes */
    uint8_t *used;
    int64_t *gid;        /* slot -> group id */
    int64_t ngroups;
    int64_t gcap;
    uint8_t *gkeys;      /* group id -> key bytes */
} table_t;

static uint64_t hash_bytes(const uint8_t *p, int n)
{
    uint64_t h = 1469598103934665603ULL;
    for (int i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ULL;
    }
    h ^= h >> 29;
    h *= 0xbf58476d1ce4e5b9ULL;
    h ^= h >> 32;
    return h;
}

static int table_init(table_t *t, int nkey, int keybytes, uint64_t cap)
{
    memset(t, 0, sizeof(*t));
    t->nkey = nkey;
    t->keybytes = keybytes;
    t->cap = cap;
    t->keys = (uint8_t *)malloc(cap * (uint64_t)keybytes);
    t->used = (uint8_t *)calloc(cap, 1);
    t->gid = (int64_t *)malloc(cap * sizeof(int64_t));
    t->gcap = 1024;
    t->gkeys = (uint8_t *)malloc((uint64_t)t->gcap * keybytes);
    return (t->keys && t->used && t->gid && t->gkeys) ? 0 : -1;
}

static void table_free(table_t *t)
{
    free(t->keys);
    free(t->used);
    free(t->gid);
    free(t->gkeys);
}

static int table_grow(table_t *t)
{
    table_t n;
    if (table_init(&n, t->nkey, t->keybytes, t->cap * 2) != 0) return -1;
    for (uint64_t s = 0; s < t->cap; ++s) {
        if (!t->used[s]) continue;
        const uint8_t *k = t->keys + s * (uint64_t)t->keybytes;
        uint64_t i = hash_bytes(k, t->keybytes) & (n.cap - 1);
        while (n.used[i]) i = (i + 1) & (n.cap - 1);
        n.used[i] = 1;
        memcpy(n.keys + i * (uint64_t)n.keybytes, k, t->keybytes);
        n.gid[i] = t->gid[s];
    }
    free(n.gkeys);
    n.gkeys = t->gkeys;
    n.gcap = t->gcap;
    n.ngroups = t->ngroups;
    free(t->keys);
    free(t->used);
    free(t->gid);
    *t = n;
    return 0;
}

/* Returns the group id of the key, inserting it (new id) if absent; -1 on allocation failure. */
static int64_t table_find_insert(table_t *t, const uint8_t *k, int *isnew)
{
    if ((uint64_t)(t->ngroups + 1) * 2 > t->cap && table_grow(t) != 0) return -1;
    uint64_t i = hash_bytes(k, t->keybytes) & (t->cap - 1);
    while (t->used[i]) {
        if (memcmp(t->keys + i * (uint64_t)t->keybytes, k, t->keybytes) == 0) {
            *isnew = 0;
            return t->gid[i];
        }
        i = (i + 1) & (t->cap - 1);
    }
    if (t->ngroups == t->gcap) {
        uint8_t *g = (uint8_t *)realloc(t->gkeys, (uint64_t)t->gcap * 2 * t->keybytes);
        if (!g) return -1;
        t->gkeys = g;
        t->gcap *= 2;
    }
    t->used[i] = 1;
    memcpy(t->keys + i * (uint64_t)t->keybytes, k, t->keybytes);
    t->gid[i] = t->ngroups;
    memcpy(t->gkeys + (uint64_t)t->ngroups * t->keybytes, k, t->keybytes);
    *isnew = 1;
    return t->ngroups++;
}

/* ---------------------------------------------------------------- aggregation */
typedef struct {
    int func, in_type, in_width, out_type, rescale;
    const void *col;
    const uint8_t *nulls; /* byte per row, 1 = null; NULL = no nulls */
    const uint8_t *mask;  /* byte per row, 1 = the row reaches this aggregator; NULL = no mask */
    int in_prec, in_scale, out_scale; /* decimal AVG: input precision / scale, output scale */
} agg_t;

typedef struct {
    /* per group, per aggregator */
    int64_t i64;      /* int sums, min/max, counts */
    i128 wide;        /* decimal sums */
    double d;         /* double sums / min / max */
    int64_t count;    /* non-null count; -1 = sticky overflow (generic int sum) */
    int8_t state;     /* ST_* */
} state_t;

typedef struct {
    int nagg;
    agg_t *aggs;
    int policy; /* 0 spark, 1 generic */
    state_t *st;
    int64_t stcap;
} aggctx_t;

static void state_init(const agg_t *a, state_t *s)
{
    memset(s, 0, sizeof(*s));
    if (a->func == F_MIN || a->func == F_MAX) {
        int w = a->in_width;
        int ow = 8;
        if (a->out_type == T_INT || a->out_type == T_DATE32) ow = 4;
        else if (a->out_type == T_SHORT) ow = 2;
        else if (a->out_type == T_BYTE || a->out_type == T_BOOLEAN) ow = 1;
        (void)w;
        if (a->in_type == T_DOUBLE || a->in_type == T_FLOAT) {
            const double lim = a->in_type == T_FLOAT ? 3.4028234663852886e38 : 1.7976931348623157e308;
            s->d = a->func == F_MIN ? lim : -lim;
        } else if (a->in_type == T_DEC128) {
            /* Decimal128 MIN/MAX start at +-(10^38 - 1) (GetMax<Decimal128>, min_aggregator.h:31-34) */
            s->wide = a->func == F_MIN ? DEC38_MAX : -DEC38_MAX;
        } else {
            int64_t mx = ow == 1 ? INT8_MAX : ow == 2 ? INT16_MAX : ow == 4 ? INT32_MAX : INT64_MAX;
            int64_t mn = ow == 1 ? INT8_MIN : ow == 2 ? INT16_MIN : ow == 4 ? INT32_MIN : INT64_MIN;
            s->i64 = a->func == F_MIN ? mx : mn;
        }
    }
}

static void state_update(const aggctx_t *c, const agg_t *a, state_t *s, int64_t r)
{
    /* A masked aggregator sees only the rows whose mask value is TRUE; a NULL or FALSE mask
     * skips the row (MaskColAggregator::ProcessGroup, mask_column_assistant_aggregator.h:44-53).
     * The row's group exists either way. */
    if (a->mask && !a->mask[r]) return;
    if (a->func == F_COUNT_ALL) {
        s->i64++;
        return;
    }
    if (a->nulls && a->nulls[r]) return;
    switch (a->func) {
        case F_COUNT_COL:
            s->i64++;
            return;
        case F_SUM:
            if (a->in_type == T_DOUBLE || a->in_type == T_FLOAT) {
                s->d += load_double(a->col, r, a->in_type, a->in_width);
                s->state = ST_NORMAL;
            } else if (a->in_type == T_DEC64 || a->in_type == T_DEC128) {
                if (s->state == ST_OVERFLOW) return;
                if (a->out_type == T_DEC128) {
                    i128 x;
                    if (a->in_type == T_DEC128) {
                        const uint64_t *p = (const uint64_t *)a->col + 2 * r;
                        x = (i128)(((unsigned __int128)p[1] << 64) | p[0]);
                    } else {
                        x = (i128)load_int(a->col, r, 8);
                    }
                    i128 res;
                    int ov = __builtin_add_overflow(s->wide, x, &res) || res > DEC38_MAX || res < -DEC38_MAX;
                    s->wide = res;
                    s->state = ov ? ST_OVERFLOW : ST_NORMAL;
                } else {
                    int64_t res;
                    int ov = __builtin_add_overflow(s->i64, load_int(a->col, r, 8), &res);
                    s->i64 = res;
                    s->state = ov ? ST_OVERFLOW : ST_NORMAL;
                }
            } else if (c->policy == 0 || a->in_width != 8) {
                /* Spark policy, or a narrower-than-int64 input under the generic policy (SumOp
                 * checks overflow only for int64 inputs, sum_aggregator.h:36-60): wrap. */
                s->i64 = (int64_t)((uint64_t)s->i64 + (uint64_t)load_int(a->col, r, a->in_width));
                s->state = ST_NORMAL;
            } else {
                if (s->count < 0) return;
                int64_t res;
                if (__builtin_add_overflow(s->i64, load_int(a->col, r, a->in_width), &res)) {
                    s->count = -1;
                } else {
                    s->i64 = res;
                    s->count++;
                }
            }
            return;
        case F_AVG:
            if (a->in_type == T_DEC64 || a->in_type == T_DEC128) {
                /* Spark decimal AVG (AverageSparkDecimalAggregator::UpdateState with SumOp,
                 * average_spark_decimal_aggregator.h:38-49, sum_aggregator.h:13-53): a checked sum,
                 * int64 for a decimal64 result and int128 within +-(10^38 - 1) otherwise; an
                 * overflow makes count -1 and stops the state. */
                if (s->count < 0) return;
                i128 x;
                if (a->in_type == T_DEC128) {
                    const uint64_t *p = (const uint64_t *)a->col + 2 * r;
                    x = (i128)(((unsigned __int128)p[1] << 64) | p[0]);
                } else {
                    x = (i128)load_int(a->col, r, 8);
                }
                if (a->out_type == T_DEC64) {
                    int64_t res;
                    if (__builtin_add_overflow((int64_t)s->wide, (int64_t)x, &res)) {
                        s->count = -1;
                        return;
                    }
                    s->wide = res;
                } else {
                    i128 res;
                    if (__builtin_add_overflow(s->wide, x, &res) || res > DEC38_MAX || res < -DEC38_MAX) {
                        s->count = -1;
                        return;
                    }
                    s->wide = res;
                }
                s->count++;
                return;
            }
            s->d += load_double(a->col, r, a->in_type, a->in_width);
            s->count++;
            return;
        case F_MIN:
        case F_MAX:
            if (a->in_type == T_DOUBLE || a->in_type == T_FLOAT) {
                double x = load_double(a->col, r, a->in_type, a->in_width);
                if (a->func == F_MIN) s->d = (x < s->d) ? x : s->d;
                else s->d = (s->d < x) ? x : s->d;
            } else if (a->in_type == T_DEC128) {
                const uint64_t *p = (const uint64_t *)a->col + 2 * r;
                const i128 x = (i128)(((unsigned __int128)p[1] << 64) | p[0]);
                if (a->func == F_MIN) s->wide = (x < s->wide) ? x : s->wide;
                else s->wide = (s->wide < x) ? x : s->wide;
            } else {
                int64_t x = load_int(a->col, r, a->in_width);
                if (a->func == F_MIN) s->i64 = (x < s->i64) ? x : s->i64;
                else s->i64 = (s->i64 < x) ? x : s->i64;
            }
            s->state = ST_NORMAL;
            return;
    }
}

static i128 pow10_i128(int n)
{
    i128 p = 1;
    for (int i = 0; i < n; ++i) p *= 10;
    return p;
}

/* MulCheckedOverflow (type/base_operations.h:30-35): product beyond +-(10^38 - 1) overflows. */
static int mul_checked(i128 a, i128 b, i128 *r)
{
    return __builtin_mul_overflow(a, b, r) || *r > DEC38_MAX || *r < -DEC38_MAX;
}

/* DivideRoundUp (type/base_operations.h:37-48): half away from zero. */
static i128 divide_round_up(i128 l, i128 r)
{
    i128 t = r / 2;
    if ((l > 0 && r < 0) || (l < 0 && r > 0)) t = -t;
    return (l + t) / r;
}

/*
 * CalcAvg (average_spark_decimal_aggregator.h:477-512) with GetDivideResultDecimalType (:522-546):
 * the quotient's scale is max(6, sumScale + 21) at precision sumPrec - sumScale + scale, cut back
 * to 38 digits keeping the integer digits and at least min(scale, 6) fractional ones; the sum
 * is rescaled to it, divided by the count (rounded half away from zero) and rescaled to the
 * output scale (multiplied, checked, or divided, rounded again).  Returns 1 on overflow.
 */
static int calc_decimal_avg(i128 sum, int64_t count, int sum_prec, int sum_scale, int out_scale, i128 *out)
{
    i128 wider;
    if (mul_checked(sum, pow10_i128((sum_scale > 0 ? sum_scale : 0) - sum_scale), &wider)) return 1;
    int scale = sum_scale + 21 > 6 ? sum_scale + 21 : 6;
    int prec = sum_prec - sum_scale + scale;
    if (prec > 38) {
        const int int_digits = prec - scale;
        const int min_scale = scale < 6 ? scale : 6;
        scale = 38 - int_digits > min_scale ? 38 - int_digits : min_scale;
    }
    i128 dividend;
    int ovf = mul_checked(sum, pow10_i128(scale - sum_scale), &dividend);
    const i128 avg = divide_round_up(dividend, (i128)count);
    const int diff = out_scale - scale;
    if (diff >= 0) {
        ovf = ovf || mul_checked(avg, pow10_i128(diff), out);
    } else {
        *out = divide_round_up(avg, pow10_i128(-diff));
    }
    return ovf;
}

/* Writes the output value of one aggregator; returns 1 if NULL, 2 on an overflow error. */
static int state_extract(const aggctx_t *c, const agg_t *a, const state_t *s, int overflow_as_null, void *out,
    int64_t g)
{
    switch (a->func) {
        case F_COUNT_ALL:
        case F_COUNT_COL:
            ((int64_t *)out)[g] = s->i64;
            return 0;
        case F_AVG:
            if (a->in_type == T_DEC64 || a->in_type == T_DEC128) {
                if (s->count < 0) return overflow_as_null ? 1 : 2;
                if (s->count == 0) return 1;
                /* a single-stage (raw input, final output) AVG sums at precision p + 10 */
                const int sum_prec = a->in_prec + 10 < 38 ? a->in_prec + 10 : 38;
                i128 res;
                if (calc_decimal_avg(s->wide, s->count, sum_prec, a->in_scale, a->out_scale, &res)) {
                    return overflow_as_null ? 1 : 2;
                }
                if (a->out_type == T_DEC128) {
                    uint64_t *o = (uint64_t *)out + 2 * g;
                    o[0] = (uint64_t)res;
                    o[1] = (uint64_t)((unsigned __int128)res >> 64);
                } else {
                    ((int64_t *)out)[g] = (int64_t)res;
                }
                return 0;
            }
            if (s->count == 0) return 1;
            ((double *)out)[g] = s->d / (double)s->count;
            return 0;
        case F_MIN:
        case F_MAX: {
            if (s->state == ST_EMPTY) return 1;
            if (a->in_type == T_DEC128) {
                uint64_t *o = (uint64_t *)out + 2 * g;
                o[0] = (uint64_t)s->wide;
                o[1] = (uint64_t)((unsigned __int128)s->wide >> 64);
                return 0;
            }
            if (a->out_type == T_DOUBLE) ((double *)out)[g] = s->d;
            else if (a->out_type == T_FLOAT) ((float *)out)[g] = (float)s->d;
            else if (a->out_type == T_INT || a->out_type == T_DATE32) ((int32_t *)out)[g] = (int32_t)s->i64;
            else if (a->out_type == T_SHORT) ((int16_t *)out)[g] = (int16_t)s->i64;
            else if (a->out_type == T_BYTE || a->out_type == T_BOOLEAN) ((int8_t *)out)[g] = (int8_t)s->i64;
            else ((int64_t *)out)[g] = s->i64;
            return 0;
        }
        case F_SUM:
            if (a->in_type == T_DOUBLE || a->in_type == T_FLOAT) {
                if (s->state == ST_EMPTY) return 1;
                ((double *)out)[g] = s->d;
                return 0;
            }
            if (a->in_type == T_DEC64 || a->in_type == T_DEC128) {
                if (s->state == ST_EMPTY) return 1;
                if (s->state == ST_OVERFLOW) return overflow_as_null ? 1 : 2;
                i128 v = a->out_type == T_DEC128 ? s->wide : (i128)s->i64;
                i128 res;
                int ov = __builtin_mul_overflow(v, pow10_i128(a->rescale), &res) || res > DEC38_MAX || res < -DEC38_MAX;
                if (ov) return overflow_as_null ? 1 : 2;
                if (a->out_type == T_DEC128) {
                    uint64_t *o = (uint64_t *)out + 2 * g;
                    o[0] = (uint64_t)res;
                    o[1] = (uint64_t)((unsigned __int128)res >> 64);
                } else {
                    ((int64_t *)out)[g] = (int64_t)res;
                }
                return 0;
            }
            if (c->policy == 0 || a->in_width != 8) {
                if (s->state == ST_EMPTY) return 1;
                ((int64_t *)out)[g] = s->i64;
                return 0;
            }
            if (s->count < 0) return overflow_as_null ? 1 : 2;
            if (s->count == 0) return 1;
            ((int64_t *)out)[g] = s->i64;
            return 0;
    }
    return 1;
}

static int pack_key(int nkey, const void **key_cols, const int32_t *key_widths, const uint8_t **key_nulls, int64_t r,
    uint8_t *k)
{
    int off = 0;
    for (int i = 0; i < nkey; ++i) {
        const int w = key_widths[i];
        const int isnull = key_nulls && key_nulls[i] && key_nulls[i][r];
        k[off++] = (uint8_t)isnull;
        if (isnull) memset(k + off, 0, w);
        else memcpy(k + off, (const uint8_t *)key_cols[i] + (int64_t)w * r, w);
        off += w;
    }
    return off;
}

/*
 * Single-stage hash aggregation over `n_rows` rows (all batches concatenated in arrival
 * order).  Outputs are written for up to `max_groups` groups: key columns (values + byte
 * nulls) and one value column per aggregator (16 bytes per row reserved for decimal128).
 * Returns the number of groups, -1 on allocation failure, -2 if an overflow must raise
 * (overflow-as-null off), -3 if max_groups is too small.
 */
int64_t orc_hashagg(int64_t n_rows, int32_t nkey, const void **key_cols, const int32_t *key_widths,
    const uint8_t **key_nulls, int32_t nagg, const int32_t *funcs, const void **agg_cols, const int32_t *in_types,
    const int32_t *in_widths, const uint8_t **agg_nulls, const int32_t *out_types, const int32_t *rescale,
    int32_t policy, int32_t overflow_as_null, int64_t max_groups, void **out_keys, uint8_t **out_key_nulls,
    void **out_vals, uint8_t **out_val_nulls, const uint8_t **agg_masks, const int32_t *dec_params)
{
    int keybytes = 0;
    for (int i = 0; i < nkey; ++i) keybytes += 1 + key_widths[i];
    table_t t;
    if (table_init(&t, nkey, keybytes, 1024) != 0) return -1;
    aggctx_t c;
    c.nagg = nagg;
    c.policy = policy;
    c.aggs = (agg_t *)calloc(nagg > 0 ? nagg : 1, sizeof(agg_t));
    c.stcap = 1024;
    c.st = (state_t *)malloc((uint64_t)c.stcap * (nagg > 0 ? nagg : 1) * sizeof(state_t));
    uint8_t *k = (uint8_t *)malloc(keybytes + 1);
    if (!c.aggs || !c.st || !k) return -1;
    for (int a = 0; a < nagg; ++a) {
        c.aggs[a].func = funcs[a];
        c.aggs[a].col = agg_cols[a];
        c.aggs[a].in_type = in_types[a];
        c.aggs[a].in_width = in_widths[a];
        c.aggs[a].nulls = agg_nulls ? agg_nulls[a] : NULL;
        c.aggs[a].out_type = out_types[a];
        c.aggs[a].rescale = rescale ? rescale[a] : 0;
        c.aggs[a].mask = agg_masks ? agg_masks[a] : NULL;
        if (dec_params) {
            c.aggs[a].in_prec = dec_params[3 * a];
            c.aggs[a].in_scale = dec_params[3 * a + 1];
            c.aggs[a].out_scale = dec_params[3 * a + 2];
        }
    }
    int64_t ret = 0;
    for (int64_t r = 0; r < n_rows; ++r) {
        pack_key(nkey, key_cols, key_widths, key_nulls, r, k);
        int isnew = 0;
        int64_t g = table_find_insert(&t, k, &isnew);
        if (g < 0) { ret = -1; goto done; }
        if (isnew) {
            if (g >= c.stcap) {
                state_t *ns = (state_t *)realloc(c.st, (uint64_t)c.stcap * 2 * (nagg > 0 ? nagg : 1) * sizeof(state_t));
                if (!ns) { ret = -1; goto done; }
                c.st = ns;
                c.stcap *= 2;
            }
            for (int a = 0; a < nagg; ++a) state_init(&c.aggs[a], &c.st[g * nagg + a]);
        }
        for (int a = 0; a < nagg; ++a) state_update(&c, &c.aggs[a], &c.st[g * nagg + a], r);
    }
    if (t.ngroups > max_groups) { ret = -3; goto done; }
    for (int64_t g = 0; g < t.ngroups; ++g) {
        const uint8_t *gk = t.gkeys + (uint64_t)g * keybytes;
        int off = 0;
        for (int i = 0; i < nkey; ++i) {
            out_key_nulls[i][g] = gk[off];
            memcpy((uint8_t *)out_keys[i] + (int64_t)key_widths[i] * g, gk + off + 1, key_widths[i]);
            off += 1 + key_widths[i];
        }
        for (int a = 0; a < nagg; ++a) {
            int rc = state_extract(&c, &c.aggs[a], &c.st[g * nagg + a], overflow_as_null, out_vals[a], g);
            if (rc == 2) { ret = -2; goto done; }
            out_val_nulls[a][g] = (uint8_t)(rc == 1);
        }
    }
    ret = t.ngroups;
done:
    free(k);
    free(c.aggs);
    free(c.st);
    table_free(&t);
    return ret;
}

/* ---------------------------------------------------------------- inner join */
typedef struct {
    int array_mode;
    int64_t min;
    uint64_t range;
    int64_t *head;   /* array: head row per key-min; hash: per slot */
    int64_t *next;   /* chain: next build row with the same key, -1 end */
    uint64_t cap;
    int64_t *hkeys;
    uint8_t *hused;
} jtable_t;

static uint64_t mix64(uint64_t k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

static int jbuild(jtable_t *t, int64_t n, const void *keys, int w, const uint8_t *nulls)
{
    memset(t, 0, sizeof(*t));
    int64_t mn = INT64_MAX, mx = INT64_MIN, cnt = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (nulls && nulls[i]) continue;
        int64_t k = load_int(keys, i, w);
        if (k < mn) mn = k;
        if (k > mx) mx = k;
        cnt++;
    }
    t->next = (int64_t *)malloc((n > 0 ? n : 1) * sizeof(int64_t));
    if (!t->next) return -1;
    if (cnt == 0) { t->array_mode = 1; t->range = 0; return 0; }
    uint64_t range = (uint64_t)mx - (uint64_t)mn + 1;
    uint64_t p2 = 1;
    while (p2 < (uint64_t)cnt) p2 <<= 1;
    if (range != 0 && range <= 8 * p2 && range <= 0xffffffffULL) {
        t->array_mode = 1;
        t->min = mn;
        t->range = range;
        t->head = (int64_t *)malloc(range * sizeof(int64_t));
        if (!t->head) return -1;
        for (uint64_t i = 0; i < range; ++i) t->head[i] = -1;
        for (int64_t i = n - 1; i >= 0; --i) {
            if (nulls && nulls[i]) continue;
            uint64_t s = (uint64_t)load_int(keys, i, w) - (uint64_t)mn;
            t->next[i] = t->head[s];
            t->head[s] = i;
        }
        return 0;
    }
    t->cap = 2 * p2;
    t->hkeys = (int64_t *)malloc(t->cap * sizeof(int64_t));
    t->hused = (uint8_t *)calloc(t->cap, 1);
    t->head = (int64_t *)malloc(t->cap * sizeof(int64_t));
    if (!t->hkeys || !t->hused || !t->head) return -1;
    for (int64_t i = n - 1; i >= 0; --i) {
        if (nulls && nulls[i]) continue;
        int64_t k = load_int(keys, i, w);
        uint64_t s = mix64((uint64_t)k) & (t->cap - 1);
        while (t->hused[s] && t->hkeys[s] != k) s = (s + 1) & (t->cap - 1);
        if (!t->hused[s]) { t->hused[s] = 1; t->hkeys[s] = k; t->head[s] = -1; }
        t->next[i] = t->head[s];
        t->head[s] = i;
    }
    return 0;
}

static int64_t jfind(const jtable_t *t, int64_t k)
{
    if (t->array_mode) {
        uint64_t d = (uint64_t)k - (uint64_t)t->min;
        if (t->range == 0 || k < t->min || d >= t->range) return -1;
        return t->head[d];
    }
    uint64_t s = mix64((uint64_t)k) & (t->cap - 1);
    while (t->hused[s]) {
        if (t->hkeys[s] == k) return t->head[s];
        s = (s + 1) & (t->cap - 1);
    }
    return -1;
}

static void jfree(jtable_t *t)
{
    free(t->head);
    free(t->next);
    free(t->hkeys);
    free(t->hused);
}

/*
 * Inner join of probe keys against build keys: writes (probe row, build row) pairs for
 * every match, probe rows in order.  Returns the number of pairs (which may exceed
 * `capacity`; only the first `capacity` are written) or -1 on allocation failure.
 */
int64_t orc_join_inner(int64_t n_build, const void *build_keys, int32_t build_width, const uint8_t *build_nulls,
    int64_t n_probe, const void *probe_keys, int32_t probe_width, const uint8_t *probe_nulls, int64_t *out_probe,
    int64_t *out_build, int64_t capacity)
{
    jtable_t t;
    if (jbuild(&t, n_build, build_keys, build_width, build_nulls) != 0) { jfree(&t); return -1; }
    int64_t n = 0;
    for (int64_t r = 0; r < n_probe; ++r) {
        if (probe_nulls && probe_nulls[r]) continue;
        for (int64_t b = jfind(&t, load_int(probe_keys, r, probe_width)); b >= 0; b = t.next[b]) {
            if (n < capacity) {
                out_probe[n] = r;
                out_build[n] = b;
            }
            n++;
        }
    }
    jfree(&t);
    return n;
}

/*
 * Equi-join of every kind a probe emits (kind: 0 inner, 1 probe-side outer, 2 build-side
 * outer, 3 full, 4 left semi, 5 left anti, 6 existence).  Writes one (probe row, build row)
 * pair per output row, -1 for the side an outer row does not have:
 *  - probe-side outer (lookup_join.cpp:1037-1105): all matches of a probe row, else (r, -1);
 *    a NULL probe key gives (r, -1);
 *  - build-side outer (:1107-1174): the matches only, marking the matched build rows; then
 *    every unmarked build row, NULL keys included, as (-1, b) (lookup_outer_join.cpp:173-374:
 *    these builds keep NULL-key rows in the table, join_hash_table_variants.cpp:80-82);
 *  - full (:1176-1245): probe-side outer rows, marking matches, then the unmarked build rows;
 *  - left semi (:1247-1311): (r, -1) once for a probe row with a match (NULL keys skipped);
 *  - left anti (:1313-1379): (r, -1) for a probe row without a match, NULL keys included;
 *  - existence (:1381-1430): (r, 1 or 0) for every probe row, 1 iff it has a match.
 * Returns the number of output rows (only the first `capacity` are written), -1 on allocation
 * failure or an unknown kind.
 */
int64_t orc_join(int32_t kind, int64_t n_build, const void *build_keys, int32_t build_width,
    const uint8_t *build_nulls, int64_t n_probe, const void *probe_keys, int32_t probe_width,
    const uint8_t *probe_nulls, int64_t *out_probe, int64_t *out_build, int64_t capacity)
{
    if (kind < 0 || kind > 6) return -1;
    jtable_t t;
    if (jbuild(&t, n_build, build_keys, build_width, build_nulls) != 0) { jfree(&t); return -1; }
    uint8_t *visited = (uint8_t *)calloc((size_t)(n_build > 0 ? n_build : 1), 1);
    if (!visited) { jfree(&t); return -1; }
    int64_t n = 0;
#define EMIT(pr, br) do { if (n < capacity) { out_probe[n] = (pr); out_build[n] = (br); } n++; } while (0)
    for (int64_t r = 0; r < n_probe; ++r) {
        const int null_key = probe_nulls && probe_nulls[r];
        const int64_t head = null_key ? -1 : jfind(&t, load_int(probe_keys, r, probe_width));
        switch (kind) {
            case 0:
            case 2:
                for (int64_t b = head; b >= 0; b = t.next[b]) { EMIT(r, b); visited[b] = 1; }
                break;
            case 1:
            case 3:
                if (head < 0) { EMIT(r, -1); break; }
                for (int64_t b = head; b >= 0; b = t.next[b]) { EMIT(r, b); visited[b] = 1; }
                break;
            case 4:
                if (head >= 0) EMIT(r, -1);
                break;
            case 5:
                if (head < 0) EMIT(r, -1);
                break;
            default:
                EMIT(r, head >= 0 ? 1 : 0);
        }
    }
    if (kind == 2 || kind == 3) {
        for (int64_t b = 0; b < n_build; ++b) {
            if (!visited[b]) EMIT(-1, b);
        }
    }
#undef EMIT
    free(visited);
    jfree(&t);
    return n;
}

/* ---------------------------------------------------------------- timed CPU baselines */
/*
 * Join probe baseline: the reference's probe loop materialising (probe key, payload columns)
 * output rows, over `nthreads` threads that each own a contiguous slice of the probe rows and
 * share the read-only build table (the reference runs one LookupJoin operator per task over a
 * shared build, join_test.cpp:525-770).  Payload columns are int32.
 */
typedef struct {
    const jtable_t *t;
    const int64_t *pkeys;
    const uint8_t *pnulls;
    int64_t r0, r1;
    int32_t npay;
    const int32_t **pay;
    int64_t *okey;
    int32_t **opay;
    int64_t n;
} jwork_t;

static void *jprobe_thread(void *arg)
{
    jwork_t *w = (jwork_t *)arg;
    int64_t n = 0;
    for (int64_t r = w->r0; r < w->r1; ++r) {
        if (w->pnulls && w->pnulls[r]) continue;
        const int64_t k = w->pkeys[r];
        for (int64_t b = jfind(w->t, k); b >= 0; b = w->t->next[b]) {
            w->okey[n] = k;
            for (int p = 0; p < w->npay; ++p) w->opay[p][n] = w->pay[p][b];
            n++;
        }
    }
    w->n = n;
    return NULL;
}

static double now_seconds(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* seconds[0] = build time, seconds[1] = probe time (output buffers allocated beforehand). */
int64_t orc_join_probe_bench(int64_t n_build, const int64_t *build_keys, const uint8_t *build_nulls, int32_t npay,
    const int32_t **payloads, int64_t n_probe, const int64_t *probe_keys, const uint8_t *probe_nulls, int32_t nthreads,
    double *seconds)
{
    jtable_t t;
    const double t0 = now_seconds();
    if (jbuild(&t, n_build, build_keys, 8, build_nulls) != 0) { jfree(&t); return -1; }
    const double t1 = now_seconds();
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    jwork_t *w = (jwork_t *)calloc(nthreads, sizeof(jwork_t));
    int64_t total = 0;
    for (int i = 0; i < nthreads; ++i) {
        w[i].t = &t;
        w[i].pkeys = probe_keys;
        w[i].pnulls = probe_nulls;
        w[i].r0 = n_probe * i / nthreads;
        w[i].r1 = n_probe * (i + 1) / nthreads;
        w[i].npay = npay;
        w[i].pay = payloads;
        const int64_t cap = (w[i].r1 - w[i].r0) * 2 + 16;
        w[i].okey = (int64_t *)malloc(cap * sizeof(int64_t));
        w[i].opay = (int32_t **)malloc(sizeof(int32_t *) * (npay > 0 ? npay : 1));
        for (int p = 0; p < npay; ++p) w[i].opay[p] = (int32_t *)malloc(cap * sizeof(int32_t));
    }
    const double t2 = now_seconds();
    for (int i = 0; i < nthreads; ++i) pthread_create(&th[i], NULL, jprobe_thread, &w[i]);
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    const double t3 = now_seconds();
    if (seconds) {
        seconds[0] = t1 - t0;
        seconds[1] = t3 - t2;
    }
    for (int i = 0; i < nthreads; ++i) {
        total += w[i].n;
        free(w[i].okey);
        for (int p = 0; p < npay; ++p) free(w[i].opay[p]);
        free(w[i].opay);
    }
    free(th);
    free(w);
    jfree(&t);
    return total;
}

/*
 * Aggregation baseline: `nthreads` operator instances each aggregate a contiguous slice of
 * the rows with orc_hashagg's row loop (partial stage); the partial groups are then merged
 * into one table (final stage) -- the reference's partial/final split.  Single int64 key,
 * aggregates SUM/COUNT/MIN/MAX of an int64 column and SUM/AVG of a double column (the
 * uniform-key workload).  Returns the number of groups.
 */
typedef struct {
    int64_t r0, r1;
    const int64_t *key, *v1;
    const double *v2;
    table_t t;
    int64_t *sum, *cnt, *mn, *mx;
    double *dsum;
    int64_t cap;
} awork_t;

static void *agg_thread(void *arg)
{
    awork_t *w = (awork_t *)arg;
    table_init(&w->t, 1, 9, 1024);
    w->cap = 1024;
    w->sum = (int64_t *)malloc(w->cap * 8);
    w->cnt = (int64_t *)malloc(w->cap * 8);
    w->mn = (int64_t *)malloc(w->cap * 8);
    w->mx = (int64_t *)malloc(w->cap * 8);
    w->dsum = (double *)malloc(w->cap * 8);
    uint8_t k[9];
    k[0] = 0;
    for (int64_t r = w->r0; r < w->r1; ++r) {
        memcpy(k + 1, &w->key[r], 8);
        int isnew = 0;
        int64_t g = table_find_insert(&w->t, k, &isnew);
        if (isnew) {
            if (g >= w->cap) {
                w->cap *= 2;
                w->sum = (int64_t *)realloc(w->sum, w->cap * 8);
                w->cnt = (int64_t *)realloc(w->cnt, w->cap * 8);
                w->mn = (int64_t *)realloc(w->mn, w->cap * 8);
                w->mx = (int64_t *)realloc(w->mx, w->cap * 8);
                w->dsum = (double *)realloc(w->dsum, w->cap * 8);
            }
            w->sum[g] = 0;
            w->cnt[g] = 0;
            w->mn[g] = INT64_MAX;
            w->mx[g] = INT64_MIN;
            w->dsum[g] = 0;
        }
        const int64_t x = w->v1[r];
        w->sum[g] = (int64_t)((uint64_t)w->sum[g] + (uint64_t)x);
        w->cnt[g]++;
        w->mn[g] = x < w->mn[g] ? x : w->mn[g];
        w->mx[g] = w->mx[g] < x ? x : w->mx[g];
        w->dsum[g] += w->v2[r];
    }
    return NULL;
}

int64_t orc_agg_bench(int64_t n, const int64_t *key, const int64_t *v1, const double *v2, int32_t nthreads)
{
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    awork_t *w = (awork_t *)calloc(nthreads, sizeof(awork_t));
    for (int i = 0; i < nthreads; ++i) {
        w[i].r0 = n * i / nthreads;
        w[i].r1 = n * (i + 1) / nthreads;
        w[i].key = key;
        w[i].v1 = v1;
        w[i].v2 = v2;
        pthread_create(&th[i], NULL, agg_thread, &w[i]);
    }
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    /* final stage: merge the partial tables */
    table_t t;
    table_init(&t, 1, 9, 1024);
    int64_t cap = 1024;
    int64_t *sum = (int64_t *)malloc(cap * 8), *cnt = (int64_t *)malloc(cap * 8);
    int64_t *mn = (int64_t *)malloc(cap * 8), *mx = (int64_t *)malloc(cap * 8);
    double *dsum = (double *)malloc(cap * 8);
    for (int i = 0; i < nthreads; ++i) {
        for (int64_t g = 0; g < w[i].t.ngroups; ++g) {
            int isnew = 0;
            int64_t h = table_find_insert(&t, w[i].t.gkeys + g * 9, &isnew);
            if (isnew) {
                if (h >= cap) {
                    cap *= 2;
                    sum = (int64_t *)realloc(sum, cap * 8);
                    cnt = (int64_t *)realloc(cnt, cap * 8);
                    mn = (int64_t *)realloc(mn, cap * 8);
                    mx = (int64_t *)realloc(mx, cap * 8);
                    dsum = (double *)realloc(dsum, cap * 8);
                }
                sum[h] = 0; cnt[h] = 0; mn[h] = INT64_MAX; mx[h] = INT64_MIN; dsum[h] = 0;
            }
            sum[h] = (int64_t)((uint64_t)sum[h] + (uint64_t)w[i].sum[g]);
            cnt[h] += w[i].cnt[g];
            mn[h] = w[i].mn[g] < mn[h] ? w[i].mn[g] : mn[h];
            mx[h] = mx[h] < w[i].mx[g] ? w[i].mx[g] : mx[h];
            dsum[h] += w[i].dsum[g];
        }
        table_free(&w[i].t);
        free(w[i].sum); free(w[i].cnt); free(w[i].mn); free(w[i].mx); free(w[i].dsum);
    }
    const int64_t groups = t.ngroups;
    table_free(&t);
    free(sum); free(cnt); free(mn); free(mx); free(dsum);
    free(th);
    free(w);
    return groups;
}

/* ---------------------------------------------------------------- checks at full configuration size */
/*
 * Order-independent row-multiset fingerprint, the same row hash the library's fingerprint
 * kernel computes on the device (a chain of the 64-bit finaliser over the column values,
 * zero-extended, 16-byte values as two words, a NULL as a per-column tag; per row
 * out[0] += 1, out[1] += mix64(h), out[2] += mix64(h ^ c)).  Two row sets with equal counts and
 * equal sums are the same multiset up to a 2^-128 chance.  Used to compare a GPU output that
 * stays on the device with the rows this file computes, without moving the rows.
 */
static uint64_t fp_row_start(void) { return 0x243f6a8885a308d3ULL; }
static uint64_t fp_null(uint64_t h, int c) { return mix64(h ^ 0x9e3779b97f4a7c15ULL ^ (uint64_t)c); }
static uint64_t fp_value(uint64_t h, const void *col, int64_t r, int w)
{
    switch (w) {
        case 1: return mix64(h ^ (uint64_t)((const uint8_t *)col)[r]);
        case 2: return mix64(h ^ (uint64_t)((const uint16_t *)col)[r]);
        case 4: return mix64(h ^ (uint64_t)((const uint32_t *)col)[r]);
        case 16: {
            const uint64_t *p = (const uint64_t *)col + 2 * r;
            return mix64(mix64(h ^ p[0]) ^ p[1]);
        }
        default: return mix64(h ^ ((const uint64_t *)col)[r]);
    }
}
static void fp_add(uint64_t *acc, uint64_t h)
{
    acc[0] += 1;
    acc[1] += mix64(h);
    acc[2] += mix64(h ^ 0xc2b2ae3d27d4eb4fULL);
}

/* Fingerprint of n rows of ncols columns (nulls: byte per row, 1 = NULL; NULL = none). */
void orc_fingerprint_cols(int64_t n, int32_t ncols, const void **cols, const int32_t *widths, const uint8_t **nulls,
    uint64_t *out)
{
    out[0] = out[1] = out[2] = 0;
    for (int64_t r = 0; r < n; ++r) {
        uint64_t h = fp_row_start();
        for (int c = 0; c < ncols; ++c) {
            h = (nulls && nulls[c] && nulls[c][r]) ? fp_null(h, c) : fp_value(h, cols[c], r, widths[c]);
        }
        fp_add(out, h);
    }
}

/* A join build kept across calls (one build, many probes of the full-size checks). */
void *orc_jtable_new(int64_t n_build, const int64_t *build_keys, const uint8_t *build_nulls)
{
    jtable_t *t = (jtable_t *)calloc(1, sizeof(jtable_t));
    if (!t) return NULL;
    if (jbuild(t, n_build, build_keys, 8, build_nulls) != 0) {
        jfree(t);
        free(t);
        return NULL;
    }
    return t;
}

void orc_jtable_free(void *t)
{
    if (t) {
        jfree((jtable_t *)t);
        free(t);
    }
}

typedef struct {
    const jtable_t *t;
    const int64_t *pkeys;
    const uint8_t *pnulls;
    int64_t r0, r1;
    int32_t npay;
    const void **pay;
    const int32_t *payw;
    uint64_t acc[3];
} jfp_work_t;

static void *jfp_thread(void *arg)
{
    jfp_work_t *w = (jfp_work_t *)arg;
    w->acc[0] = w->acc[1] = w->acc[2] = 0;
    for (int64_t r = w->r0; r < w->r1; ++r) {
        if (w->pnulls && w->pnulls[r]) continue;
        const int64_t k = w->pkeys[r];
        for (int64_t b = jfind(w->t, k); b >= 0; b = w->t->next[b]) {
            uint64_t h = mix64(fp_row_start() ^ (uint64_t)k);
            for (int p = 0; p < w->npay; ++p) h = fp_value(h, w->pay[p], b, w->payw[p]);
            fp_add(w->acc, h);
        }
    }
    return NULL;
}

/*
 * Inner-join output fingerprint: the rows (probe key, payload columns of the matched build
 * row) of every match, NULL probe keys skipped -- the rows ProbeBatchForInnerJoin emits
 * (lookup_join.cpp:924-1035) -- hashed as orc_fingerprint_cols would hash them, over
 * `nthreads` threads owning contiguous probe slices of a shared build.  Payload columns are
 * NULL-free.  out[3] as orc_fingerprint_cols; returns the probe seconds in *seconds.
 */
int32_t orc_jtable_fingerprint(const void *table, int32_t npay, const void **pay, const int32_t *payw,
    int64_t n_probe, const int64_t *probe_keys, const uint8_t *probe_nulls, int32_t nthreads, uint64_t *out,
    double *seconds)
{
    if (!table) return -1;
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    jfp_work_t *w = (jfp_work_t *)calloc(nthreads, sizeof(jfp_work_t));
    if (!th || !w) {
        free(th);
        free(w);
        return -1;
    }
    const double t0 = now_seconds();
    for (int i = 0; i < nthreads; ++i) {
        w[i].t = (const jtable_t *)table;
        w[i].pkeys = probe_keys;
        w[i].pnulls = probe_nulls;
        w[i].r0 = n_probe * i / nthreads;
        w[i].r1 = n_probe * (i + 1) / nthreads;
        w[i].npay = npay;
        w[i].pay = pay;
        w[i].payw = payw;
        pthread_create(&th[i], NULL, jfp_thread, &w[i]);
    }
    out[0] = out[1] = out[2] = 0;
    for (int i = 0; i < nthreads; ++i) {
        pthread_join(th[i], NULL);
        out[0] += w[i].acc[0];
        out[1] += w[i].acc[1];
        out[2] += w[i].acc[2];
    }
    if (seconds) *seconds = now_seconds() - t0;
    free(th);
    free(w);
    return 0;
}

/* (probe row, build row) pairs of every inner-join match against a kept build, probe rows in
 * order; returns the number of pairs (only the first `capacity` written). */
int64_t orc_jtable_pairs(const void *table, int64_t n_probe, const int64_t *probe_keys, const uint8_t *probe_nulls,
    int64_t *out_probe, int64_t *out_build, int64_t capacity)
{
    const jtable_t *t = (const jtable_t *)table;
    if (!t) return -1;
    int64_t n = 0;
    for (int64_t r = 0; r < n_probe; ++r) {
        if (probe_nulls && probe_nulls[r]) continue;
        for (int64_t b = jfind(t, probe_keys[r]); b >= 0; b = t->next[b]) {
            if (n < capacity) {
                out_probe[n] = r;
                out_build[n] = b;
            }
            n++;
        }
    }
    return n;
}

/*
 * Multi-threaded single-stage hash aggregation for checks at full configuration size.  Every
 * group's rows go to one thread (thread = hash of the packed key mod nthreads), which folds
 * them in row order with the same per-row state updates as orc_hashagg, so each group's result
 * is the one orc_hashagg computes.  Outputs as orc_hashagg (groups in thread order).
 * For every aggregator over a DOUBLE column (SUM, AVG), out_exact[a] / out_abs[a] (when given)
 * receive the group's sum of the non-NULL values accumulated in double-double arithmetic
 * (Knuth's TwoSum, error at most n * 2^-104 * sum|x|, about 10^10 times below the 1e-12
 * tolerance these checks use) and the sum of |x|.  Returns the number of groups, -1 on
 * allocation failure, -2 if an overflow must raise, -3 if max_groups is too small.
 */
typedef struct {
    int tid, nthreads;
    int64_t n_rows;
    const uint8_t *part;
    int32_t nkey;
    const void **key_cols;
    const int32_t *key_widths;
    const uint8_t **key_nulls;
    int keybytes;
    aggctx_t c;
    table_t t;
    double *ehi, *elo, *eabs; /* per group, per aggregator (double inputs only) */
    int64_t ecap;
    int rc;
} hmt_work_t;

static void two_sum(double a, double b, double *s, double *e)
{
    const double x = a + b;
    const double bv = x - a;
    *e = (a - (x - bv)) + (b - bv);
    *s = x;
}

/* (hi, lo) += x in double-double arithmetic. */
static void dd_add(double *hi, double *lo, double x)
{
    double s, e;
    two_sum(*hi, x, &s, &e);
    e += *lo;
    const double h = s + e;
    *lo = e - (h - s);
    *hi = h;
}

static void *hmt_thread(void *arg)
{
    hmt_work_t *w = (hmt_work_t *)arg;
    const int nagg = w->c.nagg;
    const int na = nagg > 0 ? nagg : 1;
    w->rc = 0;
    if (table_init(&w->t, w->nkey, w->keybytes, 1024) != 0) {
        w->rc = -1;
        return NULL;
    }
    w->c.stcap = 1024;
    w->c.st = (state_t *)malloc((uint64_t)w->c.stcap * na * sizeof(state_t));
    w->ecap = 1024;
    w->ehi = (double *)calloc((uint64_t)w->ecap * na, sizeof(double));
    w->elo = (double *)calloc((uint64_t)w->ecap * na, sizeof(double));
    w->eabs = (double *)calloc((uint64_t)w->ecap * na, sizeof(double));
    uint8_t *k = (uint8_t *)malloc(w->keybytes + 1);
    if (!w->c.st || !w->ehi || !w->elo || !w->eabs || !k) {
        w->rc = -1;
        free(k);
        return NULL;
    }
    for (int64_t r = 0; r < w->n_rows; ++r) {
        if (w->part[r] != (uint8_t)w->tid) continue;
        pack_key(w->nkey, w->key_cols, w->key_widths, w->key_nulls, r, k);
        int isnew = 0;
        const int64_t g = table_find_insert(&w->t, k, &isnew);
        if (g < 0) {
            w->rc = -1;
            break;
        }
        if (isnew) {
            if (g >= w->c.stcap) {
                state_t *ns = (state_t *)realloc(w->c.st, (uint64_t)w->c.stcap * 2 * na * sizeof(state_t));
                if (!ns) {
                    w->rc = -1;
                    break;
                }
                w->c.st = ns;
                w->c.stcap *= 2;
            }
            if (g >= w->ecap) {
                const int64_t nc = w->ecap * 2;
                double *a = (double *)realloc(w->ehi, (uint64_t)nc * na * sizeof(double));
                if (a) w->ehi = a;
                double *b = a ? (double *)realloc(w->elo, (uint64_t)nc * na * sizeof(double)) : NULL;
                if (b) w->elo = b;
                double *d = b ? (double *)realloc(w->eabs, (uint64_t)nc * na * sizeof(double)) : NULL;
                if (d) w->eabs = d;
                if (!a || !b || !d) {
                    w->rc = -1;
                    break;
                }
                w->ecap = nc;
            }
            for (int a = 0; a < nagg; ++a) {
                state_init(&w->c.aggs[a], &w->c.st[g * nagg + a]);
                w->ehi[g * na + a] = w->elo[g * na + a] = w->eabs[g * na + a] = 0.0;
            }
        }
        for (int a = 0; a < nagg; ++a) {
            const agg_t *ag = &w->c.aggs[a];
            state_update(&w->c, ag, &w->c.st[g * nagg + a], r);
            if (ag->in_type == T_DOUBLE && (ag->func == F_SUM || ag->func == F_AVG) && !(ag->nulls && ag->nulls[r]) &&
                !(ag->mask && !ag->mask[r])) {
                const double x = ((const double *)ag->col)[r];
                dd_add(&w->ehi[g * na + a], &w->elo[g * na + a], x);
                w->eabs[g * na + a] += x < 0 ? -x : x;
            }
        }
    }
    free(k);
    return NULL;
}

typedef struct {
    int64_t r0, r1;
    int32_t nkey;
    const void **key_cols;
    const int32_t *key_widths;
    const uint8_t **key_nulls;
    int keybytes;
    int nthreads;
    uint8_t *part;
} hpart_work_t;

static void *hpart_thread(void *arg)
{
    hpart_work_t *w = (hpart_work_t *)arg;
    uint8_t *k = (uint8_t *)malloc(w->keybytes + 1);
    if (!k) return NULL;
    for (int64_t r = w->r0; r < w->r1; ++r) {
        pack_key(w->nkey, w->key_cols, w->key_widths, w->key_nulls, r, k);
        w->part[r] = (uint8_t)((hash_bytes(k, w->keybytes) >> 40) % (uint64_t)w->nthreads);
    }
    free(k);
    return NULL;
}

int64_t orc_hashagg_mt(int64_t n_rows, int32_t nkey, const void **key_cols, const int32_t *key_widths,
    const uint8_t **key_nulls, int32_t nagg, const int32_t *funcs, const void **agg_cols, const int32_t *in_types,
    const int32_t *in_widths, const uint8_t **agg_nulls, const int32_t *out_types, const int32_t *rescale,
    int32_t policy, int32_t overflow_as_null, int64_t max_groups, void **out_keys, uint8_t **out_key_nulls,
    void **out_vals, uint8_t **out_val_nulls, double **out_exact, double **out_abs, int32_t nthreads,
    const uint8_t **agg_masks, const int32_t *dec_params)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 255) nthreads = 255;
    int keybytes = 0;
    for (int i = 0; i < nkey; ++i) keybytes += 1 + key_widths[i];
    uint8_t *part = (uint8_t *)malloc((size_t)(n_rows > 0 ? n_rows : 1));
    agg_t *aggs = (agg_t *)calloc(nagg > 0 ? nagg : 1, sizeof(agg_t));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    hpart_work_t *pw = (hpart_work_t *)calloc(nthreads, sizeof(hpart_work_t));
    hmt_work_t *w = (hmt_work_t *)calloc(nthreads, sizeof(hmt_work_t));
    int64_t ret = 0;
    if (!part || !aggs || !th || !pw || !w) {
        ret = -1;
        goto out;
    }
    for (int a = 0; a < nagg; ++a) {
        aggs[a].func = funcs[a];
        aggs[a].col = agg_cols[a];
        aggs[a].in_type = in_types[a];
        aggs[a].in_width = in_widths[a];
        aggs[a].nulls = agg_nulls ? agg_nulls[a] : NULL;
        aggs[a].out_type = out_types[a];
        aggs[a].rescale = rescale ? rescale[a] : 0;
        aggs[a].mask = agg_masks ? agg_masks[a] : NULL;
        if (dec_params) {
            aggs[a].in_prec = dec_params[3 * a];
            aggs[a].in_scale = dec_params[3 * a + 1];
            aggs[a].out_scale = dec_params[3 * a + 2];
        }
    }
    for (int i = 0; i < nthreads; ++i) {
        pw[i].r0 = n_rows * i / nthreads;
        pw[i].r1 = n_rows * (i + 1) / nthreads;
        pw[i].nkey = nkey;
        pw[i].key_cols = key_cols;
        pw[i].key_widths = key_widths;
        pw[i].key_nulls = key_nulls;
        pw[i].keybytes = keybytes;
        pw[i].nthreads = nthreads;
        pw[i].part = part;
        pthread_create(&th[i], NULL, hpart_thread, &pw[i]);
    }
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    for (int i = 0; i < nthreads; ++i) {
        w[i].tid = i;
        w[i].nthreads = nthreads;
        w[i].n_rows = n_rows;
        w[i].part = part;
        w[i].nkey = nkey;
        w[i].key_cols = key_cols;
        w[i].key_widths = key_widths;
        w[i].key_nulls = key_nulls;
        w[i].keybytes = keybytes;
        w[i].c.nagg = nagg;
        w[i].c.aggs = aggs;
        w[i].c.policy = policy;
        pthread_create(&th[i], NULL, hmt_thread, &w[i]);
    }
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    int64_t total = 0;
    for (int i = 0; i < nthreads; ++i) {
        if (w[i].rc != 0) {
            ret = -1;
            goto out;
        }
        total += w[i].t.ngroups;
    }
    if (total > max_groups) {
        ret = -3;
        goto out;
    }
    {
        const int na = nagg > 0 ? nagg : 1;
        int64_t base = 0;
        for (int i = 0; i < nthreads && ret == 0; ++i) {
            for (int64_t g = 0; g < w[i].t.ngroups; ++g) {
                const int64_t o = base + g;
                const uint8_t *gk = w[i].t.gkeys + (uint64_t)g * keybytes;
                int off = 0;
                for (int c = 0; c < nkey; ++c) {
                    out_key_nulls[c][o] = gk[off];
                    memcpy((uint8_t *)out_keys[c] + (int64_t)key_widths[c] * o, gk + off + 1, key_widths[c]);
                    off += 1 + key_widths[c];
                }
                for (int a = 0; a < nagg; ++a) {
                    const int rc = state_extract(&w[i].c, &aggs[a], &w[i].c.st[g * nagg + a], overflow_as_null,
                        out_vals[a], o);
                    if (rc == 2) {
                        ret = -2;
                        break;
                    }
                    out_val_nulls[a][o] = (uint8_t)(rc == 1);
                    if (out_exact && out_exact[a]) out_exact[a][o] = w[i].ehi[g * na + a] + w[i].elo[g * na + a];
                    if (out_abs && out_abs[a]) out_abs[a][o] = w[i].eabs[g * na + a];
                }
                if (ret != 0) break;
            }
            base += w[i].t.ngroups;
        }
        if (ret == 0) ret = total;
    }
out:
    if (w) {
        for (int i = 0; i < nthreads; ++i) {
            if (w[i].t.keys || w[i].t.used || w[i].t.gid || w[i].t.gkeys) table_free(&w[i].t);
            free(w[i].c.st);
            free(w[i].ehi);
            free(w[i].elo);
            free(w[i].eabs);
        }
    }
    free(part);
    free(aggs);
    free(th);
    free(pw);
    free(w);
    return ret;
}
