"""Writes agg_kats.json and join_kats.json: known-answer tests of the reference's own C++ tests,
transcribed (inputs and expected outputs as literals) with the file:line they come from.

The reference is C++ and cannot be built here, so its test vectors are carried over by reading
the test sources; each entry below restates one test's inputs and EXPECT_* values.  Run
`python tests/golden/make_golden.py` to regenerate the JSON files.
"""
import json
import struct
from pathlib import Path

HERE = Path(__file__).resolve().parent

INT64_MAX = 9223372036854775807
DEC38 = 10**38 - 1

AGG = {
    # core/test/operator/aggregation_test.cpp:4386-4422 -- Spark long SUM wraps:
    # 3 x 9223372036854774807 -> 9223372036854772805.
    "spark_sum_long_overflow": dict(
        source="core/test/operator/aggregation_test.cpp:4386-4422", policy="spark",
        func="SUM", in_type="LONG", out_type="LONG", values=[9223372036854774807] * 3,
        nulls=None, expected=9223372036854772805),
    # aggregation_test.cpp:4424-4466 -- 851451 + 9223372036854775807 = -9223372036853924358 and
    # -9223372036854775807 + -256 = 9223372036854775553 ("overflow but same with vanilla spark").
    "spark_sum_long_wrap_positive": dict(
        source="core/test/operator/aggregation_test.cpp:4424-4466", policy="spark",
        func="SUM", in_type="LONG", out_type="LONG", values=[851451, INT64_MAX], nulls=None,
        expected=-9223372036853924358),
    "spark_sum_long_wrap_negative": dict(
        source="core/test/operator/aggregation_test.cpp:4424-4466", policy="spark",
        func="SUM", in_type="LONG", out_type="LONG", values=[-INT64_MAX, -256], nulls=None,
        expected=9223372036854775553),
    # aggregation_test.cpp:4468-4500 -- Spark double SUM of three values -> 7.037035803703704E11.
    "spark_sum_double": dict(
        source="core/test/operator/aggregation_test.cpp:4468-4500", policy="spark",
        func="SUM", in_type="DOUBLE", out_type="DOUBLE",
        values=[123456789012.3456789, 234567890123.4567891, 345678901234.5678912], nulls=None,
        expected=7.037035803703704e11),
    # aggregation_test.cpp:4598-4641 -- Spark AVG of 3 x 9223372036854774807 -> 9.2233720368547748E18.
    "spark_avg_long": dict(
        source="core/test/operator/aggregation_test.cpp:4598-4641", policy="spark",
        func="AVG", in_type="LONG", out_type="DOUBLE", values=[9223372036854774807] * 3, nulls=None,
        expected=9.2233720368547748e18),
    # aggregation_test.cpp:4643-4683 -- Spark AVG of the three doubles -> 2.345678601234568E11.
    "spark_avg_double": dict(
        source="core/test/operator/aggregation_test.cpp:4643-4683", policy="spark",
        func="AVG", in_type="DOUBLE", out_type="DOUBLE",
        values=[123456789012.3456789, 234567890123.4567891, 345678901234.5678912], nulls=None,
        expected=2.345678601234568e11),
    # aggregation_test.cpp:3790-3848 / 3849-3900 -- decimal128(38,0) SUM of 3 x (10^38 - 1):
    # overflow raises with overflow-as-null off, gives NULL with it on.
    "spark_sum_decimal128_overflow": dict(
        source="core/test/operator/aggregation_test.cpp:3790-3900", policy="spark",
        func="SUM", in_type="DECIMAL128", out_type="DECIMAL128", scale=0, values=[DEC38] * 3, nulls=None,
        expected="overflow"),
    # aggregation_test.cpp:3167-3229 (sum_test, SUPPORT policy) -- SUM of 200 ones = 200; SUM of
    # an all-NULL column is NULL.
    "generic_sum_long_ones": dict(
        source="core/test/operator/aggregation_test.cpp:3167-3229", policy="generic",
        func="SUM", in_type="LONG", out_type="LONG", values=[1] * 200, nulls=None, expected=200),
    "generic_sum_all_null": dict(
        source="core/test/operator/aggregation_test.cpp:3167-3229", policy="generic",
        func="SUM", in_type="LONG", out_type="LONG", values=[0] * 200, nulls=[True] * 200, expected=None),
    "generic_sum_short_decimal_ones": dict(
        source="core/test/operator/aggregation_test.cpp:3167-3229", policy="generic",
        func="SUM", in_type="DECIMAL64", out_type="DECIMAL128", scale=0, values=[1] * 200, nulls=None,
        expected=200),
}

# aggregation_test.cpp:1292-1350 (verify_null_correctness): one group of 6 rows, all agg inputs
# are ones (BuildAggregateInput, :180-252); col 2 NULL at rows 0-4, cols 3,4,5 NULL at row 1.
# SUM(c1), AVG(c2), COUNT(c3), MIN(c4), MAX(c5) -> {key 0, 6, 1.0, 5, 1, 1}.
AGG_MULTI = {
    "verify_null_correctness": dict(
        source="core/test/operator/aggregation_test.cpp:1292-1350",
        key=[0] * 6,
        columns=[[1] * 6] * 5,
        nulls=[[False] * 6, [True] * 5 + [False], [False, True, False, False, False, False],
               [False, True, False, False, False, False], [False, True, False, False, False, False]],
        funcs=["SUM", "AVG", "COUNT_COLUMN", "MIN", "MAX"],
        out_types=["LONG", "DOUBLE", "LONG", "LONG", "LONG"],
        expected=[[0, 6, 1.0, 5, 1, 1]]),
}


def _join_one_build_op():
    # core/test/operator/join_test.cpp:52-59 (build), :81-88 (probe), :90-109 (expected), :283-305.
    build = [[1, 2, 1, 2, 3, 4, 5, 6, 7, 1], [79, 79, 70, 70, 70, 70, 70, 70, 70, 70]]
    probe = [[1, 2, 3, 4, 5, 6, 1, 1, 2, 3], [78, 78, 78, 78, 78, 78, 78, 82, 82, 65]]
    expected0 = [78, 78, 78, 78, 78, 78, 78, 82, 82, 65]
    ids = [0, 0, 0, 1, 1, 2, 3, 4, 5, 6, 6, 6, 7, 7, 7, 8, 8, 9]
    expected1 = [79, 70, 70, 79, 70, 70, 70, 70, 70, 79, 70, 70, 79, 70, 70, 79, 70, 70]
    rows = [[expected0[i], e1] for i, e1 in zip(ids, expected1)]
    return dict(source="core/test/operator/join_test.cpp:52-109,137-160,283-305", build=build, probe=probe,
                build_hash_col=0, probe_hash_col=0, probe_output_cols=[1], build_output_cols=[1],
                expected_rows=rows)


def _join_array_table_short():
    # core/test/operator/join_test.cpp:4265-4313 (TestInnerEqualityJoinOfArrayTable).
    build = [[1, 2, 3, 4, 1, 2], [111, 11, 333, 33, 20, 16]]
    probe = [[1, 2, 3, 4], [11, 22, 33, 44]]
    exp = [[1, 1, 2, 2, 3, 4], [11, 11, 22, 22, 33, 44], [1, 1, 2, 2, 3, 4], [111, 20, 11, 16, 333, 33]]
    rows = [list(r) for r in zip(*exp)]
    return dict(source="core/test/operator/join_test.cpp:4265-4313", build=build, probe=probe, build_hash_col=0,
                probe_hash_col=0, probe_output_cols=[0, 1], build_output_cols=[0, 1], expected_rows=rows)


# Join types other than inner.  Each entry restates one test of core/test/operator/join_test.cpp:
# columns are int64 unless "types" says otherwise, "*_nulls" list the NULL rows per column,
# expected rows list the probe output values then the build output values (None = NULL) in the
# probe-first order the test checks, and "outer_rows" are the rows of the LookupOuterJoin operator
# (None for an operator that is not run).  The reference tests that use VARCHAR payloads are
# restated with the strings replaced by distinct integers (STR below): joins never read payload
# values, so the pairing of rows is unchanged.
STR = {"11": 11, "22": 22, "33": 33, "44": 44, "aaa": 1001, "aa": 1002, "ccc": 1003}


def _s(vals):
    return [STR[v] for v in vals]


def _bits(vals):
    """IEEE-754 bit patterns of doubles as signed int64."""
    return [struct.unpack("<q", struct.pack("<d", v))[0] for v in vals]


JOIN_TYPED = {
    "left_join": dict(
        source="core/test/operator/join_test.cpp:773-833", join_type="LEFT", build_side="UNKNOWN",
        build=[[1, 2, 3, 4], [111, 11, 333, 33]], build_nulls=None, build_hash_col=1,
        probe=[[1, 2, 3, 4], [11, 22, 33, 44]], probe_nulls=None, probe_hash_col=1,
        probe_output_cols=[0, 1], build_output_cols=[0, 1],
        expected_rows=[[1, 11, 2, 11], [2, 22, None, None], [3, 33, 4, 33], [4, 44, None, None]],
        outer_rows=None),
    "left_join_build_left": dict(
        source="core/test/operator/join_test.cpp:835-918", join_type="LEFT", build_side="LEFT",
        build=[[1, 2, 3, 4], [111, 11, 333, 33]], build_nulls=None, build_hash_col=1,
        probe=[[1, 2, 3, 4], [11, 22, 33, 44]], probe_nulls=None, probe_hash_col=1,
        probe_output_cols=[0, 1], build_output_cols=[0, 1],
        expected_rows=[[1, 11, 2, 11], [3, 33, 4, 33]],
        outer_rows=[[None, None, 3, 333], [None, None, 1, 111]]),
    "full_join_one_build_op": dict(
        source="core/test/operator/join_test.cpp:52-109,137-170,2589-2632", join_type="FULL", build_side="UNKNOWN",
        build=[[1, 2, 1, 2, 3, 4, 5, 6, 7, 1], [79, 79, 70, 70, 70, 70, 70, 70, 70, 70]], build_nulls=None,
        build_hash_col=0,
        probe=[[1, 2, 3, 4, 5, 6, 1, 1, 2, 3], [78, 78, 78, 78, 78, 78, 78, 82, 82, 65]], probe_nulls=None,
        probe_hash_col=0, probe_output_cols=[1], build_output_cols=[1],
        expected_rows=None,  # the inner join's rows (every probe row matches): filled in main()
        outer_rows=[[None, 70]]),
    "full_join_build_null": dict(
        source="core/test/operator/join_test.cpp:2881-2973", join_type="FULL", build_side="UNKNOWN",
        build=[[1, 2, 3, 4, 5, 6], [111, 11, 333, 33, 11, 11]], build_nulls=[[], [0, 2]], build_hash_col=1,
        probe=[[1, 2, 3, 4], [11, 22, 33, 44]], probe_nulls=None, probe_hash_col=1,
        probe_output_cols=[0, 1], build_output_cols=[0, 1],
        expected_rows=[[1, 11, 2, 11], [1, 11, 5, 11], [1, 11, 6, 11], [2, 22, None, None], [3, 33, 4, 33],
                       [4, 44, None, None]],
        outer_rows=[[None, None, 1, None], [None, None, 3, None]]),
    "left_semi_join": dict(
        source="core/test/operator/join_test.cpp:3831-3889", join_type="LEFT_SEMI", build_side="UNKNOWN",
        build=[[1, 0, 3, 0, 1, 0, 2, 2], _s(["aaa", "11", "ccc", "33", "aaa", "11", "ccc", "33"])],
        build_nulls=[[1], []], build_hash_col=0,
        probe=[[0, 2, 0, 1, 0, 2, 0, 4], _s(["11", "22", "33", "44", "11", "22", "33", "44"])],
        probe_nulls=[[2], []], probe_hash_col=0, probe_output_cols=[0, 1], build_output_cols=[],
        expected_rows=[[0, 11], [2, 22], [1, 44], [0, 11], [2, 22], [0, 33]], outer_rows=None),
    "right_join": dict(
        source="core/test/operator/join_test.cpp:4014-4081", join_type="RIGHT", build_side="UNKNOWN",
        build=[[1, 0, 3, 0, 1, 0, 2, 2], _s(["aaa", "11", "ccc", "33", "aa", "11", "ccc", "33"])],
        build_nulls=None, build_hash_col=0,
        probe=[[0, 2, 0, 1], _s(["11", "22", "33", "44"])], probe_nulls=[[2], []], probe_hash_col=0,
        probe_output_cols=[0, 1], build_output_cols=[0, 1],
        expected_rows=[[0, 11, 0, 11], [0, 11, 0, 33], [0, 11, 0, 11], [2, 22, 2, 1003], [2, 22, 2, 33],
                       [1, 44, 1, 1001], [1, 44, 1, 1002], [None, 33, None, None]],
        outer_rows=None),
    "left_anti_join": dict(
        source="core/test/operator/join_test.cpp:4157-4207", join_type="LEFT_ANTI", build_side="UNKNOWN",
        build=[[1, 2, 3, 4], [111, 11, 333, 33]], build_nulls=None, build_hash_col=1,
        probe=[[1, 2, 3, 4, 3, 6], [11, 22, 33, 44, 22, 44]], probe_nulls=None, probe_hash_col=1,
        probe_output_cols=[0, 1], build_output_cols=[],
        expected_rows=[[2, 22], [4, 44], [3, 22], [6, 44]], outer_rows=None),
    # join_test.cpp:4329 lists 8 initialisers for a 7-row column: the first 7 are the data.
    "left_anti_join_array_probe": dict(
        source="core/test/operator/join_test.cpp:4323-4380", join_type="LEFT_ANTI", build_side="UNKNOWN",
        build=[[1, 2, 3, 4, 6, 7, 8], [2, 11, 7, 3, 4, 5, 5]], build_nulls=None, build_hash_col=1,
        probe=[[1, 2, 3, 4, 3, 6, 7], [28, 2, 3, 10, 0, 15, 8]], probe_nulls=None, probe_hash_col=1,
        probe_output_cols=[0, 1], build_output_cols=[],
        expected_rows=[[1, 28], [4, 10], [3, 0], [6, 15], [7, 8]], outer_rows=None),
    "full_join_array_table": dict(
        source="core/test/operator/join_test.cpp:4382-4471", join_type="FULL", build_side="UNKNOWN",
        types="SHORT",
        build=[[1, 2, 3, 4, 1, 2], [111, 11, 333, 33, 20, 16]], build_nulls=[[4, 5], []], build_hash_col=0,
        probe=[[1, 2, 3, 4], [11, 22, 33, 44]], probe_nulls=None, probe_hash_col=0,
        probe_output_cols=[0, 1], build_output_cols=[0, 1],
        expected_rows=[[1, 11, 1, 111], [2, 22, 2, 11], [3, 33, 3, 333], [4, 44, 4, 33]],
        outer_rows=[[None, None, None, 20], [None, None, None, 16]]),
    "existence_join": dict(
        source="core/test/operator/join_test.cpp:4584-4635", join_type="EXISTENCE", build_side="UNKNOWN",
        build=[[1, 2, 3, 4], [111, 11, 333, 33]], build_nulls=None, build_hash_col=1,
        probe=[[1, 2, 3, 4, 3, 6], [11, 22, 33, 44, 22, 44]], probe_nulls=None, probe_hash_col=1,
        probe_output_cols=[], build_output_cols=[],
        expected_rows=[[1], [0], [1], [0], [0], [0]], outer_rows=None),
    # Multi-column keys (short, int, long); the test reads the probe operator's rows only.
    "multi_keys_full_integer": dict(
        source="core/test/operator/join_test.cpp:4637-4704", join_type="FULL", build_side="UNKNOWN",
        types=["SHORT", "INT", "LONG"],
        build=[[1, 2, 3, 4, 5, 6], [11, 22, 33, 44, 55, 66], [111, 222, 333, 444, 555, 666]], build_nulls=None,
        build_hash_cols=[0, 1, 2],
        probe=[[1, 3, 5, 7], [11, 33, 55, 77], [111, 333, 555, 777]], probe_nulls=None, probe_hash_cols=[0, 1, 2],
        probe_output_cols=[0, 1, 2], build_output_cols=[0, 1, 2],
        expected_rows=[[1, 11, 111, 1, 11, 111], [3, 33, 333, 3, 33, 333], [5, 55, 555, 5, 55, 555],
                       [7, 77, 777, None, None, None]],
        outer_rows=None),
    # join_test.cpp:4706-4772 fills its Decimal64 key column from doubles; the values here are
    # those doubles' 64-bit patterns, which is what the decimal64 column holds.
    "multi_keys_full_decimal64": dict(
        source="core/test/operator/join_test.cpp:4706-4772", join_type="FULL", build_side="UNKNOWN",
        types=["SHORT", "INT", "LONG"],
        build=[[1, 2, 3, 4, 5, 6], [11, 22, 33, 44, 55, 66], _bits([1.11, 2.22, 3.33, 4.44, 5.55, 6.66])],
        build_nulls=None, build_hash_cols=[0, 1, 2],
        probe=[[1, 3, 5, 7], [11, 33, 55, 77], _bits([1.11, 3.33, 5.55, 7.77])], probe_nulls=None,
        probe_hash_cols=[0, 1, 2], probe_output_cols=[0, 1, 2], build_output_cols=[0, 1, 2],
        expected_rows=[[1, 11, _bits([1.11])[0], 1, 11, _bits([1.11])[0]],
                       [3, 33, _bits([3.33])[0], 3, 33, _bits([3.33])[0]],
                       [5, 55, _bits([5.55])[0], 5, 55, _bits([5.55])[0]],
                       [7, 77, _bits([7.77])[0], None, None, None]],
        outer_rows=None),
}


# aggregation_test.cpp:632-1190 (verify_group_colum_array_map_*): two batches of 21 rows built by
# BuildAggInput (:254-271): group key j % 3 (BuildHashInput, :60-175), five LONG aggregate inputs
# all 1 (BuildAggregateInput, :180-252); SUM(c1), AVG(c2), COUNT(c3), MIN(c4), MAX(c5).  Both
# batches: key NULL at rows 0 and 11, c2 NULL at rows 0-4, c3/c4/c5 NULL at rows 0 and 1; the
# second batch also has key NULL at row 20.  "resize" sets the second batch's key at row 2 to
# 1000; "switch" sets it at rows 2 and 5 to the key type's max and min (the reference builds that
# key column as a dictionary vector over those values with identity ids; restated flat here).  The
# reference runs every case for SHORT, INT, DATE32, LONG, TIMESTAMP and DECIMAL64 keys; each
# *_without_agg variant has the same keys and no aggregates.  Expected rows: (key, SUM, AVG,
# COUNT, MIN, MAX), key None = NULL, AVG None = NULL.
KEY_LIMITS = {"SHORT": (-2**15, 2**15 - 1), "INT": (-2**31, 2**31 - 1), "DATE32": (-2**31, 2**31 - 1),
              "LONG": (-2**63, 2**63 - 1), "TIMESTAMP": (-2**63, 2**63 - 1), "DECIMAL64": (-2**63, 2**63 - 1)}


def _array_map_batch(second, edits):
    keys = [j % 3 for j in range(21)]
    for row, v in edits.items():
        keys[row] = v
    key_nulls = [0, 11] + ([20] if second else [])
    agg_nulls = [[], [0, 1, 2, 3, 4], [0, 1], [0, 1], [0, 1]]
    return dict(keys=keys, key_nulls=key_nulls, agg_nulls=agg_nulls)


def _array_map_cases():
    out = {}
    for key_type, (lo, hi) in KEY_LIMITS.items():
        regular = [[None, 5, 1.0, 3, 1, 1], [0, 12, 1.0, 12, 1, 1], [1, 14, 1.0, 12, 1, 1], [2, 11, 1.0, 11, 1, 1]]
        resize = [[None, 5, 1.0, 3, 1, 1], [0, 12, 1.0, 12, 1, 1], [1, 14, 1.0, 12, 1, 1], [2, 10, 1.0, 10, 1, 1],
                  [1000, 1, None, 1, 1, 1]]
        switch = [[0, 12, 1.0, 12, 1, 1], [lo, 1, 1.0, 1, 1, 1], [1, 14, 1.0, 12, 1, 1], [hi, 1, None, 1, 1, 1],
                  [2, 9, 1.0, 9, 1, 1], [None, 5, 1.0, 3, 1, 1]]
        for name, edits, rows, src in (("regular", {}, regular, "632-718"), ("resize", {2: 1000}, resize, "804-890"),
                                       ("switch", {2: hi, 5: lo}, switch, "1000-1093")):
            batches = [_array_map_batch(False, {}), _array_map_batch(True, edits)]
            out[f"{name}_{key_type}"] = dict(source=f"core/test/operator/aggregation_test.cpp:{src}",
                                             key_type=key_type, batches=batches, expected=rows)
            out[f"{name}_without_agg_{key_type}"] = dict(
                source=f"core/test/operator/aggregation_test.cpp:{src} (without_agg variant)", key_type=key_type,
                batches=batches, expected=[[r[0]] for r in rows], no_aggs=True)
    return out


# core/test/codegen/function_test.cpp:2030-2506 -- substr over UTF-8 code points, each call as
# (string, start, length or None for SubstrVarcharWithStart, supports negative start,
# supports zero start, expected).  SubstrChar takes the same (str, strLen) and gives the same.
_MAGIC = "Magic Johnson 123@#$"
_ZH = "时欧基乌斯侧后解 hello! 回复哦黑色的and magic粉色的圣诞袜"
_ABC = "ABC efg 123 $%^"
_ZH9 = "时欧基乌斯侧后解 h"
SUBSTR = {
    "Substr": ("core/test/codegen/function_test.cpp:2030-2070", [
        (_MAGIC, 1, 20, False, False, _MAGIC), (_MAGIC, 1, 5, False, False, "Magic"),
        (_MAGIC, 10, 10, False, False, "nson 123@#"), (_MAGIC, -5, 7, False, False, "23@#$"),
        (_MAGIC, 0, 0, False, False, ""), (_MAGIC, 20, 25, False, False, "$")]),
    "SubstrZh": ("core/test/codegen/function_test.cpp:2072-2138", [
        (_ZH, 1, 37, False, False, _ZH), (_ZH, 0, 37, False, True, _ZH), (_ZH, 1, 5, False, False, "时欧基乌斯"),
        (_ZH, 0, 5, False, True, "时欧基乌斯"), (_ZH, 10, 10, False, False, "hello! 回复哦"),
        (_ZH, -5, 7, False, False, "色的圣诞袜"), (_ZH, 0, 0, False, False, ""), (_ZH, 0, 0, False, True, ""),
        (_ZH, 37, len(_ZH.encode()) + 5, False, False, "袜"), (_ZH, -38, 10, False, False, ""),
        (_ZH, -37, 37, False, False, _ZH)]),
    "SubstrChar": ("core/test/codegen/function_test.cpp:2140-2198", [
        (_MAGIC, 1, 20, False, False, _MAGIC), (_MAGIC, 0, 20, False, True, _MAGIC),
        (_MAGIC, 1, 5, False, False, "Magic"), (_MAGIC, 0, 5, False, True, "Magic"),
        (_MAGIC, 10, 10, False, False, "nson 123@#"), (_MAGIC, -5, 7, False, False, "23@#$"),
        (_MAGIC, 0, 0, False, False, ""), (_MAGIC, 0, 0, False, True, ""), (_MAGIC, 20, 25, False, False, "$")]),
    "SubstrCharZh": ("core/test/codegen/function_test.cpp:2200-2267", [
        (_ZH, 1, 37, False, False, _ZH), (_ZH, 0, 37, False, True, _ZH), (_ZH, 1, 5, False, False, "时欧基乌斯"),
        (_ZH, 0, 5, False, True, "时欧基乌斯"), (_ZH, 10, 10, False, False, "hello! 回复哦"),
        (_ZH, -5, 7, False, False, "色的圣诞袜"), (_ZH, 0, 0, False, False, ""), (_ZH, 0, 0, False, True, ""),
        (_ZH, 37, len(_ZH.encode()) + 5, False, False, "袜"), (_ZH, -38, 10, False, False, ""),
        (_ZH, -37, 37, False, False, _ZH)]),
    "SubstrWithStart": ("core/test/codegen/function_test.cpp:2269-2305", [
        (_ABC, 1, None, False, False, _ABC), (_ABC, 0, None, False, True, _ABC),
        (_ABC, 9, None, False, False, "123 $%^"), (_ABC, -3, None, False, False, "$%^"),
        (_ABC, 0, None, False, False, "")]),
    "SubstrWithZh": ("core/test/codegen/function_test.cpp:2307-2358", [
        (_ZH, 1, None, False, False, _ZH), (_ZH, 0, None, False, True, _ZH),
        (_ZH, 9, None, False, False, " hello! 回复哦黑色的and magic粉色的圣诞袜"), (_ZH, -3, None, False, False, "圣诞袜"),
        (_ZH, 0, None, False, False, ""), (_ZH, 37, None, False, False, "袜"), (_ZH, -38, None, False, False, "")]),
    "SubstrWithZhForSpark": ("core/test/codegen/function_test.cpp:2360-2414", [
        (_ZH9, -15, None, True, False, _ZH9), (_ZH9, 0, None, True, True, _ZH9), (_ZH9, -15, 5, True, False, ""),
        (_ZH9, -15, 6, True, False, "时"), (_ZH9, -15, 14, True, False, "时欧基乌斯侧后解 "),
        (_ZH9, -15, 20, True, False, _ZH9), ("apple", -7, 3, True, False, "a"),
        ("apple", -7, None, True, False, "apple")]),
    "SubstrCharWithStart": ("core/test/codegen/function_test.cpp:2416-2452", [
        (_ABC, 1, None, False, False, _ABC), (_ABC, 0, None, False, True, _ABC),
        (_ABC, 9, None, False, False, "123 $%^"), (_ABC, -3, None, False, False, "$%^"),
        (_ABC, 0, None, False, False, "")]),
    "SubstrCharWithStartZh": ("core/test/codegen/function_test.cpp:2454-2506", [
        (_ZH, 1, None, False, False, _ZH), (_ZH, 0, None, False, True, _ZH),
        (_ZH, 9, None, False, False, " hello! 回复哦黑色的and magic粉色的圣诞袜"), (_ZH, -3, None, False, False, "圣诞袜"),
        (_ZH, 0, None, False, False, ""), (_ZH, 37, None, False, False, "袜"), (_ZH, -38, None, False, False, ""),
        (_ZH, -37, None, False, False, _ZH)]),
}


def main():
    (HERE / "agg_kats.json").write_text(json.dumps({"single": AGG, "multi": AGG_MULTI,
                                                    "array_map": _array_map_cases()}, indent=1) + "\n")
    (HERE / "join_kats.json").write_text(json.dumps({"inner_join_one_build_op": _join_one_build_op(),
                                                    "array_table_short": _join_array_table_short()}, indent=1)
                                         + "\n")
    typed = dict(JOIN_TYPED)
    typed["full_join_one_build_op"] = dict(typed["full_join_one_build_op"],
                                           expected_rows=_join_one_build_op()["expected_rows"])
    (HERE / "join_type_kats.json").write_text(json.dumps(typed, indent=1) + "\n")
    substr = {name: dict(source=src, cases=[dict(string=c[0], start=c[1], length=c[2], negative=c[3], zero=c[4],
                                                 expected=c[5]) for c in cases])
              for name, (src, cases) in SUBSTR.items()}
    (HERE / "substr_kats.json").write_text(json.dumps(substr, indent=1, ensure_ascii=False) + "\n")


if __name__ == "__main__":
    main()
