"""C ABI and host-logic tests that need no GPU: the library loads, exports every symbol the
header declares, builds OmniVec batches in the reference layout, validates factory arguments
the way the reference does, and refuses to compute without a device."""
import ctypes as C
import subprocess

import numpy as np
import pytest

import omnioperator_gb300 as omg
from omnioperator_gb300 import _capi


def test_library_exports_every_header_symbol():
    syms = omg.header_symbols()
    assert len(syms) >= 45
    out = subprocess.run(["nm", "-D", "--defined-only", str(_capi.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    L = omg.lib()
    for s in syms:
        assert hasattr(L, s)


def test_version_and_policy_roundtrip():
    assert b"sm_103a" in omg.lib().omg_version()
    assert omg.lib().omg_config_get_policy() == omg.POLICY_SPARK
    omg.set_policy(omg.POLICY_GENERIC)
    assert omg.lib().omg_config_get_policy() == omg.POLICY_GENERIC
    omg.set_policy(omg.POLICY_SPARK)
    with pytest.raises(omg.OmgError):
        omg.set_policy(7)


def test_vector_layout_matches_omnivec():
    """Flat values plus LSB-first null bitmap with set bit = NULL (nulls_buffer.h:18-21)."""
    vals = np.arange(-5, 12, dtype=np.int64)
    mask = np.zeros(len(vals), bool)
    mask[[0, 3, 9, 16]] = True
    b = omg.make_batch([omg.LongType()], [vals], [mask])
    L = omg.lib()
    v = L.omg_batch_get(b, 0)
    assert L.omg_vec_size(v) == len(vals) and L.omg_vec_type(v) == omg.OMNI_LONG and L.omg_vec_width(v) == 8
    raw = (C.c_uint8 * 3).from_address(L.omg_vec_nulls(v))
    assert list(raw) == [0b00001001, 0b00000010, 0b00000001]
    assert L.omg_vec_has_null(v) == 1
    (got, gmask), = omg.batch_to_numpy(b)
    assert np.array_equal(got, vals) and np.array_equal(gmask, mask)
    omg.free_batch(b)


def test_decimal128_and_fixed_binary_vectors():
    d = np.array([[1, 0], [2**64 - 1, 2**64 - 1]], dtype=np.uint64)
    fb = np.arange(32, dtype=np.uint8).reshape(2, 16)
    b = omg.make_batch([omg.Decimal128Type(38, 2), omg.FixedBinaryType(16)], [d, fb])
    (dv, _), (fv, _) = omg.batch_to_numpy(b)
    assert np.array_equal(dv, d) and np.array_equal(fv, fb)
    omg.free_batch(b)


def test_factory_validation_matches_reference_rules():
    L = omg.LongType()
    # unsupported function id -> UNSUPPORTED (aggregation.cpp:81-85 throws for unknown types)
    with pytest.raises(omg.OmgError) as e:
        omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[L]], [9])
    assert e.value.status == -2
    # a partial decimal SUM emits (decimal sum, boolean isEmpty): two output types
    d64, d128 = omg.Decimal64Type(18, 2), omg.Decimal128Type(38, 2)
    with pytest.raises(omg.OmgError) as e:
        omg.HashAggregationOperatorFactory([0], [L], [[1]], [[d64]], [[d128]], [0], output_partials=[True])
    assert e.value.status == -1
    # under the container-vector policy a partial int64 SUM declared LONG is SumAggregator<LONG, LONG>
    # (aggregator_factory.h:26-62 picks by the output type): a flat sticky-overflow sum; a SUM
    # declared CONTAINER is refused
    omg.set_policy(omg.POLICY_GENERIC)
    try:
        omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[L]], [0], output_partials=[True]).close()
        omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[L]], [0], input_raws=[False]).close()
        with pytest.raises(omg.OmgError):
            omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[omg.ContainerType()]], [0],
                                               output_partials=[True])
    finally:
        omg.set_policy(omg.POLICY_SPARK)
    # a partial AVG emits (double sum, long count): two output types
    with pytest.raises(omg.OmgError) as e:
        omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[omg.DoubleType()]], [omg.OMNI_AGGREGATION_TYPE_AVG],
                                           output_partials=[True])
    assert e.value.status == -1
    omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[omg.DoubleType(), L]],
                                       [omg.OMNI_AGGREGATION_TYPE_AVG], output_partials=[True]).close()
    # every join type of planNode.h:406-414 builds; an unknown one is UNSUPPORTED
    for jt in range(7):
        omg.HashBuilderOperatorFactory(jt, [L], [0]).close()
    with pytest.raises(omg.OmgError) as e:
        omg.HashBuilderOperatorFactory(7, [L], [0])
    assert e.value.status == -2
    with pytest.raises(omg.OmgError) as e:
        omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_LEFT, [L], [0], build_side=5)
    assert e.value.status == -1
    # a semi join emits probe columns only; the outer-join operator follows full and
    # build-side outer joins only
    sf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_LEFT_SEMI, [L, L], [0])
    with pytest.raises(omg.OmgError) as e:
        omg.LookupJoinOperatorFactory([L], [0], [0], [1], [L], sf)
    assert e.value.status == -2
    with pytest.raises(omg.OmgError) as e:
        omg.LookupOuterJoinOperatorFactory([L], [0], [1], [L], sf)
    assert e.value.status == -2
    sf.close()
    ff = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_FULL, [L, L], [0])
    omg.LookupOuterJoinOperatorFactory([L], [0], [1], [L], ff).close()
    ff.close()
    # join filters: compiled on the host when the factory is made; comparisons / AND / OR / NOT /
    # IS NULL and INT / LONG / DOUBLE arithmetic over integer-like and DOUBLE columns are accepted,
    # anything else is refused with UNSUPPORTED (lookup_join.cpp:175-187 refuses what its code
    # generator cannot compile)
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, L], [0])
    ok = omg.Binary(omg.EXPR_AND, omg.Binary(omg.EXPR_NEQ, omg.Field(0, L), omg.Field(2, L)),
                    omg.Not(omg.IsNull(omg.Field(1, L))))
    omg.LookupJoinOperatorFactory([L, L], [0], [0], [1], [L], bf, filter_expr=ok).close()
    arith = omg.Binary(omg.EXPR_GT, omg.Binary(omg.EXPR_ADD, omg.Field(0, L), omg.Field(2, L), L),
                       omg.Literal(5, L))
    omg.LookupJoinOperatorFactory([L, L], [0], [0], [1], [L], bf, filter_expr=arith).close()
    for bad in (omg.Binary(omg.EXPR_ADD, omg.Field(0, L), omg.Field(2, L)),  # arithmetic with a BOOLEAN result
                omg.Binary(omg.EXPR_EQ, omg.Field(0, omg.VarcharType(4)), omg.Field(2, L))):  # string = long
        with pytest.raises(omg.OmgError) as e:
            omg.LookupJoinOperatorFactory([omg.VarcharType(4), L], [0], [0], [1], [L], bf, filter_expr=bad)
        assert e.value.status == -2
    with pytest.raises(omg.OmgError) as e:  # column 9 is past probe + build columns
        omg.LookupJoinOperatorFactory([L, L], [0], [0], [1], [L], bf,
                                      filter_expr=omg.Binary(omg.EXPR_EQ, omg.Field(9, L), omg.Field(0, L)))
    assert e.value.status == -1
    with pytest.raises(TypeError):
        omg.LookupJoinOperatorFactory([L], [0], [0], [1], [L], bf, filter_expr=object())
    bf.close()
    # strings: VARCHAR columns, literals and substr results compare with one another; substr takes a
    # string and INT / LONG positions; other functions, mixed comparisons and a string-valued
    # filter are refused
    V, I = omg.VarcharType(8), omg.IntType()
    sf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, V], [0])
    sub = omg.Func("substr", [omg.Field(1, V), omg.Literal(1, I), omg.Literal(3, L)], V)
    for good in (omg.Binary(omg.EXPR_NEQ, sub, omg.Field(3, V)),
                 omg.Binary(omg.EXPR_LT, omg.Field(1, V), omg.Literal("abc", V)),
                 omg.IsNull(omg.Func("substr", [omg.Field(3, V), omg.Field(0, L)], V))):
        omg.LookupJoinOperatorFactory([L, V], [0], [0], [1], [V], sf, filter_expr=good).close()
    C8 = omg.DataType(omg.OMNI_CHAR, 0, 0, 8)
    bf_c = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, C8], [0])
    omg.LookupJoinOperatorFactory([L, C8], [0], [0], [1], [C8], bf_c, filter_expr=omg.Binary(
        omg.EXPR_GT, omg.Func("length", [omg.Field(1, C8)], L), omg.Literal(3, L))).close()
    with pytest.raises(omg.OmgError) as e:  # StartsWith is registered for VARCHAR only
        omg.LookupJoinOperatorFactory([L, C8], [0], [0], [1], [C8], bf_c, filter_expr=omg.Func(
            "StartsWith", [omg.Field(1, C8), omg.Literal("a", V)], omg.BooleanType()))
    assert e.value.status == -2
    bf_c.close()
    # numeric CAST: integer-like to integer-like or DOUBLE, DOUBLE to LONG / INT
    omg.LookupJoinOperatorFactory([L, V], [0], [0], [1], [V], sf, filter_expr=omg.Binary(
        omg.EXPR_GT, omg.Func("CAST", [omg.Field(0, L)], omg.DoubleType()), omg.Literal(0.5, omg.DoubleType()))).close()
    for bad_cast in (omg.Func("CAST", [omg.Field(1, V)], L),
                     omg.Func("CAST", [omg.Literal(1.5, omg.DoubleType())], omg.ShortType())):
        with pytest.raises(omg.OmgError) as e:
            omg.LookupJoinOperatorFactory([L, V], [0], [0], [1], [V], sf, filter_expr=omg.Binary(
                omg.EXPR_EQ, bad_cast, omg.Literal(1, bad_cast.dtype)))
        assert e.value.status == -2
    for bad in (omg.Func("upper", [omg.Field(1, V)], V),
                omg.Binary(omg.EXPR_EQ, sub, omg.Field(0, L)),
                omg.Binary(omg.EXPR_AND, omg.Field(1, V), omg.Literal(1, omg.BooleanType())),
                omg.Binary(omg.EXPR_EQ, omg.Func("substr", [omg.Field(0, L), omg.Literal(1, I)], V),
                           omg.Field(3, V)),
                omg.Binary(omg.EXPR_EQ, omg.Func("substr", [omg.Field(1, V), omg.Literal(1.5, omg.DoubleType())],
                                                 V), omg.Field(3, V)),
                sub):
        with pytest.raises(omg.OmgError) as e:
            omg.LookupJoinOperatorFactory([L, V], [0], [0], [1], [V], sf, filter_expr=bad)
        assert e.value.status == -2
    # conditionals and sets: operands of one type (strings interchangeable), IN / BETWEEN over the
    # types the reference's code generator handles, a BOOLEAN root
    S = omg.ShortType()
    for good in (omg.In(omg.Field(0, L), [omg.Literal(1, L), omg.Field(2, L)]),
                 omg.Between(omg.Field(1, V), omg.Literal("a", omg.VarcharType(2)), omg.Field(3, V)),
                 omg.If(omg.IsNull(omg.Field(1, V)), omg.Literal(1, omg.BooleanType()),
                        omg.Binary(omg.EXPR_EQ, omg.Coalesce(omg.Field(1, V), omg.Literal("x", V)), omg.Field(3, V))),
                 omg.Switch([(omg.IsNull(omg.Field(1, V)), omg.Literal(0, omg.BooleanType()))],
                            omg.Literal(1, omg.BooleanType()))):
        omg.LookupJoinOperatorFactory([L, V], [0], [0], [1], [V], sf, filter_expr=good).close()
    for bad in (omg.In(omg.Field(0, L), [omg.Literal(1, I)]),  # LONG IN (INT)
                omg.In(omg.Literal(1, S), [omg.Literal(1, S)]),  # SHORT: not an IN type
                omg.Between(omg.Field(0, L), omg.Literal(1, L), omg.Literal(2.0, omg.DoubleType())),
                omg.If(omg.IsNull(omg.Field(1, V)), omg.Field(1, V), omg.Literal(1, omg.BooleanType())),
                omg.Binary(omg.EXPR_ADD, omg.Field(0, L), omg.Field(2, L), L)):  # not BOOLEAN
        with pytest.raises(omg.OmgError) as e:
            omg.LookupJoinOperatorFactory([L, V], [0], [0], [1], [V], sf, filter_expr=bad)
        assert e.value.status == -2
    sf.close()
    assert omg.get_substr_rules() == (1, 1)
    omg.set_substr_rules(0, 0)
    assert omg.get_substr_rules() == (0, 0)
    omg.set_substr_rules(1, 1)
    with pytest.raises(omg.OmgError):
        omg.set_substr_rules(2, 1)


def test_operator_state_machine_without_gpu():
    """AddInput takes ownership and queues; compute refuses loudly without a device."""
    if omg.device_available():
        pytest.skip("a GPU is visible: covered by the gpu tests")
    L = omg.LongType()
    fac = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[L]], [0])
    op = fac.create_operator()
    assert op.get_status() == omg.OMNI_STATUS_NORMAL
    assert op.get_output() == (0, None)  # no input yet: group_aggregation.cpp:456-458
    op.add_input(omg.make_batch([L, L], [np.arange(4, dtype=np.int64), np.arange(4, dtype=np.int64)]))
    with pytest.raises(omg.OmgError) as e:
        op.get_output()
    assert e.value.status == -8
    op.delete()
    fac.close()
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L], [0])
    bop = bf.create_operator()
    bop.add_input(omg.make_batch([L], [np.arange(4, dtype=np.int64)]))
    bop.set_no_more_input(False)
    assert bop.get_output() == (0, None) and bop.get_status() == omg.OMNI_STATUS_NORMAL  # hash_builder.cpp:184-187
    bop.set_no_more_input(True)
    with pytest.raises(omg.OmgError) as e:
        bop.get_output()
    assert e.value.status == -8
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [0], [L], bf)
    pop = pf.create_operator()
    assert pop.is_blocked()  # kWaitForJoinBuild until the build finished (lookup_join.cpp:270-277)
    pop.delete()
    bop.delete()
    pf.close()
    bf.close()


def test_align_schema_needs_a_raw_partial_plan():
    """AlignSchema of a single-stage aggregation is refused before any device work (and frees
    the batch, as the reference's AlignSchema does)."""
    L = omg.LongType()
    fac = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[L]], [omg.OMNI_AGGREGATION_TYPE_SUM])
    op = fac.create_operator()
    with pytest.raises(omg.OmgError) as e:
        op.align_schema(omg.make_batch([L, L], [np.arange(4, dtype=np.int64)] * 2))
    assert e.value.status == -2
    op.delete()
    fac.close()


def test_device_alloc_fault_injection_is_host_side():
    omg.lib().omg_debug_fail_next_allocs(2)
    omg.lib().omg_debug_fail_next_allocs(0)
    assert omg.lib().omg_last_error() == b""


def test_null_handles_are_rejected():
    L = omg.lib()
    assert L.omg_op_add_input(None, None, None) == -1
    assert b"null" in L.omg_last_error()
    assert L.omg_batch_row_count(None) == -1


def test_batched_aggregation_rejects_sticky_overflow_plans_and_empty_tasks():
    """Batched tasks run only plans without order-dependent (sticky-overflow) sums; that and the
    task list are checked before any device work."""
    L = omg.LongType()
    d64, d128 = omg.Decimal64Type(18, 2), omg.Decimal128Type(38, 2)
    fac = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[d64]], [[d128]], [omg.OMNI_AGGREGATION_TYPE_SUM])
    b = omg.make_batch([L, d64], [np.arange(10, dtype=np.int64), np.arange(10, dtype=np.int64)])
    with pytest.raises(omg.OmgError) as ei:
        omg.AggBatch(fac, [b])
    assert ei.value.status == -2  # OMG_ERR_UNSUPPORTED
    fac2 = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[L]], [omg.OMNI_AGGREGATION_TYPE_SUM])
    empty = omg.make_batch([L, L], [np.zeros(0, np.int64), np.zeros(0, np.int64)])
    with pytest.raises(omg.OmgError) as ei:
        omg.AggBatch(fac2, [b, empty])
    assert ei.value.status == -1  # OMG_ERR_INVALID_ARG
    omg.free_batches([b, empty])
    fac.close()
    fac2.close()


def test_dictionary_vectors_on_the_host():
    """VectorHelper::CreateDictionaryVector: ids index a flat dictionary whose buffers the new vector
    shares; NULL-ness comes from the dictionary row; out-of-range ids are refused."""
    L = omg.lib()
    d = omg.new_host_vector(omg.LongType(), np.array([5, 6, 7], dtype=np.int64), np.array([False, True, False]))
    v = omg.new_dictionary_vector(np.array([2, 1, 0, 2], dtype=np.int32), d)
    assert L.omg_vec_encoding(v) == 1 and L.omg_vec_encoding(d) == 0
    assert L.omg_vec_size(v) == 4 and L.omg_vec_type(v) == omg.OMNI_LONG and L.omg_vec_width(v) == 8
    assert L.omg_vec_has_null(v) == 1
    for bad in ([0, 3], [-1]):
        with pytest.raises(omg.OmgError) as ei:
            omg.new_dictionary_vector(np.array(bad, dtype=np.int32), d)
        assert ei.value.status == -1
    L.omg_vec_free(d)
    L.omg_vec_free(v)


def test_noalloc_entry_refuses_string_columns_before_touching_a_device():
    V, L = omg.VarcharType(8), omg.LongType()
    f = omg.HashAggregationOperatorFactory([0], [V], [[1]], [[L]], [[L]], [omg.OMNI_AGGREGATION_TYPE_SUM])
    n = C.c_int64(0)
    rc = omg.lib().omg_hashagg_run_noalloc(f.handle, None, None, 0, 0, None, None, 0, 16, C.byref(n), None)
    assert rc == -2
    f.close()


def test_mask_columns_are_checked_on_the_host():
    """A mask list has one entry per aggregator; the allocation-free entry refuses masked plans
    (their NULL bitmaps are per-call device allocations) before it touches a device."""
    L = omg.LongType()
    with pytest.raises(ValueError):
        omg.HashAggregationOperatorFactory([0], [L], [[1], [1]], [[L], [L]], [[L], [L]],
                                           [omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_MIN],
                                           mask_cols=[2, 0xFFFFFFFF, 2])
    f = omg.HashAggregationOperatorFactory([0], [L], [[1], [1]], [[L], [L]], [[L], [L]],
                                           [omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_MIN],
                                           mask_cols=[2, 0xFFFFFFFF])
    n = C.c_int64(0)
    rc = omg.lib().omg_hashagg_run_noalloc(f.handle, None, None, 0, 0, None, None, 0, 16, C.byref(n), None)
    assert rc == -2
    f.close()


def test_two_stage_decimal_sum_plans_are_checked_on_the_host():
    """Partial decimal SUM: (decimal sum, boolean isEmpty) outputs; a merging stage reads the
    pair; the wrong shapes are refused while the factory compiles its plan."""
    L, B, D128 = omg.LongType(), omg.BooleanType(), omg.Decimal128Type(38, 2)
    SUM = omg.OMNI_AGGREGATION_TYPE_SUM
    for cols, ins, outs, raw, partial in (([[1]], [[D128]], [[D128, B]], True, True),
                                          ([[1, 2]], [[D128, B]], [[D128]], False, False),
                                          ([[1, 2]], [[D128, B]], [[D128, B]], False, True)):
        omg.HashAggregationOperatorFactory([0], [L], cols, ins, outs, [SUM], input_raws=[raw],
                                           output_partials=[partial]).close()
    for cols, ins, outs in (([[1]], [[D128]], [[D128]]), ([[1, 2]], [[D128, L]], [[D128]])):
        with pytest.raises(omg.OmgError) as e:
            omg.HashAggregationOperatorFactory([0], [L], cols, ins, outs, [SUM], input_raws=[len(cols[0]) == 1],
                                               output_partials=[len(cols[0]) == 1])
        assert e.value.status == -1


def test_spill_settings_are_checked_on_the_host():
    """Spill takes fixed-width plans (order-dependent sums included) and VARCHAR keys, not
    VARCHAR MIN/MAX, and needs a budget."""
    L, V = omg.LongType(), omg.VarcharType(8)
    ok = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[L]], [omg.OMNI_AGGREGATION_TYPE_SUM])
    op = ok.create_operator()
    op.set_spill(True, 1 << 20)
    assert op.spilled_bytes() == 0
    with pytest.raises(omg.OmgError) as e:
        op.set_spill(True, 0)
    assert e.value.status == -1
    op.delete()
    ok.close()
    d64, d128 = omg.Decimal64Type(18, 2), omg.Decimal128Type(38, 2)
    # VARCHAR keys spill as dictionary ids; MIN/MAX of VARCHAR values does not spill
    fac = omg.HashAggregationOperatorFactory([0], [V], [[1]], [[L]], [[L]], [omg.OMNI_AGGREGATION_TYPE_SUM])
    op = fac.create_operator()
    op.set_spill(True, 1 << 20)
    op.delete()
    fac.close()
    fac = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[V]], [[V]], [omg.OMNI_AGGREGATION_TYPE_MIN])
    op = fac.create_operator()
    with pytest.raises(omg.OmgError) as e:
        op.set_spill(True, 1 << 20)
    assert e.value.status == -2
    op.delete()
    fac.close()
    # order-dependent (sticky-overflow) sums spill through the order-preserving partition pass
    fac = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[d64]], [[d128]], [omg.OMNI_AGGREGATION_TYPE_SUM])
    op = fac.create_operator()
    op.set_spill(True, 1 << 20)
    op.delete()
    fac.close()


def test_learned_join_strategy_choice():
    """JOIN_LEARNED reads a hot key off the learned splits (a run of equal splits longer than 7.5%
    of the partitions): then the direct probe, otherwise hash partitions."""
    L = omg.LongType()
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, L], [0])
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1], [L], bf)
    op = pf.create_operator()
    spread = np.arange(15, dtype=np.int64) * 100  # 2^4 - 1 distinct splits
    hot = np.array([0, 100, 200, 500, 500, 500, 500, 500, 600, 700, 800, 900, 1000, 1100, 1200], dtype=np.int64)
    op.set_join_strategy(omg.JOIN_LEARNED, 4, spread)
    assert op.join_strategy() == omg.JOIN_HASH_PARTITIONED
    op.set_join_strategy(omg.JOIN_LEARNED, 4, hot)  # a run of 5 of 16 splits
    assert op.join_strategy() == omg.JOIN_DIRECT
    op.set_join_strategy(omg.JOIN_RANGE_PARTITIONED, 4, hot)
    assert op.join_strategy() == omg.JOIN_RANGE_PARTITIONED
    op.delete()
    pf.close()
    bf.close()


def test_quantile_join_strategy_choice():
    """JOIN_QUANTILE takes the choice from exact sample quantiles (no network): a key holding a
    share q of the sample repeats as about q * 2^bits splits, and a run longer than 15% of the
    partitions selects the direct probe."""
    rng = np.random.default_rng(3)
    L = omg.LongType()
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, L], [0])
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1], [L], bf)
    op = pf.create_operator()
    for share, want in ((0.30, omg.JOIN_DIRECT), (0.05, omg.JOIN_HASH_PARTITIONED)):
        sample = rng.integers(0, 2**40, 65536).astype(np.int64)
        sample[: int(share * len(sample))] = 12345
        splits = omg.quantile_splits(sample, bits=8)
        assert np.all(np.diff(splits) >= 0)
        ranks = np.searchsorted(np.sort(sample), splits, side="left")
        assert np.all(np.abs(ranks - np.arange(1, 256) * len(sample) // 256) <= share * len(sample) + 1)
        op.set_join_strategy(omg.JOIN_QUANTILE, 8, splits)
        assert op.join_strategy() == want
    op.delete()
    pf.close()
    bf.close()


def test_container_avg_types_accepted_only_for_avg():
    """A partial AVG may emit one CONTAINER column and a merging AVG may read one; other
    aggregators refuse container types (CPU: plan compilation only)."""
    L, D, C_ = omg.LongType(), omg.DoubleType(), omg.ContainerType()
    AVG, SUM = omg.OMNI_AGGREGATION_TYPE_AVG, omg.OMNI_AGGREGATION_TYPE_SUM
    omg.HashAggregationOperatorFactory([0], [L], [[1]], [[D]], [[C_]], [AVG], output_partials=[True]).close()
    omg.HashAggregationOperatorFactory([0], [L], [[1]], [[C_]], [[D]], [AVG], input_raws=[False]).close()
    omg.HashAggregationOperatorFactory([0], [L], [[1]], [[C_]], [[C_]], [AVG], input_raws=[False],
                                       output_partials=[True]).close()
    for args, kw in [(([0], [L], [[1]], [[L]], [[C_]], [SUM]), {}),
                     (([0], [L], [[1]], [[C_]], [[L]], [SUM]), {"input_raws": [False]}),
                     (([0], [L], [[1]], [[C_]], [[D]], [AVG]), {})]:
        with pytest.raises(omg.OmgError) as e:
            omg.HashAggregationOperatorFactory(*args, **kw)
        assert e.value.status == -1
