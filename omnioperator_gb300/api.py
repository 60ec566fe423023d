"""Python mirror of OmniOperator's operator interface for the hash aggregation / hash join path.

Names and argument meaning follow the reference's C++ API (operator/operator.h,
operator/aggregation/group_aggregation.h:217-249, operator/join/hash_builder.h:28-31,
operator/join/lookup_join.h:148-152); every call goes through the C ABI of
libomniop_gb300.so.  Batches are OmniVec VectorBatch handles: ``make_batch`` builds a host
batch from numpy columns, ``batch_to_numpy`` reads one back.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._capi import OmgDataType, OmgError, check, lib

# DataTypeId (type/data_type.h:40-74)
OMNI_INT, OMNI_LONG, OMNI_DOUBLE, OMNI_BOOLEAN, OMNI_SHORT = 1, 2, 3, 4, 5
OMNI_DECIMAL64, OMNI_DECIMAL128, OMNI_DATE32, OMNI_DATE64, OMNI_TIMESTAMP = 6, 7, 8, 9, 12
OMNI_BYTE, OMNI_FLOAT, OMNI_FIXEDBINARY = 18, 19, 40
OMNI_VARCHAR, OMNI_CHAR, OMNI_CONTAINER = 15, 16, 17
# FunctionType (operator/util/function_type.h:11-27)
OMNI_AGGREGATION_TYPE_SUM, OMNI_AGGREGATION_TYPE_COUNT_COLUMN = 0, 1
OMNI_AGGREGATION_TYPE_COUNT_ALL, OMNI_AGGREGATION_TYPE_AVG = 2, 3
OMNI_AGGREGATION_TYPE_MAX, OMNI_AGGREGATION_TYPE_MIN = 5, 6
# JoinType (plannode/planNode.h:406-414)
OMNI_JOIN_TYPE_INNER, OMNI_JOIN_TYPE_LEFT, OMNI_JOIN_TYPE_RIGHT, OMNI_JOIN_TYPE_FULL = 0, 1, 2, 3
OMNI_JOIN_TYPE_LEFT_SEMI, OMNI_JOIN_TYPE_LEFT_ANTI, OMNI_JOIN_TYPE_EXISTENCE = 4, 5, 6
OMNI_BUILD_UNKNOWN, OMNI_BUILD_LEFT, OMNI_BUILD_RIGHT = 0, 1, 2
# OmniStatus (operator/status.h:9-13)
OMNI_STATUS_NORMAL, OMNI_STATUS_FINISHED, OMNI_STATUS_ERROR = 0, 1, -1
# SupportContainerVecRule (util/policy.h:160-167)
POLICY_SPARK, POLICY_GENERIC = 0, 1
AGG_STRATEGY_AUTO, AGG_STRATEGY_SMEM, AGG_STRATEGY_GLOBAL, AGG_STRATEGY_PARTITIONED = 0, 1, 2, 3
AGG_SIZING_SAMPLE, AGG_SIZING_HLL = 0, 1

_NP = {OMNI_INT: np.int32, OMNI_LONG: np.int64, OMNI_DOUBLE: np.float64, OMNI_BOOLEAN: np.int8,
       OMNI_SHORT: np.int16, OMNI_DECIMAL64: np.int64, OMNI_DATE32: np.int32, OMNI_DATE64: np.int64,
       OMNI_TIMESTAMP: np.int64, OMNI_BYTE: np.int8, OMNI_FLOAT: np.float32}
_WIDTH = {OMNI_DECIMAL128: 16, **{k: np.dtype(v).itemsize for k, v in _NP.items()}}


@dataclass(frozen=True)
class DataType:
    id: int
    precision: int = 0
    scale: int = 0
    width: int = 0

    @property
    def byte_width(self) -> int:
        if self.id in (OMNI_VARCHAR, OMNI_CHAR, OMNI_CONTAINER):
            return 0  # variable length, or a container of field vectors
        return self.width if self.id == OMNI_FIXEDBINARY else _WIDTH[self.id]


def IntType():
    return DataType(OMNI_INT)


def LongType():
    return DataType(OMNI_LONG)


def ShortType():
    return DataType(OMNI_SHORT)


def DoubleType():
    return DataType(OMNI_DOUBLE)


def BooleanType():
    return DataType(OMNI_BOOLEAN)


def Decimal64Type(precision=18, scale=0):
    return DataType(OMNI_DECIMAL64, precision, scale)


def ContainerType():
    """OMNI_CONTAINER: a partial AVG's (double sum, long count) as one container column, the
    output type of a partial AVG (and the input type of a final AVG) under the container-vector
    policy (operator/aggregation/container_vector.h)."""
    return DataType(OMNI_CONTAINER)


def Decimal128Type(precision=38, scale=0):
    return DataType(OMNI_DECIMAL128, precision, scale)


def FixedBinaryType(width):
    return DataType(OMNI_FIXEDBINARY, 0, 0, width)


def VarcharType(width=0):
    """VARCHAR of at most `width` bytes (type/data_type.h VarcharDataType)."""
    return DataType(OMNI_VARCHAR, 0, 0, width)


def _types(types):
    arr = (OmgDataType * max(len(types), 1))()
    for i, t in enumerate(types):
        arr[i] = OmgDataType(t.id, t.precision, t.scale, t.width)
    return arr


def _i32(vals):
    return (C.c_int32 * max(len(vals), 1))(*vals)


def _u32(vals):
    return (C.c_uint32 * max(len(vals), 1))(*vals)


def set_policy(policy: int) -> None:
    """ConfigUtil::SetSupportContainerVecRule: POLICY_SPARK (default) or POLICY_GENERIC."""
    check(lib().omg_config_set_policy(policy))


def set_substr_rules(negative: int, zero: int) -> None:
    """ConfigUtil::SetNegativeStartIndexOutOfBoundsRule / SetZeroStartIndexSupportRule for join
    factories created afterwards: negative 1 INTERCEPT_FROM_BEYOND (default) or 0 EMPTY_STRING,
    zero 1 IS_SUPPORT (default) or 0 IS_NOT_SUPPORT."""
    check(lib().omg_config_set_substr_rules(negative, zero))


def get_substr_rules() -> tuple[int, int]:
    n, z = C.c_int32(), C.c_int32()
    check(lib().omg_config_get_substr_rules(C.byref(n), C.byref(z)))
    return n.value, z.value


def device_available() -> bool:
    return bool(lib().omg_device_available())


# ----------------------------------------------------------------------------------- vectors
def _np_view(ptr: int, dtype, count: int) -> np.ndarray:
    if count == 0:
        return np.zeros(0, dtype=dtype)
    buf = (C.c_uint8 * (count * np.dtype(dtype).itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype, count=count)


def new_host_vector(dtype: DataType, values: np.ndarray, nulls: np.ndarray | None = None) -> int:
    """A host (pinned) OmniVec flat vector holding `values` (decimal128: (n, 2) uint64 low/high;
    fixed binary: (n, width) uint8) with an optional boolean null mask."""
    n = len(values)
    out = C.c_void_p()
    if dtype.id in (OMNI_VARCHAR, OMNI_CHAR):
        # values: a sequence of bytes / str
        enc = [v.encode() if isinstance(v, str) else bytes(v) for v in values]
        offs = np.zeros(n + 1, dtype=np.int32)
        if n:
            offs[1:] = np.cumsum([len(v) for v in enc])
        data = b"".join(enc)
        check(lib().omg_vec_new_varchar(dtype.id, n, len(data), C.byref(out)))
        vec = out.value
        C.memmove(lib().omg_vec_offsets(vec), offs.ctypes.data, offs.nbytes)
        if data:
            C.memmove(lib().omg_vec_values(vec), data, len(data))
        if nulls is not None and np.any(nulls):
            bits = np.packbits(np.asarray(nulls, dtype=bool), bitorder="little")
            C.memmove(lib().omg_vec_nulls(vec), bits.ctypes.data, bits.size)
            check(lib().omg_vec_set_null_flag(vec, 1))
        return vec
    if dtype.id == OMNI_FIXEDBINARY:
        check(lib().omg_vec_new_fixed(dtype.width, n, C.byref(out)))
    else:
        check(lib().omg_vec_new(dtype.id, n, C.byref(out)))
    vec = out.value
    raw = np.ascontiguousarray(values).view(np.uint8).reshape(-1)
    if raw.size:
        C.memmove(lib().omg_vec_values(vec), raw.ctypes.data, raw.size)
    if nulls is not None and np.any(nulls):
        bits = np.packbits(np.asarray(nulls, dtype=bool), bitorder="little")
        C.memmove(lib().omg_vec_nulls(vec), bits.ctypes.data, bits.size)
        check(lib().omg_vec_set_null_flag(vec, 1))
    return vec


def new_dictionary_vector(ids, dictionary: int) -> int:
    """A dictionary-encoded host vector: row i is row ids[i] of the flat vector `dictionary`
    (which stays the caller's)."""
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    out = C.c_void_p()
    check(lib().omg_vec_new_dictionary(ids.ctypes.data if ids.size else None, len(ids), dictionary, C.byref(out)))
    return out.value


def make_dict_batch(types, columns, nulls=None, encode=()) -> int:
    """make_batch, with the columns whose indices are in `encode` dictionary-encoded: each such
    column becomes ids into a dictionary of its distinct (value, null) entries, in reverse order
    of first appearance so that ids differ from row numbers."""
    n = len(columns[0]) if columns else 0
    out = C.c_void_p()
    check(lib().omg_batch_new(n, C.byref(out)))
    batch = out.value
    for i, (t, col) in enumerate(zip(types, columns)):
        m = None if nulls is None else nulls[i]
        if i not in encode:
            check(lib().omg_batch_append(batch, new_host_vector(t, col, m)))
            continue
        keys = {}
        ids = np.empty(n, dtype=np.int32)
        for r in range(n):
            isnull = m is not None and bool(m[r])
            v = col[r]
            k = (True, None) if isnull else (False, bytes(v) if isinstance(v, (bytes, bytearray, str)) else
                                               np.asarray(v).tobytes())
            ids[r] = keys.setdefault(k, len(keys))
        order = list(keys.items())[::-1]
        remap = {old: new for new, (_, old) in enumerate(order)}
        ids = np.array([remap[x] for x in ids], dtype=np.int32)
        first = {}
        for r in range(n):
            first.setdefault(ids[r], r)
        rows = [first[j] for j in range(len(order))]
        dvals = [col[r] for r in rows] if col.dtype == object else np.asarray(col)[rows]
        if col.dtype == object:
            dvals = np.array(dvals, dtype=object)
        dnull = None if m is None else np.asarray(m)[rows]
        dvec = new_host_vector(t, dvals, dnull)
        try:
            check(lib().omg_batch_append(batch, new_dictionary_vector(ids, dvec)))
        finally:
            check(lib().omg_vec_free(dvec))
    return batch


def make_batch(types, columns, nulls=None) -> int:
    """A host VectorBatch from numpy columns (all of equal length)."""
    n = len(columns[0]) if columns else 0
    out = C.c_void_p()
    check(lib().omg_batch_new(n, C.byref(out)))
    batch = out.value
    for i, (t, col) in enumerate(zip(types, columns)):
        m = None if nulls is None else nulls[i]
        check(lib().omg_batch_append(batch, new_host_vector(t, col, m)))
    return batch


def wrap_device_batch(types, rows: int, value_ptrs, null_ptrs=None) -> int:
    """A VectorBatch of non-owning DEVICE vectors over caller memory (e.g. torch tensors)."""
    out = C.c_void_p()
    check(lib().omg_batch_new(rows, C.byref(out)))
    batch = out.value
    for i, (t, vp) in enumerate(zip(types, value_ptrs)):
        v = C.c_void_p()
        np_ = None if null_ptrs is None else null_ptrs[i]
        check(lib().omg_vec_wrap_device(t.id, t.width, rows, C.c_void_p(vp), C.c_void_p(np_) if np_ else None,
                                        C.byref(v)))
        check(lib().omg_batch_append(batch, v.value))
    return batch


def batch_to_device(batch: int) -> int:
    out = C.c_void_p()
    check(lib().omg_batch_to_device(batch, C.byref(out)))
    return out.value


def batch_to_host(batch: int) -> int:
    out = C.c_void_p()
    check(lib().omg_batch_to_host(batch, C.byref(out)))
    return out.value


def free_batch(batch: int | None) -> None:
    if batch:
        check(lib().omg_batch_free(batch))


def batch_row_count(batch: int) -> int:
    return lib().omg_batch_row_count(batch)


def free_batches(batches) -> None:
    """Free many batches with one call (omg_batch_free_many)."""
    n = len(batches)
    if n:
        arr = (C.c_void_p * n)(*batches)
        check(lib().omg_batch_free_many(arr, n))


def batch_to_numpy(batch: int):
    """[(values, null_mask)] of a host batch (copies); a container vector (a partial AVG under
    the container-vector policy) gives ("container", [(values, null_mask) per field])."""
    L = lib()
    n = L.omg_batch_row_count(batch)
    cols = []
    for i in range(L.omg_batch_vector_count(batch)):
        v = L.omg_batch_get(batch, i)
        nf = L.omg_vec_num_fields(v)
        if nf > 0:
            cols.append(("container", [_vec_to_numpy(L, L.omg_vec_field(v, f), n) for f in range(nf)]))
            continue
        cols.append(_vec_to_numpy(L, v, n))
    return cols


def _vec_to_numpy(L, v, n):
    if True:
        if L.omg_vec_is_device(v):
            raise ValueError("device batch: copy it to the host first (batch_to_host)")
        t = L.omg_vec_type(v)
        w = L.omg_vec_width(v)
        ptr = L.omg_vec_values(v)
        if t in (OMNI_VARCHAR, OMNI_CHAR):
            offs = _np_view(L.omg_vec_offsets(v), np.int32, n + 1).copy() if n else np.zeros(1, np.int32)
            total = int(offs[-1]) if n else 0
            raw = bytes(_np_view(ptr, np.uint8, total)) if total else b""
            vals = np.empty(n, dtype=object)
            for j in range(n):
                vals[j] = raw[offs[j]:offs[j + 1]]
        elif t == OMNI_DECIMAL128:
            vals = _np_view(ptr, np.uint64, 2 * n).reshape(n, 2).copy()
        elif t == OMNI_FIXEDBINARY:
            vals = _np_view(ptr, np.uint8, w * n).reshape(n, w).copy()
        else:
            vals = _np_view(ptr, _NP[t], n).copy()
        nptr = L.omg_vec_nulls(v)
        if nptr:
            bits = _np_view(nptr, np.uint8, (n + 7) // 8)
            mask = np.unpackbits(bits, bitorder="little")[:n].astype(bool)
        else:
            mask = np.zeros(n, dtype=bool)
        return vals, mask


# --------------------------------------------------------------------------------- operators
class Operator:
    """operator/operator.h:22-266 through the C ABI."""

    def __init__(self, handle: int):
        self.handle = handle

    def init(self):
        check(lib().omg_op_init(self.handle))

    def add_input(self, batch: int) -> int:
        """Operator::AddInput: the operator takes ownership of `batch`."""
        ret = C.c_int32(0)
        check(lib().omg_op_add_input(self.handle, batch, C.byref(ret)))
        return ret.value

    def get_output(self):
        """Operator::GetOutput -> (return value, batch handle or None)."""
        out = C.c_void_p()
        ret = C.c_int32(0)
        check(lib().omg_op_get_output(self.handle, C.byref(out), C.byref(ret)))
        return ret.value, out.value

    def add_inputs(self, batches) -> None:
        """AddInput of each batch in order, one C call (omg_op_add_inputs).  `batches` is a
        sequence of handles or a prepared ctypes array of c_void_p."""
        arr = batches if isinstance(batches, C.Array) else (C.c_void_p * len(batches))(*batches)
        consumed = C.c_int32(0)
        check(lib().omg_op_add_inputs(self.handle, arr, len(arr), C.byref(consumed)))

    def get_outputs(self, max_batches: int = 4096):
        """GetOutput until no batch is produced or `max_batches` were returned, one C call
        (omg_op_get_outputs) -> (list of batch handles, total rows)."""
        arr = getattr(self, "_outs", None)
        if arr is None or len(arr) < max_batches:
            arr = self._outs = (C.c_void_p * max_batches)()  # reused across calls
        n = C.c_int32(0)
        rows = C.c_int64(0)
        check(lib().omg_op_get_outputs(self.handle, arr, max_batches, C.byref(n), C.byref(rows)))
        return list(arr[: n.value]), rows.value

    def set_join_strategy(self, strategy: int, bits: int = 12, splits=None):
        """LookupJoin probe strategy (JOIN_DIRECT, JOIN_HASH_PARTITIONED, JOIN_RANGE_PARTITIONED)."""
        if splits is None:
            check(lib().omg_op_set_join_strategy(self.handle, strategy, bits, None, 0))
        else:
            a = np.ascontiguousarray(splits, dtype=np.int64)
            check(lib().omg_op_set_join_strategy(self.handle, strategy, bits,
                                                 a.ctypes.data_as(C.POINTER(C.c_int64)), len(a)))

    def join_strategy(self) -> int:
        """The probe strategy in effect (JOIN_LEARNED resolved)."""
        out = C.c_int32(0)
        check(lib().omg_op_join_strategy(self.handle, C.byref(out)))
        return out.value

    def sizing_log(self) -> dict:
        """HashAggregation sizing record (omg_op_get_sizing_log)."""
        arr = (C.c_int64 * 32)()
        n = C.c_int32(0)
        check(lib().omg_op_get_sizing_log(self.handle, arr, 32, C.byref(n)))
        v = list(arr[: n.value])
        return {"rows": v[0], "sketch": v[1:17], "estimate": v[17], "part_bits": v[18], "groups": v[19],
                "plain_estimate": v[20], "learned": bool(v[21]), "smem_front": bool(v[22]), "raw": v}

    def get_status(self) -> int:
        return lib().omg_op_status(self.handle)

    def no_more_input(self):
        check(lib().omg_op_no_more_input(self.handle))

    def set_no_more_input(self, flag: bool):
        check(lib().omg_op_set_no_more_input(self.handle, 1 if flag else 0))

    def needs_input(self) -> bool:
        return bool(lib().omg_op_needs_input(self.handle))

    def is_blocked(self) -> bool:
        return bool(lib().omg_op_is_blocked(self.handle))

    def get_hashmap_unique_keys(self) -> int:
        return lib().omg_op_hashmap_unique_keys(self.handle)

    def align_schema(self, batch: int) -> int:
        """AlignSchema: the batch (consumed) as one-row partial results; a new batch handle."""
        out = C.c_void_p()
        check(lib().omg_op_align_schema(self.handle, batch, C.byref(out)))
        return out.value

    def set_stream(self, stream_handle: int):
        check(lib().omg_op_set_stream(self.handle, C.c_void_p(stream_handle)))

    def set_device_output(self, on: bool):
        check(lib().omg_op_set_device_output(self.handle, 1 if on else 0))

    def set_agg_strategy(self, strategy: int, capacity_hint: int = 0):
        check(lib().omg_op_set_agg_strategy(self.handle, strategy, capacity_hint))

    def set_agg_sizing(self, mode: int):
        """AGG_SIZING_SAMPLE (row-sample key sketch, default) or AGG_SIZING_HLL (HyperLogLog of
        every row's key) for the group-count estimate."""
        check(lib().omg_op_set_agg_sizing(self.handle, mode))

    def set_spill(self, enabled: bool, device_budget_bytes: int = 0):
        """Aggregation spill to pinned host memory above a device-memory budget."""
        check(lib().omg_op_set_spill(self.handle, 1 if enabled else 0, device_budget_bytes))

    def spilled_bytes(self) -> int:
        return lib().omg_op_spilled_bytes(self.handle)

    def counters(self):
        arr = (C.c_int64 * 12)()
        check(lib().omg_op_get_counters(self.handle, arr, 12))
        return {"launches": arr[0], "resizes": arr[1], "retried_rows": arr[2], "groups": arr[3],
                "ordered_groups": arr[4], "output_rows": arr[5], "kernel_ns": arr[6], "kernel_launches": arr[7],
                "launch_host_ns": arr[8], "wait_ns": arr[9], "carve_ns": arr[10], "free_input_ns": arr[11]}

    def close(self):
        check(lib().omg_op_close(self.handle))

    def delete(self):
        """Operator::DeleteOperator (Close + delete)."""
        if self.handle:
            check(lib().omg_op_delete(self.handle))
            self.handle = None

    def drain(self):
        """GetOutput until nothing more comes: list of output batch handles."""
        outs = []
        while True:
            _, b = self.get_output()
            if not b:
                return outs
            outs.append(b)


class OperatorFactory:
    def __init__(self, handle: int):
        self.handle = handle

    def create_operator(self) -> Operator:
        out = C.c_void_p()
        check(lib().omg_factory_create_operator(self.handle, C.byref(out)))
        return Operator(out.value)

    def close(self):
        if self.handle:
            check(lib().omg_factory_destroy(self.handle))
            self.handle = None


class HashAggregationOperatorFactory(OperatorFactory):
    """HashAggregationOperatorFactory(groupByCol, groupInputTypes, aggsCols, aggInputTypes,
    aggOutputTypes, aggFuncTypes, maskColsVector, inputRaws, outputPartials, overflowAsNull)."""

    def __init__(self, group_by_cols, group_input_types, aggs_cols, agg_input_types, agg_output_types,
                 agg_func_types, mask_cols=None, input_raws=None, output_partials=None, overflow_as_null=False):
        n_agg = len(agg_func_types)
        col_off, cols, in_types = [0], [], []
        for c, t in zip(aggs_cols, agg_input_types):
            cols.extend(c)
            in_types.extend(t)
            col_off.append(len(cols))
        out_off, out_types = [0], []
        for t in agg_output_types:
            out_types.extend(t)
            out_off.append(len(out_types))
        if mask_cols is not None and len(mask_cols) != n_agg:
            raise ValueError("one mask column entry per aggregator is required")
        masks = [-1] * n_agg if mask_cols is None else [(-1 if m in (None, -1, 0xFFFFFFFF) else m) for m in mask_cols]
        raws = [1] * n_agg if input_raws is None else [1 if r else 0 for r in input_raws]
        partials = [0] * n_agg if output_partials is None else [1 if p else 0 for p in output_partials]
        out = C.c_void_p()
        check(lib().omg_hashagg_factory_create(
            _u32(group_by_cols), _types(group_input_types), len(group_by_cols), _u32(agg_func_types), n_agg,
            _i32(col_off), _u32(cols), _types(in_types), _i32(out_off), _types(out_types), _i32(masks),
            (C.c_uint8 * max(n_agg, 1))(*raws), (C.c_uint8 * max(n_agg, 1))(*partials),
            1 if overflow_as_null else 0, C.byref(out)))
        super().__init__(out.value)
        self._sizer = None

    def set_sizer(self, model) -> None:
        """Size the operators created afterwards with a learned model (sizer.SizingModel), or
        the plain sketch estimate when `model` is None."""
        check(lib().omg_hashagg_factory_set_sizer(self.handle, None if model is None else model.handle))
        self._sizer = model  # keep the model alive while the factory may use it


class HashBuilderOperatorFactory(OperatorFactory):
    """HashBuilderOperatorFactory::CreateHashBuilderOperatorFactory(joinType[, buildSide],
    buildTypes, buildHashCols, buildHashColsCount, operatorCount)."""

    def __init__(self, join_type, build_types, build_hash_cols, operator_count=1, build_side=None):
        out = C.c_void_p()
        if build_side is None:
            check(lib().omg_hashbuilder_factory_create(join_type, _types(build_types), len(build_types),
                                                       _i32(build_hash_cols), len(build_hash_cols), operator_count,
                                                       C.byref(out)))
        else:
            check(lib().omg_hashbuilder_factory_create_side(join_type, build_side, _types(build_types),
                                                            len(build_types), _i32(build_hash_cols),
                                                            len(build_hash_cols), operator_count, C.byref(out)))
        super().__init__(out.value)


# --------------------------------------------------------------------------- join filter expressions
EXPR_EQ, EXPR_NEQ, EXPR_LT, EXPR_LTE, EXPR_GT, EXPR_GTE, EXPR_AND, EXPR_OR, EXPR_NOT = range(9)
EXPR_ADD, EXPR_SUB, EXPR_MUL, EXPR_DIV, EXPR_MOD, EXPR_TRY_ADD, EXPR_TRY_SUB, EXPR_TRY_MUL, EXPR_TRY_DIV = range(9, 18)


class Field:
    """FieldExpr: column `col` of the joined row (probe columns first, then build columns)."""

    def __init__(self, col: int, dtype: DataType):
        self.col, self.dtype = col, dtype


class Literal:
    """LiteralExpr of an integer-like / BOOLEAN (int value), DOUBLE (float value) or VARCHAR/CHAR
    (bytes or str value, str as UTF-8) type."""

    def __init__(self, value, dtype: DataType, is_null: bool = False):
        self.value, self.dtype, self.is_null = value, dtype, is_null


class Binary:
    """BinaryExpr(op, left, right[, dtype]): a comparison / AND / OR (BOOLEAN), or arithmetic
    (EXPR_ADD .. EXPR_TRY_DIV) whose result type `dtype` is INT, LONG or DOUBLE."""

    def __init__(self, op: int, left, right, dtype: DataType | None = None):
        self.op, self.left, self.right, self.dtype = op, left, right, dtype


class Func:
    """FuncExpr(name, args, dtype): a function call; the join filter compiles "substr" (a string,
    then INT or LONG start and optional length), returning VARCHAR/CHAR `dtype`."""

    def __init__(self, name: str, args: list, dtype: DataType):
        self.name, self.args, self.dtype = name, list(args), dtype


class If:
    """IfExpr(cond, then, else): `then` when cond is TRUE, else `else_`."""

    def __init__(self, cond, then, else_):
        self.cond, self.then, self.else_ = cond, then, else_


class Switch:
    """SwitchExpr: CASE WHEN whens[0][0] THEN whens[0][1] ... ELSE else_ END."""

    def __init__(self, whens: list, else_):
        self.whens, self.else_ = [tuple(w) for w in whens], else_


class Coalesce:
    def __init__(self, value1, value2):
        self.value1, self.value2 = value1, value2


class In:
    """InExpr: value IN (items...)."""

    def __init__(self, value, items: list):
        self.value, self.items = value, list(items)


class Between:
    def __init__(self, value, lower, upper):
        self.value, self.lower, self.upper = value, lower, upper


class Not:
    def __init__(self, child):
        self.child = child


class IsNull:
    def __init__(self, child):
        self.child = child


def _expr_handle(e) -> int:
    """The C expression tree of `e` (the caller frees the root with omg_expr_free)."""
    out = C.c_void_p()
    L = lib()
    if isinstance(e, Field):
        t = _types([e.dtype])
        check(L.omg_expr_field(e.col, t, C.byref(out)))
    elif isinstance(e, Literal) and e.dtype.id in (OMNI_VARCHAR, OMNI_CHAR):
        raw = b"" if e.is_null else (e.value.encode() if isinstance(e.value, str) else bytes(e.value))
        check(L.omg_expr_literal_string(raw, len(raw), _types([e.dtype]), 1 if e.is_null else 0, C.byref(out)))
    elif isinstance(e, (Func, If, Switch, Coalesce, In, Between)):
        if isinstance(e, Func):
            kids = e.args
        elif isinstance(e, If):
            kids = [e.cond, e.then, e.else_]
        elif isinstance(e, Switch):
            kids = [x for w in e.whens for x in w] + [e.else_]
        elif isinstance(e, Coalesce):
            kids = [e.value1, e.value2]
        elif isinstance(e, In):
            kids = [e.value] + e.items
        else:
            kids = [e.value, e.lower, e.upper]
        hs = []
        try:
            for a in kids:
                hs.append(_expr_handle(a))
        except Exception:
            for h in hs:
                L.omg_expr_free(h)
            raise

        def arr(xs):
            return (C.c_void_p * max(len(xs), 1))(*xs)

        if isinstance(e, Func):
            rc = L.omg_expr_func(e.name.encode(), arr(hs), len(hs), _types([e.dtype]), C.byref(out))
        elif isinstance(e, If):
            rc = L.omg_expr_if(hs[0], hs[1], hs[2], C.byref(out))
        elif isinstance(e, Switch):
            rc = L.omg_expr_switch(arr(hs[0:-1:2]), arr(hs[1:-1:2]), len(e.whens), hs[-1], C.byref(out))
        elif isinstance(e, Coalesce):
            rc = L.omg_expr_coalesce(hs[0], hs[1], C.byref(out))
        elif isinstance(e, In):
            rc = L.omg_expr_in(arr(hs), len(hs), C.byref(out))
        else:
            rc = L.omg_expr_between(hs[0], hs[1], hs[2], C.byref(out))
        if rc != 0:
            for h in hs:
                L.omg_expr_free(h)
        check(rc)
    elif isinstance(e, Literal):
        if e.dtype.id == OMNI_DOUBLE:
            check(L.omg_expr_literal_double(float(e.value), 1 if e.is_null else 0, C.byref(out)))
        else:
            check(L.omg_expr_literal_long(int(e.value), _types([e.dtype]), 1 if e.is_null else 0, C.byref(out)))
    elif isinstance(e, Binary):
        left = _expr_handle(e.left)
        try:
            right = _expr_handle(e.right)
        except Exception:
            L.omg_expr_free(left)
            raise
        rc = (L.omg_expr_binary(e.op, left, right, C.byref(out)) if e.dtype is None else
              L.omg_expr_binary_typed(e.op, left, right, _types([e.dtype]), C.byref(out)))
        if rc != 0:
            L.omg_expr_free(left)
            L.omg_expr_free(right)
        check(rc)
    elif isinstance(e, (Not, IsNull)):
        child = _expr_handle(e.child)
        rc = (L.omg_expr_unary(EXPR_NOT, child, C.byref(out)) if isinstance(e, Not)
              else L.omg_expr_is_null(child, C.byref(out)))
        if rc != 0:
            L.omg_expr_free(child)
        check(rc)
    else:
        raise TypeError(f"not a filter expression node: {e!r}")
    return out.value


class LookupJoinOperatorFactory(OperatorFactory):
    """LookupJoinOperatorFactory::CreateLookupJoinOperatorFactory(probeTypes, probeOutputCols,
    probeHashCols, buildOutputCols, buildOutputTypes, hashBuilderFactoryAddr, filterExpr,
    isShuffleExchangeBuildPlan, overflowConfig)."""

    def __init__(self, probe_types, probe_output_cols, probe_hash_cols, build_output_cols, build_output_types,
                 hash_builder_factory: HashBuilderOperatorFactory, filter_expr=None,
                 is_shuffle_exchange_build_plan=False):
        out = C.c_void_p()
        expr = _expr_handle(filter_expr) if filter_expr is not None else None
        try:
            check(lib().omg_lookupjoin_factory_create(
                _types(probe_types), len(probe_types), _i32(probe_output_cols), len(probe_output_cols),
                _i32(probe_hash_cols), len(probe_hash_cols), _i32(build_output_cols), len(build_output_cols),
                _types(build_output_types), int(hash_builder_factory.handle), expr,
                1 if is_shuffle_exchange_build_plan else 0, C.byref(out)))
        finally:
            if expr is not None:
                lib().omg_expr_free(expr)
        super().__init__(out.value)


class LookupOuterJoinOperatorFactory(OperatorFactory):
    """LookupOuterJoinOperatorFactory::CreateLookupOuterJoinOperatorFactory(probeTypes,
    probeOutputCols, probeOutputColsCount, buildOutputCols, buildOutputTypes,
    hashBuilderFactoryAddr[, buildSide]): the unmatched build rows of a full or build-side outer
    join, read after every probe operator drained."""

    def __init__(self, probe_types, probe_output_cols, build_output_cols, build_output_types,
                 hash_builder_factory: HashBuilderOperatorFactory, build_side=OMNI_BUILD_UNKNOWN):
        out = C.c_void_p()
        check(lib().omg_lookupouterjoin_factory_create(
            _types(probe_types), len(probe_types), _i32(probe_output_cols), len(probe_output_cols),
            _i32(build_output_cols), len(build_output_cols), _types(build_output_types),
            int(hash_builder_factory.handle), build_side, C.byref(out)))
        super().__init__(out.value)


# --------------------------------------------------------------------------- batched aggregation
BATCH_DEVICE_OUTPUT, BATCH_NO_GRAPH, BATCH_NO_TUNE, BATCH_DEBUG_TINY_TABLES, BATCH_DEBUG_TINY_GROW = 1, 2, 4, 8, 16
_BATCH_INFO = ["tasks", "rows", "table_slots", "reruns", "threads", "ctas_per_sm", "runs", "groups", "tune_us",
               "prepare_us", "run_us", "learned", "graph", "grown", "operator_reruns"]


class AggBatch:
    """Many HashAggregation tasks of one factory in one launch (omg_agg_batch_*).  `tasks` are
    batch handles the caller keeps alive (and frees) until close()."""

    def __init__(self, factory, tasks, sizer=None, flags=0):
        arr = (C.c_void_p * len(tasks))(*tasks)
        out = C.c_void_p()
        check(lib().omg_agg_batch_create(factory.handle, arr, len(tasks), None if sizer is None else sizer.handle,
                                         flags, C.byref(out)))
        self.handle = out.value
        self._sizer = sizer

    def run(self, stream: int | None = None):
        check(lib().omg_agg_batch_run(self.handle, C.c_void_p(stream) if stream else None))

    def outputs(self, chunk: int = 1 << 14):
        """[(task, batch handle)] of the last run (the caller frees the batches)."""
        res = []
        out = (C.c_void_p * chunk)()
        task = (C.c_int32 * chunk)()
        n = C.c_int32(0)
        while True:
            check(lib().omg_agg_batch_outputs(self.handle, out, task, chunk, C.byref(n)))
            if n.value == 0:
                return res
            res.extend(zip(task[: n.value], out[: n.value]))

    def info(self) -> dict:
        arr = (C.c_int64 * 32)()
        n = C.c_int32(0)
        check(lib().omg_agg_batch_info(self.handle, arr, 32, C.byref(n)))
        return dict(zip(_BATCH_INFO, arr[: n.value]))

    def sizing_logs(self):
        info = self.info()
        total = info["tasks"] * 23
        arr = (C.c_int64 * total)()
        n = C.c_int64(0)
        check(lib().omg_agg_batch_sizing_logs(self.handle, arr, total, C.byref(n)))
        v = list(arr[: n.value])
        return [v[i:i + 23] for i in range(0, len(v), 23)]

    def close(self):
        if self.handle:
            check(lib().omg_agg_batch_destroy(self.handle))
            self.handle = None


JOIN_DIRECT, JOIN_HASH_PARTITIONED, JOIN_RANGE_PARTITIONED, JOIN_LEARNED, JOIN_QUANTILE = 0, 1, 2, 3, 4


def quantile_splits(sample, bits: int = 12) -> np.ndarray:
    """2^bits - 1 range splits from the exact quantiles of a sample of probe keys (no network)."""
    a = np.ascontiguousarray(sample, dtype=np.int64)
    out = np.zeros((1 << bits) - 1, dtype=np.int64)
    check(lib().omg_join_quantile_splits(a.ctypes.data_as(C.POINTER(C.c_int64)), len(a), bits,
                                         out.ctypes.data_as(C.POINTER(C.c_int64))))
    return out


def learn_splits(sample, bits: int = 12, epochs: int = 2000, seed: int = 1) -> np.ndarray:
    """2^bits - 1 range splits learned on the GPU from a sample of probe keys."""
    a = np.ascontiguousarray(sample, dtype=np.int64)
    out = np.zeros((1 << bits) - 1, dtype=np.int64)
    check(lib().omg_join_learn_splits(a.ctypes.data_as(C.POINTER(C.c_int64)), len(a), bits, epochs, seed,
                                      out.ctypes.data_as(C.POINTER(C.c_int64))))
    return out


def batches_fingerprint(batches):
    """(rows, f1, f2): order-independent fingerprint of the rows of the batches (GPU)."""
    arr = (C.c_void_p * max(len(batches), 1))(*batches)
    out = (C.c_uint64 * 3)()
    check(lib().omg_batches_fingerprint(arr, len(batches), out))
    return tuple(out)
