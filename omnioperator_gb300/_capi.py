"""ctypes binding of libomniop_gb300.so (declared in include/omniop_gb300.h).

The library is the product: there is no CPU fallback.  Loading fails loudly when the shared
library is missing or does not export the full C ABI.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libomniop_gb300.so"
HEADER = PKG.parent / "include" / "omniop_gb300.h"

P, I32, I64, U8P = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_uint8)


class OmgDataType(C.Structure):
    _fields_ = [("id", I32), ("precision", I32), ("scale", I32), ("width", I32)]


_SIGS = {
    "omg_last_error": (C.c_char_p, []),
    "omg_version": (C.c_char_p, []),
    "omg_device_available": (I32, []),
    "omg_config_set_policy": (I32, [I32]),
    "omg_config_get_policy": (I32, []),
    "omg_config_set_substr_rules": (I32, [I32, I32]),
    "omg_config_get_substr_rules": (I32, [C.POINTER(I32), C.POINTER(I32)]),
    "omg_debug_fail_next_allocs": (I32, [I32]),
    "omg_debug_set_wait_budget": (I32, [I64]),
    "omg_debug_set_staged_probe": (I32, [I32]),
    "omg_debug_set_bulk_probe": (I32, [I32]),
    "omg_debug_last_probe_kernel": (I32, []),
    "omg_debug_set_fused_training": (I32, [I32]),
    "omg_op_set_agg_sizing": (I32, [P, I32]),
    "omg_debug_set_agg_flush_rows": (I32, [I64]),
    "omg_debug_set_probe_chunk_rows": (I32, [I64]),
    "omg_vec_new": (I32, [I32, I32, C.POINTER(P)]),
    "omg_vec_new_fixed": (I32, [I32, I32, C.POINTER(P)]),
    "omg_vec_new_varchar": (I32, [I32, I32, I64, C.POINTER(P)]),
    "omg_vec_offsets": (P, [P]),
    "omg_vec_data_bytes": (I64, [P]),
    "omg_vec_new_device": (I32, [I32, I32, I32, C.POINTER(P)]),
    "omg_vec_wrap_device": (I32, [I32, I32, I32, P, P, C.POINTER(P)]),
    "omg_vec_free": (I32, [P]),
    "omg_vec_new_dictionary": (I32, [P, I32, P, C.POINTER(P)]),
    "omg_vec_encoding": (I32, [P]),
    "omg_vec_num_fields": (I32, [P]),
    "omg_vec_field": (P, [P, I32]),
    "omg_vec_values": (P, [P]),
    "omg_vec_nulls": (P, [P]),
    "omg_vec_size": (I32, [P]),
    "omg_vec_type": (I32, [P]),
    "omg_vec_width": (I32, [P]),
    "omg_vec_is_device": (I32, [P]),
    "omg_vec_has_null": (I32, [P]),
    "omg_vec_set_null_flag": (I32, [P, I32]),
    "omg_batch_new": (I32, [I32, C.POINTER(P)]),
    "omg_batch_append": (I32, [P, P]),
    "omg_batch_get": (P, [P, I32]),
    "omg_batch_row_count": (I32, [P]),
    "omg_batch_vector_count": (I32, [P]),
    "omg_batch_free": (I32, [P]),
    "omg_batch_to_device": (I32, [P, C.POINTER(P)]),
    "omg_batch_to_host": (I32, [P, C.POINTER(P)]),
    "omg_hashagg_factory_create": (I32, [P, P, I32, P, I32, P, P, P, P, P, P, P, P, I32, C.POINTER(P)]),
    "omg_hashbuilder_factory_create": (I32, [I32, P, I32, P, I32, I32, C.POINTER(P)]),
    "omg_expr_field": (I32, [I32, P, C.POINTER(P)]),
    "omg_expr_literal_long": (I32, [I64, P, I32, C.POINTER(P)]),
    "omg_expr_literal_double": (I32, [C.c_double, I32, C.POINTER(P)]),
    "omg_expr_literal_string": (I32, [C.c_char_p, I32, P, I32, C.POINTER(P)]),
    "omg_expr_func": (I32, [C.c_char_p, C.POINTER(P), I32, P, C.POINTER(P)]),
    "omg_expr_binary": (I32, [I32, P, P, C.POINTER(P)]),
    "omg_expr_binary_typed": (I32, [I32, P, P, P, C.POINTER(P)]),
    "omg_expr_unary": (I32, [I32, P, C.POINTER(P)]),
    "omg_expr_is_null": (I32, [P, C.POINTER(P)]),
    "omg_expr_if": (I32, [P, P, P, C.POINTER(P)]),
    "omg_expr_switch": (I32, [C.POINTER(P), C.POINTER(P), I32, P, C.POINTER(P)]),
    "omg_expr_coalesce": (I32, [P, P, C.POINTER(P)]),
    "omg_expr_in": (I32, [C.POINTER(P), I32, C.POINTER(P)]),
    "omg_expr_between": (I32, [P, P, P, C.POINTER(P)]),
    "omg_expr_free": (I32, [P]),
    "omg_lookupjoin_factory_create": (I32, [P, I32, P, I32, P, I32, P, I32, P, I64, P, I32, C.POINTER(P)]),
    "omg_hashbuilder_factory_create_side": (I32, [I32, I32, P, I32, P, I32, I32, C.POINTER(P)]),
    "omg_lookupouterjoin_factory_create": (I32, [P, I32, P, I32, P, I32, P, I64, I32, C.POINTER(P)]),
    "omg_factory_create_operator": (I32, [P, C.POINTER(P)]),
    "omg_factory_destroy": (I32, [P]),
    "omg_op_init": (I32, [P]),
    "omg_op_add_input": (I32, [P, P, C.POINTER(I32)]),
    "omg_op_get_output": (I32, [P, C.POINTER(P), C.POINTER(I32)]),
    "omg_op_add_inputs": (I32, [P, C.POINTER(P), I32, C.POINTER(I32)]),
    "omg_op_get_outputs": (I32, [P, C.POINTER(P), I32, C.POINTER(I32), C.POINTER(I64)]),
    "omg_batch_free_many": (I32, [C.POINTER(P), I32]),
    "omg_op_get_sizing_log": (I32, [P, C.POINTER(I64), I32, C.POINTER(I32)]),
    "omg_sizer_create": (I32, [C.POINTER(I32), I32, C.c_uint64, C.POINTER(P)]),
    "omg_sizer_destroy": (I32, [P]),
    "omg_sizer_num_params": (I32, [P, C.POINTER(I64)]),
    "omg_sizer_get_params": (I32, [P, C.POINTER(C.c_float), I64]),
    "omg_sizer_set_params": (I32, [P, C.POINTER(C.c_float), I64]),
    "omg_sizer_predict": (I32, [P, C.POINTER(C.c_float), I32, C.POINTER(C.c_float)]),
    "omg_sizer_gradients": (I32, [P, C.POINTER(C.c_float), C.POINTER(C.c_float), I32, C.POINTER(C.c_float),
                                  C.POINTER(C.c_float)]),
    "omg_sizer_train": (I32, [P, C.POINTER(C.c_float), C.POINTER(C.c_float), I32, I32, C.c_float,
                              C.POINTER(C.c_float)]),
    "omg_sizer_features": (I32, [C.POINTER(I64), I32, C.POINTER(C.c_float)]),
    "omg_sizer_target": (I32, [C.POINTER(I64), I32, I64, C.POINTER(C.c_float)]),
    "omg_sizer_estimate": (I32, [C.POINTER(I64), I32, C.c_float, C.POINTER(I64)]),
    "omg_hashagg_factory_set_sizer": (I32, [P, P]),
    "omg_agg_batch_create": (I32, [P, C.POINTER(P), I32, P, I32, C.POINTER(P)]),
    "omg_agg_batch_run": (I32, [P, P]),
    "omg_agg_batch_outputs": (I32, [P, C.POINTER(P), C.POINTER(I32), I32, C.POINTER(I32)]),
    "omg_agg_batch_info": (I32, [P, C.POINTER(I64), I32, C.POINTER(I32)]),
    "omg_agg_batch_sizing_logs": (I32, [P, C.POINTER(I64), I64, C.POINTER(I64)]),
    "omg_agg_batch_destroy": (I32, [P]),
    "omg_op_set_join_strategy": (I32, [P, I32, I32, C.POINTER(I64), I32]),
    "omg_op_join_strategy": (I32, [P, C.POINTER(I32)]),
    "omg_batches_fingerprint": (I32, [C.POINTER(P), I32, C.POINTER(C.c_uint64)]),
    "omg_join_learn_splits": (I32, [C.POINTER(I64), I64, I32, I32, C.c_uint64, C.POINTER(I64)]),
    "omg_join_quantile_splits": (I32, [C.POINTER(I64), I64, I32, C.POINTER(I64)]),
    "omg_op_status": (I32, [P]),
    "omg_op_no_more_input": (I32, [P]),
    "omg_op_set_no_more_input": (I32, [P, I32]),
    "omg_op_needs_input": (I32, [P]),
    "omg_op_is_blocked": (I32, [P]),
    "omg_op_hashmap_unique_keys": (I64, [P]),
    "omg_op_align_schema": (I32, [P, P, C.POINTER(P)]),
    "omg_op_close": (I32, [P]),
    "omg_op_delete": (I32, [P]),
    "omg_op_set_stream": (I32, [P, P]),
    "omg_op_set_device_output": (I32, [P, I32]),
    "omg_op_set_agg_strategy": (I32, [P, I32, I64]),
    "omg_op_set_spill": (I32, [P, I32, I64]),
    "omg_op_spilled_bytes": (I64, [P]),
    "omg_op_get_counters": (I32, [P, C.POINTER(I64), I32]),
    "omg_hashagg_run_noalloc": (I32, [P, P, P, I32, I64, P, P, I32, I64, C.POINTER(I64), P]),
}

_lib = None


def header_symbols() -> list[str]:
    """Names of every function the C header declares."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(omg_[a-z0-9_]+)\s*\(", text)))


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH.name} is not built: run omnioperator_gb300.build.build() "
                               "(the GB300 operators have no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class OmgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status
        self.message = message


def check(status: int) -> None:
    if status != 0:
        raise OmgError(status, lib().omg_last_error().decode(errors="replace"))
