"""Learned sizing for HashAggregation.

A small network (12 sketch features -> hidden ReLU layers -> 1) predicts log2(groups / d), the
ratio of the group count to the distinct keys d of the operator's own row sample.  Its training
data are the sizing records the plain operator logs (omg_op_get_sizing_log: the key sketch of
the first flush and the group count found), and it is trained on the GPU by the library's
forward / backward / Adam kernels.  Attached to a factory (HashAggregationOperatorFactory.
set_sizer), its estimate pre-sizes the table and picks the strategy; the exact resize path
still corrects any misprediction, so outputs do not depend on the model.
"""
from __future__ import annotations

import ctypes as C
import json

import numpy as np

from ._capi import check, lib

N_FEATURES = 12
DEFAULT_DIMS = (N_FEATURES, 64, 64, 1)


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


def _log_arr(log):
    arr = (C.c_int64 * len(log))(*[int(v) for v in log])
    return arr, len(log)


def features(log) -> np.ndarray:
    arr, n = _log_arr(log)
    out = (C.c_float * N_FEATURES)()
    check(lib().omg_sizer_features(arr, n, out))
    return np.array(out[:], dtype=np.float32)


def target(log, groups: int) -> float:
    arr, n = _log_arr(log)
    out = C.c_float(0)
    check(lib().omg_sizer_target(arr, n, int(groups), C.byref(out)))
    return out.value


def estimate(log, y: float) -> int:
    arr, n = _log_arr(log)
    out = C.c_int64(0)
    check(lib().omg_sizer_estimate(arr, n, float(y), C.byref(out)))
    return out.value


class SizingModel:
    """The network behind omg_sizer_* (parameters in HBM)."""

    def __init__(self, dims=DEFAULT_DIMS, seed: int = 1):
        self.dims = tuple(int(d) for d in dims)
        arr = (C.c_int32 * len(self.dims))(*self.dims)
        out = C.c_void_p()
        check(lib().omg_sizer_create(arr, len(self.dims), seed, C.byref(out)))
        self.handle = out.value

    def close(self):
        if self.handle:
            check(lib().omg_sizer_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        n = C.c_int64(0)
        check(lib().omg_sizer_num_params(self.handle, C.byref(n)))
        return n.value

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.num_params, dtype=np.float32)
        check(lib().omg_sizer_get_params(self.handle, out.ctypes.data_as(C.POINTER(C.c_float)), len(out)))
        return out

    def set_params(self, params) -> None:
        a, p = _f32(params)
        check(lib().omg_sizer_set_params(self.handle, p, len(a)))

    def predict(self, X) -> np.ndarray:
        X, px = _f32(X)
        out = np.zeros(len(X), dtype=np.float32)
        check(lib().omg_sizer_predict(self.handle, px, len(X), out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def gradients(self, X, T):
        X, px = _f32(X)
        T, pt = _f32(T)
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = C.c_float(0)
        check(lib().omg_sizer_gradients(self.handle, px, pt, len(X), g.ctypes.data_as(C.POINTER(C.c_float)),
                                        C.byref(loss)))
        return g, loss.value

    def train(self, X, T, epochs: int = 2000, lr: float = 3e-3) -> float:
        X, px = _f32(X)
        T, pt = _f32(T)
        loss = C.c_float(0)
        check(lib().omg_sizer_train(self.handle, px, pt, len(X), epochs, lr, C.byref(loss)))
        return loss.value

    def save(self, path) -> None:
        with open(path, "w") as f:
            json.dump({"dims": list(self.dims), "params": [float(v) for v in self.get_params()]}, f)

    @classmethod
    def load(cls, path) -> "SizingModel":
        with open(path) as f:
            d = json.load(f)
        m = cls(d["dims"])
        m.set_params(np.array(d["params"], dtype=np.float32))
        return m


def record_from_operator(op) -> tuple[list[int], int]:
    """(sizing record, group count) of a finished HashAggregation operator."""
    s = op.sizing_log()
    return s["raw"], s["groups"]


def dataset(records):
    """Features and targets of [(sizing record, group count)]."""
    X = np.stack([features(r) for r, _ in records])
    T = np.array([target(r, g) for r, g in records], dtype=np.float32)
    return X, T
