"""CPU oracle of the hash aggregation / inner hash join path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may import this
package, and only as the checker or the timed CPU baseline; the product never does.

``oracle.c`` restates the reference's algorithms (file:line citations at its top).  The
reference itself cannot be compiled here or on the GPU machine: its hot-path translation units need
jemalloc, libboundscheck (securec), LLVM (via filter_and_project.h), nlohmann-json and JNI
logging, and the build uses the reference's own CMake.  Parity of the restatement is pinned by
the reference's test vectors in tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.c"
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

_lib = None

# Type / function ids (reference numbering, type/data_type.h:40-74, function_type.h:11-27).
T_INT, T_LONG, T_DOUBLE, T_BOOLEAN, T_SHORT, T_DEC64, T_DEC128 = 1, 2, 3, 4, 5, 6, 7
T_DATE32, T_BYTE, T_FLOAT = 8, 18, 19
F_SUM, F_COUNT_COL, F_COUNT_ALL, F_AVG, F_MAX, F_MIN = 0, 1, 2, 3, 5, 6

WIDTH = {T_INT: 4, T_LONG: 8, T_DOUBLE: 8, T_BOOLEAN: 1, T_SHORT: 2, T_DEC64: 8, T_DEC128: 16,
         T_DATE32: 4, T_BYTE: 1, T_FLOAT: 4}


def build() -> Path:
    """Compile oracle.c with gcc (portable flags: the same source builds on x86 and Arm)."""
    BUILD.mkdir(exist_ok=True)
    if not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(".tmp.so")
        subprocess.run(["gcc", "-O3", "-fPIC", "-shared", "-std=gnu11", "-o", str(tmp), str(SRC), "-lpthread"],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P, I32, I64 = C.c_void_p, C.c_int32, C.c_int64
        L.orc_hashagg.restype = I64
        L.orc_hashagg.argtypes = [I64, I32, P, P, P, I32, P, P, P, P, P, P, P, I32, I32, I64, P, P, P, P, P, P]
        L.orc_join_inner.restype = I64
        L.orc_join_inner.argtypes = [I64, P, I32, P, I64, P, I32, P, P, P, I64]
        L.orc_join.restype = I64
        L.orc_join.argtypes = [I32, I64, P, I32, P, I64, P, I32, P, P, P, I64]
        L.orc_join_probe_bench.restype = I64
        L.orc_join_probe_bench.argtypes = [I64, P, P, I32, P, I64, P, P, I32, P]
        L.orc_agg_bench.restype = I64
        L.orc_agg_bench.argtypes = [I64, P, P, P, I32]
        L.orc_fingerprint_cols.restype = None
        L.orc_fingerprint_cols.argtypes = [I64, I32, P, P, P, P]
        L.orc_jtable_new.restype = P
        L.orc_jtable_new.argtypes = [I64, P, P]
        L.orc_jtable_free.restype = None
        L.orc_jtable_free.argtypes = [P]
        L.orc_jtable_fingerprint.restype = I32
        L.orc_jtable_fingerprint.argtypes = [P, I32, P, P, I64, P, P, I32, P, P]
        L.orc_jtable_pairs.restype = I64
        L.orc_jtable_pairs.argtypes = [P, I64, P, P, P, P, I64]
        L.orc_hashagg_mt.restype = I64
        L.orc_hashagg_mt.argtypes = [I64, I32, P, P, P, I32, P, P, P, P, P, P, P, I32, I32, I64, P, P, P, P, P, P,
                                     I32, P, P]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _ptr_array(arrs):
    return (C.c_void_p * max(len(arrs), 1))(*[(a.ctypes.data if a is not None else None) for a in arrs])


def _dec_params(aggs):
    """Per aggregator (input precision, input scale, output scale) of a decimal AVG."""
    return np.array([[a.get("in_prec", 18), a.get("in_scale", 0), a.get("out_scale", 0)] for a in aggs] or [[0, 0, 0]],
                    dtype=np.int32).reshape(-1)


def _masks(aggs):
    """Per aggregator: a byte per row, 1 where the row reaches the aggregator (its mask value
    is TRUE and not NULL), or None for an aggregator without a mask column."""
    out = []
    for a in aggs:
        m = a.get("mask")
        if m is None:
            out.append(None)
            continue
        m = np.asarray(m, dtype=bool)
        mn = a.get("mask_nulls")
        if mn is not None:
            m = m & ~np.asarray(mn, dtype=bool)
        out.append(np.ascontiguousarray(m, dtype=np.uint8))
    return out


def hashagg(keys, key_types, key_nulls, aggs, policy=0, overflow_as_null=False):
    """Single-stage hash aggregation with the reference's semantics.

    keys: list of value arrays (int types as their numpy ints, decimal128 as (n, 2) uint64).
    key_nulls: list of bool arrays or None.  aggs: list of dicts with keys func, col (array or
    None for COUNT(*)), in_type, out_type, nulls (bool array or None), rescale (int), for a
    decimal AVG in_prec / in_scale / out_scale, and
    optionally mask / mask_nulls (bool arrays: the aggregator's mask column; a row reaches it
    only where the mask is TRUE and not NULL).
    Returns (key_values, key_nulls, agg_values, agg_nulls) per group (unordered), or raises
    OverflowError when an overflow must raise (overflow-as-null off)."""
    L = lib()
    n = len(keys[0]) if keys else 0
    kw = [WIDTH[t] for t in key_types]
    kcols = [np.ascontiguousarray(k) for k in keys]
    knulls = [None if m is None else np.ascontiguousarray(m, dtype=np.uint8) for m in key_nulls]
    funcs = np.array([a["func"] for a in aggs], dtype=np.int32)
    cols, in_types, in_widths, anulls, out_types, rescale = [], [], [], [], [], []
    for a in aggs:
        col = a.get("col")
        if col is None:
            col = np.zeros(max(n, 1), dtype=np.int64)
            in_types.append(T_LONG)
        else:
            in_types.append(a["in_type"])
        cols.append(np.ascontiguousarray(col))
        in_widths.append(WIDTH[in_types[-1]])
        m = a.get("nulls")
        anulls.append(None if m is None else np.ascontiguousarray(m, dtype=np.uint8))
        out_types.append(a["out_type"])
        rescale.append(a.get("rescale", 0))
    in_types = np.array(in_types, dtype=np.int32)
    in_widths = np.array(in_widths, dtype=np.int32)
    out_types = np.array(out_types, dtype=np.int32)
    rescale = np.array(rescale, dtype=np.int32)
    maxg = max(n, 1)
    okeys = [np.zeros((maxg, 2) if w == 16 else maxg, dtype=np.uint64 if w == 16 else
                      {1: np.int8, 2: np.int16, 4: np.int32, 8: np.int64}[w]) for w in kw]
    oknulls = [np.zeros(maxg, dtype=np.uint8) for _ in kw]
    ovals = [np.zeros((maxg, 2), dtype=np.uint64) for _ in aggs]
    ovnulls = [np.zeros(maxg, dtype=np.uint8) for _ in aggs]
    masks = _masks(aggs)  # kept alive across the call (the pointer array holds raw addresses)
    g = L.orc_hashagg(n, len(keys), _ptr_array(kcols), _ptr(np.array(kw, dtype=np.int32)),
                      _ptr_array(knulls), len(aggs), _ptr(funcs), _ptr_array(cols), _ptr(in_types),
                      _ptr(in_widths), _ptr_array(anulls), _ptr(out_types), _ptr(rescale), policy,
                      1 if overflow_as_null else 0, maxg, _ptr_array(okeys), _ptr_array(oknulls),
                      _ptr_array(ovals), _ptr_array(ovnulls), _ptr_array(masks), _ptr(_dec_params(aggs)))
    if g == -2:
        raise OverflowError("sum_aggregator overflow.")
    if g < 0:
        raise RuntimeError(f"oracle hashagg failed ({g})")
    vals = []
    for a, ov in zip(aggs, ovals):
        t = a["out_type"]
        raw = ov.reshape(-1)  # the oracle writes a dense array of the output type
        if t == T_DEC128:
            vals.append(raw.reshape(maxg, 2)[:g].copy())
        else:
            dt = {T_DOUBLE: np.float64, T_FLOAT: np.float32, T_INT: np.int32, T_DATE32: np.int32,
                  T_SHORT: np.int16, T_BYTE: np.int8, T_BOOLEAN: np.int8}.get(t, np.int64)
            vals.append(raw.view(np.uint8).view(dt)[:g].copy())
    return ([k[:g] for k in okeys], [m[:g].astype(bool) for m in oknulls], vals,
            [m[:g].astype(bool) for m in ovnulls])


def join_inner(build_keys, build_nulls, probe_keys, probe_nulls):
    """(probe_row, build_row) index pairs of the inner equi-join, NULL keys never matching."""
    L = lib()
    bk = np.ascontiguousarray(build_keys)
    pk = np.ascontiguousarray(probe_keys)
    bn = None if build_nulls is None else np.ascontiguousarray(build_nulls, dtype=np.uint8)
    pn = None if probe_nulls is None else np.ascontiguousarray(probe_nulls, dtype=np.uint8)
    cap = max(len(pk), 1)
    while True:
        op = np.empty(cap, dtype=np.int64)
        ob = np.empty(cap, dtype=np.int64)
        n = L.orc_join_inner(len(bk), _ptr(bk), bk.dtype.itemsize, _ptr(bn), len(pk), _ptr(pk),
                             pk.dtype.itemsize, _ptr(pn), _ptr(op), _ptr(ob), cap)
        if n < 0:
            raise RuntimeError("oracle join failed")
        if n <= cap:
            return op[:n], ob[:n]
        cap = n


JOIN_KINDS = {"inner": 0, "probe_outer": 1, "build_outer": 2, "full": 3, "semi": 4, "anti": 5, "existence": 6}


JOIN_TYPES = {"INNER": 0, "LEFT": 1, "RIGHT": 2, "FULL": 3, "LEFT_SEMI": 4, "LEFT_ANTI": 5, "EXISTENCE": 6}
BUILD_SIDES = {"UNKNOWN": 0, "LEFT": 1, "RIGHT": 2}


def join_kind(join_type, build_side="UNKNOWN"):
    """The probe a join type selects (lookup_join.cpp:330-411): a LEFT (RIGHT) join built on its
    left (right) input keeps unmatched build rows, otherwise unmatched probe rows."""
    if join_type in ("LEFT", "RIGHT"):
        return "build_outer" if build_side == join_type else "probe_outer"
    return {"INNER": "inner", "FULL": "full", "LEFT_SEMI": "semi", "LEFT_ANTI": "anti",
            "EXISTENCE": "existence"}[join_type]


def join(kind, build_keys, build_nulls, probe_keys, probe_nulls):
    """(probe_row, build_row) pairs of one output row each for a join kind (JOIN_KINDS); -1
    marks the side an outer row lacks, and for "existence" build_row is the 0/1 flag."""
    L = lib()
    bk = np.ascontiguousarray(build_keys)
    pk = np.ascontiguousarray(probe_keys)
    bn = None if build_nulls is None else np.ascontiguousarray(build_nulls, dtype=np.uint8)
    pn = None if probe_nulls is None else np.ascontiguousarray(probe_nulls, dtype=np.uint8)
    cap = max(len(pk) + len(bk), 1)
    while True:
        op = np.empty(cap, dtype=np.int64)
        ob = np.empty(cap, dtype=np.int64)
        n = L.orc_join(JOIN_KINDS[kind], len(bk), _ptr(bk), bk.dtype.itemsize, _ptr(bn), len(pk), _ptr(pk),
                       pk.dtype.itemsize, _ptr(pn), _ptr(op), _ptr(ob), cap)
        if n < 0:
            raise RuntimeError("oracle join failed")
        if n <= cap:
            return op[:n], ob[:n]
        cap = n


def utf8_offset(data: bytes, pos: int, count: int) -> int:
    """Byte offset of the code point `count` places after byte `pos`, or -1 when the string ends
    first (utf8_util.h:22-60, OffsetOfCodePoint).  The reference adds the continuation bytes
    (10xxxxxx) it passes to the target index until it reaches it; the answer is the
    (count + 1)-th byte from `pos` that is not a continuation byte."""
    n = len(data)
    if n - pos <= count:
        return -1
    if count == 0:
        return pos
    seen = 0
    for i in range(pos, n):
        if data[i] & 0xC0 != 0x80:
            seen += 1
            if seen == count + 1:
                return i
    return -1


def utf8_count(data: bytes) -> int:
    """Code points: bytes less continuation bytes (utf8_util.h:62-91, CountCodePoints)."""
    return len(data) - sum(1 for c in data if c & 0xC0 == 0x80)


def _i32(x: int) -> int:
    """The int32 parameter of OffsetOfCodePoint receiving an int64 (two's-complement truncation)."""
    return ((x + 2**31) % 2**32) - 2**31


def substr(data: bytes, start: int, length=None, negative: bool = True, zero: bool = True) -> bytes:
    """substr over UTF-8 code points (stringfunctions.h:215-250 SubstrVarcharWithStart when
    length is None, :258-318 SubstrVarchar).  negative: NegativeStartIndexOutOfBoundsRule
    INTERCEPT_FROM_BEYOND (a start before the string keeps the part inside it; EMPTY_STRING
    otherwise); zero: ZeroStartIndexSupportRule IS_SUPPORT (start 0 means 1).  Both default to
    the Spark policy (policy.h:160-167).  Where the reference reads outside the string (a
    negative start into malformed UTF-8) the result is empty."""
    n = len(data)
    if zero and start == 0:
        start = 1
    if start == 0 or (length is not None and length <= 0) or n == 0 or start > n:
        return b""
    if start > 0:
        si = utf8_offset(data, 0, _i32(start - 1))
        if si < 0:
            return b""
        if length is None:
            return data[si:]
        ei = utf8_offset(data, si, _i32(length))
        return data[si:n if ei < 0 else ei]
    points = utf8_count(data)
    sp = start + points
    ln = 0 if length is None else length
    if sp < 0:
        if not negative or (length is not None and sp + ln <= 0):
            return b""
        ln += sp
        sp = 0
    si = utf8_offset(data, 0, _i32(sp))
    if si < 0:
        return b""
    if length is None or sp + ln >= points:
        return data[si:]
    ei = utf8_offset(data, si, _i32(ln))
    return data[si:n if ei < si else ei]


def str_compare(a: bytes, b: bytes) -> int:
    """Byte-wise unsigned comparison, then by length: -1, 0 or 1 (stringfunctions.cpp:86-98,
    StrCompare; StrEquals at :75-84 after equal lengths)."""
    return -1 if a < b else (1 if a > b else 0)


def string_function(name: str, args: list, char_width=None):
    """The buffer-free string functions of a filter (codegen/functions/stringfunctions.cpp:
    2064-2092 length / char_length, 2801-2820 InStr, 2822-2844 StartsWith / EndsWith, 2900-2944
    Contains / Greatest / Least) over bytes arguments, None for NULL: NULL in gives NULL out
    (the INPUT_DATA registrations) except Greatest / Least, which return the other argument when
    one is NULL.  char_width: length of a CHAR argument is its declared width."""
    if name in ("Greatest", "Least"):
        a, b = args
        if a is None or b is None:
            return b if a is None else a
        c = str_compare(a, b)
        return b if (c < 0 if name == "Greatest" else c > 0) else a
    if any(x is None for x in args):
        return None
    if name in ("length", "char_length"):
        return char_width if char_width is not None else utf8_count(args[0])
    s, sub = args
    if name == "instr":
        pos = s.find(sub) if len(sub) <= len(s) else -1
        return 0 if pos < 0 else utf8_count(s[:pos]) + 1
    if name == "StartsWith":
        return int(s.startswith(sub))
    if name == "EndsWith":
        return int(s.endswith(sub))
    if name == "Contains":
        return int(sub in s)
    raise ValueError(name)


def join_filtered(kind, build_keys, build_nulls, probe_keys, probe_nulls, passes):
    """join() with a join filter: a (probe, build) pair whose keys are equal counts as a match
    only when passes(probe_rows, build_rows) (a vectorised predicate over pair arrays) is true.
    Restates the reference's filtered probes (lookup_join.cpp:1037-1438, the filter evaluated
    per candidate at :1440-1466; unmatched build rows, lookup_outer_join.cpp:173-374): inner
    rows are the passing pairs; outer kinds add the probe (build) rows without a passing pair,
    with -1 on the missing side; semi keeps probe rows with one, anti those without; existence
    flags every probe row."""
    pi, bi = join_inner(build_keys, build_nulls, probe_keys, probe_nulls)
    ok = np.asarray(passes(pi, bi), dtype=bool) if len(pi) else np.zeros(0, bool)
    pp, pb = pi[ok], bi[ok]
    n_probe, n_build = len(probe_keys), len(build_keys)
    probe_has = np.zeros(n_probe, bool)
    probe_has[pp] = True
    build_has = np.zeros(n_build, bool)
    build_has[pb] = True
    none_p = np.nonzero(~probe_has)[0]
    none_b = np.nonzero(~build_has)[0]
    neg_p = -np.ones(len(none_b), np.int64)
    neg_b = -np.ones(len(none_p), np.int64)
    if kind == "inner":
        return pp, pb
    if kind == "probe_outer":
        return np.concatenate([pp, none_p]), np.concatenate([pb, neg_b])
    if kind == "build_outer":
        return np.concatenate([pp, neg_p]), np.concatenate([pb, none_b])
    if kind == "full":
        return np.concatenate([pp, none_p, neg_p]), np.concatenate([pb, neg_b, none_b])
    if kind == "semi":
        rows = np.nonzero(probe_has)[0]
        return rows, -np.ones(len(rows), np.int64)
    if kind == "anti":
        return none_p, neg_b
    if kind == "existence":
        return np.arange(n_probe, dtype=np.int64), probe_has.astype(np.int64)
    raise ValueError(kind)


def exact_group_sums(group_ids: np.ndarray, values: np.ndarray, valid: np.ndarray | None, ngroups: int):
    """Correctly rounded per-group sums (math.fsum) and per-group sums of |x|, the reference
    values of the double tolerance."""
    if valid is not None:
        group_ids = group_ids[valid]
        values = values[valid]
    order = np.argsort(group_ids, kind="stable")
    g = group_ids[order]
    v = values[order]
    bounds = np.searchsorted(g, np.arange(ngroups + 1))
    exact = np.zeros(ngroups)
    absum = np.zeros(ngroups)
    for i in range(ngroups):
        seg = v[bounds[i]:bounds[i + 1]]
        if len(seg):
            exact[i] = math.fsum(seg.tolist())
            absum[i] = math.fsum(np.abs(seg).tolist())
    return exact, absum


# ------------------------------------------------------------------ checks at full configuration size
def fingerprint_cols(cols, nulls=None):
    """(rows, f1, f2): the order-independent fingerprint of the rows of `cols` (numpy arrays,
    decimal128 as (n, 2) uint64; `nulls` bool arrays or None), the row hash the library's
    fingerprint kernel computes on the device (omg_batches_fingerprint)."""
    L = lib()
    cols = [np.ascontiguousarray(c) for c in cols]
    n = len(cols[0]) if cols else 0
    widths = np.array([c.dtype.itemsize * (2 if c.ndim == 2 else 1) for c in cols], dtype=np.int32)
    nl = [None if m is None else np.ascontiguousarray(m, dtype=np.uint8) for m in (nulls or [None] * len(cols))]
    out = (C.c_uint64 * 3)()
    L.orc_fingerprint_cols(n, len(cols), _ptr_array(cols), _ptr(widths), _ptr_array(nl), out)
    return tuple(int(x) for x in out)


class JoinTable:
    """A build side (int64 keys, bool NULL mask or None) kept for many probes of the checks."""

    def __init__(self, keys, nulls=None):
        self._keys = np.ascontiguousarray(keys, dtype=np.int64)
        self._nulls = None if nulls is None else np.ascontiguousarray(nulls, dtype=np.uint8)
        self.handle = lib().orc_jtable_new(len(self._keys), _ptr(self._keys), _ptr(self._nulls))
        if not self.handle:
            raise MemoryError("oracle join table")

    def fingerprint(self, payloads, probe_keys, probe_nulls=None, threads=1):
        """(fingerprint of the inner-join rows (probe key, payload columns), probe seconds)."""
        pays = [np.ascontiguousarray(p) for p in payloads]
        pw = np.array([p.dtype.itemsize for p in pays], dtype=np.int32)
        pk = np.ascontiguousarray(probe_keys, dtype=np.int64)
        pn = None if probe_nulls is None else np.ascontiguousarray(probe_nulls, dtype=np.uint8)
        out = (C.c_uint64 * 3)()
        secs = C.c_double(0.0)
        rc = lib().orc_jtable_fingerprint(self.handle, len(pays), _ptr_array(pays), _ptr(pw), len(pk), _ptr(pk),
                                          _ptr(pn), threads, out, C.byref(secs))
        if rc != 0:
            raise RuntimeError("oracle join fingerprint failed")
        return tuple(int(x) for x in out), secs.value

    def pairs(self, probe_keys, probe_nulls=None):
        """(probe row, build row) index pairs of the inner join, probe rows in order."""
        pk = np.ascontiguousarray(probe_keys, dtype=np.int64)
        pn = None if probe_nulls is None else np.ascontiguousarray(probe_nulls, dtype=np.uint8)
        cap = max(len(pk), 1)
        while True:
            op = np.empty(cap, dtype=np.int64)
            ob = np.empty(cap, dtype=np.int64)
            n = lib().orc_jtable_pairs(self.handle, len(pk), _ptr(pk), _ptr(pn), _ptr(op), _ptr(ob), cap)
            if n < 0:
                raise RuntimeError("oracle join failed")
            if n <= cap:
                return op[:n], ob[:n]
            cap = n

    def close(self):
        if self.handle:
            lib().orc_jtable_free(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


def hashagg_mt(keys, key_types, key_nulls, aggs, policy=0, overflow_as_null=False, threads=1, max_groups=None):
    """hashagg() over `threads` threads (each group's rows folded in row order by one thread).
    Returns (key_values, key_nulls, agg_values, agg_nulls, exact, absum): for aggregates over a
    DOUBLE column, exact[j] / absum[j] are per-group double-double sums of the non-NULL values
    and sums of |x| (None for other aggregates).  Output arrays hold `max_groups` groups
    (default: one per row); more groups raise."""
    L = lib()
    n = len(keys[0]) if keys else 0
    kw = [WIDTH[t] for t in key_types]
    kcols = [np.ascontiguousarray(k) for k in keys]
    knulls = [None if m is None else np.ascontiguousarray(m, dtype=np.uint8) for m in key_nulls]
    funcs = np.array([a["func"] for a in aggs], dtype=np.int32)
    cols, in_types, in_widths, anulls, out_types, rescale = [], [], [], [], [], []
    for a in aggs:
        col = a.get("col")
        if col is None:
            col = np.zeros(max(n, 1), dtype=np.int64)
            in_types.append(T_LONG)
        else:
            in_types.append(a["in_type"])
        cols.append(np.ascontiguousarray(col))
        in_widths.append(WIDTH[in_types[-1]])
        m = a.get("nulls")
        anulls.append(None if m is None else np.ascontiguousarray(m, dtype=np.uint8))
        out_types.append(a["out_type"])
        rescale.append(a.get("rescale", 0))
    in_types_a = np.array(in_types, dtype=np.int32)
    maxg = max(n if max_groups is None else min(n, max_groups), 1)
    okeys = [np.zeros((maxg, 2) if w == 16 else maxg, dtype=np.uint64 if w == 16 else
                      {1: np.int8, 2: np.int16, 4: np.int32, 8: np.int64}[w]) for w in kw]
    oknulls = [np.zeros(maxg, dtype=np.uint8) for _ in kw]
    ovals = [np.zeros(maxg * (2 if t == T_DEC128 else 1), dtype=np.uint64) for t in out_types]
    ovnulls = [np.zeros(maxg, dtype=np.uint8) for _ in aggs]
    dbl = [a["func"] in (F_SUM, F_AVG) and t == T_DOUBLE for a, t in zip(aggs, in_types)]
    exact = [np.zeros(maxg) if d else None for d in dbl]
    absum = [np.zeros(maxg) if d else None for d in dbl]
    masks = _masks(aggs)  # kept alive across the call (the pointer array holds raw addresses)
    g = L.orc_hashagg_mt(n, len(keys), _ptr_array(kcols), _ptr(np.array(kw, dtype=np.int32)), _ptr_array(knulls),
                         len(aggs), _ptr(funcs), _ptr_array(cols), _ptr(in_types_a),
                         _ptr(np.array(in_widths, dtype=np.int32)), _ptr_array(anulls),
                         _ptr(np.array(out_types, dtype=np.int32)), _ptr(np.array(rescale, dtype=np.int32)), policy,
                         1 if overflow_as_null else 0, maxg, _ptr_array(okeys), _ptr_array(oknulls),
                         _ptr_array(ovals), _ptr_array(ovnulls), _ptr_array(exact), _ptr_array(absum), threads,
                         _ptr_array(masks), _ptr(_dec_params(aggs)))
    if g == -2:
        raise OverflowError("sum_aggregator overflow.")
    if g == -3:
        raise RuntimeError(f"more than max_groups = {maxg} groups")
    if g < 0:
        raise RuntimeError(f"oracle hashagg failed ({g})")
    vals = []
    for t, ov in zip(out_types, ovals):
        if t == T_DEC128:
            vals.append(ov.reshape(maxg, 2)[:g].copy())
        else:
            dt = {T_DOUBLE: np.float64, T_FLOAT: np.float32, T_INT: np.int32, T_DATE32: np.int32,
                  T_SHORT: np.int16, T_BYTE: np.int8, T_BOOLEAN: np.int8}.get(t, np.int64)
            vals.append(ov.view(np.uint8).view(dt)[:g].copy())
    return ([k[:g] for k in okeys], [m[:g].astype(bool) for m in oknulls], vals,
            [m[:g].astype(bool) for m in ovnulls], [None if e is None else e[:g] for e in exact],
            [None if a is None else a[:g] for a in absum])


# ------------------------------------------------------------------ two-stage decimal SUM
DEC38_MAX = 10**38 - 1


def decimal_sum_merge(keys, sums, sum_nulls, empties, partial=False, rescale=0):
    """The merging stage of the Spark decimal SUM over partial rows in arrival order
    (AddDecimalUseRowIndex, sum_spark_decimal_aggregator.h:14-66): per group the state starts
    EMPTY; a row with a NULL partial sum makes it OVERFLOWED; a row whose isEmpty is true is
    skipped; any other row is added with the checked addition (a result beyond +-(10^38 - 1)
    overflows); an OVERFLOWED state takes no further rows.  Output (ExtractValues, :165-241):
    final -- NULL for an overflowed or empty group ("overflow" marks the former), else the sum
    times 10^rescale (NULL-or-error if that overflows); partial -- (sum or NULL, isEmpty), the sum
    0 for an empty group.  Pure Python, for small cases.  Returns {key: (value or None, flag)}
    where flag is "overflow"/"empty"/None (final) or the isEmpty boolean (partial)."""
    state = {}
    for k, s, n, e in zip(keys, sums, sum_nulls, empties):
        st = state.setdefault(k, ["empty", 0])
        if st[0] == "overflow":
            continue
        if n:
            st[0] = "overflow"
            continue
        if e:
            continue
        v = st[1] + int(s)
        if abs(v) > DEC38_MAX:
            st[0] = "overflow"
        else:
            st[0], st[1] = "normal", v
    out = {}
    for k, (kind, v) in state.items():
        if partial:
            if kind == "overflow":
                out[k] = (None, False)
            elif kind == "empty":
                out[k] = (0, True)
            else:
                r = v * 10**rescale
                out[k] = (None if abs(r) > DEC38_MAX else r, False)
        else:
            if kind != "normal":
                out[k] = (None, kind)
            else:
                r = v * 10**rescale
                out[k] = (None, "overflow") if abs(r) > DEC38_MAX else (r, None)
    return out
