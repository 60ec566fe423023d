"""Shared test helpers: run the GPU operators through the C ABI and compare with the oracle."""
from __future__ import annotations

import math

import numpy as np

import omnioperator_gb300 as omg
import oracle

# Map api DataType ids to oracle ids (same numbering).
DOUBLE_TOL = 1e-12


def split(n, sizes):
    """Row ranges of consecutive batches with the given (cycled) sizes."""
    out, s, i = [], 0, 0
    while s < n:
        e = min(n, s + sizes[i % len(sizes)])
        out.append((s, e))
        s, i = e, i + 1
    return out


def run_agg(group_cols, group_types, aggs_cols, agg_in_types, agg_out_types, funcs, columns, types, nulls=None,
            batch_sizes=(4096,), overflow_as_null=False, strategy=None, capacity_hint=0, device_input=False,
            pipeline=False, mask_cols=None, spill_budget=None):
    """Run HashAggregation on the GPU; returns (output columns as [(values, mask)], op counters)."""
    fac = omg.HashAggregationOperatorFactory(group_cols, group_types, aggs_cols, agg_in_types, agg_out_types, funcs,
                                             mask_cols=mask_cols, overflow_as_null=overflow_as_null)
    op = fac.create_operator()
    try:
        if strategy is not None:
            op.set_agg_strategy(strategy, capacity_hint)
        if spill_budget is not None:
            op.set_spill(True, spill_budget)
        if pipeline:
            op.set_no_more_input(False)
        n = len(columns[0])
        for s, e in split(n, list(batch_sizes)):
            b = omg.make_batch(types, [c[s:e] for c in columns],
                               None if nulls is None else [None if m is None else m[s:e] for m in nulls])
            if device_input:
                d = omg.batch_to_device(b)
                omg.free_batch(b)
                b = d
            op.add_input(b)
        if pipeline:
            op.no_more_input()
        outs = op.drain()
        assert op.get_status() == omg.OMNI_STATUS_FINISHED
        cols = None
        for b in outs:
            c = omg.batch_to_numpy(b)
            omg.free_batch(b)
            cols = c if cols is None else [(np.concatenate([a[0], x[0]]), np.concatenate([a[1], x[1]]))
                                           for a, x in zip(cols, c)]
        counters = op.counters()
        counters["sizing"] = op.sizing_log()
    finally:
        op.delete()
        fac.close()
    return cols, counters


def canon_key(vals, mask):
    """Hashable per-row key values (None for NULL)."""
    out = []
    for i in range(len(mask)):
        if mask[i]:
            out.append(None)
        else:
            v = vals[i]
            out.append(tuple(int(x) for x in v) if np.ndim(v) else (float(v) if isinstance(v, np.floating) else int(v)))
    return out


def rows_by_key(cols, nkeys):
    keys = list(zip(*[canon_key(v, m) for v, m in cols[:nkeys]]))
    res = {}
    for i, k in enumerate(keys):
        assert k not in res, f"duplicate group {k}"
        res[k] = i
    return res


def assert_agg_equal(gpu_cols, ora, nkeys, double_aggs=(), exact=None):
    """Compare GPU output columns with oracle.hashagg output.  Integer/decimal/count/min/max
    columns must match bit for bit (and NULLs exactly); double SUM/AVG columns (indices in
    `double_aggs`) must lie within DOUBLE_TOL * max(|exact|, sum|x|) of the exact sum, where
    `exact[j] = (exact_values_by_group_key, abs_sum_by_group_key, divisor_by_group_key)`."""
    okeys, oknulls, ovals, onulls = ora
    ng = len(okeys[0]) if okeys else 0
    if gpu_cols is None:
        assert ng == 0
        return
    assert len(gpu_cols[0][0]) == ng, f"group count {len(gpu_cols[0][0])} != {ng}"
    gi = rows_by_key(gpu_cols, nkeys)
    okey_rows = list(zip(*[canon_key(k, m) for k, m in zip(okeys, oknulls)]))
    for orow, k in enumerate(okey_rows):
        assert k in gi, f"group {k} missing on GPU"
        grow = gi[k]
        for j in range(len(ovals)):
            gv, gm = gpu_cols[nkeys + j]
            assert bool(gm[grow]) == bool(onulls[j][orow]), f"null mismatch group {k} agg {j}"
            if onulls[j][orow]:
                continue
            if j in double_aggs:
                ex, ab, div = exact[j]
                e, a, d = ex[k], ab[k], div[k]
                target = e / d
                tol = DOUBLE_TOL * max(abs(e), a) / d
                got = float(gv[grow])
                assert abs(got - target) <= tol, f"double agg {j} group {k}: gpu {got!r} exact {target!r} tol {tol}"
            else:
                g = gv[grow]
                o = ovals[j][orow]
                if np.ndim(g):
                    assert tuple(int(x) for x in g) == tuple(int(x) for x in o), f"agg {j} group {k}: {g} != {o}"
                elif isinstance(g, np.floating):
                    assert (g == o) or (np.isnan(g) and np.isnan(o)), f"agg {j} group {k}: {g!r} != {o!r}"
                else:
                    assert int(g) == int(o), f"agg {j} group {k}: {g} != {o}"


def exact_by_key(key_cols, key_nulls, values, valid, divide_by_count=False):
    """{group key: correctly rounded sum}, {key: sum |x|}, {key: count or 1} for a double agg."""
    keys = list(zip(*[canon_key(k, np.zeros(len(k), bool) if m is None else m) for k, m in zip(key_cols, key_nulls)]))
    uniq = {}
    gid = np.empty(len(keys), dtype=np.int64)
    for i, k in enumerate(keys):
        gid[i] = uniq.setdefault(k, len(uniq))
    ex, ab = oracle.exact_group_sums(gid, values.astype(np.float64), valid, len(uniq))
    cnt = np.bincount(gid[valid] if valid is not None else gid, minlength=len(uniq))
    inv = {v: k for k, v in uniq.items()}
    exd = {inv[i]: ex[i] for i in range(len(uniq))}
    abd = {inv[i]: ab[i] for i in range(len(uniq))}
    dv = {inv[i]: (float(cnt[i]) if divide_by_count else 1.0) for i in range(len(uniq))}
    return exd, abd, dv


def run_join(build_types, build_cols, build_nulls, build_hash_cols, probe_types, probe_cols, probe_nulls,
             probe_hash_cols, probe_out, build_out, batch_sizes=(4096,), build_batch=1 << 20, pipeline=False,
             device_input=False, device_output=False):
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, build_types, build_hash_cols)
    bop = bf.create_operator()
    pf = pop = None
    try:
        nb = len(build_cols[0])
        for s, e in split(nb, [build_batch]):
            bop.add_input(omg.make_batch(build_types, [c[s:e] for c in build_cols],
                                         None if build_nulls is None else
                                         [None if m is None else m[s:e] for m in build_nulls]))
        bop.get_output()
        assert bop.get_status() == omg.OMNI_STATUS_FINISHED
        pf = omg.LookupJoinOperatorFactory(probe_types, probe_out, probe_hash_cols, build_out,
                                           [build_types[c] for c in build_out], bf)
        pop = pf.create_operator()
        assert not pop.is_blocked()
        if device_output:
            pop.set_device_output(True)
        if pipeline:
            pop.set_no_more_input(False)
        n = len(probe_cols[0])
        outs = []
        for s, e in split(n, list(batch_sizes)):
            b = omg.make_batch(probe_types, [c[s:e] for c in probe_cols],
                               None if probe_nulls is None else [None if m is None else m[s:e] for m in probe_nulls])
            if device_input:
                d = omg.batch_to_device(b)
                omg.free_batch(b)
                b = d
            pop.add_input(b)
            if not pipeline:
                outs.extend(pop.drain())
        if pipeline:
            outs.extend(pop.drain())
            pop.no_more_input()
            outs.extend(pop.drain())
        assert pop.get_status() == omg.OMNI_STATUS_FINISHED
        cols = None
        max_rows = 0
        for b in outs:
            max_rows = max(max_rows, omg.batch_row_count(b))
            if device_output:
                h = omg.batch_to_host(b)
                omg.free_batch(b)
                b = h
            c = omg.batch_to_numpy(b)
            omg.free_batch(b)
            cols = c if cols is None else [(np.concatenate([a[0], x[0]]), np.concatenate([a[1], x[1]]))
                                           for a, x in zip(cols, c)]
        return cols, max_rows
    finally:
        if pop:
            pop.delete()
        bop.delete()
        if pf:
            pf.close()
        bf.close()


def join_rows_canonical(cols):
    """Sorted row tuples (NULL as None) of output columns."""
    if cols is None:
        return []
    per = [canon_key(v, m) for v, m in cols]
    rows = list(zip(*per))
    return sorted(rows, key=lambda r: tuple((x is None, x if x is not None else 0) for x in r))


def expected_join_rows(probe_cols, probe_nulls, build_cols, build_nulls, pk, bk, probe_out, build_out):
    pn = None if probe_nulls is None else probe_nulls[pk]
    bn = None if build_nulls is None else build_nulls[bk]
    pi, bi = oracle.join_inner(build_cols[bk], bn, probe_cols[pk], pn)
    cols = []
    for c in probe_out:
        m = probe_nulls[c] if probe_nulls is not None and probe_nulls[c] is not None else np.zeros(len(probe_cols[c]), bool)
        cols.append((probe_cols[c][pi], m[pi]))
    for c in build_out:
        m = build_nulls[c] if build_nulls is not None and build_nulls[c] is not None else np.zeros(len(build_cols[c]), bool)
        cols.append((build_cols[c][bi], m[bi]))
    return join_rows_canonical(cols)


def kat_columns(k):
    """Build/probe columns and NULL masks of a typed join KAT ("types": one type for all
    columns or a list per column)."""
    dts = {"SHORT": np.int16, "INT": np.int32, "LONG": np.int64}
    t = k.get("types", "LONG")

    def side(cols, nulls):
        kinds = t if isinstance(t, list) else [t] * len(cols)
        vals = [np.array(c, dtype=dts[kd]) for c, kd in zip(cols, kinds)]
        masks = [np.zeros(len(c), bool) for c in cols]
        for m, rows in zip(masks, nulls or []):
            m[rows] = True
        return vals, masks
    return side(k["build"], k["build_nulls"]), side(k["probe"], k["probe_nulls"])


def kat_hash_cols(k, side):
    """Key columns of a KAT side ("build"/"probe"): one column or a list."""
    v = k.get(side + "_hash_cols", k.get(side + "_hash_col"))
    return v if isinstance(v, list) else [v]


def tuple_ids(build_keys, build_masks, probe_keys, probe_masks):
    """Dense ids of key tuples over both sides (equal tuples, equal ids; decimal128 as (n, 2)
    words) and each row's NULL flag (any key column NULL): a multi-column key restated as one
    column for the oracle's join."""
    nb = len(build_keys[0])
    cols = []
    for bk, pk in zip(build_keys, probe_keys):
        a = np.concatenate([np.asarray(bk), np.asarray(pk)])
        if a.ndim == 2:
            cols += [a[:, 0].astype(np.int64), a[:, 1].astype(np.int64)]
        else:
            cols.append(a.astype(np.int64))
    mat = np.stack(cols, axis=1)
    _, inv = np.unique(mat, axis=0, return_inverse=True)
    inv = np.asarray(inv).reshape(-1).astype(np.int64)
    nulls = np.zeros(len(mat), bool)
    for bm, pm in zip(build_masks, probe_masks):
        nulls |= np.concatenate([bm, pm])
    return inv[:nb], nulls[:nb], inv[nb:], nulls[nb:]


def oracle_join_rows(k):
    """(probe-side rows, outer-join rows) of a typed join KAT computed by the oracle: probe
    output values, then build output values or the existence flag; None = NULL."""
    (b, bm), (p, pm) = kat_columns(k)
    kind = oracle.join_kind(k["join_type"], k["build_side"])
    bh, ph = kat_hash_cols(k, "build"), kat_hash_cols(k, "probe")
    bid, bn, pid, pn = tuple_ids([b[c] for c in bh], [bm[c] for c in bh], [p[c] for c in ph], [pm[c] for c in ph])
    pi, bi = oracle.join(kind, bid, bn, pid, pn)
    rows, outer = [], []
    for i, j in zip(pi.tolist(), bi.tolist()):
        r = [None if i < 0 or pm[c][i] else int(p[c][i]) for c in k["probe_output_cols"]]
        if kind == "existence":
            r.append(j)
        else:
            r += [None if j < 0 or bm[c][j] else int(b[c][j]) for c in k["build_output_cols"]]
        (outer if i < 0 else rows).append(r)
    return rows, outer


def row_key(r):
    return tuple((v is None, 0 if v is None else v) for v in r)


def rows_matrix(cols):
    """Row multiset of output columns [(values, NULL mask)] as a lexicographically sorted int64
    matrix with a (NULL flag, value) pair per column (value 0 when NULL)."""
    if not cols:
        return np.zeros((0, 0), dtype=np.int64)
    parts = []
    for v, m in cols:
        m = np.asarray(m, dtype=bool)
        parts.append(m.astype(np.int64))
        parts.append(np.where(m, 0, np.asarray(v).astype(np.int64)))
    mat = np.stack(parts, axis=1)
    order = np.lexsort(mat.T[::-1])
    return mat[order]
