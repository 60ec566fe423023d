"""The oracle's helpers for checks at full configuration size (CPU only): the multi-threaded
aggregation equals the single-threaded restatement group for group, its double-double sums
agree with math.fsum, the row fingerprint equals a plain-Python restatement of the device
kernel's row hash, and the kept join build's fingerprint and pairs equal the inner join's rows."""
import math

import numpy as np
import pytest

import oracle

M64 = (1 << 64) - 1


def _mix(k):
    k ^= k >> 33
    k = (k * 0xff51afd7ed558ccd) & M64
    k ^= k >> 33
    k = (k * 0xc4ceb9fe1a85ec53) & M64
    k ^= k >> 33
    return k


def _py_fingerprint(cols, nulls):
    """The device kernel's row hash (util.cu FingerprintKernel) in plain Python."""
    acc = [0, 0, 0]
    for r in range(len(cols[0])):
        h = 0x243f6a8885a308d3
        for c, col in enumerate(cols):
            if nulls[c] is not None and nulls[c][r]:
                h = _mix(h ^ 0x9e3779b97f4a7c15 ^ c)
            elif col.ndim == 2:
                h = _mix(h ^ int(col[r, 0]))
                h = _mix(h ^ int(col[r, 1]))
            else:
                w = col.dtype.itemsize
                h = _mix(h ^ (int(col[r]) & ((1 << (8 * w)) - 1)))
        acc[0] += 1
        acc[1] = (acc[1] + _mix(h)) & M64
        acc[2] = (acc[2] + _mix(h ^ 0xc2b2ae3d27d4eb4f)) & M64
    return tuple(acc)


def _groups(res):
    keys, knulls, vals, vnulls = res[:4]
    out = {}
    for i in range(len(keys[0])):
        k = tuple(None if m[i] else (tuple(int(x) for x in v[i]) if v.ndim == 2 else int(v[i]))
                  for v, m in zip(keys, knulls))
        out[k] = tuple(None if vn[i] else (tuple(int(x) for x in v[i]) if v.ndim == 2 else v[i].item())
                       for v, vn in zip(vals, vnulls))
    return out


@pytest.mark.parametrize("threads", [1, 3, 16])
def test_hashagg_mt_equals_hashagg(threads):
    rng = np.random.default_rng(threads)
    n = 120_000
    k1 = rng.integers(0, 40, n).astype(np.int32)
    k2 = rng.integers(-2**62, 2**62, 300, dtype=np.int64)[rng.integers(0, 300, n)]
    km = rng.random(n) < 0.01
    dec = rng.integers(-10**9, 10**9, n).astype(np.int64)
    dn = rng.random(n) < 0.02
    d = rng.standard_normal(n)
    dd = rng.random(n) < 0.02
    v = rng.integers(-10**6, 10**6, n).astype(np.int64)
    aggs = [dict(func=oracle.F_SUM, col=dec, in_type=oracle.T_DEC64, out_type=oracle.T_DEC128, nulls=dn),
            dict(func=oracle.F_COUNT_ALL, col=None, in_type=oracle.T_LONG, out_type=oracle.T_LONG),
            dict(func=oracle.F_AVG, col=d, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=dd),
            dict(func=oracle.F_SUM, col=d, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=dd),
            dict(func=oracle.F_MIN, col=v, in_type=oracle.T_LONG, out_type=oracle.T_LONG),
            dict(func=oracle.F_MAX, col=v, in_type=oracle.T_LONG, out_type=oracle.T_LONG)]
    ktypes = [oracle.T_INT, oracle.T_LONG]
    single = oracle.hashagg([k1, k2], ktypes, [None, km], aggs)
    multi = oracle.hashagg_mt([k1, k2], ktypes, [None, km], aggs, threads=threads)
    assert _groups(single) == _groups(multi)
    # Double-double sums and sums of |x| against math.fsum, group by group.
    exact, absum = multi[4], multi[5]
    assert exact[0] is None and exact[1] is None and exact[4] is None
    keys = [tuple(x) for x in zip(k1.tolist(), np.where(km, -1, k2).tolist(), km.tolist())]
    by = {}
    for i, k in enumerate(keys):
        if not dd[i]:
            by.setdefault(k, []).append(d[i])
    mk = multi[0]
    for g in range(len(mk[0])):
        k = (int(mk[0][g]), -1 if multi[1][1][g] else int(mk[1][g]), bool(multi[1][1][g]))
        xs = by.get(k, [])
        assert exact[2][g] == math.fsum(xs) and exact[3][g] == math.fsum(xs)
        assert abs(absum[2][g] - math.fsum(abs(x) for x in xs)) <= 1e-9 * max(1.0, absum[2][g])


def test_fingerprint_cols_equals_python_restatement():
    rng = np.random.default_rng(3)
    n = 300
    cols = [rng.integers(-2**63, 2**63 - 1, n, dtype=np.int64), rng.integers(-2**31, 2**31, n).astype(np.int32),
            rng.integers(-9, 9, n).astype(np.int16), rng.integers(0, 2**64 - 1, (n, 2), dtype=np.uint64),
            rng.integers(-100, 100, n).astype(np.int8)]
    nulls = [None, rng.random(n) < 0.2, None, rng.random(n) < 0.1, rng.random(n) < 0.5]
    assert oracle.fingerprint_cols(cols, nulls) == _py_fingerprint(cols, nulls)
    # Order-independent, and sensitive to a changed value.
    perm = rng.permutation(n)
    assert oracle.fingerprint_cols([c[perm] for c in cols], [None if m is None else m[perm] for m in nulls]) == \
        oracle.fingerprint_cols(cols, nulls)
    c0 = cols[0].copy()
    c0[7] ^= 1
    assert oracle.fingerprint_cols([c0] + cols[1:], nulls) != oracle.fingerprint_cols(cols, nulls)


@pytest.mark.parametrize("dense", [True, False])
def test_join_table_fingerprint_and_pairs(dense):
    rng = np.random.default_rng(11)
    nb = 5000
    bkey = rng.permutation(nb).astype(np.int64) if dense else 2 * rng.choice(2**39, nb, replace=False)
    bnull = rng.random(nb) < 0.01
    p1 = rng.integers(-2**31, 2**31, nb).astype(np.int32)
    p2 = rng.integers(-2**62, 2**62, nb, dtype=np.int64)
    pkey = np.where(rng.random(80_000) < 0.8, bkey[rng.integers(0, nb, 80_000)], 2 * nb + 1)
    pnull = rng.random(80_000) < 0.01
    jt = oracle.JoinTable(bkey, bnull)
    try:
        pi, bi = jt.pairs(pkey, pnull)
        ri, rb = oracle.join_inner(bkey, bnull, pkey, pnull)
        assert np.array_equal(pi, ri) and np.array_equal(bi, rb)
        for threads in (1, 5):
            fp, _ = jt.fingerprint([p1, p2], pkey, pnull, threads=threads)
            assert fp == oracle.fingerprint_cols([pkey[pi], p1[bi], p2[bi]])
    finally:
        jt.close()


def test_masked_aggregator_equals_aggregator_over_kept_rows():
    """The oracle's mask rule (MaskColAggregator::ProcessGroup): a masked aggregator equals the
    unmasked one over the rows whose mask is TRUE and not NULL, and every row still makes its
    group (groups without kept rows give NULL / 0)."""
    rng = np.random.default_rng(8)
    n = 20_000
    key = rng.integers(0, 300, n).astype(np.int64)
    v = rng.integers(-10**6, 10**6, n).astype(np.int64)
    vn = rng.random(n) < 0.05
    mask = rng.random(n) < 0.5
    mask[key < 20] = False
    mn = rng.random(n) < 0.1
    funcs = (oracle.F_SUM, oracle.F_COUNT_COL, oracle.F_COUNT_ALL, oracle.F_MIN, oracle.F_MAX)
    masked = oracle.hashagg_mt([key], [oracle.T_LONG], [None],
                               [dict(func=f, col=v, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=vn,
                                     mask=mask, mask_nulls=mn) for f in funcs], threads=3)
    keep = mask & ~mn
    plain = oracle.hashagg([key[keep]], [oracle.T_LONG], [None],
                           [dict(func=f, col=v[keep], in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=vn[keep])
                            for f in funcs])
    got, want = _groups(masked), _groups(plain)

    assert len(got) == len(np.unique(key))
    for k, vals in got.items():
        if k in want:
            assert vals == want[k]
        else:  # no kept row: NULL SUM/MIN/MAX, zero counts
            assert vals == (None, 0, 0, None, None)


def test_decimal128_min_max_restatement():
    """The oracle's decimal128 MIN / MAX against Python integers, group by group."""
    rng = np.random.default_rng(12)
    n = 5000
    key = rng.integers(0, 60, n).astype(np.int64)
    vals = [int(rng.integers(-2**62, 2**62)) * (1 << 64) + int(rng.integers(0, 2**63)) for _ in range(n)]
    dec = np.array([[v & M64, (v >> 64) & M64] for v in vals], dtype=np.uint64)
    nulls = rng.random(n) < 0.1
    nulls[key == 3] = True
    res = oracle.hashagg([key], [oracle.T_LONG], [None],
                         [dict(func=f, col=dec, in_type=oracle.T_DEC128, out_type=oracle.T_DEC128, nulls=nulls)
                          for f in (oracle.F_MIN, oracle.F_MAX)])
    got = _groups(res)
    for k in np.unique(key):
        xs = [vals[i] for i in range(n) if key[i] == k and not nulls[i]]
        g = got[(int(k),)]
        if not xs:
            assert g == (None, None)
            continue
        lo, hi = min(xs), max(xs)
        assert g == ((lo & M64, (lo >> 64) & M64), (hi & M64, (hi >> 64) & M64))


def _py_decimal_avg(vals, in_prec, in_scale, out_scale, out_dec64=False):
    """Spark's decimal AVG in Python integers: checked sum (None on overflow), then CalcAvg."""
    big = 10**38 - 1
    s, n = 0, 0
    for v in vals:
        s += v
        n += 1
        if (out_dec64 and not -2**63 <= s < 2**63) or (not out_dec64 and abs(s) > big):
            return None
    if n == 0:
        return None

    def rnd(a, b):  # half away from zero
        q = (abs(a) + abs(b) // 2) // abs(b)
        return q if (a >= 0) == (b > 0) else -q
    sp = min(in_prec + 10, 38)
    scale = max(6, in_scale + 21)
    prec = sp - in_scale + scale
    if prec > 38:
        scale = max(38 - (prec - scale), min(scale, 6))
    dividend = s * 10**(scale - in_scale)
    ovf = abs(dividend) > big
    avg = rnd(dividend, n)
    diff = out_scale - scale
    if diff >= 0:
        out = avg * 10**diff
        ovf = ovf or abs(out) > big
    else:
        out = rnd(avg, 10**-diff)
    if ovf:
        return None
    # a decimal64 result is the 128-bit value cut to 64 bits (static_cast<int64_t>)
    return ((out + 2**63) % 2**64) - 2**63 if out_dec64 else out


@pytest.mark.parametrize("case", ["dec64_to_dec128", "dec128_to_dec128", "dec64_to_dec64"])
def test_decimal_avg_restatement(case):
    """AVG of decimals (AverageSparkDecimalAggregator): a hand-checked value, then random groups
    (with overflowing ones for the 128-bit cases) against a Python-integer restatement."""
    # 1.00, 2.00, 2.00 as decimal(18,2) -> decimal(22,6): 5.00 / 3 at scale 12, then scale 6 = 1.666667
    got = oracle.hashagg([np.zeros(3, np.int64)], [oracle.T_LONG], [None],
                         [dict(func=oracle.F_AVG, col=np.array([100, 200, 200], np.int64), in_type=oracle.T_DEC64,
                               out_type=oracle.T_DEC128, in_prec=18, in_scale=2, out_scale=6)])
    assert int(got[2][0][0][0]) == 1666667
    rng = np.random.default_rng(4)
    n = 20_000
    key = rng.integers(0, 400, n).astype(np.int64)
    nulls = rng.random(n) < 0.05
    if case == "dec128_to_dec128":
        vals = [int(rng.integers(-10**18, 10**18)) * 10**int(rng.integers(0, 19)) for _ in range(n)]
        in_t, out_t, prec, sc, osc = oracle.T_DEC128, oracle.T_DEC128, 38, 4, 8
        col = np.array([[v & M64, (v >> 64) & M64] for v in vals], dtype=np.uint64)
    else:
        vals = [int(x) for x in rng.integers(-10**17, 10**17, n)]
        in_t, prec, sc = oracle.T_DEC64, 18, 2
        out_t, osc = (oracle.T_DEC64, 6) if case == "dec64_to_dec64" else (oracle.T_DEC128, 6)
        col = np.array(vals, dtype=np.int64)
    res = oracle.hashagg([key], [oracle.T_LONG], [None],
                         [dict(func=oracle.F_AVG, col=col, in_type=in_t, out_type=out_t, nulls=nulls, in_prec=prec,
                               in_scale=sc, out_scale=osc)], overflow_as_null=True)
    keys, _, vals_out, vnulls = res
    for i in range(len(keys[0])):
        k = int(keys[0][i])
        xs = [vals[j] for j in range(n) if key[j] == k and not nulls[j]]
        want = _py_decimal_avg(xs, prec, sc, osc, out_dec64=out_t == oracle.T_DEC64)
        if want is None:
            assert vnulls[0][i]
            continue
        assert not vnulls[0][i]
        v = vals_out[0][i]
        got = (int(v[1]) << 64 | int(v[0])) if np.ndim(v) else int(v)
        if np.ndim(v) and got >> 127:
            got -= 1 << 128
        assert got == want, (k, got, want)
