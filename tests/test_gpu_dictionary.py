"""Dictionary-encoded input vectors (VectorHelper::CreateDictionaryVector,
vector/vector_helper.h:381-420) through the GPU operators.

Row i of a dictionary vector is row ids[i] of its dictionary, NULL when that dictionary row is.
The operators flatten such vectors on the device when they take a batch, so every result must
equal the result on the same rows in flat vectors: group results bit-exact against the oracle
(doubles within 1e-12 * max(|exact|, sum|x|) of the correctly rounded sum), join row multisets
exact.  Here the helpers' batches are built with some columns dictionary-encoded (ids in reverse
order of first appearance, so ids are never row numbers)."""
import ctypes as C

import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import assert_agg_equal, exact_by_key, join_rows_canonical, run_agg, run_join

pytestmark = pytest.mark.gpu

L, D, I, V = omg.LongType(), omg.DoubleType(), omg.IntType(), omg.VarcharType(32)
SUM, CNT, AVG, MAX, MIN = (omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN,
                           omg.OMNI_AGGREGATION_TYPE_AVG, omg.OMNI_AGGREGATION_TYPE_MAX,
                           omg.OMNI_AGGREGATION_TYPE_MIN)


@pytest.fixture
def encode(monkeypatch):
    """Make the helpers' batches dictionary-encode the given column indices."""
    def use(cols):
        monkeypatch.setattr(omg, "make_batch",
                            lambda types, columns, nulls=None: omg.make_dict_batch(types, columns, nulls,
                                                                                   encode=set(cols)))
    return use


@pytest.mark.parametrize("cols", [(0,), (1, 2), (0, 1, 2)])
@pytest.mark.parametrize("device_input", [False, True])
def test_aggregation_over_dictionary_columns(encode, cols, device_input):
    rng = np.random.default_rng(len(cols) * 3 + device_input)
    n = 60_000
    key = rng.integers(-50, 50, n).astype(np.int64)
    km = rng.random(n) < 0.02
    v1 = rng.integers(-1000, 1000, n).astype(np.int64)
    m1 = rng.random(n) < 0.05
    v2 = np.round(rng.random(n), 3)  # few distinct doubles: a real dictionary
    m2 = rng.random(n) < 0.05
    encode(cols)
    gpu, _ = run_agg([0], [L], [[1], [1], [1], [1], [2], [2]], [[L], [L], [L], [L], [D], [D]],
                     [[L], [L], [L], [L], [D], [D]], [SUM, CNT, MIN, MAX, SUM, AVG], [key, v1, v2], [L, L, D],
                     nulls=[km, m1, m2], batch_sizes=(4096, 1000), device_input=device_input)
    ora = oracle.hashagg(
        [key], [oracle.T_LONG], [km],
        [dict(func=f, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1)
         for f in (oracle.F_SUM, oracle.F_COUNT_COL, oracle.F_MIN, oracle.F_MAX)] +
        [dict(func=f, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=m2)
         for f in (oracle.F_SUM, oracle.F_AVG)])
    ex_s = exact_by_key([key], [km], v2, ~m2)
    ex_a = exact_by_key([key], [km], v2, ~m2, divide_by_count=True)
    assert_agg_equal(gpu, ora, 1, double_aggs=(4, 5), exact={4: ex_s, 5: ex_a})


def test_varchar_dictionary_group_key(encode):
    rng = np.random.default_rng(4)
    n = 40_000
    words = np.array([b"", b"alpha", b"beta", b"gamma", b"alphabet", b"x" * 31], dtype=object)
    keys = words[rng.integers(0, len(words), n)]
    km = rng.random(n) < 0.03
    v = rng.integers(0, 100, n).astype(np.int64)
    encode((0,))
    cols, _ = run_agg([0], [V], [[1], [1]], [[L], [L]], [[L], [L]], [SUM, CNT], [keys, v], [V, L],
                      nulls=[km, None], batch_sizes=(4096, 333))
    got = {(None if m else bytes(k)): (int(s), int(c))
           for k, m, s, c in zip(cols[0][0], cols[0][1], cols[1][0], cols[2][0])}
    want = {}
    for k, m, x in zip(keys, km, v):
        g = None if m else bytes(k)
        s, c = want.get(g, (0, 0))
        want[g] = (s + int(x), c + 1)
    assert got == want


@pytest.mark.parametrize("side", ["probe", "build", "both"])
def test_join_with_dictionary_columns(monkeypatch, side):
    rng = np.random.default_rng(len(side))
    nb, npr = 5000, 40_000
    bkey = rng.permutation(nb).astype(np.int64) * 3
    p1 = rng.integers(0, 7, nb).astype(np.int32)  # few distinct payloads
    p1m = rng.random(nb) < 0.1
    pkey = rng.integers(0, 3 * nb, npr).astype(np.int64)
    pkm = rng.random(npr) < 0.02
    flat, _ = run_join([L, I], [bkey, p1], [None, p1m], [0], [L], [pkey], [pkm], [0], [0], [1],
                       batch_sizes=(4096, 777))
    real = omg.make_batch

    def make(types, columns, nulls=None):
        is_build = len(types) == 2
        if (side == "both") or (side == "build") == is_build:
            return omg.make_dict_batch(types, columns, nulls, encode=set(range(len(types))))
        return real(types, columns, nulls)

    monkeypatch.setattr(omg, "make_batch", make)
    enc, _ = run_join([L, I], [bkey, p1], [None, p1m], [0], [L], [pkey], [pkm], [0], [0], [1],
                      batch_sizes=(4096, 777))
    assert join_rows_canonical(enc) == join_rows_canonical(flat)
    assert len(join_rows_canonical(enc)) > 0


def test_dictionary_batch_copies_flatten():
    """batch_to_device / batch_to_host of a dictionary batch give the flat rows."""
    vals = np.array([10, 20, 30, 40], dtype=np.int64)
    dm = np.array([False, True, False, False])
    d = omg.new_host_vector(L, vals, dm)
    ids = np.array([3, 0, 1, 1, 2, 3, 0], dtype=np.int32)
    v = omg.new_dictionary_vector(ids, d)
    omg.lib().omg_vec_free(d)  # the dictionary vector keeps the shared buffers alive
    out = C.c_void_p()
    omg.check(omg.lib().omg_batch_new(len(ids), C.byref(out)))
    omg.check(omg.lib().omg_batch_append(out.value, v))
    dev = omg.batch_to_device(out.value)
    host = omg.batch_to_host(dev)
    (got, mask), = omg.batch_to_numpy(host)
    for h in (out.value, dev, host):
        omg.free_batch(h)
    assert list(mask) == [False, False, True, True, False, False, False]
    assert [int(x) for x, m in zip(got, mask) if not m] == [40, 10, 30, 40, 10]


def test_reference_inner_join_on_dictionary_keys():
    """join_test.cpp:1333-1398 (TestInnerEqualityJoinDictionary): build (long, dictionary long)
    and probe (long, dictionary long) joined on their dictionary columns -> (1, 11, 2, 11) and
    (3, 33, 4, 33)."""
    ids = np.array([0, 1, 2, 3], dtype=np.int32)

    def batch(flat, dict_values):
        d = omg.new_host_vector(L, np.array(dict_values, dtype=np.int64))
        out = C.c_void_p()
        omg.check(omg.lib().omg_batch_new(4, C.byref(out)))
        omg.check(omg.lib().omg_batch_append(out.value, omg.new_host_vector(L, np.array(flat, dtype=np.int64))))
        omg.check(omg.lib().omg_batch_append(out.value, omg.new_dictionary_vector(ids, d)))
        omg.lib().omg_vec_free(d)
        return out.value

    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, L], [1])
    bop = bf.create_operator()
    bop.add_input(batch([1, 2, 3, 4], [111, 11, 333, 33]))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L, L], [0, 1], [1], [0, 1], [L, L], bf)
    pop = pf.create_operator()
    pop.add_input(batch([1, 2, 3, 4], [11, 22, 33, 44]))
    rows = []
    for b in pop.drain():
        cols = omg.batch_to_numpy(b)
        omg.free_batch(b)
        rows += [tuple(int(v[i]) for v, _ in cols) for i in range(len(cols[0][0]))]
    pop.delete()
    pf.close()
    bop.delete()
    bf.close()
    assert sorted(rows) == [(1, 11, 2, 11), (3, 33, 4, 33)]
