"""The oracle's restatement of the merging decimal SUM (CPU): hand-made partial rows with
empty groups, NULL (overflowed) partial sums, an order-dependent overflow and rescaling."""
import oracle

BIG = 6 * 10**37


def test_merge_final_and_partial_semantics():
    keys = [1, 1, 2, 2, 3, 3, 3, 4, 5, 5]
    sums = [5, 7, 0, 0, BIG, BIG, -BIG, 0, 0, 3]
    nulls = [False, False, False, False, False, False, False, True, False, False]
    empties = [False, False, True, True, False, False, False, False, True, False]
    fin = oracle.decimal_sum_merge(keys, sums, nulls, empties)
    assert fin[1] == (12, None)
    assert fin[2] == (None, "empty")
    # 6e37 + 6e37 exceeds 10^38 - 1 on the second row: sticky, though the total is 6e37.
    assert fin[3] == (None, "overflow")
    assert fin[4] == (None, "overflow")  # a NULL partial sum is an overflowed partial
    assert fin[5] == (3, None)
    part = oracle.decimal_sum_merge(keys, sums, nulls, empties, partial=True)
    assert part[1] == (12, False) and part[2] == (0, True) and part[3] == (None, False)
    assert part[4] == (None, False) and part[5] == (3, False)
    # Rescaling by 10^1: 3 -> 30; a rescale beyond 38 digits overflows.
    assert oracle.decimal_sum_merge([1], [3], [False], [False], rescale=1)[1] == (30, None)
    assert oracle.decimal_sum_merge([1], [BIG], [False], [False], rescale=1)[1] == (None, "overflow")
