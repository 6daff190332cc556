"""The oracle's result consumers — MatrixColumnCount, MatrixRowOrSum,
SemiJoin<N> — against independent numpy / Python-set computations of the
reference's semantics (matrix_column_count.cpp:19-87,
matrix_row_or_sum.cpp:14-54, semi_join.cpp:58-262; the reference's own
SemiJoin tests only print their results, so these are the pins)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import bool_to_words

A, B, K = 1, 2, 9


def rand_matrix(rng, rows, cols, density=0.05):
    return rng.random((rows, cols)) < density


@pytest.mark.parametrize("kind", [O.VARROW, O.COLMAIN])
@pytest.mark.parametrize("order", [0, 1, 2])
def test_matrix_column_count(kind, order):
    rng = np.random.default_rng(3)
    m = rand_matrix(rng, 150, 400, 0.03)
    cmap = rng.permutation(10_000)[:400].astype(np.uint32)
    t = O.Table(kind, [A, B], words=bool_to_words(m), mrows=150, mcols=400, col_map=cmap)
    cols, cnt = O.matrix_column_count(t, order)
    pairs = [(int(m[:, c].sum()), int(cmap[c])) for c in range(400)]
    if order == 1:
        pairs.sort()
    elif order == 2:
        pairs.sort(reverse=True)
    assert list(zip(cnt.tolist(), cols.tolist())) == pairs


def test_matrix_row_or_sum():
    rng = np.random.default_rng(4)
    m = rand_matrix(rng, 90, 500, 0.004)
    t = O.Table(O.VARROW, [A, B], words=bool_to_words(m), mrows=90, mcols=500)
    assert O.matrix_row_or_sum(t).tolist() == [c for c in range(500) if m[:, c].any()]


def test_semi_join_flat_flat():
    rng = np.random.default_rng(5)
    a = [rng.integers(0, 50, 300).astype(np.uint32), rng.integers(0, 20, 300).astype(np.int64)]
    b = [rng.integers(0, 50, 200).astype(np.uint32), rng.integers(0, 20, 200).astype(np.int64)]
    ta = O.Table(O.FLAT, [A, K], cols=a)
    tb = O.Table(O.FLAT, [B, K], cols=b)
    keys = set(b[1].tolist())
    exp = [(int(x), int(k)) for x, k in zip(*a) if int(k) in keys]
    var, cols, count = O.semi_join(ta, tb, [K])
    assert var == [A, K] and count == len(exp)
    assert list(zip(cols[0].tolist(), cols[1].tolist())) == exp
    assert O.semi_join(ta, tb, [K], only_count=True)[2] == len(exp)
    # two keys
    tb2 = O.Table(O.FLAT, [K, A], cols=[b[1], b[0]])
    pairs = set(zip(b[0].tolist(), b[1].tolist()))
    exp2 = [(int(x), int(k)) for x, k in zip(*a) if (int(x), int(k)) in pairs]
    assert O.semi_join(ta, tb2, [A, K], only_count=True)[2] == len(exp2)


@pytest.mark.parametrize("b_kind", ["flat", "varrow"])
def test_semi_join_matrix_left(b_kind):
    """VarRow a (rows = a values, cols = b values): keep the bits whose (a, b)
    pair occurs in b; the result is a's matrix with the other bits cleared."""
    rng = np.random.default_rng(6)
    rows, cols = 70, 300
    m = rand_matrix(rng, rows, cols, 0.05)
    rmap = rng.permutation(1000)[:rows].astype(np.uint32)
    ta = O.Table(O.VARROW, [A, B], words=bool_to_words(m), mrows=rows, mcols=cols, row_map=rmap)
    if b_kind == "flat":
        pa = rng.choice(rmap, 2000).astype(np.uint32)
        pb = rng.integers(0, cols, 2000).astype(np.uint32)
        tb = O.Table(O.FLAT, [B, A], cols=[pb, pa])
        pairs = set(zip(pa.tolist(), pb.tolist()))
    else:
        m2 = rand_matrix(rng, rows, cols, 0.3)
        tb = O.Table(O.VARROW, [A, B], words=bool_to_words(m2), mrows=rows, mcols=cols, row_map=rmap)
        pairs = {(int(rmap[r]), c) for r, c in zip(*np.nonzero(m2))}
    keep = np.zeros_like(m)
    for r, c in zip(*np.nonzero(m)):
        keep[r, c] = (int(rmap[r]), int(c)) in pairs
    words, count = O.semi_join(ta, tb, [A, B])
    assert count == int(keep.sum()) > 0
    assert np.array_equal(words, bool_to_words(keep))
    assert O.semi_join(ta, tb, [A, B], only_count=True)[1] == count


def test_semi_join_one_key_against_a_matrix():
    """N = 1 with a VarRow b: b's set is the values of its rows (or columns) holding bits."""
    rng = np.random.default_rng(7)
    m2 = rand_matrix(rng, 40, 60, 0.01)
    tb = O.Table(O.VARROW, [A, B], words=bool_to_words(m2), mrows=40, mcols=60)
    a = rng.integers(0, 60, 500).astype(np.uint32)
    ta = O.Table(O.FLAT, [B], cols=[a])
    present = set(np.nonzero(m2.any(axis=0))[0].tolist())
    assert O.semi_join(ta, tb, [B], only_count=True)[2] == sum(int(x) in present for x in a)
    ta2 = O.Table(O.FLAT, [A], cols=[a % 40])
    present_r = set(np.nonzero(m2.any(axis=1))[0].tolist())
    assert O.semi_join(ta2, tb, [A], only_count=True)[2] == sum(int(x) in present_r for x in a % 40)


def value_bits(values, universe):
    """A bitset (uint64 words) over `universe` values with the given values set."""
    bits = np.zeros((universe + 63) // 64, np.uint64)
    for v in values:
        if v < universe:
            bits[v >> 6] |= np.uint64(1) << np.uint64(v & 63)
    return bits


@pytest.mark.parametrize("kind", [O.VARROW, O.COLMAIN])
def test_matrix_filter(kind):
    """MatrixTableFilter (big_operators2.hh:142-170): a bit (r, c) survives when
    the predicate holds on its mapped (row value, column value), checked against
    a Python loop over the set bits (the reference has no filter test)."""
    rng = np.random.default_rng(11)
    rows, cols = 130, 300
    m = rand_matrix(rng, rows, cols, 0.08)
    rmap = rng.permutation(5000)[:rows].astype(np.uint32)
    cmap = rng.permutation(7000)[:cols].astype(np.uint32)
    rkeep = set(rng.choice(rmap, rows // 2, replace=False).tolist())
    ckeep = set(rng.choice(cmap, cols // 3, replace=False).tolist())
    bits = [(int(rmap[r]), int(cmap[c])) for r, c in zip(*np.nonzero(m))]
    listed = sorted({(r << 32) | c for r, c in bits[::3]} | {(4999 << 32) | 1})
    listed_set = set(listed)
    cases = [dict(row_keep=value_bits(rkeep, 5000), row_values=5000),
             dict(col_keep=value_bits(ckeep, 7000), col_values=7000),
             dict(col_keep=value_bits(ckeep, 6000), col_values=6000),  # values >= 6000 fail
             dict(pairs=np.array(listed, np.uint64), pairs_mode=1),
             dict(pairs=np.array(listed, np.uint64), pairs_mode=2),
             dict(row_keep=value_bits(rkeep, 5000), row_values=5000, col_keep=value_bits(ckeep, 7000),
                  col_values=7000, pairs=np.array(listed, np.uint64), pairs_mode=2)]
    for kw in cases:
        t = O.Table(kind, [A, B], words=bool_to_words(m), mrows=rows, mcols=cols, row_map=rmap, col_map=cmap)

        def keep(r, c):
            if "row_keep" in kw and not (r < kw["row_values"] and r in rkeep):
                return False
            if "col_keep" in kw and not (c < kw["col_values"] and c in ckeep):
                return False
            if kw.get("pairs_mode"):
                return (((r << 32) | c) in listed_set) == (kw["pairs_mode"] == 1)
            return True

        exp = np.zeros_like(m)
        for r, c in zip(*np.nonzero(m)):
            exp[r, c] = keep(int(rmap[r]), int(cmap[c]))
        cleared = O.matrix_filter(t, **kw)
        assert np.array_equal(t.words, bool_to_words(exp))
        assert cleared == int(m.sum() - exp.sum())


def test_vertex_mask_any_neighbor():
    rng = np.random.default_rng(12)
    V, n_other = 400, 90
    deg = rng.integers(0, 6, V)
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.int64)
    adj = rng.integers(0, n_other, int(off[-1])).astype(np.uint32)
    prop = (rng.random(n_other) < 0.2).astype(np.uint8)
    mask = O.vertex_mask_any_neighbor(off, adj, V, prop, 1)
    exp = [v for v in range(V) if any(prop[u] == 1 for u in adj[off[v]:off[v + 1]])]
    assert np.array_equal(mask, value_bits(exp, V))
