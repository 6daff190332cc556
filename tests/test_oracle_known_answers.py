"""Pin the CPU oracle to the known answers of the reference's own unit tests.

HashJoin{FlatFlat,FlatMat,MatFlat,MatMat}[CountOnly] -> 18
  (src/objects/operator/join.cpp:451-920)
Mintersect{FlatFlatFlat,FlatMatMat} -> 3 (src/objects/operator/mintersect.cpp:347-511)
TableConvertVRtoCM[_T] exactness (src/objects/operator/big_operators2.cpp:215-296)
VarRow/ColMain iterator round trip (src/objects/execution/bit_matrix_table.cpp:363-483)
DenseMatrix set-all/count (src/objects/storage/bitmap.cpp:1303-1336)
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import bool_to_words, words_to_bool

# variable ids standing in for the reference's variable names
A, B, C, K = 1, 2, 3, 9
VA = np.arange(1, 9, dtype=np.uint32)           # {1..8}
VK = np.array([1, 1, 1, 2, 2, 3, 3, 4], dtype=np.uint32)  # {1,1,1,2,2,3,3,4}


def flat(var, *cols):
    return O.Table(O.FLAT, var, cols=list(cols))


def key_matrix(rows, cols, row_vals, keys, pad_keys=True):
    """ColMain (row var, key var): set(row_vals[i], k_map[keys[i]]), col_map = distinct keys;
    extra physical columns get keys that match nothing."""
    k_map = {}
    k_mapv = []
    for x in keys:
        if int(x) not in k_map:
            k_map[int(x)] = len(k_map)
            k_mapv.append(int(x))
    m = np.zeros((rows, cols), dtype=bool)
    for r, k in zip(row_vals, keys):
        m[int(r), k_map[int(k)]] = True
    cmap = np.array(k_mapv + [1000 + i for i in range(cols - len(k_mapv))], dtype=np.uint32)
    return bool_to_words(m), cmap


def colmain(var, rows, cols, row_vals, keys):
    w, cmap = key_matrix(rows, cols, row_vals, keys)
    return O.Table(O.COLMAIN, var, words=w, mrows=rows, mcols=cols, col_map=cmap)


def sorted_rows(cols):
    return sorted(zip(*[c.tolist() for c in cols]))


@pytest.mark.parametrize("only_count", [False, True])
def test_hash_join_flat_flat(only_count):
    a = flat([A, K], VA, VK.astype(np.int64))
    b = flat([B, K], VA, VK.astype(np.int64))
    var, cols, count = O.hash_join(a, b, K, only_count)
    assert count == 18
    if not only_count:
        assert var == [A, K, B] and len(cols[0]) == 18
        expect = sorted((int(x), int(k), int(y)) for x, k in zip(VA, VK) for y, k2 in zip(VA, VK) if k == k2)
        assert sorted_rows(cols) == expect


@pytest.mark.parametrize("only_count", [False, True])
def test_hash_join_flat_mat(only_count):
    a = flat([A, K], VA, VK)
    b = colmain([B, K], 10, 4, VA, VK)
    var, cols, count = O.hash_join(a, b, K, only_count)
    assert count == 18
    if not only_count:
        assert var == [A, K, B]
        expect = sorted((int(x), int(k), int(y)) for x, k in zip(VA, VK) for y, k2 in zip(VA, VK) if k == k2)
        assert sorted_rows(cols) == expect


@pytest.mark.parametrize("only_count", [False, True])
def test_hash_join_mat_flat(only_count):
    a = flat([A, K], VA, VK)
    b = colmain([B, K], 10, 10, VA, VK)
    var, cols, count = O.hash_join(a, b, K, only_count)
    assert count == 18


@pytest.mark.parametrize("only_count", [False, True])
def test_hash_join_mat_mat(only_count):
    a = colmain([A, K], 10, 4, VA, VK)
    b = colmain([B, K], 10, 4, VA, VK)
    var, cols, count = O.hash_join(a, b, K, only_count)
    assert count == 18
    if not only_count:
        assert var == [A, K, B]
        expect = sorted((int(x), int(k), int(y)) for x, k in zip(VA, VK) for y, k2 in zip(VA, VK) if k == k2)
        assert sorted_rows(cols) == expect


def test_mintersect_flat_flat_flat():
    base = flat([A, B], VA, VK)
    d1 = flat([A, C], VA, VK)
    d2 = flat([B, C], VA, VK)
    var, cols, count = O.mintersect(base, [d1, d2], C, 16)
    assert count == 3 and len(cols[0]) == 3
    assert var == [A, B, C]
    assert sorted_rows(cols) == [(1, 1, 1), (2, 1, 1), (3, 1, 1)]
    _, _, c2 = O.mintersect(base, [d1, d2], C, 16, only_count=True)
    assert c2 == 3


def test_mintersect_flat_mat_mat():
    base = flat([A, B], VA, VK)
    w1, m1 = key_matrix(10, 10, VK, VA)   # set(c[i], k_map[a[i]])
    d1 = O.Table(O.COLMAIN, [C, A], words=w1, mrows=10, mcols=10, col_map=m1)
    w2, m2 = key_matrix(10, 10, VK, VA)
    d2 = O.Table(O.COLMAIN, [C, B], words=w2, mrows=10, mcols=10, col_map=m2)
    var, cols, count = O.mintersect(base, [d1, d2], C, 16)
    assert count == 3
    assert sorted_rows(cols) == [(1, 1, 1), (2, 1, 1), (3, 1, 1)]


@pytest.mark.parametrize("transpose", [False, True])
def test_table_convert_exact(transpose):
    rng = np.random.default_rng(123)
    rows, cols = 1000, 10000
    m = rng.random((rows, cols)) < 0.5
    w = bool_to_words(m)
    out = O.table_convert(w, rows, cols, transpose, stack_row_count=512)
    if transpose:
        assert np.array_equal(words_to_bool(out, cols), m.T)
    else:
        assert np.array_equal(words_to_bool(out, rows), m)


def test_varrow_iterator_round_trip():
    rng = np.random.default_rng(123)
    rows, cols = 2000, 10000
    m = rng.random((rows, cols)) < 0.5
    w = bool_to_words(m)
    r, c = O.matrix_iterate(w, rows, cols, stack_row_count=512)
    assert len(r) == int(m.sum()) == O.matrix_count(w, rows, cols, 512)
    pairs = set(zip(r.tolist(), c.tolist()))
    assert len(pairs) == len(r)
    rr, cc = np.nonzero(m)
    assert pairs == set(zip(rr.tolist(), cc.tolist()))


def test_dense_matrix_count_all_set():
    rows, cols = 200, 1000
    m = np.ones((rows, cols), dtype=bool)
    assert O.matrix_count(bool_to_words(m), rows, cols) == rows * cols


def test_matrix_select_matches_columns():
    rng = np.random.default_rng(7)
    rows, cols = 300, 500
    m = rng.random((rows, cols)) < 0.3
    t = rng.integers(0, cols, 77).astype(np.uint32)
    out = O.matrix_select(bool_to_words(m), rows, cols, t)
    assert np.array_equal(words_to_bool(out, rows), m[:, t])
