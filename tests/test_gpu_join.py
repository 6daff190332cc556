"""GPU HashJoin parity against the oracle: the reference's eight known-answer
cases (join.cpp:451-920, 18 tuples / count 18) through the C ABI, then seeded
random joins (skewed keys, int64 keys including -1, matrix operands with and
without column maps, empty sides, output bounds).  Join output order is not
defined (the reference pushes tuples from parallel threads), so tuple
multisets are compared."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import bool_to_words
from tests.test_oracle_known_answers import VA, VK, key_matrix

pytestmark = pytest.mark.gpu

A, B, K = 1, 2, 9


def rows_of(cols):
    """Canonical (sorted) tuple multiset as an int64 array of shape (n, ncols)."""
    if not len(cols) or len(cols[0]) == 0:
        return np.zeros((0, len(cols)), np.int64)
    m = np.stack([np.asarray(c).astype(np.int64) for c in cols], axis=1)
    order = np.lexsort(m.T[::-1])
    return m[order]


def gpu_mat(vs, words, rows, cols, col_map=None, row_map=None, kind=2):
    return vs.BitMatrix.from_logical(words, rows, cols, kind=kind, row_map=row_map, col_map=col_map)


@pytest.mark.parametrize("only_count", [False, True])
def test_known_answer_flat_flat(vs, only_count):
    a = vs.FlatTable.from_columns([VA, VK.astype(np.int64)])
    b = vs.FlatTable.from_columns([VA, VK.astype(np.int64)])
    out, count, trunc = vs.hash_join(a, b, 1, 1, only_count)
    assert count == 18 and not trunc
    if not only_count:
        ob = O.hash_join(O.Table(O.FLAT, [A, K], cols=[VA, VK.astype(np.int64)]),
                         O.Table(O.FLAT, [B, K], cols=[VA, VK.astype(np.int64)]), K)
        assert np.array_equal(rows_of(out.columns()), rows_of(ob[1]))


@pytest.mark.parametrize("only_count", [False, True])
@pytest.mark.parametrize("shape", [("flat", "mat", 4), ("flat", "mat", 10), ("mat", "mat", 4)])
def test_known_answer_with_matrices(vs, only_count, shape):
    ka, kb, ncols = shape
    w, cmap = key_matrix(10, ncols, VA, VK)
    if ka == "flat":
        ga = vs.FlatTable.from_columns([VA, VK])
        oa = O.Table(O.FLAT, [A, K], cols=[VA, VK])
    else:
        ga = gpu_mat(vs, w, 10, ncols, col_map=cmap)
        oa = O.Table(O.COLMAIN, [A, K], words=w, mrows=10, mcols=ncols, col_map=cmap)
    gb = gpu_mat(vs, w, 10, ncols, col_map=cmap)
    ob = O.Table(O.COLMAIN, [B, K], words=w, mrows=10, mcols=ncols, col_map=cmap)
    out, count, _ = vs.hash_join(ga, gb, 1, 1, only_count)
    assert count == 18
    _, ocols, ocount = O.hash_join(oa, ob, K, only_count)
    assert ocount == 18
    if not only_count:
        assert np.array_equal(rows_of(out.columns()), rows_of(ocols))


def zipf_keys(rng, n, V, a=1.3):
    """90% uniform keys, 10% Zipf-skewed (hot keys repeat thousands of times)."""
    k = rng.integers(0, V, n)
    hot = rng.random(n) < 0.1
    k[hot] = rng.zipf(a, int(hot.sum())) % V
    return k.astype(np.uint32)


@pytest.mark.parametrize("na,nb", [(1000, 5000), (20000, 3000), (0, 100), (100, 0), (50000, 50000)])
def test_random_flat_flat(vs, na, nb):
    rng = np.random.default_rng(na * 7 + nb)
    V = 5000
    ka, kb = zipf_keys(rng, na, V), zipf_keys(rng, nb, V)
    pa = rng.integers(0, 1 << 31, na).astype(np.uint32)
    pb = rng.integers(-(1 << 40), 1 << 40, nb).astype(np.int64)
    ga = vs.FlatTable.from_columns([pa, ka])
    gb = vs.FlatTable.from_columns([kb, pb])
    _, count_only, _ = vs.hash_join(ga, gb, 1, 0, True)
    out, count, _ = vs.hash_join(ga, gb, 1, 0, False)
    _, ocols, ocount = O.hash_join(O.Table(O.FLAT, [A, K], cols=[pa, ka]),
                                   O.Table(O.FLAT, [K, B], cols=[kb, pb]), K)
    assert count == count_only == ocount
    assert np.array_equal(rows_of(out.columns()), rows_of(ocols))


def test_int64_keys_with_all_ones(vs):
    ka = np.array([-1, -1, 5, 7, -1, 1 << 40], dtype=np.int64)
    kb = np.array([-1, 5, 5, -2, 1 << 40], dtype=np.int64)
    pa = np.arange(len(ka), dtype=np.uint32)
    pb = np.arange(len(kb), dtype=np.uint32) + 100
    out, count, _ = vs.hash_join(vs.FlatTable.from_columns([pa, ka]), vs.FlatTable.from_columns([pb, kb]), 1, 1)
    _, ocols, ocount = O.hash_join(O.Table(O.FLAT, [A, K], cols=[pa, ka]),
                                   O.Table(O.FLAT, [B, K], cols=[pb, kb]), K)
    assert count == ocount == 3 + 2 + 1
    assert np.array_equal(rows_of(out.columns()), rows_of(ocols))


@pytest.mark.parametrize("maps", [(False, False), (True, False), (False, True), (True, True)])
def test_random_mat_mat(vs, maps):
    rng = np.random.default_rng(sum(maps) + 5)
    ra, rb, ca, cb = 150, 70, 300, 260
    ma = rng.random((ra, ca)) < 0.05
    mb = rng.random((rb, cb)) < 0.05
    cma = rng.permutation(400)[:ca].astype(np.uint32) if maps[0] else None
    cmb = rng.permutation(400)[:cb].astype(np.uint32) if maps[1] else None
    rma = rng.integers(0, 1 << 30, ra).astype(np.uint32)
    wa, wb = bool_to_words(ma), bool_to_words(mb)
    ga = gpu_mat(vs, wa, ra, ca, col_map=cma, row_map=rma)
    gb = gpu_mat(vs, wb, rb, cb, col_map=cmb)
    oa = O.Table(O.COLMAIN, [A, K], words=wa, mrows=ra, mcols=ca, col_map=cma, row_map=rma)
    ob = O.Table(O.COLMAIN, [B, K], words=wb, mrows=rb, mcols=cb, col_map=cmb)
    _, c1, _ = vs.hash_join(ga, gb, 1, 1, True)
    out, c2, _ = vs.hash_join(ga, gb, 1, 1, False)
    _, ocols, ocount = O.hash_join(oa, ob, K)
    assert c1 == c2 == ocount
    assert np.array_equal(rows_of(out.columns()), rows_of(ocols))


def test_flat_mat_random_and_mat_flat(vs):
    rng = np.random.default_rng(11)
    rows, cols = 90, 500
    m = rng.random((rows, cols)) < 0.04
    w = bool_to_words(m)
    cm = rng.permutation(2000)[:cols].astype(np.uint32)
    keys = rng.choice(cm, 3000).astype(np.uint32)
    keys[:100] = 1999  # keys missing from the matrix
    pay = rng.integers(0, 1 << 31, 3000).astype(np.uint32)
    gf = vs.FlatTable.from_columns([pay, keys])
    gm = gpu_mat(vs, w, rows, cols, col_map=cm)
    of = O.Table(O.FLAT, [A, K], cols=[pay, keys])
    om = O.Table(O.COLMAIN, [B, K], words=w, mrows=rows, mcols=cols, col_map=cm)
    for first_flat in (True, False):
        x, y = (gf, gm) if first_flat else (gm, gf)
        ox, oy = (of, om) if first_flat else (om, of)
        _, cc, _ = vs.hash_join(x, y, 1, 1, True)
        out, c, _ = vs.hash_join(x, y, 1, 1, False)
        _, ocols, ocount = O.hash_join(ox, oy, K)
        assert cc == c == ocount
        assert np.array_equal(rows_of(out.columns()), rows_of(ocols))


def test_output_bound_reports_capacity(vs):
    k = np.zeros(300, dtype=np.uint32)
    a = vs.FlatTable.from_columns([np.arange(300, dtype=np.uint32), k])
    out, count, trunc = vs.hash_join(a, a, 1, 1, False, max_rows=1000)
    assert count == 90000 and trunc
    assert out.info()[1] == 1000
    cols = out.columns()
    assert np.all(cols[1] == 0)


def test_key_type_mismatch_rejected(vs):
    a = vs.FlatTable.from_columns([VA, VK.astype(np.int64)])
    b = vs.FlatTable.from_columns([VA, VK])
    with pytest.raises(vs.VsError):
        vs.hash_join(a, b, 1, 1, False)
