"""GPU result consumers — MatrixColumnCount, MatrixRowOrSum, SemiJoin<1|2> —
against the oracle, exact: column counts in column order and both sorted
orders (ties broken by column value as std::less / std::greater on the pair),
non-empty columns, semi-join rows (as multisets of a's rows, in a's order)
and masked matrices bit for bit."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import bool_to_words
from vertexsurge_gb300 import graphgen

pytestmark = pytest.mark.gpu

A, B, K = 1, 2, 9


def gmat(vs, m, kind=1, row_map=None, col_map=None):
    rows, cols = m.shape
    return vs.BitMatrix.from_logical(bool_to_words(m), rows, cols, kind=kind, row_map=row_map, col_map=col_map)


@pytest.mark.parametrize("shape", [(10, 10), (150, 400), (3000, 70_000)])
@pytest.mark.parametrize("kind", [1, 2])
@pytest.mark.parametrize("mapped", [False, True])
def test_matrix_column_count(vs, shape, kind, mapped):
    rng = np.random.default_rng(shape[1] + kind)
    rows, cols = shape
    m = rng.random((rows, cols)) < (3.0 / rows)
    cmap = rng.permutation(cols * 3)[:cols].astype(np.uint32) if mapped else None
    g = gmat(vs, m, kind, col_map=cmap)
    t = O.Table(O.VARROW if kind == 1 else O.COLMAIN, [A, B], words=bool_to_words(m), mrows=rows, mcols=cols,
                col_map=cmap)
    for order in (0, 1, 2):
        got = vs.matrix_column_count(g, order).columns()
        ocols, ocnt = O.matrix_column_count(t, order)
        assert np.array_equal(got[0], ocols), order
        assert np.array_equal(got[1], ocnt), order


def test_column_count_and_row_or_sum_of_an_expand(vs):
    g = graphgen.rmat(11, 8, seed=4)
    dg = vs.DeviceGraph.from_host(g)
    src = graphgen.sample_sources(g.V, 300, seed=3)
    m, _, _ = vs.expand(dg, src, 1, 2, "shortest", "forward")
    w, _, _ = O.vexpand(g, src, 1, 2, "shortest", "forward")
    t = O.Table(O.VARROW, [A, B], words=w, mrows=len(src), mcols=g.V, row_map=src)
    for order in (0, 2):
        got = vs.matrix_column_count(m, order).columns()
        oc, on = O.matrix_column_count(t, order)
        assert np.array_equal(got[0], oc) and np.array_equal(got[1], on)
    got = vs.matrix_row_or_sum(m).columns()[0]
    assert np.array_equal(got, O.matrix_row_or_sum(t)) and len(got) > 0


@pytest.mark.parametrize("mapped", [False, True])
def test_matrix_row_or_sum(vs, mapped):
    rng = np.random.default_rng(9)
    m = rng.random((90, 5000)) < 0.002
    cmap = rng.permutation(20000)[:5000].astype(np.uint32) if mapped else None
    got = vs.matrix_row_or_sum(gmat(vs, m, 1, col_map=cmap)).columns()[0]
    exp = O.matrix_row_or_sum(O.Table(O.VARROW, [A, B], words=bool_to_words(m), mrows=90, mcols=5000,
                                      col_map=cmap))
    assert np.array_equal(got, exp)


def flat_pair(vs, rng, n, hi0, hi1, i64=False):
    c0 = rng.integers(0, hi0, n).astype(np.uint32)
    c1 = rng.integers(0, hi1, n).astype(np.int64 if i64 else np.uint32)
    return [c0, c1]


@pytest.mark.parametrize("i64", [False, True])
def test_semi_join_flat_flat(vs, i64):
    rng = np.random.default_rng(11)
    a = flat_pair(vs, rng, 20000, 500, 300, i64)
    b = flat_pair(vs, rng, 5000, 500, 300, i64)
    ga, gb = vs.FlatTable.from_columns(a), vs.FlatTable.from_columns(b)
    ta, tb = O.Table(O.FLAT, [A, K], cols=a), O.Table(O.FLAT, [B, K], cols=b)
    out, count = vs.semi_join(ga, gb, [1], [1])
    var, ocols, ocount = O.semi_join(ta, tb, [K])
    assert count == ocount > 0
    got = out.columns()
    assert all(np.array_equal(x, y) for x, y in zip(got, ocols))  # a's order is kept
    assert vs.semi_join(ga, gb, [1], [1], only_count=True)[1] == ocount
    if not i64:  # two vertex-id keys, the right input's columns in the other order
        tb2 = O.Table(O.FLAT, [K, A], cols=[b[1], b[0]])
        gb2 = vs.FlatTable.from_columns([b[1], b[0]])
        _, c2 = vs.semi_join(ga, gb2, [0, 1], [1, 0], only_count=True)
        assert c2 == O.semi_join(ta, tb2, [A, K], only_count=True)[2]


@pytest.mark.parametrize("b_kind", ["flat", "varrow"])
def test_semi_join_matrix_left(vs, b_kind):
    rng = np.random.default_rng(12)
    rows, cols = 200, 3000
    m = rng.random((rows, cols)) < 0.02
    rmap = rng.permutation(10_000)[:rows].astype(np.uint32)
    ga = gmat(vs, m, 1, row_map=rmap)
    ta = O.Table(O.VARROW, [A, B], words=bool_to_words(m), mrows=rows, mcols=cols, row_map=rmap)
    if b_kind == "flat":
        pa = rng.choice(rmap, 30000).astype(np.uint32)
        pb = rng.integers(0, cols, 30000).astype(np.uint32)
        gb = vs.FlatTable.from_columns([pb, pa])
        tb = O.Table(O.FLAT, [B, A], cols=[pb, pa])
        bkeys = [1, 0]
    else:
        m2 = rng.random((rows, cols)) < 0.4
        gb = gmat(vs, m2, 1, row_map=rmap)
        tb = O.Table(O.VARROW, [A, B], words=bool_to_words(m2), mrows=rows, mcols=cols, row_map=rmap)
        bkeys = [0, 1]
    out, count = vs.semi_join(ga, gb, [0, 1], bkeys)
    ow, ocount = O.semi_join(ta, tb, [A, B])
    assert count == ocount > 0
    assert np.array_equal(out.download(), ow)
    assert vs.semi_join(ga, gb, [0, 1], bkeys, only_count=True)[1] == ocount


def test_semi_join_one_key_against_a_matrix(vs):
    rng = np.random.default_rng(13)
    m2 = rng.random((40, 600)) < 0.001
    gb = gmat(vs, m2, 1)
    tb = O.Table(O.VARROW, [A, B], words=bool_to_words(m2), mrows=40, mcols=600)
    a = rng.integers(0, 600, 5000).astype(np.uint32)
    ga = vs.FlatTable.from_columns([a])
    for bkey, var, vals in ((1, B, a), (0, A, a % 40)):
        gav = vs.FlatTable.from_columns([vals])
        _, count = vs.semi_join(gav, gb, [0], [bkey], only_count=True)
        tav = O.Table(O.FLAT, [var], cols=[vals])
        assert count == O.semi_join(tav, tb, [var], only_count=True)[2]
    del ga


def test_semi_join_rejects_colmain_and_wide_keys(vs):
    m = np.zeros((8, 8), bool)
    cm = gmat(vs, m, 2)
    f = vs.FlatTable.from_columns([np.arange(8, dtype=np.uint32)] * 3)
    with pytest.raises(vs.VsError):
        vs.semi_join(f, cm, [0], [0])
    with pytest.raises(vs.VsError):
        vs.semi_join(f, f, [0, 1, 2], [0, 1, 2])


def test_select_ids_in_range(vs):
    import torch
    rng = np.random.default_rng(3)
    for dt in (torch.uint8, torch.int16, torch.int32, torch.int64):
        v = torch.from_numpy(rng.integers(0, 50, 10_000).astype(np.int64)).to(dt).cuda()
        got = vs.select_ids_in_range(v, 10, 20).columns()[0]
        h = v.cpu().numpy()
        assert np.array_equal(got, np.nonzero((h >= 10) & (h <= 20))[0].astype(np.uint32)), dt
    assert np.array_equal(vs.select_ids_in_range(77, 0, 0).columns()[0], np.arange(77, dtype=np.uint32))
