"""MatrixTableFilter on the GPU against the oracle: every predicate form
(row-value bitset, column-value bitset, kept or dropped pair list, all three
together) on VarRow and ColMain matrices with row and column maps, bit for
bit; argument errors; and the reference's tcr1 plan shape
(ldbc-finbench/tcr1.cpp:41-60): VExpand with distances, then a filter that
keeps the accounts with a neighbour medium whose isBlocked flag is set."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import bool_to_words
from tests.test_oracle_consumers import value_bits
from vertexsurge_gb300 import graphgen

pytestmark = pytest.mark.gpu

A, B = 1, 2


def rand_bits(rng, rows, cols, density):
    return rng.random((rows, cols)) < density


@pytest.mark.parametrize("kind", [1, 2])  # VarRow, ColMain
def test_filter_forms_match_oracle(vs, kind):
    rng = np.random.default_rng(21)
    rows, cols = 300, 2000
    m = rand_bits(rng, rows, cols, 0.05)
    rmap = rng.permutation(4000)[:rows].astype(np.uint32)
    cmap = rng.permutation(9000)[:cols].astype(np.uint32)
    rkeep = value_bits(rng.choice(rmap, rows // 2, replace=False).tolist(), 4000)
    ckeep = value_bits(rng.choice(cmap, cols // 3, replace=False).tolist(), 9000)
    nz = list(zip(*np.nonzero(m)))
    listed = np.array(sorted({(int(rmap[r]) << 32) | int(cmap[c]) for r, c in nz[::4]}), np.uint64)
    cases = [dict(row_keep=rkeep, row_values=4000),
             dict(col_keep=ckeep, col_values=9000),
             dict(col_keep=ckeep, col_values=5000),
             dict(pairs=listed, pairs_mode=1),
             dict(pairs=listed, pairs_mode=2),
             dict(pairs=np.zeros(0, np.uint64), pairs_mode=1),
             dict(row_keep=rkeep, row_values=4000, col_keep=ckeep, col_values=9000, pairs=listed, pairs_mode=2)]
    for kw in cases:
        words = bool_to_words(m)
        g = vs.BitMatrix.from_logical(words, rows, cols, kind=kind, row_map=rmap, col_map=cmap)
        vs.matrix_filter(g, **kw)
        t = O.Table(O.VARROW if kind == 1 else O.COLMAIN, [A, B], words=words.copy(), mrows=rows, mcols=cols,
                    row_map=rmap, col_map=cmap)
        O.matrix_filter(t, **kw)
        assert np.array_equal(g.download(), t.words), {k: v for k, v in kw.items() if k.endswith("mode")}
        g.free()


def test_filter_rejects_bad_arguments(vs):
    full = np.full((10, 1), np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64)
    m = vs.BitMatrix.from_logical(full, 64, 10)
    with pytest.raises(vs.VsError):  # a pair list out of order
        vs.matrix_filter(m, pairs=np.array([5, 3], np.uint64), pairs_mode=1)
    with pytest.raises(vs.VsError):  # unknown mode
        vs.matrix_filter(m, pairs=np.array([3, 5], np.uint64), pairs_mode=3)
    assert np.array_equal(m.download(), full)
    # a host bitset is copied in: rows 0..31 kept
    host = np.array([0xFFFFFFFF], np.uint64)
    assert vs.lib().vs_matrix_filter(m.h, host.ctypes.data, 64, None, 0, None, 0, 0, None) == 0
    assert np.array_equal(m.download(), np.full((10, 1), 0xFFFFFFFF, np.uint64))
    m.free()


def test_tcr1_plan_shape(vs):
    """VExpand(Shortest, with distances, [1,3]) from account sources, then
    MatrixTableFilter keeping the accounts signed in to a blocked medium."""
    g = graphgen.rmat(13, 8, 0.57, 0.19, 0.19, seed=31)  # accounts and their transfers
    dg = vs.DeviceGraph.from_host(g)
    rng = np.random.default_rng(32)
    n_acc, n_medium = g.V, 3000
    # signIn edges account -> medium, mediums numbered after the accounts
    ne = 3 * n_acc
    sig = graphgen.from_edges(n_acc + n_medium, rng.integers(0, n_acc, ne),
                              n_acc + rng.integers(0, n_medium, ne))
    dsig = vs.DeviceGraph.from_host(sig)
    prop = np.zeros(n_acc + n_medium, np.uint8)
    prop[n_acc:] = rng.random(n_medium) < 0.1  # Medium.isBlocked
    mask = vs.vertex_mask_any_neighbor(dsig, prop, 1)
    omask = O.vertex_mask_any_neighbor(sig.fwd_off, sig.fwd_dst, sig.V, prop, 1)
    assert np.array_equal(mask, omask)
    kept = sum(int(x).bit_count() for x in mask)
    assert 0 < kept < n_acc
    src = graphgen.sample_sources(g.V, 200, seed=33)
    layers = vs.expand_layers(dg, src, 1, 3, "shortest", "forward")
    assert len(layers) == 3
    for h, m in layers:
        vs.matrix_filter(m, col_keep=mask, col_values=n_acc)
        exp, _, _ = O.vexpand(g, src, h, h, "shortest", "forward")
        t = O.Table(O.VARROW, [A, B], words=exp, mrows=len(src), mcols=g.V, row_map=src)
        O.matrix_filter(t, col_keep=omask, col_values=n_acc)
        assert np.array_equal(m.download(), t.words), h
        m.free()
