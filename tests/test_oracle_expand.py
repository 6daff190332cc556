"""Pin the expand oracle (a restatement of VExpand/Expand, which the reference's
own tests only log) against an independent reachability computation, and
check the graph generator's output invariants."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import words_to_bool
from tests import graphs as G
from vertexsurge_gb300 import graphgen


@pytest.fixture(scope="module")
def small():
    return G.small_graphs()


def test_generator_clean_and_consistent(small):
    for name, g in small.items():
        for v in range(0, g.V, max(1, g.V // 200)):
            lst = g.fwd_dst[g.fwd_off[v]:g.fwd_off[v + 1]]
            assert np.all(np.diff(lst.astype(np.int64)) > 0), name  # sorted, no duplicates
            assert not np.any(lst == v), name                       # no self loops
        # reverse CSR holds exactly the transposed edges
        src = np.repeat(np.arange(g.V, dtype=np.uint64), np.diff(g.fwd_off))
        fw = np.sort(src * g.V + g.fwd_dst)
        dst = np.repeat(np.arange(g.V, dtype=np.uint64), np.diff(g.rev_off))
        rv = np.sort(g.rev_src.astype(np.uint64) * g.V + dst)
        assert np.array_equal(fw, rv), name


def test_generator_deterministic():
    a = graphgen.rmat(10, 8, seed=5)
    b = graphgen.rmat(10, 8, seed=5)
    assert np.array_equal(a.fwd_dst, b.fwd_dst) and np.array_equal(a.fwd_off, b.fwd_off)
    assert graphgen.hash64(1, 2, 3) == graphgen.hash64(1, 2, 3)
    assert not np.array_equal(graphgen.rmat(10, 8, seed=6).fwd_dst[:100], a.fwd_dst[:100])


CASES = [
    ("any", 1, 3, "forward"), ("any", 0, 2, "forward"), ("any", 2, 4, "backward"),
    ("any", 1, 2, "both"), ("shortest", 1, 3, "forward"), ("shortest", 0, 3, "both"),
    ("shortest", 2, 5, "forward"), ("shortest", 1, 8, "backward"), ("shortest", 3, 3, "forward"),
]


@pytest.mark.parametrize("path,k_min,k_max,direction", CASES)
def test_oracle_expand_matches_bfs(small, path, k_min, k_max, direction):
    for name, g in small.items():
        S = 70
        src = graphgen.sample_sources(g.V, S, seed=21)
        words, _, st = O.vexpand(g, src, k_min, k_max, path, direction, hop_stats=True)
        got = words_to_bool(words, S)
        if path == "any":
            exp = G.reach_any(g, src, k_min, k_max, direction)
        else:
            exp = G.reach_shortest(g, src, k_min, k_max, direction)
        assert np.array_equal(got, exp), (name, path, k_min, k_max, direction)


def test_oracle_find_shortest(small):
    g = small["rmat10"]
    S = 100
    src = graphgen.sample_sources(g.V, S, seed=31)
    tgt = graphgen.sample_sources(g.V, S, seed=32)
    tgt[:5] = src[:5]  # distance 0 cases
    _, dist, _ = O.vexpand(g, src, 1, 50, "find_shortest", "forward", targets=tgt)
    assert np.array_equal(dist, G.find_shortest(g, src, tgt))


def test_oracle_duplicate_sources_and_stack_sizes(small):
    g = small["rmat10"]
    src = np.array([5, 5, 17, 900, 5, 17], dtype=np.uint32)
    for path in ("any", "shortest"):
        w1, _, _ = O.vexpand(g, src, 1, 3, path, "forward", stack_row_count=1024)
        w2, _, _ = O.vexpand(g, src, 1, 3, path, "forward", stack_row_count=512)
        assert np.array_equal(w1, w2)
        exp = (G.reach_any if path == "any" else G.reach_shortest)(g, src, 1, 3)
        assert np.array_equal(words_to_bool(w1, len(src)), exp)


def test_oracle_self_ring_counts(small):
    """e1-style counts: |{(a,b) in SxS : dist <= 3}| and the Any[1,3] diagonal."""
    g = small["rmat10"]
    src = graphgen.sample_sources(g.V, 64, seed=41)
    w, _, _ = O.vexpand(g, src, 0, 3, "shortest", "both")
    sel = O.matrix_select(w, len(src), g.V, src)
    d = G.bfs_dist(g, src, "both")[:, src]
    assert O.matrix_count(sel, len(src), len(src)) == int((d <= 3).sum())
    w2, _, _ = O.vexpand(g, src, 1, 3, "any", "forward")
    R = words_to_bool(w2, len(src))
    diag = int(R[np.arange(len(src)), src].sum())
    assert diag == int(G.reach_any(g, src, 1, 3)[np.arange(len(src)), src].sum())


# ---- the reference's BlockHilbert hop over its flat edge layout -------------

@pytest.mark.parametrize("path,k_min,k_max,direction", CASES)
def test_blockhilbert_equals_csr_pull(small, path, k_min, k_max, direction):
    for name, g in small.items():
        S = 70
        src = graphgen.sample_sources(g.V, S, seed=21)
        want, _, st_want = O.vexpand(g, src, k_min, k_max, path, direction, hop_stats=True)
        for n_blocks in (1, 7, 64):
            b = O.FlatBlocks(g, direction, n_blocks)
            got, _, st = O.vexpand(g, src, k_min, k_max, path, direction, hop_stats=True, blocks=b)
            assert np.array_equal(got, want), (name, n_blocks)
            assert st == st_want, (name, n_blocks)


def test_blockhilbert_find_shortest_and_stacks(small):
    g = small["rmat11_skew"]
    b = O.FlatBlocks(g, "forward", 16)
    src = graphgen.sample_sources(g.V, 100, seed=31)
    tgt = graphgen.sample_sources(g.V, 100, seed=32)
    tgt[:5] = src[:5]
    _, dist, _ = O.vexpand(g, src, 1, 50, "find_shortest", "forward", targets=tgt, blocks=b)
    assert np.array_equal(dist, G.find_shortest(g, src, tgt))
    # three 512-row stacks, the last one partly used
    src = graphgen.sample_sources(g.V, 1300, seed=33)
    for path in ("any", "shortest"):
        want, _, _ = O.vexpand(g, src, 1, 3, path, "forward", stack_row_count=512)
        got, _, _ = O.vexpand(g, src, 1, 3, path, "forward", stack_row_count=512, blocks=b)
        assert np.array_equal(got, want), path


def test_blockhilbert_layout_is_the_importers(small):
    """The blocks are the reference importer's partitioned hilbert lists of the
    forward direction: the same block bounds and pair order as graph_dir's
    restatement of partition_by_dst + sort_edge_in_peano2."""
    from vertexsurge_gb300 import graph_dir as GD
    for name in ("rmat10", "zipf3000"):
        g = small[name]
        count = 13
        off, pairs = O.FlatBlocks(g, "forward", count).export()
        src = np.repeat(np.arange(g.V, dtype=np.uint32), np.diff(g.fwd_off).astype(np.int64))
        dst = np.asarray(g.fwd_dst, np.uint32)
        by_dst = GD._pair_order(dst, src)
        s_, t_ = src[by_dst], dst[by_dst]
        bounds = GD.partition_by_dst(t_, count)
        assert [int(x) for x in off] == [b for b, _ in bounds] + [len(t_)], name
        for b, e in bounds:
            perm = GD.order_edges(s_[b:e], t_[b:e], "hilbert", g.V, g.V)
            assert np.array_equal(pairs[b:e, 0], s_[b:e][perm]), name
            assert np.array_equal(pairs[b:e, 1], t_[b:e][perm]), name


def test_blockhilbert_more_blocks_than_targets():
    g = graphgen.from_edges(6, np.array([0, 1, 2], np.uint32), np.array([3, 3, 4], np.uint32))
    b = O.FlatBlocks(g, "forward", 64)
    off, pairs = b.export()
    assert len(pairs) == 3 and off[0] == 0 and int(off[-1]) == 3
    assert np.all(np.diff(off.astype(np.int64)) >= 0)
    src = np.array([0, 1, 2, 5], np.uint32)
    for path in ("any", "shortest"):
        want, _, _ = O.vexpand(g, src, 1, 2, path, "forward")
        got, _, _ = O.vexpand(g, src, 1, 2, path, "forward", blocks=b)
        assert np.array_equal(got, want)
    with pytest.raises(ValueError):
        O.vexpand(g, src, 1, 2, "any", "backward", blocks=b)
