"""GPU Mintersect parity against the oracle: the reference's two known-answer
cases (mintersect.cpp:347-511, 3 tuples) through the C ABI, the triangle plan
shape (VarRow base + two transposed ColMain dependencies, p3-tri3-1), random
matrix/flat dependencies, and adjacency dependencies (triangle closing over
sorted CSR lists) checked against a CPU set intersection."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests import graphs as G
from tests.conftest import bool_to_words
from tests.test_gpu_join import rows_of
from tests.test_oracle_known_answers import VA, VK, key_matrix
from vertexsurge_gb300 import graphgen

pytestmark = pytest.mark.gpu

A, B, C = 1, 2, 3


@pytest.mark.parametrize("only_count", [False, True])
def test_known_answer_flat_flat_flat(vs, only_count):
    base = vs.FlatTable.from_columns([VA, VK])
    d1 = vs.FlatTable.from_columns([VA, VK])
    d2 = vs.FlatTable.from_columns([VA, VK])
    deps = [dict(flat=d1, u_col=0, nv_col=1, base_col=0), dict(flat=d2, u_col=0, nv_col=1, base_col=1)]
    out, count, _ = vs.mintersect(base, deps, 16, only_count)
    assert count == 3
    if not only_count:
        assert rows_of(out.columns()).tolist() == [[1, 1, 1], [2, 1, 1], [3, 1, 1]]


@pytest.mark.parametrize("only_count", [False, True])
def test_known_answer_flat_mat_mat(vs, only_count):
    base = vs.FlatTable.from_columns([VA, VK])
    w1, m1 = key_matrix(10, 10, VK, VA)
    w2, m2 = key_matrix(10, 10, VK, VA)
    d1 = vs.BitMatrix.from_logical(w1, 10, 10, kind=2, col_map=m1)
    d2 = vs.BitMatrix.from_logical(w2, 10, 10, kind=2, col_map=m2)
    deps = [dict(mat=d1, base_col=0), dict(mat=d2, base_col=1)]
    out, count, _ = vs.mintersect(base, deps, 16, only_count)
    assert count == 3
    if not only_count:
        assert rows_of(out.columns()).tolist() == [[1, 1, 1], [2, 1, 1], [3, 1, 1]]


def test_triangle_plan_shape(vs):
    """p3-tri3-1: p12 VarRow base, p13^T and p23^T ColMain deps, through expand,
    select and transpose on the GPU, against the oracle chain."""
    g = graphgen.rmat(11, 16, seed=21, undirected=True)
    dg = vs.DeviceGraph.from_host(g)
    sa = graphgen.sample_sources(g.V, 150, seed=1)
    sb = graphgen.sample_sources(g.V, 130, seed=2)
    sc = graphgen.sample_sources(g.V, 140, seed=3)

    def gexp(src, tgt):
        m, _, _ = vs.expand(dg, src, 0, 2, "shortest", "both")
        return m.select(tgt)

    def oexp(src, tgt):
        w, _, _ = O.vexpand(g, src, 0, 2, "shortest", "both")
        return O.matrix_select(w, len(src), g.V, tgt)

    p12, p13, p23 = gexp(sa, sb), gexp(sa, sc), gexp(sb, sc)
    p13t, p23t = p13.convert(True), p23.convert(True)
    for only_count in (True, False):
        out, count, _ = vs.mintersect(p12, [dict(mat=p13t, base_col=0), dict(mat=p23t, base_col=1)],
                                      g.V, only_count)
        o12, o13, o23 = oexp(sa, sb), oexp(sa, sc), oexp(sb, sc)
        t13 = O.table_convert(o13, len(sa), len(sc), True)
        t23 = O.table_convert(o23, len(sb), len(sc), True)
        base = O.Table(O.VARROW, [A, B], words=o12, mrows=len(sa), mcols=len(sb), row_map=sa, col_map=sb)
        d13 = O.Table(O.COLMAIN, [C, A], words=t13, mrows=len(sc), mcols=len(sa), row_map=sc, col_map=sa)
        d23 = O.Table(O.COLMAIN, [C, B], words=t23, mrows=len(sc), mcols=len(sb), row_map=sc, col_map=sb)
        _, ocols, ocount = O.mintersect(base, [d13, d23], C, g.V, only_count)
        assert count == ocount > 0
        if not only_count:
            assert np.array_equal(rows_of(out.columns()), rows_of(ocols))


def test_random_flat_and_mat_deps(vs):
    rng = np.random.default_rng(5)
    nb, Vn = 2000, 300
    base_a = rng.integers(0, 200, nb).astype(np.uint32)
    base_b = rng.integers(0, 150, nb).astype(np.uint32)
    m = rng.random((Vn, 200)) < 0.2  # rows = new vertex, cols = a
    w = bool_to_words(m)
    fu = rng.integers(0, 150, 20000).astype(np.uint32)
    fv = rng.integers(0, Vn, 20000).astype(np.uint32)
    gbase = vs.FlatTable.from_columns([base_a, base_b])
    gm = vs.BitMatrix.from_logical(w, Vn, 200, kind=2)
    gf = vs.FlatTable.from_columns([fu, fv])
    out, count, _ = vs.mintersect(gbase, [dict(mat=gm, base_col=0), dict(flat=gf, u_col=0, nv_col=1, base_col=1)],
                                  Vn, False)
    obase = O.Table(O.FLAT, [A, B], cols=[base_a, base_b])
    om = O.Table(O.COLMAIN, [C, A], words=w, mrows=Vn, mcols=200)
    of = O.Table(O.FLAT, [B, C], cols=[fu, fv])
    _, ocols, ocount = O.mintersect(obase, [om, of], C, Vn)
    assert count == ocount
    assert np.array_equal(rows_of(out.columns()), rows_of(ocols))


@pytest.fixture(scope="module")
def hub_graphs(vs):
    """An R-MAT graph and a power-law graph with many vertices of degree >= 1024
    (adjacency bitmaps)."""
    z = graphgen.zipf(20_000, 600_000, 1.6, 6000, seed=5)
    zt = graphgen.HostGraph(z.V, z.E, z.rev_off, z.rev_src, z.fwd_off, z.fwd_dst, True)  # in-degree hubs
    gs = {"rmat12": graphgen.rmat(12, 16, seed=33), "zipf20k": z, "zipf20k_t": zt}
    return {k: (g, vs.DeviceGraph.from_host(g)) for k, g in gs.items()}


@pytest.mark.parametrize("algo", ["auto", "binary", "merge", "bitmap"])
@pytest.mark.parametrize("gname", ["rmat12", "zipf20k"])
def test_adjacency_triangle_closing(vs, hub_graphs, algo, gname):
    """Base (a, b) edges; deps = out-lists of a and of b: triangles a->b, a->c,
    b->c, under every membership method (bitmap, window merge, binary search)."""
    g, dg = hub_graphs[gname]
    rng = np.random.default_rng(1)
    src = np.repeat(np.arange(g.V, dtype=np.uint32), np.diff(g.fwd_off))
    pick = rng.choice(g.E, 30000, replace=False)
    a, b = src[pick], g.fwd_dst[pick]
    base = vs.FlatTable.from_columns([a, b])
    deps = [dict(graph=dg, direction="forward", base_col=0, algo=algo),
            dict(graph=dg, direction="forward", base_col=1, algo=algo)]
    out, count, _ = vs.mintersect(base, deps, g.V, False)
    _, c2, _ = vs.mintersect(base, deps, g.V, True)
    exp = []
    for x, y in zip(a.tolist(), b.tolist()):
        na = g.fwd_dst[g.fwd_off[x]:g.fwd_off[x + 1]]
        nb = g.fwd_dst[g.fwd_off[y]:g.fwd_off[y + 1]]
        for z in np.intersect1d(na, nb).tolist():
            exp.append((x, y, z))
    exp = np.array(sorted(exp), dtype=np.int64).reshape(-1, 3)
    assert count == c2 == len(exp) > 0
    assert np.array_equal(rows_of(out.columns()), exp)
    if algo == "auto":
        # the same through flat edge tables (pair-hash membership)
        fe = vs.FlatTable.from_columns([src, g.fwd_dst])
        deps_f = [dict(flat=fe, u_col=0, nv_col=1, base_col=0), dict(flat=fe, u_col=0, nv_col=1, base_col=1)]
        _, c3, _ = vs.mintersect(base, deps_f, g.V, True)
        assert c3 == count


@pytest.mark.parametrize("algo", ["auto", "binary"])
def test_pair_count_long_walks_beyond_the_piece_list(vs, algo):
    """Count-only closing over two adjacency lists cuts walks above 64
    candidates into pieces; here 600 base tuples each walk 30,000 candidates
    (70,800 pieces, more than the first pass's list holds), so the call counts
    again with room for every piece.  Source 0 reaches 1..30000; hubs 1..600
    each reach 10000..39999: every hub tuple closes 20,001 triangles."""
    V, D, H = 40_000, 30_000, 600
    src = np.concatenate([np.zeros(D, np.uint32), np.repeat(np.arange(1, H + 1, dtype=np.uint32), D)])
    dst = np.concatenate([np.arange(1, D + 1, dtype=np.uint32), np.tile(np.arange(10_000, 10_000 + D, dtype=np.uint32), H)])
    g = graphgen.from_edges(V, src, dst)
    dg = vs.DeviceGraph.from_host(g)
    a = np.zeros(D, np.uint32)
    b = np.arange(1, D + 1, dtype=np.uint32)
    base = vs.FlatTable.from_columns([a, b])
    deps = [dict(graph=dg, direction="forward", base_col=0, algo=algo),
            dict(graph=dg, direction="forward", base_col=1, algo=algo)]
    _, count, _ = vs.mintersect(base, deps, V, True)
    # the general kernel (a forced window merge keeps it) on the same base
    merge = [dict(d, algo="merge") for d in deps]
    _, c_general, _ = vs.mintersect(base, merge, V, True)
    assert count == c_general == H * (D - 10_000 + 1)


@pytest.mark.parametrize("algo", ["auto", "merge", "bitmap"])
def test_adjacency_in_lists(vs, hub_graphs, algo):
    """Backward (in-list) adjacency on a directed graph: common in-neighbours of
    (a, b) pairs, every method against numpy."""
    g, dg = hub_graphs["zipf20k_t"]
    rng = np.random.default_rng(2)
    a = rng.integers(0, g.V, 5000).astype(np.uint32)
    b = rng.integers(0, g.V, 5000).astype(np.uint32)
    base = vs.FlatTable.from_columns([a, b])
    deps = [dict(graph=dg, direction="backward", base_col=0, algo=algo),
            dict(graph=dg, direction="backward", base_col=1, algo=algo)]
    _, count, _ = vs.mintersect(base, deps, g.V, True)
    exp = 0
    for x, y in zip(a.tolist(), b.tolist()):
        exp += len(np.intersect1d(g.rev_src[g.rev_off[x]:g.rev_off[x + 1]], g.rev_src[g.rev_off[y]:g.rev_off[y + 1]]))
    assert count == exp


def test_unknown_intersection_method_is_rejected(vs, hub_graphs):
    g, dg = hub_graphs["rmat12"]
    base = vs.FlatTable.from_columns([np.zeros(4, np.uint32), np.ones(4, np.uint32)])
    with pytest.raises(vs.VsError):
        vs.mintersect(base, [dict(graph=dg, base_col=0, algo=7), dict(graph=dg, base_col=1)], g.V, True)


def test_output_bound(vs):
    base = vs.FlatTable.from_columns([VA, VK])
    w1, m1 = key_matrix(10, 10, VK, VA)
    d1 = vs.BitMatrix.from_logical(w1, 10, 10, kind=2, col_map=m1)
    out, count, trunc = vs.mintersect(base, [dict(mat=d1, base_col=0), dict(mat=d1, base_col=1)], 16,
                                      False, max_rows=2)
    assert count == 3 and trunc and out.info()[1] == 2
