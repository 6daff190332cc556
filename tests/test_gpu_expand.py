"""GPU parity of the expand (VExpand) against the CPU oracle, bit-exact,
through the C ABI.  Covers every path type, direction, hop range, every
pull kernel variant (row widths from 1 to 256 words), forced strategies,
hub CTAs, multi-slice rows, duplicate sources and FindShortest."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import words_to_bool
from tests import graphs as G
from vertexsurge_gb300 import graphgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graphs(vs):
    hg = G.small_graphs()
    return {k: (g, vs.DeviceGraph.from_host(g)) for k, g in hg.items()}


def run_both(vs, g, dg, src, k_min, k_max, path, direction, **kw):
    m, _, st = vs.expand(dg, src, k_min, k_max, path, direction, stats=True, **kw)
    got = m.download()
    exp, _, _ = O.vexpand(g, src, k_min, k_max, path, direction)
    return got, exp, st


@pytest.mark.parametrize("path", ["any", "shortest"])
@pytest.mark.parametrize("direction", ["forward", "backward", "both"])
@pytest.mark.parametrize("krange", [(0, 2), (1, 3), (2, 4), (1, 1), (2, 2), (0, 0)])
def test_expand_parity_paths(vs, graphs, path, direction, krange):
    for name, (g, dg) in graphs.items():
        src = graphgen.sample_sources(g.V, 96, seed=7)
        got, exp, st = run_both(vs, g, dg, src, krange[0], krange[1], path, direction)
        assert np.array_equal(got, exp), (name, path, direction, krange, st)


@pytest.mark.parametrize("S", [1, 31, 64, 65, 128, 200, 512, 1000, 2048, 4096, 8192, 16384])
def test_expand_parity_row_widths(vs, graphs, S):
    g, dg = graphs["rmat11_skew"]
    src = graphgen.sample_sources(g.V, min(S, g.V), seed=S)
    if S > g.V:
        src = np.resize(src, S).astype(np.uint32)  # repeated sources are independent rows
    for path in ("any", "shortest"):
        got, exp, _ = run_both(vs, g, dg, src, 1, 3, path, "forward")
        assert np.array_equal(got, exp), (S, path)


@pytest.mark.parametrize("strategy", ["pull", "sparse", "push", "auto"])
@pytest.mark.parametrize("path", ["any", "shortest"])
def test_expand_forced_strategies(vs, graphs, strategy, path):
    for name, (g, dg) in graphs.items():
        src = graphgen.sample_sources(g.V, 150, seed=3)
        got, exp, st = run_both(vs, g, dg, src, 1, 4, path, "forward", strategy=strategy)
        assert np.array_equal(got, exp), (name, strategy, path, st)


def test_expand_hub_ctas_and_slices(vs, graphs):
    for name, (g, dg) in graphs.items():
        src = graphgen.sample_sources(g.V, 300, seed=9)
        for kw in ({"hub_threshold": 8}, {"slice_words": 2}, {"slice_words": 4, "hub_threshold": 16},
                   {"strategy": "pull", "slice_words": 2}):
            for path in ("any", "shortest"):
                got, exp, _ = run_both(vs, g, dg, src, 1, 3, path, "both", **kw)
                assert np.array_equal(got, exp), (name, kw, path)


def test_expand_sparse_overflow_falls_back(vs, graphs):
    g, dg = graphs["rmat10"]
    src = graphgen.sample_sources(g.V, 200, seed=5)
    for path in ("any", "shortest"):
        got, exp, st = run_both(vs, g, dg, src, 1, 4, path, "forward", strategy="sparse",
                                pair_capacity=300)
        assert np.array_equal(got, exp), st


def test_expand_duplicate_sources(vs, graphs):
    g, dg = graphs["rmat10"]
    src = np.array([5, 5, 17, 900, 5, 17, 0, 0], dtype=np.uint32)
    for path in ("any", "shortest"):
        for kr in ((0, 3), (1, 3), (2, 5)):
            got, exp, _ = run_both(vs, g, dg, src, kr[0], kr[1], path, "forward")
            assert np.array_equal(got, exp), (path, kr)


def test_expand_early_stop_hops_run(vs, graphs):
    g, dg = graphs["rmat10"]
    src = graphgen.sample_sources(g.V, 64, seed=1)
    m, _, st = vs.expand(dg, src, 1, 30, "shortest", "forward", stats=True)
    _, _, ost = O.vexpand(g, src, 1, 30, "shortest", "forward", hop_stats=True)
    assert st["hops_run"] == ost["hops_run"] < 30
    assert st["visit_count"] == ost["visit_count"][-1]
    exp, _, _ = O.vexpand(g, src, 1, 30, "shortest", "forward")
    assert np.array_equal(m.download(), exp)


def test_expand_find_shortest(vs, graphs):
    for name, (g, dg) in graphs.items():
        S = 120
        src = graphgen.sample_sources(g.V, S, seed=31)
        tgt = graphgen.sample_sources(g.V, S, seed=32)
        tgt[:7] = src[:7]
        _, dist, _ = vs.expand(dg, src, 1, 50, "find_shortest", "forward", targets=tgt)
        _, odist, _ = O.vexpand(g, src, 1, 50, "find_shortest", "forward", targets=tgt)
        assert np.array_equal(dist, odist), name


def test_expand_stats_active_edges(vs, graphs):
    g, dg = graphs["zipf3000"]
    src = graphgen.sample_sources(g.V, 256, seed=2)
    for path in ("any", "shortest"):
        _, _, st = vs.expand(dg, src, 1, 3, path, "forward", stats=True)
        _, _, ost = O.vexpand(g, src, 1, 3, path, "forward", hop_stats=True)
        assert st["active_edges"][1:] == ost["active_edges"][1:], (path, st, ost)


@pytest.mark.parametrize("path,k0,k1", [("shortest", 1, 3), ("shortest", 2, 4), ("shortest", 0, 2),
                                         ("any", 1, 3), ("any", 2, 2), ("any", 1, 1)])
def test_plan_rerun_is_clean(vs, graphs, path, k0, k1):
    """A reused plan gives the right answer for another source set: the rows
    the previous run left in its result and frontier matrices are cleared,
    and the result's column-occupancy flags (used by counts) stay exact."""
    g, dg = graphs["rmat11_skew"]
    p = vs.make_params(k0, k1, path, "forward")
    plan = vs.ExpandPlan(dg, 256, p)
    for seed in (1, 2, 1, 3):
        src = graphgen.sample_sources(g.V, 256 if seed != 3 else 40, seed=seed)
        if len(src) < 256:  # fewer distinct vertices: repeat the last one (rows are independent)
            src = np.concatenate([src, np.full(256 - len(src), src[-1], np.uint32)])
        plan.run(src)
        got = plan.result().download()
        exp, _, _ = O.vexpand(g, src, k0, k1, path, "forward")
        assert np.array_equal(got, exp), seed
        assert plan.result().count() == O.matrix_count(exp, 256, g.V), seed


@pytest.mark.parametrize("path,k0,k1", [("shortest", 1, 2), ("shortest", 2, 3), ("any", 1, 2)])
def test_rerun_across_strategies(vs, graphs, path, k0, k1):
    """One plan run under alternating per-hop strategies: a Shortest run whose
    last hop is SPARSE keeps no next-layer rows (flag 2), and the runs after
    it (PULL, PUSH, SPARSE) still find clean buffers; every run equals the
    oracle, and so do the stats' per-hop new-bit counts."""
    g, dg = graphs["rmat11_skew"]
    plan = vs.ExpandPlan(dg, 192, vs.make_params(k0, k1, path, "forward"))
    plan.set_tuning(push_frac=0.5)
    seq = [("sparse", 1), ("pull", 2), ("sparse", 3), ("push", 1), ("sparse", 2), ("auto", 4)]
    for strat, seed in seq:
        plan.set_hop_strategies([0] + [strat] * k1)
        src = graphgen.sample_sources(g.V, 192, seed=seed)
        plan.run(src)
        exp, _, ost = O.vexpand(g, src, k0, k1, path, "forward", hop_stats=True)
        assert np.array_equal(plan.result().download(), exp), (strat, seed)
        assert plan.result().count() == O.matrix_count(exp, 192, g.V), (strat, seed)
        st = plan.stats()
        if path == "shortest":
            assert st["visit_count"] == ost["visit_count"][st["hops_run"]], (strat, seed)


def test_expand_empty_and_isolated(vs):
    # a graph with isolated vertices and a single edge
    g = graphgen.from_edges(10, [1], [2])
    dg = vs.DeviceGraph.from_host(g)
    src = np.array([0, 1, 2, 9], dtype=np.uint32)
    for path in ("any", "shortest"):
        m, _, _ = vs.expand(dg, src, 0, 3, path, "both")
        exp, _, _ = O.vexpand(g, src, 0, 3, path, "both")
        assert np.array_equal(m.download(), exp)
    m, _, _ = vs.expand(dg, np.zeros(0, np.uint32), 1, 3, "any", "forward")
    assert m.shape == (0, 10) and m.count() == 0


def test_expand_rejects_bad_arguments(vs, graphs):
    g, dg = graphs["rmat10"]
    with pytest.raises(vs.VsError):
        vs.expand(dg, np.array([1], np.uint32), 3, 2, "any", "forward")
    with pytest.raises(vs.VsError):
        vs.expand(dg, np.array([1], np.uint32), 1, 65, "any", "forward")


def test_expand_rejects_out_of_range_ids(vs, graphs):
    g, dg = graphs["rmat10"]
    with pytest.raises(vs.VsError):
        vs.expand(dg, np.array([1, g.V + 5], np.uint32), 1, 2, "shortest", "forward")
    with pytest.raises(vs.VsError):
        vs.expand(dg, np.array([1, 2], np.uint32), 1, 5, "find_shortest", "forward",
                  targets=np.array([3, g.V], np.uint32))


@pytest.mark.parametrize("path", ["any", "shortest"])
@pytest.mark.parametrize("strategy", ["auto", "pull", "push", "sparse"])
def test_batched_queries_equal_solo_runs(vs, graphs, path, strategy):
    """Queries packed into one plan (row ranges, per-row hop limits) give each
    query exactly its solo result."""
    g, dg = graphs["rmat11_skew"]
    sizes, kmaxs = [70, 5, 130, 64, 33], [2, 5, 3, 1, 4]
    srcs = [graphgen.sample_sources(g.V, n, seed=100 + i) for i, n in enumerate(sizes)]
    allsrc = np.concatenate(srcs).astype(np.uint32)
    limits = np.concatenate([np.full(n, k, np.uint8) for n, k in zip(sizes, kmaxs)])
    plan = vs.ExpandPlan(dg, len(allsrc), vs.make_params(1, max(kmaxs), path, "forward", strategy=strategy))
    plan.set_row_limits(limits)
    plan.run(allsrc)
    got = words_to_bool(plan.result().download(), len(allsrc))
    r0 = 0
    for src, k in zip(srcs, kmaxs):
        exp, _, _ = O.vexpand(g, src, 1, k, path, "forward")
        assert np.array_equal(got[r0:r0 + len(src)], words_to_bool(exp, len(src))), (k, path, strategy)
        r0 += len(src)


def test_autotuner_settings_keep_results(vs, graphs):
    from vertexsurge_gb300 import autotune
    g, dg = graphs["rmat11_skew"]
    src = graphgen.sample_sources(g.V, 200, seed=12)
    t = autotune.tune(dg, src, 1, 3, "shortest", "forward", repeats=1, pull_kinds=(0, 3),
                      sparse_fracs=(0.001, 0.05), hub_thresholds=(0, 64))
    assert len(t["table"]) == 16 and t["ms"] > 0  # x2: short mode on and off
    assert {r["short_share"] for r in t["table"]} == {0.0, -1.0}
    exp, _, _ = O.vexpand(g, src, 1, 3, "shortest", "forward")
    for row in t["table"]:
        plan = autotune.make_plan(dg, len(src), 1, 3, "shortest", "forward", row)
        plan.run(src)
        assert np.array_equal(plan.result().download(), exp), row
        m, _, _ = vs.expand(dg, src, 1, 3, "shortest", "forward", **autotune.params_kw(row))
        assert np.array_equal(m.download(), exp), row


def test_captured_graph_equals_direct_run(vs, graphs):
    import torch
    g, dg = graphs["zipf3000"]
    src = graphgen.sample_sources(g.V, 300, seed=14)
    dsrc = torch.from_numpy(src.view(np.int32)).cuda()
    stream = torch.cuda.Stream()
    for path in ("any", "shortest"):
        plan = vs.ExpandPlan(dg, len(src), vs.make_params(1, 4, path, "forward"))
        plan.run(dsrc, stream=stream)  # first run on the stream, outside the capture
        stream.synchronize()
        with vs.Captured(stream, keep=(plan, dsrc)) as cg:
            plan.run(dsrc, stream=stream)
        assert cg.kernels > 0
        exp, _, _ = O.vexpand(g, src, 1, 4, path, "forward")
        for _ in range(2):
            n0 = vs.kernel_launches()
            cg.launch(stream)
            stream.synchronize()
            assert vs.kernel_launches() - n0 == cg.kernels
            assert np.array_equal(plan.result().download(stream), exp)
        # the replay reads the sources buffer at every launch
        src2 = graphgen.sample_sources(g.V, 300, seed=15)
        dsrc.copy_(torch.from_numpy(src2.view(np.int32)))
        cg.launch(stream)
        stream.synchronize()
        exp2, _, _ = O.vexpand(g, src2, 1, 4, path, "forward")
        assert np.array_equal(plan.result().download(stream), exp2)
        dsrc.copy_(torch.from_numpy(src.view(np.int32)))
        cg.free()
        plan.free()


@pytest.mark.parametrize("path", ["any", "shortest"])
def test_device_row_limits_equal_solo(vs, graphs, path):
    """Row limits set from a device array: each query's rows equal its solo
    result; rows past n never grow; the run stops after the largest limit."""
    import torch
    g, dg = graphs["rmat11_skew"]
    sizes, kmaxs = [40, 70, 25, 90], [1, 3, 2, 2]
    srcs = [graphgen.sample_sources(g.V, n, seed=30 + i) for i, n in enumerate(sizes)]
    allsrc = np.concatenate(srcs).astype(np.uint32)
    S = len(allsrc) + 20  # 20 trailing rows without a limit entry
    padded = np.concatenate([allsrc, np.zeros(20, np.uint32)])
    limits = np.concatenate([np.full(n, k, np.uint8) for n, k in zip(sizes, kmaxs)])
    plan = vs.ExpandPlan(dg, S, vs.make_params(1, 5, path, "forward"))
    plan.set_tuning(collect_stats=True)
    dl = torch.from_numpy(limits).cuda()
    plan.set_row_limits_device(dl, len(limits))
    plan.run(padded)
    st = plan.stats()
    assert st["hops_run"] <= max(kmaxs)
    got = words_to_bool(plan.result().download(), S)
    r0 = 0
    for src, k in zip(srcs, kmaxs):
        exp, _, _ = O.vexpand(g, src, 1, k, path, "forward")
        assert np.array_equal(got[r0:r0 + len(src)], words_to_bool(exp, len(src))), (k, path)
        r0 += len(src)
    # rows without a limit keep at most their seed (no hop may grow them)
    assert got[r0:].sum(axis=1).max() <= 1
    plan.free()


def test_device_row_limit_above_kmax_is_an_error(vs, graphs):
    import torch
    g, dg = graphs["rmat11_skew"]
    src = graphgen.sample_sources(g.V, 64, seed=3)
    plan = vs.ExpandPlan(dg, 64, vs.make_params(1, 2, "shortest", "forward"))
    plan.set_row_limits_device(torch.full((64,), 3, dtype=torch.uint8, device="cuda"), 64)
    plan.set_tuning(collect_stats=True)
    plan.run(src)
    with pytest.raises(vs.VsError):
        plan.stats()
    plan.free()


@pytest.mark.parametrize("path", ["any", "shortest"])
@pytest.mark.parametrize("krange", [(0, 3), (2, 4), (1, 1), (1, 8)])
def test_expand_layers_with_distance(vs, graphs, path, krange):
    """with_distance: layer h equals the expand over [h, h]; the layers stop at
    the last hop run (a Shortest expand ends when a hop adds nothing)."""
    g, dg = graphs["rmat11_skew"]
    src = graphgen.sample_sources(g.V, 130, seed=8)
    k0, k1 = krange
    layers = vs.expand_layers(dg, src, k0, k1, path, "forward")
    _, _, st = O.vexpand(g, src, k0, k1, path, "forward", hop_stats=True)
    k_actual = min(st["hops_run"], k1) if path == "shortest" else k1
    assert len(layers) == max(0, k_actual - k0 + 1)
    total = 0
    for h, m in layers:
        exp, _, _ = O.vexpand(g, src, h, h, path, "forward")
        got = m.download()
        assert np.array_equal(got, exp), (path, krange, h)
        total += O.matrix_count(exp, len(src), g.V)
    if layers:
        f = vs.layers_to_flat(layers)
        r, c, d = f.columns()
        assert len(r) == total
        assert set(np.unique(d).tolist()) <= set(range(k0, k_actual + 1))
        if path == "shortest":  # layers are disjoint: every (source, vertex) pair once
            assert len(set(zip(r.tolist(), c.tolist()))) == total


@pytest.mark.parametrize("path,krange", [("any", (1, 3)), ("any", (2, 4)), ("any", (0, 2)), ("shortest", (1, 3))])
def test_layers_to_flat_first_distance(vs, graphs, path, krange):
    """VExpand's CSR output with distances: each (source, vertex) pair once at
    the smallest layer it appears in (merge_to_Flat; for Any a pair reached by
    walks of several lengths keeps the shortest in range).  Checked against the
    oracle's per-layer matrices; for Shortest it equals the plain layer list."""
    g, dg = graphs["rmat11_skew"]
    src = graphgen.sample_sources(g.V, 130, seed=8)
    k0, k1 = krange
    layers = vs.expand_layers(dg, src, k0, k1, path, "forward")
    first = {}
    for h, _ in layers:
        exp, _, _ = O.vexpand(g, src, h, h, path, "forward")
        bits = np.unpackbits(exp.view(np.uint8), axis=1, bitorder="little")[:, : len(src)]
        for v, i in zip(*np.nonzero(bits)):
            first.setdefault((int(src[i]), int(v)), h)
    r, c, d = vs.layers_to_flat(layers, first=True).columns()
    got = {(int(a), int(b)): int(x) for a, b, x in zip(r, c, d)}
    assert len(got) == len(r) == len(first)
    assert got == first
    if path == "shortest":
        r2, c2, d2 = vs.layers_to_flat(layers).columns()
        assert sorted(zip(r2.tolist(), c2.tolist(), d2.tolist())) == sorted(zip(r.tolist(), c.tolist(), d.tolist()))


def test_malformed_csr_is_rejected(vs):
    g = graphgen.from_edges(10, [1, 2], [2, 3])
    bad = g.fwd_dst.copy()
    bad[0] = 10  # a target outside the vertex range
    with pytest.raises(vs.VsError):
        vs.DeviceGraph(g.V, g.E, g.fwd_off, bad, g.rev_off, g.rev_src)
    off = g.fwd_off.copy()
    off[5], off[6] = off[6] + 1, off[6]  # offsets that go down
    with pytest.raises(vs.VsError):
        vs.DeviceGraph(g.V, g.E, off, g.fwd_dst, g.rev_off, g.rev_src)
    vs.DeviceGraph(g.V, g.E, g.fwd_off, g.fwd_dst, g.rev_off, g.rev_src)  # the well-formed one loads


@pytest.mark.parametrize("path", ["any", "shortest"])
@pytest.mark.parametrize("direction", ["forward", "backward", "both"])
def test_short_pull_parity(vs, graphs, path, direction):
    """Short-mode PULL (rows with at most 15 bits read from their id slots,
    longer rows gathered whole) against the oracle, forced on every PULL hop:
    slots written by the PULL epilogue (warp and hub CTA) and by the build
    pass after SPARSE hops or the seed; rows of 1 to 128 uint4; with
    short mode off no hop uses it and the results are the same."""
    n_short, n_edges = 0, 0
    for name in ("rmat11_skew", "zipf3000", "rmat10"):
        g, dg = graphs[name]
        for S in (20, 40, 300, 1000, 4000) + ((8192, 16384) if name == "rmat10" else ()):
            src = graphgen.sample_sources(g.V, min(S, g.V), seed=S + 1)
            if S > g.V:
                src = np.resize(src, S).astype(np.uint32)
            exp, _, _ = O.vexpand(g, src, 1, 4, path, direction)
            for strategy in ("pull", "auto"):
                for share in (2.0, -1.0):
                    m, _, st = vs.expand(dg, src, 1, 4, path, direction, strategy=strategy, stats=True,
                                         short_share=share, hub_threshold=64)
                    assert np.array_equal(m.download(), exp), (name, S, path, direction, strategy, share)
                    for h in range(1, st["hops_run"] + 1):
                        if st["strategy"][h] == vs.STRAT_PULL:
                            assert bool(st["short_pull"][h]) == (share > 0), (h, st["short_pull"])
                            n_short += share > 0
                            n_edges += st["short_edges"][h]
                        else:
                            assert not st["short_pull"][h]
    assert n_short > 50 and n_edges > 0


@pytest.mark.parametrize("path", ["any", "shortest"])
@pytest.mark.parametrize("S", [700, 8192])
def test_short_rows_counted(vs, graphs, path, S):
    """The PULL epilogue's counts of short rows (at most 15 bits for rows of
    up to 64 words, 31 for 128 words) and of rows with their ids inline in
    the tiny word (one or two bits), in every layer it writes words for,
    equal the counts over the oracle's layer."""
    g, dg = graphs["zipf3000"]
    src = graphgen.sample_sources(g.V, min(S, g.V), seed=8)
    if S > g.V:
        src = np.resize(src, S).astype(np.uint32)
    _, _, st = vs.expand(dg, src, 1, 4, path, "forward", strategy="pull", stats=True, short_share=2.0)
    W = (len(src) + 63) // 64
    W += W & 1
    short_max = 15 if W <= 64 else 31 if W <= 128 else 63
    checked = 0
    for h in range(1, min(st["hops_run"], 3) + 1):  # hop 4 is the last: no slots
        layer, _, _ = O.vexpand(g, src, h, h, path, "forward")
        bits = words_to_bool(layer, len(src)).sum(axis=0) if layer.size else np.zeros(g.V)
        assert st["short_rows"][h] == int(((bits >= 1) & (bits <= short_max)).sum()), h
        assert st["tiny_rows"][h] == int(((bits >= 1) & (bits <= 2)).sum()), h
        checked += 1
    assert checked == 3


@pytest.mark.parametrize("share", [2.0, 0.0])
@pytest.mark.parametrize("hops", [["pull", "push", "pull", "pull"], ["pull", "pull", "push", "pull"],
                                  ["sparse", "pull", "pull", "push"], ["pull", "pull", "pull", "pull"]])
def test_slot_only_rows_materialize(vs, graphs, share, hops):
    """Short rows a PULL hop leaves only in their slots (flag 2) are written
    out whole before a hop that reads rows (PUSH, or a dense PULL when short
    mode is not chosen) and are skipped by the row clears; a reused plan
    stays exact across runs and path types."""
    for name in ("zipf3000", "rmat11_skew"):
        g, dg = graphs[name]
        for path in ("shortest", "any"):
            plan = vs.ExpandPlan(dg, 300, vs.make_params(1, 4, path, "forward", short_share=share))
            plan.set_hop_strategies([0] + hops)
            for seed in (1, 2):
                src = graphgen.sample_sources(g.V, 300, seed=seed)
                plan.run(src)
                exp, _, _ = O.vexpand(g, src, 1, 4, path, "forward")
                assert np.array_equal(plan.result().download(), exp), (name, path, hops, share, seed)


@pytest.mark.parametrize("cap", [0, 300])
def test_short_words_from_pairs_or_rows(vs, graphs, cap):
    """After a SPARSE hop (or the seed) the short-row words and slots come
    from its pair list; when that list overflowed (cap 300) they come from the
    rows.  Both give the oracle's result."""
    for name in ("rmat10", "zipf3000"):
        g, dg = graphs[name]
        src = graphgen.sample_sources(g.V, 200, seed=5)
        for hops in (["sparse", "pull", "pull", "pull"], ["pull", "sparse", "pull", "pull"]):
            for path in ("shortest", "any"):
                plan = vs.ExpandPlan(dg, len(src), vs.make_params(1, 4, path, "forward", short_share=2.0,
                                                                  pair_capacity=cap))
                plan.set_hop_strategies([0] + hops)
                plan.run(src)
                exp, _, _ = O.vexpand(g, src, 1, 4, path, "forward")
                assert np.array_equal(plan.result().download(), exp), (name, hops, path, cap)


def test_short_pull_find_shortest(vs, graphs):
    """FindShortest with short mode forced on every PULL hop (its layers keep
    their rows, which the target check reads) gives the oracle's distances."""
    for name, (g, dg) in graphs.items():
        src = graphgen.sample_sources(g.V, 150, seed=41)
        tgt = graphgen.sample_sources(g.V, 150, seed=42)
        tgt[:5] = src[:5]
        for strategy in ("pull", "auto"):
            _, dist, _ = vs.expand(dg, src, 1, 30, "find_shortest", "forward", targets=tgt, strategy=strategy,
                                   short_share=2.0)
            _, odist, _ = O.vexpand(g, src, 1, 30, "find_shortest", "forward", targets=tgt)
            assert np.array_equal(dist, odist), (name, strategy)


def test_short_pull_default_rule(vs, graphs):
    """With the default share, frontiers that fit in half of L2 keep the
    dense PULL (every small test graph), and the results agree."""
    g, dg = graphs["rmat11_skew"]
    src = graphgen.sample_sources(g.V, 500, seed=3)
    m, _, st = vs.expand(dg, src, 1, 4, "shortest", "forward", strategy="pull", stats=True)
    assert not any(st["short_pull"])
    exp, _, _ = O.vexpand(g, src, 1, 4, "shortest", "forward")
    assert np.array_equal(m.download(), exp)


def test_short_pull_with_row_limits_and_layers(vs, graphs):
    """Short mode under batched per-row hop limits and with per-distance layers."""
    import torch
    g, dg = graphs["rmat11_skew"]
    sizes, kmaxs = [50, 90, 30], [1, 3, 2]
    srcs = [graphgen.sample_sources(g.V, n, seed=60 + i) for i, n in enumerate(sizes)]
    allsrc = np.concatenate(srcs).astype(np.uint32)
    plan = vs.ExpandPlan(dg, len(allsrc), vs.make_params(1, 3, "shortest", "forward", strategy="pull",
                                                         short_share=2.0))
    plan.set_row_limits_device(torch.from_numpy(np.concatenate(
        [np.full(n, k, np.uint8) for n, k in zip(sizes, kmaxs)])).cuda(), len(allsrc))
    plan.run(allsrc)
    got = words_to_bool(plan.result().download(), len(allsrc))
    r0 = 0
    for src, k in zip(srcs, kmaxs):
        exp, _, _ = O.vexpand(g, src, 1, k, "shortest", "forward")
        assert np.array_equal(got[r0:r0 + len(src)], words_to_bool(exp, len(src)))
        r0 += len(src)
    src = graphgen.sample_sources(g.V, 200, seed=4)
    for h, m in vs.expand_layers(dg, src, 1, 4, "shortest", "forward", strategy="pull", short_share=2.0):
        exp, _, _ = O.vexpand(g, src, h, h, "shortest", "forward")
        assert np.array_equal(m.download(), exp), h


def test_one_shot_plan_cache(vs, graphs):
    """One-shot expands keep their plans: results lent out at the same time
    stay exact, a plan reused for other sources gives exact results, FindShortest
    reuses without a matrix, a result outlives its graph, and a result is
    read-only."""
    g, dg = graphs["zipf3000"]
    srcs = [graphgen.sample_sources(g.V, 200, seed=s) for s in (1, 2, 3, 4)]
    exp = [O.vexpand(g, s, 1, 3, "shortest", "forward")[0] for s in srcs]
    m0, _, _ = vs.expand(dg, srcs[0], 1, 3, "shortest", "forward")
    m1, _, _ = vs.expand(dg, srcs[1], 1, 3, "shortest", "forward")  # m0 still lent: another plan
    assert np.array_equal(m0.download(), exp[0]) and np.array_equal(m1.download(), exp[1])
    m0.free()
    m2, _, _ = vs.expand(dg, srcs[2], 1, 3, "shortest", "forward")  # reuses m0's plan
    assert np.array_equal(m2.download(), exp[2]) and np.array_equal(m1.download(), exp[1])
    import ctypes
    zeros = np.zeros_like(exp[2])
    assert vs.lib().vs_bitmat_upload(m2.h, zeros.ctypes.data_as(ctypes.c_void_p), None) != 0  # read-only
    m1.free()
    m2.free()
    for s, e in zip(srcs, exp):  # every call on a reused plan
        m, _, _ = vs.expand(dg, s, 1, 3, "shortest", "forward")
        assert np.array_equal(m.download(), e)
        assert m.count() == O.matrix_count(e, len(s), g.V)
        m.free()
    tgt = graphgen.sample_sources(g.V, 200, seed=9)
    for _ in range(2):
        _, dist, _ = vs.expand(dg, srcs[0], 1, 20, "find_shortest", "forward", targets=tgt)
        _, odist, _ = O.vexpand(g, srcs[0], 1, 20, "find_shortest", "forward", targets=tgt)
        assert np.array_equal(dist, odist)
    # a result outlives its graph; the plan is freed, not kept, on release
    h = graphgen.from_edges(64, list(range(63)), list(range(1, 64)))
    dh = vs.DeviceGraph.from_host(h)
    src = np.array([0, 5, 9], np.uint32)
    m, _, _ = vs.expand(dh, src, 1, 2, "any", "forward")
    e, _, _ = O.vexpand(h, src, 1, 2, "any", "forward")
    dh.free()
    assert np.array_equal(m.download(), e)
    m.free()
    vs.release_cached()
    m, _, _ = vs.expand(dg, srcs[3], 1, 3, "shortest", "forward")
    assert np.array_equal(m.download(), exp[3])
    m.free()
