"""The learned strategy picker: CUDA forward/backward against the CPU
restatement (oracle/mlp_ref.py), training on the GPU, inference inside the
expand's decide kernel, per-hop overrides and feature logging."""
import numpy as np
import pytest

from oracle import mlp_ref as M
from oracle import pyoracle as O
from tests import graphs as G
from vertexsurge_gb300 import graphgen

pytestmark = pytest.mark.gpu


def test_forward_and_gradient_match_cpu(vs):
    pk = vs.Picker(seed=3)
    rng = np.random.default_rng(1)
    p = rng.normal(0, 0.2, M.NPARAM).astype(np.float32)
    pk.set_params(p)
    assert np.array_equal(pk.params(), p)
    X = rng.normal(0, 1, (300, M.NF)).astype(np.float32)
    y = rng.integers(0, 3, 300).astype(np.int32)
    z_gpu = pk.forward(X)
    z_cpu, _ = M.forward(p, X)
    assert np.allclose(z_gpu, z_cpu, rtol=1e-4, atol=1e-4)
    g_gpu, loss_gpu = pk.backward(X, y)
    loss_cpu, g_cpu = M.loss_and_grad(p, X, y)
    assert abs(loss_gpu - loss_cpu) < 1e-4 * max(1.0, abs(loss_cpu))
    # float32 sums in different orders: 1e-4 relative plus a small absolute floor
    assert np.allclose(g_gpu, g_cpu, rtol=1e-3, atol=2e-6), np.abs(g_gpu - g_cpu).max()


def test_training_learns_a_separable_rule(vs):
    rng = np.random.default_rng(2)
    X = rng.random((20000, M.NF)).astype(np.float32)
    y = np.where(X[:, 0] > 0.6, 0, np.where(X[:, 1] > 0.5, 1, 2)).astype(np.int32)
    pk = vs.Picker(seed=5)
    _, l0 = pk.backward(X, y)
    l1 = pk.train(X, y, epochs=25, batch=512, lr=3e-3)
    assert l1 < l0 * 0.5
    acc = (pk.predict(X) == y).mean()
    assert acc > 0.9, acc


def constant_picker(vs, cls):
    p = np.zeros(M.NPARAM, dtype=np.float32)
    off = M.NPARAM - 3
    p[off + cls] = 10.0  # b3: always this class
    pk = vs.Picker()
    pk.set_params(p)
    return pk


@pytest.mark.parametrize("cls,strategy", [(0, 1), (1, 2), (2, 3)])
def test_picker_drives_the_planner_and_results_stay_exact(vs, cls, strategy):
    g = graphgen.rmat(12, 16, seed=4)
    dg = vs.DeviceGraph.from_host(g)
    src = graphgen.sample_sources(g.V, 300, seed=8)
    for path, push_on in (("any", True), ("shortest", True), ("shortest", False)):
        plan = vs.ExpandPlan(dg, len(src), vs.make_params(1, 4, path, "forward", use_picker=True))
        plan.set_picker(constant_picker(vs, cls))
        if push_on:  # PUSH is opt-in: the picker chooses it only where the plan launches its kernels
            plan.set_tuning(push_frac=1e-9)
        plan.run(src)
        st = plan.stats()
        exp, _, _ = O.vexpand(g, src, 1, 4, path, "forward")
        assert np.array_equal(plan.result().download(), exp)
        got = st["strategy"][1:]
        if strategy == 3:  # sparse runs while its pair list is valid, then falls back
            assert got[0] == 3
        elif strategy == 2 and not push_on:  # the next-best class instead
            assert all(s == 1 for s in got), got
        else:
            assert all(s == strategy for s in got), got


def test_hop_overrides_and_feature_logging(vs):
    g = graphgen.rmat(12, 16, seed=4)
    dg = vs.DeviceGraph.from_host(g)
    src = graphgen.sample_sources(g.V, 200, seed=9)
    plan = vs.ExpandPlan(dg, len(src), vs.make_params(1, 4, "shortest", "forward"))
    plan.set_hop_strategies([0, "sparse", "push", "pull", "push"])
    plan.log_features(True)
    plan.run(src)
    st = plan.stats()
    n = st["hops_run"]
    assert n >= 3 and st["strategy"][1:] == [3, 2, 1, 2][:n]
    exp, _, _ = O.vexpand(g, src, 1, 4, "shortest", "forward")
    assert np.array_equal(plan.result().download(), exp)
    f = plan.features()[1:n + 1]
    assert np.all(np.isfinite(f)) and f.max() <= 4.0 and f.min() >= 0.0
    assert np.allclose(f[:, 16:].sum(axis=1), 1.0, atol=1e-5)  # degree histogram normalised


@pytest.mark.parametrize("path", ["shortest", "any"])
def test_frontier_statistics_same_under_every_strategy(vs, path):
    """E_active and the out-degree histogram of a hop's frontier come from the
    seed (hop 1), from the SPARSE hop that wrote the layer (counted as its rows
    became non-zero) or from a pass over the frontier flags after a PULL or
    PUSH hop: the features they give are the same under every strategy, E_active
    equals the oracle's, and hop 1's histogram is that of the distinct sources."""
    g = graphgen.rmat(12, 16, seed=4)
    dg = vs.DeviceGraph.from_host(g)
    src = graphgen.sample_sources(g.V, 200, seed=9)
    src[:6] = src[6:12]  # repeated sources: each distinct vertex is one row
    _, _, ost = O.vexpand(g, src, 1, 4, path, "forward", hop_stats=True)
    feats = {}
    for strat in ("sparse", "pull", "push"):
        plan = vs.ExpandPlan(dg, len(src), vs.make_params(1, 4, path, "forward"))
        plan.set_hop_strategies([0] + [strat] * 4)
        plan.log_features(True)
        plan.set_tuning(collect_stats=True)
        plan.run(src)
        st = plan.stats()
        n = st["hops_run"]
        assert st["active_edges"][1:] == ost["active_edges"][1:n + 1], (strat, st["active_edges"])
        feats[strat] = plan.features()[1:n + 1]
        plan.free()
    for strat in ("pull", "push"):
        k = min(len(feats[strat]), len(feats["sparse"]))
        assert np.array_equal(feats[strat][:k, 16:], feats["sparse"][:k, 16:]), strat
        assert np.array_equal(feats[strat][:k, 10:12], feats["sparse"][:k, 10:12]), strat
    d = np.diff(g.fwd_off)[np.unique(src)]
    bins = np.minimum(15, np.floor(np.log2(d + 1.0)).astype(int))
    h1 = np.bincount(bins, minlength=16) / len(d)
    assert np.allclose(feats["sparse"][0, 16:], h1, atol=1e-6)


@pytest.mark.parametrize("cls", [0, 1, 2])
def test_intersection_method_picker_keeps_results(vs, cls):
    """A network choosing the adjacency membership method (binary search,
    window merge, hub bitmap) on the device: every choice gives the count of
    the per-tuple rule; the call's features are finite and normalised."""
    g = graphgen.zipf(20_000, 600_000, 1.6, 6000, seed=5)
    dg = vs.DeviceGraph.from_host(g)
    src = graphgen.sample_sources(g.V, 500, seed=3)
    P, _, _ = vs.expand(dg, src, 1, 1, "any", "forward")
    deps = [dict(graph=dg, direction="forward", base_col=0), dict(graph=dg, direction="forward", base_col=1)]
    _, exp, _ = vs.mintersect(P, deps, g.V, True)
    out, count, _, feat = vs.mintersect(P, deps, g.V, False, method_picker=constant_picker(vs, cls), features=True)
    assert count == exp > 0 and out.info()[1] == exp
    assert np.all(np.isfinite(feat)) and feat.min() >= 0.0 and feat.max() <= 4.0
    assert abs(feat[16:24].sum() - 1.0) < 1e-4  # walked-list length histogram
    assert feat[13] == 1.0  # the graph has adjacency bitmaps (degrees >= 1024)


def test_trained_hop_picker_beats_the_fixed_planner(vs):
    """The committed network against the fixed planner on fresh logged hops
    (graphs and queries it was not trained on): it picks the fastest strategy
    more often, and its per-hop choices cost less time in total."""
    from vertexsurge_gb300 import picker_train as T
    pk = vs.Picker()
    pk.set_params(np.load(T.WEIGHTS_FILE))
    graphs = [graphgen.rmat(17, 16, 0.6, 0.175, 0.175, seed=77), graphgen.zipf(300_000, 6_000_000, 2.1, 50_000, seed=78)]
    samples = T.collect(40, seed=99, graphs=graphs, log=None)
    X, y, times, fixed, _ = samples.arrays()
    rep = T.evaluate(pk, X, y, times, fixed)
    assert rep["accuracy"] > rep["fixed_accuracy"], rep
    assert rep["slowdown_vs_best"] <= rep["fixed_slowdown_vs_best"] * 1.02, rep
