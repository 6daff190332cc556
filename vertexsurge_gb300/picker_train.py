"""Training data, training and evaluation of the learned per-hop strategy picker.

Data comes from the method's own runs.  For every logged query the expand is
run once per strategy family — every hop PULL; PUSH at every hop whose
frontier holds under PUSH_CAP of the vertices (a PUSH hop over a denser
frontier is an atomic write per edge and row, always far slower than PULL, and
is counted as not chosen); SPARSE for as long as its pair list lasts — with
per-hop CUDA-event timing and feature logging on.  All runs of a query see the
same frontier at every hop (the strategy never changes a result), so each hop
yields samples (features, fastest strategy):
  * from the SPARSE run while SPARSE is still possible (features say a pair
    list exists): label = fastest of PULL / PUSH / SPARSE at that hop;
  * from the PULL run (features say no pair list): label = fastest of
    PULL / PUSH.
The network (vs_picker, CUDA training kernels) is trained on these samples.
Evaluation on held-out queries compares, per hop, the time of the picker's
choice with the exhaustive best and with the fixed planner's choice, using
the logged times of the same hops.
"""
from __future__ import annotations

import json
import math
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _abi as vs
from . import graphgen

WEIGHTS_FILE = Path(__file__).resolve().parent / "picker_weights.npy"
STRATS = (vs.STRAT_PULL, vs.STRAT_PUSH, vs.STRAT_SPARSE)  # class 0, 1, 2
PUSH_CAP = 0.05  # PUSH is timed at hops whose frontier holds fewer than this fraction of V


@dataclass
class Samples:
    X: list = field(default_factory=list)       # features (32,)
    y: list = field(default_factory=list)       # fastest class
    times: list = field(default_factory=list)   # (3,) ms per class, inf when unavailable
    fixed: list = field(default_factory=list)   # class the fixed planner chose in the same context
    query: list = field(default_factory=list)   # query index (for held-out splits)

    def arrays(self):
        return (np.asarray(self.X, np.float32), np.asarray(self.y, np.int32),
                np.asarray(self.times, np.float64), np.asarray(self.fixed, np.int32),
                np.asarray(self.query, np.int64))


def graph_suite(scales=(20, 21, 22, 23, 24), skews=(0.45, 0.57, 0.65),
                zipf=((1_000_000, 30_000_000), (10_000_000, 300_000_000)), small=(16,)):
    """R-MAT graphs at `scales` x skews a (b = c = (1 - a - 0.05) / 2), the
    small R-MAT of the plain-method configuration and the power-law graphs of
    the pattern query (10M vertices, and its 1M-vertex instance)."""
    gs = []
    for sc in scales:
        for a in skews:
            b = (1.0 - a - 0.05) / 2
            gs.append(graphgen.rmat(sc, 16, a, b, b, seed=sc * 100 + int(a * 100)))
    for sc in small:
        gs.append(graphgen.rmat(sc, 16, 0.57, 0.19, 0.19, seed=1))
    for V, E in zipf:
        gs.append(graphgen.zipf(V, E, 2.1, min(50_000, V // 4), seed=3))
    return gs


def _run(plan, src, strategies):
    plan.set_hop_strategies([0] + list(strategies))
    plan.run(src)
    st = plan.stats()
    return st, plan.features()


def log_query(dg, g, S, k_max, path, direction, seed, out: Samples, qid: int):
    src = graphgen.sample_sources(g.V, min(S, g.V), seed=seed)
    plan = vs.ExpandPlan(dg, len(src), vs.make_params(1, k_max, path, direction))
    plan.set_tuning(timing=True)
    plan.log_features(True)
    try:
        _log_runs(plan, src, k_max, g.V, out, qid)
    finally:
        plan.free()


def _log_runs(plan, src, k_max, V, out: Samples, qid: int):
    runs = {vs.STRAT_PULL: _run(plan, src, [vs.STRAT_PULL] * k_max)}
    av = runs[vs.STRAT_PULL][0]["active_vertices"]
    push_at = [h for h in range(1, k_max + 1) if h - 1 < len(av) and av[h - 1] < PUSH_CAP * V]
    runs[vs.STRAT_PUSH] = _run(plan, src, [vs.STRAT_PUSH if h in push_at else vs.STRAT_PULL
                                           for h in range(1, k_max + 1)])
    runs[vs.STRAT_SPARSE] = _run(plan, src, [vs.STRAT_SPARSE] * k_max)
    st_auto, f_auto = _run(plan, src, [vs.STRAT_AUTO] * k_max)
    hops = runs[vs.STRAT_PULL][0]["hops_run"]
    for h in range(1, hops + 1):
        t = {s: runs[s][0]["hop_ms"][h] if h <= runs[s][0]["hops_run"] else math.inf for s in STRATS}
        if h not in push_at:
            t[vs.STRAT_PUSH] = math.inf
        sp_st = runs[vs.STRAT_SPARSE][0]
        sparse_ok = h <= sp_st["hops_run"] and sp_st["strategy"][h] == vs.STRAT_SPARSE
        fixed_class = STRATS.index(st_auto["strategy"][h]) if h <= st_auto["hops_run"] else 0
        # context with a pair list: the SPARSE run's features
        if sparse_ok:
            times = [t[vs.STRAT_PULL], t[vs.STRAT_PUSH], t[vs.STRAT_SPARSE]]
            out.X.append(runs[vs.STRAT_SPARSE][1][h])
            out.y.append(int(np.argmin(times)))
            out.times.append(times)
            # the fixed planner's choice where it also had a pair list
            fc = fixed_class if (h == 1 or st_auto["strategy"][h - 1] == vs.STRAT_SPARSE) else None
            out.fixed.append(fc if fc is not None else int(np.argmin(times[:2])))
            out.query.append(qid)
        if h >= 2 or not sparse_ok:
            times = [t[vs.STRAT_PULL], t[vs.STRAT_PUSH], math.inf]
            out.X.append(runs[vs.STRAT_PULL][1][h])
            out.y.append(int(np.argmin(times)))
            out.times.append(times)
            out.fixed.append(0 if fixed_class == 2 else fixed_class)
            out.query.append(qid)


def collect(n_queries: int, seed: int = 1, graphs=None, log=print, minutes: float = 0.0,
            target_samples: int = 0) -> Samples:
    """Log up to n_queries queries (stopping early after `minutes` of logging or
    at `target_samples` samples); graphs are drawn with weight 1/E so small and
    large graphs contribute similar logging time."""
    rng = np.random.default_rng(seed)
    graphs = graphs or graph_suite()
    dgs = [vs.DeviceGraph.from_host(g) for g in graphs]
    w = np.array([1.0 / max(1, g.E) for g in graphs])
    w /= w.sum()
    out = Samples()
    t0 = time.time()
    for q in range(n_queries):
        if minutes and time.time() - t0 > 60 * minutes:
            break
        if target_samples and len(out.y) >= target_samples:
            break
        gi = int(rng.choice(len(graphs), p=w))
        S = int(round(math.exp(rng.uniform(math.log(64), math.log(8192)))))
        S = max(1, min(S, graphs[gi].V))
        k_max = int(rng.integers(2, 7))
        path = "shortest" if rng.random() < 0.7 else "any"
        direction = "forward" if rng.random() < 0.7 else "both"
        if path == "any":
            k_max = min(k_max, 4)
        log_query(dgs[gi], graphs[gi], S, k_max, path, direction, int(rng.integers(1 << 30)), out, q)
        if log and (q + 1) % 200 == 0:
            log(f"  {q + 1} queries, {len(out.y)} samples, {time.time() - t0:.0f}s")
    return out


def evaluate(pk, X, y, times, fixed):
    """Per-hop times of the picker's, the fixed planner's and the best choices."""
    pred = pk.predict(X)
    # the picker never chooses an unavailable strategy (the decide kernel masks it)
    avail = np.isfinite(times)
    logits = pk.forward(X)
    logits[~avail] = -np.inf
    pred = logits.argmax(axis=1)
    t_best = times.min(axis=1).sum()
    t_pick = times[np.arange(len(pred)), pred].sum()
    t_fix = times[np.arange(len(fixed)), fixed].sum()
    return {"samples": int(len(y)), "accuracy": float((pred == y).mean()),
            "fixed_accuracy": float((fixed == y).mean()),
            "slowdown_vs_best": float(t_pick / t_best), "fixed_slowdown_vs_best": float(t_fix / t_best),
            "speedup_vs_fixed": float(t_fix / t_pick)}


def train_and_evaluate(samples: Samples, epochs=40, seed=3, holdout=0.2):
    X, y, times, fixed, qid = samples.arrays()
    rng = np.random.default_rng(seed)
    queries = np.unique(qid)
    test_q = set(rng.choice(queries, max(1, int(len(queries) * holdout)), replace=False).tolist())
    te = np.array([q in test_q for q in qid])
    pk = vs.Picker(seed=seed)
    loss = pk.train(X[~te], y[~te], epochs=epochs, batch=512, lr=2e-3, seed=seed)
    rep = evaluate(pk, X[te], y[te], times[te], fixed[te])
    rep["train_loss"] = loss
    rep["train_samples"] = int((~te).sum())
    return pk, rep


def main():
    import argparse
    ap = argparse.ArgumentParser(description="log, train and evaluate the strategy picker")
    ap.add_argument("--queries", type=int, default=100_000)
    ap.add_argument("--samples", type=int, default=100_000, help="stop logging at this many samples")
    ap.add_argument("--minutes", type=float, default=0.0, help="stop logging after this long (0: no limit)")
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--out", default=str(WEIGHTS_FILE))
    ap.add_argument("--report", default="")
    ap.add_argument("--scales", default="20,21,22,23,24")
    ap.add_argument("--no-zipf", action="store_true", help="leave out the power-law graphs")
    args = ap.parse_args()
    vs.init(0)
    scales = tuple(int(x) for x in args.scales.split(","))
    t0 = time.time()
    graphs = graph_suite(scales=scales, zipf=() if args.no_zipf else ((1_000_000, 30_000_000),
                                                                       (10_000_000, 300_000_000)))
    samples = collect(args.queries, graphs=graphs, minutes=args.minutes, target_samples=args.samples)
    t_log = time.time() - t0
    pk, rep = train_and_evaluate(samples, epochs=args.epochs)
    rep["logging_s"] = t_log
    rep["queries"] = int(len(np.unique(samples.query)))
    rep["graphs"] = [{"V": g.V, "E": g.E} for g in graphs]
    rep["label_share"] = np.bincount(np.asarray(samples.y), minlength=3).tolist()
    np.save(args.out, pk.params())
    print(json.dumps(rep))
    if args.report:
        Path(args.report).write_text(json.dumps(rep, indent=1))


if __name__ == "__main__":
    main()
