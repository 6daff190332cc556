"""Training data, training and evaluation of the learned choice of the
intersection's adjacency membership method.

A logged call is the triangle-closing intersection of the pattern query:
base pairs (a, b) = the out-edges of S sources (the rows of an Any [1,1]
expand), dependencies = the adjacency lists of a and of b (forward, or both
backward).  Each call is timed (CUDA events around the whole call, best of
two after a warm run) under every method the network can choose — binary
search everywhere, hub bitmap wherever one exists, and the per-tuple rule
(`algo='auto'`, which is also the fixed planner it is compared with); the
call's 32 features come from the same device code that feeds the network.
Results never depend on the method (checked on every logged call).
Evaluation on held-out calls: the network's slowdown against the best
choice and its speedup over the rule.
"""
from __future__ import annotations

import json
import math
import sys
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _abi as vs
from . import graphgen

WEIGHTS_FILE = Path(__file__).resolve().parent / "isect_picker_weights.npy"
METHODS = ("auto", "binary", "bitmap")  # network classes 0, 1, 2 (auto: the per-tuple rule)


@dataclass
class Calls:
    X: list = field(default_factory=list)
    times: list = field(default_factory=list)   # (3,) ms per class
    rule: list = field(default_factory=list)    # ms of the per-tuple rule
    call: list = field(default_factory=list)

    def arrays(self):
        return (np.asarray(self.X, np.float32), np.asarray(self.times, np.float64),
                np.asarray(self.rule, np.float64), np.asarray(self.call, np.int64))


def graph_suite(scales=(18, 19, 20, 21, 22), skews=(0.45, 0.57, 0.65), zipf=((1_000_000, 30_000_000),
                                                                                (10_000_000, 300_000_000))):
    gs = []
    for sc in scales:
        for a in skews:
            b = (1.0 - a - 0.05) / 2
            gs.append(graphgen.rmat(sc, 16, a, b, b, seed=sc * 10 + int(a * 100)))
    for V, E in zipf:
        gs.append(graphgen.zipf(V, E, 2.1, min(50_000, V // 4), seed=V % 991))
    return gs


def _time(fn, stream):
    import torch
    fn()
    best = math.inf
    for _ in range(2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = fn()
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best, r


def log_call(dg, g, S, direction, seed, out: Calls, cid: int, stream=None):
    import torch
    stream = stream or torch.cuda.current_stream()
    src = graphgen.sample_sources(g.V, min(S, g.V), seed=seed)
    P, _, _ = vs.expand(dg, src, 1, 1, "any", "forward", stream=stream)
    try:
        def deps(algo):
            return [dict(graph=dg, direction=direction, base_col=0, algo=algo),
                    dict(graph=dg, direction=direction, base_col=1, algo=algo)]
        *_, feat = vs.mintersect(P, deps("auto"), g.V, True, stream=stream, features=True)
        times, counts = [], []
        for m in METHODS:
            ms, r = _time(lambda m=m: vs.mintersect(P, deps(m), g.V, True, stream=stream), stream)
            times.append(ms)
            counts.append(r[1])
        ms_rule = times[0]
        if len(set(counts)) != 1:
            raise RuntimeError(f"intersection methods disagree: {counts}")
    finally:
        P.free()
    out.X.append(feat)
    out.times.append(times)
    out.rule.append(ms_rule)
    out.call.append(cid)


def collect(n_calls: int, graphs=None, seed: int = 2, minutes: float = 0.0, log=print) -> Calls:
    rng = np.random.default_rng(seed)
    graphs = graphs or graph_suite()
    dgs = [vs.DeviceGraph.from_host(g) for g in graphs]
    out = Calls()
    t0 = time.time()
    for c in range(n_calls):
        if minutes and time.time() - t0 > 60 * minutes:
            break
        gi = int(rng.integers(len(graphs)))
        S = int(round(math.exp(rng.uniform(math.log(16), math.log(4096)))))
        direction = "forward" if rng.random() < 0.7 else "backward"
        log_call(dgs[gi], graphs[gi], S, direction, int(rng.integers(1 << 30)), out, c)
        if log and (c + 1) % 100 == 0:
            log(f"  {c + 1} calls, {time.time() - t0:.0f}s")
    return out


def evaluate(pk, X, times, rule):
    pred = pk.predict(X)
    best = times.min(axis=1).sum()
    pick = times[np.arange(len(pred)), pred].sum()
    y = times.argmin(axis=1)
    return {"calls": int(len(X)), "accuracy": float((pred == y).mean()),
            "slowdown_vs_best": float(pick / best), "rule_slowdown_vs_best": float(rule.sum() / best),
            "speedup_vs_rule": float(rule.sum() / pick),
            "best_fixed_method": METHODS[int(times.sum(axis=0).argmin())],
            "best_fixed_method_slowdown": float(times.sum(axis=0).min() / best)}


def train_and_evaluate(calls: Calls, epochs=60, seed=3, holdout=0.25):
    X, times, rule, cid = calls.arrays()
    y = times.argmin(axis=1).astype(np.int32)
    rng = np.random.default_rng(seed)
    te = rng.random(len(X)) < holdout
    pk = vs.Picker(seed=seed)
    loss = pk.train(X[~te], y[~te], epochs=epochs, batch=256, lr=2e-3, seed=seed)
    rep = evaluate(pk, X[te], times[te], rule[te])
    rep["train_loss"] = loss
    rep["train_calls"] = int((~te).sum())
    rep["label_share"] = np.bincount(y, minlength=3).tolist()
    return pk, rep


def main():
    import argparse
    ap = argparse.ArgumentParser(description="log, train and evaluate the intersection-method picker")
    ap.add_argument("--calls", type=int, default=6000)
    ap.add_argument("--minutes", type=float, default=0.0)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--out", default=str(WEIGHTS_FILE))
    ap.add_argument("--report", default="")
    ap.add_argument("--scales", default="18,19,20,21,22")
    args = ap.parse_args()
    vs.init(0)
    graphs = graph_suite(scales=tuple(int(x) for x in args.scales.split(",")))
    t0 = time.time()
    calls = collect(args.calls, graphs=graphs, minutes=args.minutes,
                    log=lambda m: print(m, file=sys.stderr, flush=True))
    pk, rep = train_and_evaluate(calls, epochs=args.epochs)
    rep["logging_s"] = time.time() - t0
    rep["graphs"] = [{"V": g.V, "E": g.E} for g in graphs]
    np.save(args.out, pk.params())
    print(json.dumps(rep))
    if args.report:
        Path(args.report).write_text(json.dumps(rep, indent=1))


if __name__ == "__main__":
    main()
