"""Serving loop with continuous batching for pattern queries on a resident graph.

A query is the expand + join + intersect pattern of one user:
  A = VExpand(its sources, Shortest, [1, l], Forward)      -> visited count
  J = HashJoin(A, its (key, payload) table) on vertex id  -> count
  T = Mintersect(VExpand(its sources, Any, [1, 1]); out-list of a, out-list of b) -> triangle count
Results are exact integers, so a query's answer is the same whether it runs
alone or among others.

The server keeps the graph in HBM and admits requests continuously: a request
that has arrived is started as soon as a slot is free and the device bytes its
plans need (vs_expand_plan_footprint) fit in the memory budget; finishing
requests return their slot and bytes at once, so new arrivals join work
already on the GPU instead of waiting for a batch boundary.  Every slot is a
host thread with its own CUDA stream (the C ABI releases the GIL), so the
kernels of concurrent queries overlap on the device.  Latency is completion
time minus arrival time (queueing included).
"""
from __future__ import annotations

import math
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _abi as vs
from . import graphgen


@dataclass
class Request:
    rid: int
    arrival: float                # seconds after the start of the trace
    sources: np.ndarray
    k_max: int
    keys: np.ndarray              # join table: uint32 vertex keys
    payload: np.ndarray
    # filled by the server
    start: float = 0.0
    done: float = 0.0
    result: tuple = ()
    bytes: int = 0


def make_trace(g, n: int, rate_qps: float, s_range=(64, 2048), l_max=5, join_rows=(1000, 100_000),
               seed: int = 5) -> list:
    """Poisson arrivals; source counts log-uniform in s_range; hop ranges [1, l] with l
    uniform in 2..l_max; a join table per query with Zipf-skewed keys."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate_qps)
        S = int(round(math.exp(rng.uniform(math.log(s_range[0]), math.log(s_range[1])))))
        S = max(1, min(S, g.V))
        src = graphgen.sample_sources(g.V, S, seed=int(rng.integers(1 << 30)))
        l = int(rng.integers(2, l_max + 1))
        nj = int(round(math.exp(rng.uniform(math.log(join_rows[0]), math.log(join_rows[1])))))
        keys = np.minimum(rng.zipf(1.3, nj) - 1, g.V - 1).astype(np.uint32)
        payload = rng.integers(0, 1 << 31, nj).astype(np.uint32)
        out.append(Request(i, t, src, l, keys, payload))
    return out


class Server:
    def __init__(self, dg: vs.DeviceGraph, budget_bytes: int, slots: int = 4, picker=None, tuned=None,
                 make_stream=None):
        self.dg = dg
        self.budget = int(budget_bytes)
        self.slots = slots
        self.picker = picker
        self.tuned = tuned or {}
        self.adj = [dict(graph=dg, direction="forward", base_col=0), dict(graph=dg, direction="forward", base_col=1)]
        self.make_stream = make_stream  # a slot's stream (default: a new CUDA stream per slot)

    def _params(self, S, k_min, k_max, path):
        from .autotune import params_kw
        return vs.make_params(k_min, k_max, path, "forward", use_picker=self.picker is not None,
                              **params_kw(self.tuned.get(path)))

    def footprint(self, r: Request) -> int:
        """Device bytes the query holds at its peak: its two expand plans run
        one after the other, so the larger of the two."""
        S = len(r.sources)
        return max(vs.plan_footprint(self.dg, S, self._params(S, 1, r.k_max, "shortest")),
                   vs.plan_footprint(self.dg, S, self._params(S, 1, 1, "any")))

    def run_query(self, r: Request, stream) -> tuple:
        """The query's stages on its own stream; returns exact counts."""
        S = len(r.sources)
        pa = vs.ExpandPlan(self.dg, S, self._params(S, 1, r.k_max, "shortest"))
        try:
            if self.picker is not None:
                pa.set_picker(self.picker)
            pa.run(r.sources, stream=stream)
            A = pa.result()
            visited = A.count(stream=stream)
            jt = vs.FlatTable.from_columns([r.payload, r.keys], stream=stream)
            _, jc, _ = vs.hash_join(jt, A, 1, 1, only_count=True, stream=stream)
            jt.free()
        finally:
            pa.free()
        pp = vs.ExpandPlan(self.dg, S, self._params(S, 1, 1, "any"))
        try:
            if self.picker is not None:
                pp.set_picker(self.picker)
            pp.run(r.sources, stream=stream)
            _, tc, _ = vs.mintersect(pp.result(), self.adj, self.dg.V, only_count=True, stream=stream)
        finally:
            pp.free()
        return (visited, jc, tc)

    def serve(self, trace: list, time_scale: float = 1.0) -> dict:
        """Replay the trace: arrivals follow the trace clock (scaled), admission is
        continuous under the slot and byte limits."""
        pending = sorted(trace, key=lambda r: r.arrival)
        if self.make_stream is None:
            import torch
            make_stream = torch.cuda.Stream
        else:
            make_stream = self.make_stream
        for r in pending:
            r.bytes = self.footprint(r)
            if r.bytes > self.budget:
                raise ValueError(f"request {r.rid} needs {r.bytes} bytes, above the budget {self.budget}")
        lock = threading.Condition()
        state = {"used": 0, "active": 0, "next": 0, "peak_used": 0, "peak_active": 0}
        t0 = time.perf_counter()
        errors = []

        def worker():
            stream = make_stream()
            while True:
                with lock:
                    while True:
                        i = state["next"]
                        if i >= len(pending):
                            return
                        r = pending[i]
                        now = time.perf_counter() - t0
                        arrived = r.arrival * time_scale <= now
                        fits = state["used"] + r.bytes <= self.budget
                        if arrived and fits:
                            state["next"] += 1
                            state["used"] += r.bytes
                            state["active"] += 1
                            state["peak_used"] = max(state["peak_used"], state["used"])
                            state["peak_active"] = max(state["peak_active"], state["active"])
                            break
                        lock.wait(timeout=max(0.0005, r.arrival * time_scale - now) if not arrived else 0.002)
                r.start = time.perf_counter() - t0
                try:
                    r.result = self.run_query(r, stream)
                except Exception as e:  # reported after the run
                    errors.append((r.rid, repr(e)))
                r.done = time.perf_counter() - t0
                with lock:
                    state["used"] -= r.bytes
                    state["active"] -= 1
                    lock.notify_all()

        threads = [threading.Thread(target=worker, daemon=True) for _ in range(self.slots)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        wall = time.perf_counter() - t0
        if errors:
            raise RuntimeError(f"{len(errors)} queries failed: {errors[:3]}")
        lat = np.array([r.done - r.arrival * time_scale for r in pending]) * 1000.0
        svc = np.array([r.done - r.start for r in pending]) * 1000.0
        return {"queries": len(pending), "wall_s": wall, "queries_per_s": len(pending) / wall,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "service_p50_ms": float(np.percentile(svc, 50)), "peak_bytes": state["peak_used"],
                "peak_concurrent": state["peak_active"], "budget_bytes": self.budget}


def solo_results(dg, trace: list, picker=None, tuned=None) -> list:
    """Every request run alone, one after another (the reference answer of the mix)."""
    import torch
    srv = Server(dg, budget_bytes=1 << 62, slots=1, picker=picker, tuned=tuned)
    stream = torch.cuda.Stream()
    return [srv.run_query(r, stream) for r in trace]


def main():
    """Serving benchmark: R-MAT graph resident in HBM, Poisson arrivals of
    pattern queries, byte-budget admission; the plain fixed planner and the
    learned picker replay the same trace."""
    import argparse
    import json

    import torch

    from . import picker_train
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=27)
    ap.add_argument("--queries", type=int, default=200)
    ap.add_argument("--rate", type=float, default=20.0, help="mean arrivals per second")
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--s-max", type=int, default=2048)
    ap.add_argument("--l-max", type=int, default=5)
    ap.add_argument("--check", type=int, default=20, help="queries re-run alone to check the mix")
    args = ap.parse_args()
    vs.init(0)
    t0 = time.time()
    g = graphgen.rmat(args.scale, 16, 0.57, 0.19, 0.19, seed=27)
    t_gen = time.time() - t0
    dg = vs.DeviceGraph.from_host(g)
    trace = make_trace(g, args.queries, args.rate, s_range=(64, args.s_max), l_max=args.l_max)
    report = {"graph": {"scale": args.scale, "V": g.V, "E": g.E, "gen_s": t_gen},
              "trace": {"queries": args.queries, "rate_qps": args.rate, "s_range": [64, args.s_max],
                        "l_max": args.l_max}}
    del g
    budget = int(args.budget_gb * (1 << 30))
    pickers = {"plain": None}
    if picker_train.WEIGHTS_FILE.exists():
        pk = vs.Picker()
        pk.set_params(np.load(picker_train.WEIGHTS_FILE))
        pickers["learned"] = pk
    results = {}
    for name, pk in pickers.items():
        srv = Server(dg, budget, slots=args.slots, picker=pk)
        for r in trace:
            r.result = ()
        report[name] = srv.serve(trace)
        results[name] = [r.result for r in trace]
    torch.cuda.synchronize()
    # every answer is the same alone and in the mix (and under both planners)
    solo = solo_results(dg, trace[: args.check])
    report["check"] = {"queries": len(solo),
                       "same_alone_and_in_mix": all(results["plain"][i] == solo[i] for i in range(len(solo))),
                       "same_under_picker": all(results[n] == results["plain"] for n in results)}
    print(json.dumps(report))


if __name__ == "__main__":
    main()
