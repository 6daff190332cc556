"""Batched queries: many expand + join queries in one CUDA-graph launch.

Query q (sources s_q, last hop l_q, key table K_q of vertex ids):
  A_q = VExpand(s_q, Shortest, [1, l_q], Forward)
  J_q = count of HashJoin(A_q, K_q) on the vertex id
The reference runs one VExpand and one HashJoin per query.  Here the queries
are sorted by l_q and packed into waves of at most `wave_rows` source rows.  A
wave is one run of a shared expand plan whose row i belongs to one query and
stops growing after that query's last hop (per-row hop masks, set on the
device from a per-wave limit array), followed by one row-block join count
that gives every query of the wave its J_q.  The whole batch — every wave's
limits, expand and join counts — is recorded once on a stream and replayed as
a single graph launch; a query's rows, and so its counts, are the ones it gets
when run alone.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import _abi as vs
from . import graphgen


@dataclass
class Query:
    sources: np.ndarray   # uint32 vertex ids
    k_max: int            # hop range [1, k_max]
    keys: np.ndarray      # uint32 vertex ids of the joined table


def zipf_keys(rng, n: int, V: int, perm: np.ndarray, s: float = 1.2) -> np.ndarray:
    """n vertex ids Zipf-skewed over V: rank r has probability ~ r^-s (Pareto
    inverse transform, ranks folded into [0, V)), and ranks map to vertices
    through a fixed permutation so the hot keys are spread over the graph."""
    u = rng.random(n)
    r = np.floor(np.power(1.0 - u, -1.0 / (s - 1.0))).astype(np.float64) - 1.0
    r = np.mod(r, V).astype(np.int64)
    return perm[r].astype(np.uint32)


def make_queries(g, n: int, s_range=(64, 8192), l_range=(2, 6), join_rows=(100_000, 10_000_000),
                 seed: int = 4, key_skew: float = 1.2) -> list:
    """Source counts log-uniform in s_range, last hop uniform in l_range, key
    tables of (key, payload) pairs with row counts uniform in join_rows and
    keys Zipf-skewed over the vertices (only the key column enters a count)."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(g.V).astype(np.uint32)
    out = []
    for _ in range(n):
        S = int(round(math.exp(rng.uniform(math.log(s_range[0]), math.log(s_range[1])))))
        S = max(1, min(S, g.V))
        src = graphgen.sample_sources(g.V, S, seed=int(rng.integers(1 << 30)))
        l = int(rng.integers(l_range[0], l_range[1] + 1))
        nk = int(rng.integers(join_rows[0], join_rows[1] + 1))
        out.append(Query(src, l, zipf_keys(rng, nk, g.V, perm, key_skew)))
    return out


def pack(queries: list, wave_rows: int) -> list:
    """Waves of query indices: queries sorted by last hop (longest first), then
    filled greedily up to wave_rows rows."""
    if any(len(q.sources) > wave_rows for q in queries):
        raise ValueError(f"a query has more than {wave_rows} sources")
    order = sorted(range(len(queries)), key=lambda i: (-queries[i].k_max, i))
    waves, cur, rows = [], [], 0
    for i in order:
        n = len(queries[i].sources)
        if cur and rows + n > wave_rows:
            waves.append(cur)
            cur, rows = [], 0
        cur.append(i)
        rows += n
    if cur:
        waves.append(cur)
    return waves


class Batch:
    """Device-resident batch of queries; `capture` records the whole batch on
    `stream`, `launch` replays it, `counts` reads the per-query join counts.

    lanes > 1 runs the waves on that many concurrent branches of the captured
    graph, wave w on lane w mod lanes, each lane with its own expand plan and
    stream: while one wave is in a hop that leaves SMs idle (pair-list hops,
    decide and clear kernels, the tail of a PULL hop) another wave's kernels
    fill them."""

    def __init__(self, dg, queries: list, wave_rows: int, stream, path="shortest", direction="forward",
                 setting: dict | None = None, picker=None, lanes: int = 1):
        import torch
        from .autotune import params_kw
        self.dg, self.queries, self.stream = dg, queries, stream
        self.waves = pack(queries, wave_rows)
        self.S = max(sum(len(queries[i].sources) for i in w) for w in self.waves)
        self.k_max = max(q.k_max for q in queries)
        params = vs.make_params(1, self.k_max, path, direction, use_picker=picker is not None, **params_kw(setting))
        # every lane holds a plan: no more lanes than the free device memory takes twice over
        free_b, _ = torch.cuda.mem_get_info()
        fits = max(1, int(free_b // (2 * vs.plan_footprint(dg, self.S, params))))
        self.lanes = max(1, min(int(lanes), len(self.waves), fits))
        self.plans = []
        for _ in range(self.lanes):
            pl = vs.ExpandPlan(dg, self.S, params)
            if picker is not None:
                pl.set_picker(picker)
            self.plans.append(pl)
        self.plan = self.plans[0]
        self.streams = [stream] + [torch.cuda.Stream() for _ in range(self.lanes - 1)]
        nw = len(self.waves)
        src = np.zeros((nw, self.S), np.uint32)       # padding rows start at vertex 0 and never grow
        lim = np.zeros((nw, self.S), np.uint8)
        key_order, self.blocks, self.slot = [], [], np.zeros(len(queries), np.int64)
        koff, slot = 0, 0
        for wi, w in enumerate(self.waves):
            r0, blocks = 0, []
            for i in w:
                q = queries[i]
                n = len(q.sources)
                src[wi, r0:r0 + n] = q.sources
                lim[wi, r0:r0 + n] = q.k_max
                blocks.append((r0, r0 + n, koff, koff + len(q.keys)))
                key_order.append(q.keys)
                self.slot[i] = slot
                r0 += n
                koff += len(q.keys)
                slot += 1
            if len(blocks) > vs.MAX_ROW_BLOCKS:
                raise ValueError(f"more than {vs.MAX_ROW_BLOCKS} queries in one wave")
            self.blocks.append(blocks)
        self.key_rows = koff
        dev = torch.device("cuda")
        with torch.cuda.stream(stream):
            self.d_src = torch.from_numpy(src.view(np.int32)).to(dev, non_blocking=False)
            self.d_lim = torch.from_numpy(lim).to(dev)
            self.d_keys = torch.from_numpy(np.concatenate(key_order).view(np.int32)).to(dev)
            self.d_counts = torch.zeros(len(queries), dtype=torch.int64, device=dev)
        stream.synchronize()
        self.graph = None

    def h2d_bytes(self) -> int:
        return self.d_src.numel() * 4 + self.d_lim.numel() + self.d_keys.numel() * 4

    def run_eager(self):
        """Every wave: row limits, expand, row-block join counts, ordered on its
        lane's stream; the lanes fork from and join back into `stream`."""
        import torch
        if self.lanes > 1:
            fork = torch.cuda.Event()
            fork.record(self.stream)
            for st in self.streams[1:]:
                st.wait_event(fork)
        off = 0
        for wi, blocks in enumerate(self.waves):
            k = wi % self.lanes
            plan, st = self.plans[k], self.streams[k]
            plan.set_row_limits_device(self.d_lim[wi], self.S, stream=st)
            plan.run(self.d_src[wi], stream=st)
            nb = len(self.blocks[wi])
            vs.join_count_row_blocks(plan.result(), self.d_keys, self.blocks[wi],
                                     self.d_counts[off:off + nb], stream=st)
            off += nb
        for st in self.streams[1:]:
            join = torch.cuda.Event()
            join.record(st)
            self.stream.wait_event(join)

    def capture(self):
        self.run_eager()  # every plan's first run on its stream happens outside the capture
        for st in self.streams:
            st.synchronize()
        with vs.Captured(self.stream, keep=(*self.plans, self.d_src, self.d_lim, self.d_keys,
                                            self.d_counts)) as cg:
            self.run_eager()
        self.graph = cg
        return cg

    def launch(self):
        self.graph.launch(self.stream)

    def counts(self) -> np.ndarray:
        """Join count per query, in the order of `queries`."""
        self.stream.synchronize()
        return self.d_counts.cpu().numpy()[self.slot].astype(np.uint64)

    def free(self):
        if self.graph is not None:
            self.graph.free()
            self.graph = None
        for pl in self.plans:
            pl.free()


def solo_counts(dg, queries: list, path="shortest", direction="forward", stream=None) -> np.ndarray:
    """Every query alone through the one-query operators: VExpand, then a
    HashJoin with its key table (count only)."""
    out = np.zeros(len(queries), np.uint64)
    for i, q in enumerate(queries):
        A, _, _ = vs.expand(dg, q.sources, 1, q.k_max, path, direction, stream=stream)
        kt = vs.FlatTable.from_columns([q.keys], stream=stream)
        _, c, _ = vs.hash_join(kt, A, 0, 1, only_count=True, stream=stream)
        out[i] = c
        kt.free()
        A.free()
    return out


def tune_wave_rows(dg, queries, stream, candidates=(16384, 32768), setting=None, repeats=1,
                   picker=None, short_shares=(0.0, -1.0), lanes=(1,)) -> dict:
    """Time one captured batch per wave width, short-mode setting and lane
    count (the waves' hop limits and mixed sizes decide whether short-row PULL
    and concurrent waves pay, so they are tuned here on the batch itself);
    returns {'wave_rows', 'short_share', 'lanes', 'ms', 'table'}."""
    import torch
    table = []
    widest = max(len(q.sources) for q in queries)
    for wr, sh, ln in [(wr, sh, ln) for wr in candidates for sh in short_shares for ln in lanes]:
        if wr < widest:
            continue
        st = dict(setting or {})
        st["short_share"] = sh
        b = Batch(dg, queries, wr, stream, setting=st, picker=picker, lanes=ln)
        try:
            b.capture()
            b.launch()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(repeats)]
            for e0, e1 in ev:
                e0.record(stream)
                b.launch()
                e1.record(stream)
            stream.synchronize()
            ms = min(e0.elapsed_time(e1) for e0, e1 in ev)
            table.append({"wave_rows": wr, "short_share": sh, "lanes": b.lanes, "waves": len(b.waves), "ms": ms})
        finally:
            b.free()
    best = min(table, key=lambda r: r["ms"])
    return {"wave_rows": best["wave_rows"], "short_share": best["short_share"], "lanes": best["lanes"],
            "ms": best["ms"], "table": table}
