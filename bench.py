#!/usr/bin/env python3
"""Benchmark: the power-law pattern query on one GB300.

Workload (default "zipf10M_pattern"): a power-law graph with 10M vertices and
~300M directed edges (out-degree ~ Zipf(2.1) capped at 50k, uniform targets,
uint32 CSR).  One step is the whole pattern query:
  A  = VExpand(4,096 sources, Shortest, hops [1,4], Forward)
  B  = VExpand(4,096 other sources, Shortest, hops [1,2], Forward)
  J  = HashJoin(A, B) on the vertex id, exact count
  P  = VExpand(the A sources, Any, hops [1,1])  (edges a -> b)
  T  = Mintersect(P; out-list of a, out-list of b): triangles a->b, a->c, b->c, count
The metric is multi-source expand throughput, Gsrc-edges/s =
sum over the three expands and their hops of S * E_active(h), divided by the
whole step's time (join and intersection included).

value   : device-resident inputs (sources in HBM, reusable expand plans),
          CUDA events on the launching stream around exactly --steps steps.
e2e     : the same query through the one-shot C-ABI calls with the source
          lists in pinned host memory (host->device copies and the device->host
          result reads inside the timed region).
--impl reference : the CPU restatement of the reference's operators (the
          oracle, OpenMP over every host core) on a bounded sample of the same
          workload: VExpand(1,024 of the A sources, Shortest, [1,4]).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
NOMINAL_HBM_GBS = 7900.0  # GB300 HBM3e, nominal
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    "zipf10M_pattern": dict(kind="zipf", V=10_000_000, E=300_000_000, alpha=2.1, cap=50_000, seed=3,
                            S_a=4096, hops_a=(1, 4), S_b=4096, hops_b=(1, 2), cpu_S=1024),
    # smaller instances of the same query (for profiling runs)
    "zipf1M_pattern": dict(kind="zipf", V=1_000_000, E=30_000_000, alpha=2.1, cap=50_000, seed=3,
                           S_a=4096, hops_a=(1, 4), S_b=4096, hops_b=(1, 2), cpu_S=1024),
    "rmat16_pattern": dict(kind="rmat", scale=16, ef=16, seed=1, S_a=512, hops_a=(1, 3), S_b=512,
                           hops_b=(1, 2), cpu_S=512),
    # 256 queries (sources log-uniform in 64..8192, hops [1,l], l in 2..6, a join of
    # 1e5..1e7 vertex-id keys each) on the 10M-vertex graph, one CUDA-graph launch per batch
    "zipf10M_batched256": dict(kind="zipf", V=10_000_000, E=300_000_000, alpha=2.1, cap=50_000, seed=3,
                               batched=dict(n=256, s_range=(64, 8192), l_range=(2, 6),
                                            join_rows=(100_000, 10_000_000), waves=(8192, 16384, 32768),
                                            cpu_queries=3, check=6)),
    # Flat x Flat count-only HashJoin of two uint32 key columns of N rows each,
    # keys Zipf-skewed over 10M vertex ids (the key tables of the batched workload)
    "join_zipf10M": dict(kind="join", V=10_000_000, sizes=(100_000, 1_000_000, 10_000_000), skew=1.2, seed=4,
                         cpu_rows=1_000_000),
    # config 5: the serving loop on a resident R-MAT graph (scale 27: 134M vertices, 2.1B edges), Poisson
    # arrivals of pattern queries (expand + join + triangles), admission by plan bytes under a budget
    "serving_rmat27": dict(kind="serving", scale=27, queries=100, rate=1.5, budget_gb=150.0, slots=8,
                           s_max=2048, l_max=5, check=20, oracle_queries=2),
    "zipf1M_batched64": dict(kind="zipf", V=1_000_000, E=30_000_000, alpha=2.1, cap=50_000, seed=3,
                             batched=dict(n=64, s_range=(64, 8192), l_range=(2, 6),
                                          join_rows=(100_000, 1_000_000), waves=(8192, 16384, 32768),
                                          cpu_queries=3, check=6)),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def make_graph(w):
    from vertexsurge_gb300 import graphgen
    if w["kind"] == "zipf":
        return graphgen.zipf(w["V"], w["E"], w["alpha"], w["cap"], seed=w["seed"])
    return graphgen.rmat(w["scale"], w["ef"], 0.57, 0.19, 0.19, seed=w["seed"])


def sources(g, w):
    from vertexsurge_gb300 import graphgen
    sa = graphgen.sample_sources(g.V, w["S_a"], seed=101)
    sb = graphgen.sample_sources(g.V, w["S_b"], seed=102)
    return sa, sb


def profiled_traffic(workload: str, kernel: str = "k_pull"):
    """DRAM bytes per launch of the roofline kernel, from the committed ncu
    summary of this kernel and workload (the line `traffic_bytes_per_launch:
    N`), or None."""
    f = ROOT / "profiles" / f"{kernel}_{workload}.md"
    try:
        for line in f.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":", 1)[1].strip())
    except (OSError, ValueError):
        pass
    return None


def peaks():
    try:
        p = json.loads(PEAKS_FILE.read_text())
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in Path(self.f.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()),
                                   default=None)}


def expand_bytes(V, W, e_act, shortest, acc, gathers=True):
    """Algorithmic bytes of one hop: CSR offsets + targets, one row gather per
    active edge (32-byte sector minimum) and P streaming passes over the V x S
    matrices (P = 4 for the frontier/next pair plus visited or accumulator
    read+write each).  gathers=False gives the compulsory bytes alone (every
    frontier row read once instead of once per edge):
    8(V+1) + 4 E_act + P 8W V."""
    P = 2 + (2 if shortest else 0) + (2 if acc else 0)
    return 8 * (V + 1) + 4 * e_act + (e_act * max(32, 8 * W) if gathers else 0) + P * 8 * W * V


def pattern_config(args, g, w, world):
    """The workload's `config` object, the same in the GPU and reference arms."""
    Sa, Sb = w["S_a"], w["S_b"]
    W = (Sa + 63) // 64
    csr_gb = (16 * (g.V + 1) + 8 * g.E) / 1e9
    mat_gb = 8 * (W + (W & 1)) * g.V / 1e9
    return {"workload": args.workload, "V": g.V, "E": g.E, "S_a": Sa, "hops_a": list(w["hops_a"]),
            "S_b": Sb, "hops_b": list(w["hops_b"]), "join": "A x B on vertex id, exact count",
            "intersect": "triangle closing over out-lists, exact count",
            "l2": f"inputs larger than L2 (CSR {csr_gb:.1f} GB, {mat_gb:.2f} GB per bit matrix)"
            if mat_gb > 0.126 else "matrices fit in L2 (launch-bound workload)",
            "parallelism": f"replicas{world}"}


def batched_config(args, g, queries, world):
    """The batched workload's `config` object, the same in both arms."""
    return {"workload": args.workload, "V": g.V, "E": g.E, "queries": len(queries),
            "sources": int(sum(len(q.sources) for q in queries)),
            "key_rows": int(sum(len(q.keys) for q in queries)), "l2": "inputs larger than L2",
            "parallelism": f"replicas{world}"}


def cpu_model() -> str:
    """The host CPU as /proc/cpuinfo names it: the model name on x86, the
    implementer and part numbers on Arm (0x41 / 0xd4f is Neoverse V2, the
    Grace core)."""
    import platform
    import re
    try:
        txt = Path("/proc/cpuinfo").read_text()
    except OSError:
        return platform.machine()
    m = re.search(r"^model name\s*:\s*(.+)$", txt, re.M)
    if m:
        return m.group(1).strip()
    imp = re.search(r"^CPU implementer\s*:\s*(\S+)", txt, re.M)
    part = re.search(r"^CPU part\s*:\s*(\S+)", txt, re.M)
    if imp and part:
        name = " (Neoverse V2)" if (imp.group(1), part.group(1)) == ("0x41", "0xd4f") else ""
        return f"{platform.machine()} implementer {imp.group(1)} part {part.group(1)}{name}"
    return platform.machine()


# Block count of the reference's BlockHilbert edge layout in the CPU legs: the
# importer's -b 1000 of the reference's documented import commands (256 blocks
# ran within 4% of it on the 10M-vertex graph).
CPU_BLOCKS = 1000


def cpu_blocks(g):
    """The forward direction's BlockHilbert layout (the reference importer's
    partitioned hilbert lists), built once per graph outside any timed region,
    as the reference reads it from its graph directory."""
    from oracle import pyoracle as O
    return O.FlatBlocks(g, "forward", CPU_BLOCKS)


def cpu_baseline(g, w, sa):
    """Oracle VExpand on the host cores: the bounded sample and its throughput,
    and the sample's matrix (logical words, V x S/64) for the parity check.
    The matrix comes from the CSR pull, the timed run from the reference's
    BlockHilbert hop; both give the same layers (tests/test_oracle_expand.py)."""
    from oracle import pyoracle as O
    S = w["cpu_S"]
    src = sa[:S]
    k0, k1 = w["hops_a"]
    words, _, st = O.vexpand(g, src, k0, k1, "shortest", "forward", want_matrix=True, hop_stats=True)
    src_edges = S * sum(st["active_edges"][1:])
    blk = cpu_blocks(g)
    t = time.perf_counter()
    O.vexpand(g, src, k0, k1, "shortest", "forward", want_matrix=False, blocks=blk)
    dt = time.perf_counter() - t
    return {"value": src_edges / dt / 1e9, "unit": "Gsrc-edges/s", "cores": O.lib().oracle_get_threads(),
            "kind": "port", "cpu_model": cpu_model(),
            "sample": f"VExpand(Shortest, [{k0},{k1}], Forward) from the first {S} A sources on the full "
                      f"graph, the reference's BlockHilbert hop over {CPU_BLOCKS} target blocks, one run of "
                      f"{dt:.1f} s ({src_edges / 1e9:.2f} Gsrc-edges)"}, words


def batched_queries(g, w):
    from vertexsurge_gb300 import batch
    bw = w["batched"]
    return batch.make_queries(g, bw["n"], bw["s_range"], bw["l_range"], bw["join_rows"], seed=4)


def cpu_batched(g, w, queries, blk):
    """Oracle VExpand (the BlockHilbert hop over `blk`) + TableConvert +
    HashJoin (count) per query, one query at a time as the reference runs
    them, on a bounded sample: the first queries of the trace with at most
    2,048 sources."""
    from oracle import pyoracle as O
    idx = [i for i, q in enumerate(queries) if len(q.sources) <= 2048][: w["batched"]["cpu_queries"]]
    t = time.perf_counter()
    counts = []
    for q in (queries[i] for i in idx):
        words, _, _ = O.vexpand(g, q.sources, 1, q.k_max, "shortest", "forward", blocks=blk)
        # the reference's HashJoin takes ColMain matrices: TableConvert first
        cm = O.table_convert(words, len(q.sources), g.V, False)
        a = O.Table(O.COLMAIN, [0, 1], words=cm, mrows=len(q.sources), mcols=g.V, row_map=q.sources)
        k = O.Table(O.FLAT, [1], cols=[q.keys])
        counts.append(O.hash_join(k, a, 1, only_count=True)[2])
        del words, cm, a
    dt = time.perf_counter() - t
    return idx, counts, dt


def run_reference_batched(args, w):
    from oracle import pyoracle as O
    t0 = time.time()
    g = make_graph(w)
    queries = batched_queries(g, w)
    log(f"graph {g.V} vertices {g.E} edges, {len(queries)} queries in {time.time() - t0:.1f}s")
    blk = cpu_blocks(g)
    times, n = [], 0
    for i in range(args.steps + min(args.warmup, 1)):
        sample, _, dt = cpu_batched(g, w, queries, blk)
        if i >= min(args.warmup, 1):
            times.append(dt)
            n += len(sample)
    value = n / sum(times)
    cores = O.lib().oracle_get_threads()
    desc = (f"{len(sample)} queries per step, one at a time (the first with <= 2048 sources: "
            f"VExpand(Shortest, [1,l]) then HashJoin count with the key table)")
    line = {"impl": "reference", "metric": "batched queries/s", "value": value, "unit": "queries/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": min(args.warmup, 1),
            "ms_per_step": 1000 * sum(times) / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded power-law graph, uniform sources)",
            "config": batched_config(args, g, queries, args.gpus),
            "cpu_baseline": {"value": value, "unit": "queries/s", "cores": cores, "kind": "port", "cpu_model": cpu_model(),
                             "sample": desc},
            "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu_batched(args, w, rank, world, local_rank):
    """Batched queries: the whole batch as one CUDA-graph launch per step."""
    import torch
    import vertexsurge_gb300 as vs
    from vertexsurge_gb300 import autotune, batch, picker_train
    from vertexsurge_gb300 import build as b
    b.build_all()
    torch.cuda.set_device(local_rank)
    vs.init(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    bw = w["batched"]
    t0 = time.time()
    g = make_graph(w)
    queries = batched_queries(g, w)
    nq = len(queries)
    key_rows = sum(len(q.keys) for q in queries)
    src_rows = sum(len(q.sources) for q in queries)
    log(f"[rank {rank}] graph {g.V} vertices {g.E} edges, {nq} queries ({src_rows} sources, "
        f"{key_rows} key rows) in {time.time() - t0:.1f}s")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dg = vs.DeviceGraph.from_host(g, stream=stream)
    # autotune: planner knobs on a wave-sized sample, then the wave width (untimed)
    t0 = time.time()
    from vertexsurge_gb300 import graphgen
    tsrc = graphgen.sample_sources(g.V, min(bw["waves"]), seed=77)
    tc = args.tune_cache or None
    setting = autotune.tune(dg, tsrc, 1, 4, "shortest", "forward", stream=stream, repeats=1,
                            pull_kinds=(0,), sparse_fracs=(0.002, 0.02), hub_thresholds=(0, 256),
                            cache_file=tc)
    setting = {k: setting.get(k, 0.0) for k in ("pull_kind", "sparse_frac", "hub_threshold", "slice_words",
                                                "short_share", "ms")}
    wkey = f"waves|{args.workload}"
    cached = json.loads(Path(tc).read_text()) if tc and Path(tc).exists() else {}
    if wkey in cached:
        waves = cached[wkey]
    else:
        waves = batch.tune_wave_rows(dg, queries, stream, candidates=bw["waves"], setting=setting)
        # then concurrent waves at the best width and short-mode setting
        more = batch.tune_wave_rows(dg, queries, stream, candidates=(waves["wave_rows"],),
                                    setting=dict(setting, short_share=waves["short_share"]),
                                    short_shares=(waves["short_share"],), lanes=(2, 3))
        table = waves["table"] + more["table"]
        if more["ms"] < waves["ms"]:
            waves = more
        # and the SPARSE threshold, tuned above on one sample query, on the batch itself
        waves["sparse_frac"] = setting["sparse_frac"]
        for sf in (0.002, 0.02):
            if sf == setting["sparse_frac"]:
                continue
            alt = batch.tune_wave_rows(dg, queries, stream, candidates=(waves["wave_rows"],),
                                       setting=dict(setting, sparse_frac=sf, short_share=waves["short_share"]),
                                       short_shares=(waves["short_share"],), lanes=(waves["lanes"],))
            for r in alt["table"]:
                r["sparse_frac"] = sf
            table += alt["table"]
            if alt["ms"] < waves["ms"]:
                waves = dict(alt, sparse_frac=sf)
        waves["table"] = table
        if tc:
            cached = json.loads(Path(tc).read_text()) if Path(tc).exists() else {}
            cached[wkey] = waves
            Path(tc).write_text(json.dumps(cached, indent=1))
    setting["short_share"] = waves.get("short_share", setting["short_share"])
    setting["sparse_frac"] = waves.get("sparse_frac", setting["sparse_frac"])
    log(f"[rank {rank}] autotune {time.time() - t0:.1f}s: {setting} waves {waves}")
    bt = batch.Batch(dg, queries, waves["wave_rows"], stream, setting=setting, lanes=waves.get("lanes", 1))
    cg = bt.capture()
    for _ in range(args.warmup):
        bt.launch()
    counts = bt.counts()
    # bit-exact against running queries alone (a bounded subset)
    chk = sorted(range(nq), key=lambda i: len(queries[i].sources))[: bw["check"] // 2] + \
        list(range(nq))[: bw["check"] - bw["check"] // 2]
    solo = batch.solo_counts(dg, [queries[i] for i in chk], stream=stream)
    assert np.array_equal(counts[chk], solo), "batched counts differ from solo runs"
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local_rank)
    launches0 = vs.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")
    ev0.record(stream)
    for _ in range(args.steps):
        bt.launch()
    ev1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    launches = vs.kernel_launches() - launches0
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = world * nq * args.steps / (ms / 1e3)
    assert np.array_equal(bt.counts(), counts)
    # e2e: every step copies the batch's inputs (sources, limits, keys) from pinned
    # host memory into the batch's device buffers, replays the graph and reads the counts
    h_src, h_lim, h_keys = (bt.d_src.cpu().pin_memory(), bt.d_lim.cpu().pin_memory(),
                            bt.d_keys.cpu().pin_memory())
    h_cnt = torch.zeros_like(bt.d_counts, device="cpu").pin_memory()

    def step_e2e():
        bt.d_src.copy_(h_src, non_blocking=True)
        bt.d_lim.copy_(h_lim, non_blocking=True)
        bt.d_keys.copy_(h_keys, non_blocking=True)
        bt.launch()
        h_cnt.copy_(bt.d_counts, non_blocking=True)

    step_e2e()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step_e2e()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1)
    assert np.array_equal(h_cnt.numpy()[bt.slot].astype(np.uint64), counts)
    e2e = {"value": world * nq * args.steps / (ms_e2e / 1e3), "unit": "queries/s",
           "h2d_bytes_per_step": int(bt.h2d_bytes()), "d2h_bytes_per_step": int(8 * nq),
           "ms_per_step": ms_e2e / args.steps}
    kernels = cg.kernels
    bt.free()
    # learned picker: the same batch with the trained network choosing each hop
    learned = None
    if picker_train.WEIGHTS_FILE.exists():
        pk = vs.Picker()
        pk.set_params(np.load(picker_train.WEIGHTS_FILE))
        bl = batch.Batch(dg, queries, waves["wave_rows"], stream, setting=setting, picker=pk,
                         lanes=waves.get("lanes", 1))
        bl.capture()
        for _ in range(max(1, min(args.warmup, 3))):
            bl.launch()
        l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0.record(stream)
        for _ in range(args.steps):
            bl.launch()
        l1.record(stream)
        torch.cuda.synchronize()
        assert np.array_equal(bl.counts(), counts), "learned-picker counts differ"
        ms_l = l0.elapsed_time(l1) / args.steps
        learned = {"queries_per_s": world * nq / (ms_l / 1e3), "ms_per_step": ms_l}
        bl.free()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cpu = None
    parity = None
    if world == 1 and not args.no_cpu:
        sample, ccounts, dt = cpu_batched(g, w, queries, cpu_blocks(g))
        assert [int(counts[i]) for i in sample] == ccounts, "oracle counts differ from the batch"
        parity = {"queries": len(sample), "equal": True,
                  "against": "oracle VExpand(Shortest, [1,l]) + TableConvert + HashJoin count per query "
                             f"(queries {sample}); the batch also equals {len(chk)} solo GPU runs"}
        from oracle import pyoracle as O
        cpu = {"value": len(sample) / dt, "unit": "queries/s", "cores": O.lib().oracle_get_threads(),
               "kind": "port", "cpu_model": cpu_model(), "sample": f"{len(sample)} queries with <= 2048 sources, one at a time, {dt:.1f} s"}
    line = {"metric": "batched queries/s", "value": value, "unit": "queries/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded power-law graph, uniform sources and keys)",
            "config": batched_config(args, g, queries, world),
            "batch": {"wave_rows": waves["wave_rows"], "waves": len(bt.waves), "lanes": bt.lanes,
                      "graph_kernels": kernels},
            "queries_per_s": {"plain": value, "learned": learned["queries_per_s"] if learned else None},
            "learned_picker": learned, "autotune": {"planner": setting, "waves": waves},
            "results": {"count_sum": int(counts.sum()), "checked_against_solo": len(chk)},
            "roofline": None, "cpu_baseline": cpu, "parity": parity, "e2e": e2e, "gpu_launches": launches,
            "clocks": clk}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def join_inputs(w, n):
    from vertexsurge_gb300 import batch
    rng = np.random.default_rng(w["seed"] + n)
    perm = rng.permutation(w["V"]).astype(np.uint32)
    return (batch.zipf_keys(rng, n, w["V"], perm, w["skew"]), batch.zipf_keys(rng, n, w["V"], perm, w["skew"]))


def join_bytes(n_build, n_probe):
    """Algorithmic bytes of a count-only Flat x Flat join of 4-byte keys
    (the hash join's compulsory bytes, no output): both key columns read, the
    table cleared (16 B per slot: key and count, capacity the power of two
    >= 2 N_b, at least 64), one 16-byte insert per build row and at least one
    32-byte sector per probe."""
    cap = 64
    while cap < 2 * n_build:
        cap *= 2
    return 4 * n_build + 4 * n_probe + 16 * cap + 16 * n_build + 32 * n_probe


def run_join(args, w, rank, world, local_rank, reference=False):
    """Count-only Flat x Flat HashJoin of two key columns per size."""
    from oracle import pyoracle as O
    rows = []
    if reference:
        from vertexsurge_gb300 import build as b
        b.build_oracle()
        b.build_gen()
        n = w["cpu_rows"]
        ka, kb = join_inputs(w, n)
        ta, tb = O.Table(O.FLAT, [0, 1], cols=[ka, ka]), O.Table(O.FLAT, [2, 1], cols=[kb, kb])
        times = []
        for i in range(args.steps + 1):
            t = time.perf_counter()
            cnt = O.hash_join(ta, tb, 1, only_count=True)[2]
            if i:
                times.append(time.perf_counter() - t)
        value = 2 * n * args.steps / sum(times) / 1e6
        line = {"impl": "reference", "metric": "count-only hash join Mrows/s", "value": value, "unit": "Mrows/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": 1, "ms_per_step": 1000 * sum(times) / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                "data": "synthetic (Zipf-skewed vertex-id keys)",
                "config": {"workload": args.workload, "V": w["V"], "sizes": list(w["sizes"])},
                "cpu_baseline": {"value": value, "unit": "Mrows/s", "cores": O.lib().oracle_get_threads(),
                                 "kind": "port", "cpu_model": cpu_model(), "sample": f"HashJoin count of two {n}-row key columns"},
                "e2e": {"value": value, "unit": "Mrows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    import torch
    import vertexsurge_gb300 as vs
    from vertexsurge_gb300 import build as b
    b.build_all()
    torch.cuda.set_device(local_rank)
    vs.init(local_rank)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    peak, peak_kind = peaks()
    launches0 = vs.kernel_launches()
    total_ms = 0.0
    total_rows = 0
    clocks = ClockSampler(local_rank)
    for n in w["sizes"]:
        ka, kb = join_inputs(w, n)
        fa, fb = vs.FlatTable.from_columns([ka], stream), vs.FlatTable.from_columns([kb], stream)
        exp = None
        for _ in range(args.warmup):
            _, c, _ = vs.hash_join(fa, fb, 0, 0, only_count=True, stream=stream)
        # exact count: sum over keys of multiplicity_a * multiplicity_b
        ua, ca = np.unique(ka, return_counts=True)
        ub, cb = np.unique(kb, return_counts=True)
        _, ia, ib = np.intersect1d(ua, ub, assume_unique=True, return_indices=True)
        exp = int(np.sum(ca[ia].astype(np.int64) * cb[ib].astype(np.int64)))
        assert c == exp, (n, c, exp)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            vs.hash_join(fa, fb, 0, 0, only_count=True, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        byt = join_bytes(n, n)
        rows.append({"rows_per_side": n, "ms": ms, "Mrows_per_s": 2 * n / ms / 1e3, "count": c, "bytes": byt,
                     "GB_per_s": byt / ms / 1e6, "frac": byt / ms / 1e6 / peak})
        total_ms += ms
        total_rows += 2 * n
        fa.free()
        fb.free()
    clk = clocks.stop()
    big = rows[-1]
    line = {"metric": "count-only hash join Mrows/s", "value": total_rows / total_ms / 1e3, "unit": "Mrows/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (Zipf-skewed vertex-id keys)",
            "config": {"workload": args.workload, "V": w["V"], "sizes": list(w["sizes"])},
            "sizes": rows,
            "roofline": {"bound": "hbm", "achieved": big["GB_per_s"], "peak": peak, "unit": "GB/s",
                         "frac": big["frac"], "frac_nominal": big["GB_per_s"] / NOMINAL_HBM_GBS,
                         "traffic": None, "peak_source": peak_kind,
                         "bytes": "4 N_b + 4 N_p + 16 cap + 16 N_b + 32 N_p (largest size)"},
            "cpu_baseline": None, "parity": {"sizes": len(rows), "equal": True,
                                             "against": "numpy sum of multiplicity products per key"},
            "e2e": None, "gpu_launches": vs.kernel_launches() - launches0, "clocks": clk}
    print(json.dumps(line), flush=True)


def serving_oracle(g, trace, n):
    """The n queries of the trace with the fewest source-hops, each on the CPU:
    visited = the oracle's VExpand(Shortest, [1, l]) bit count; join = the
    count of HashJoin(A, key table) on the vertex id, i.e. the sum over key
    rows of the popcount of A's column for that key (numpy over the oracle's
    words); triangles = sum over the sources' edges a -> b of |N+(a) & N+(b)|
    (numpy over the sorted, duplicate-free lists)."""
    from oracle import pyoracle as O
    idx = sorted(range(len(trace)), key=lambda i: (len(trace[i].sources) * trace[i].k_max, i))[:n]
    out = []
    t = time.perf_counter()
    for i in idx:
        r = trace[i]
        words, _, _ = O.vexpand(g, r.sources, 1, r.k_max, "shortest", "forward")
        colcnt = np.bitwise_count(words).sum(axis=1, dtype=np.int64)
        del words
        tri = 0
        for a in r.sources:
            na = g.fwd_dst[g.fwd_off[a]:g.fwd_off[a + 1]]
            for b in na:
                nb = g.fwd_dst[g.fwd_off[b]:g.fwd_off[b + 1]]
                if len(nb):  # members of na in the sorted nb
                    tri += int(np.count_nonzero(nb[np.minimum(np.searchsorted(nb, na), len(nb) - 1)] == na))
        out.append((int(colcnt.sum()), int(colcnt[r.keys].sum()), tri))
    return idx, out, time.perf_counter() - t


def run_serving(args, w, rank, world, local_rank):
    """Config 5: the serving loop (vertexsurge_gb300.serve) replaying a Poisson
    trace under a byte budget, the fixed planner and the learned pickers on the
    same trace; latency = completion - arrival.  Every query's host inputs are
    copied in and its three counts read back inside the served interval."""
    from vertexsurge_gb300 import graphgen, picker_train, serve
    if args.impl == "reference":  # the oracle on the sample the GPU arm checks, one query at a time
        from vertexsurge_gb300 import build as b
        b.build_oracle()
        b.build_gen()
        g = graphgen.rmat(w["scale"], 16, 0.57, 0.19, 0.19, seed=27)
        trace = serve.make_trace(g, w["queries"], w["rate"], s_range=(64, w["s_max"]), l_max=w["l_max"])
        idx, _, dt = serving_oracle(g, trace, w["oracle_queries"])
        from oracle import pyoracle as O
        value = len(idx) / dt
        print(json.dumps({"impl": "reference", "metric": "served queries/s", "value": value, "unit": "queries/s",
                          "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": 1000 * dt,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
                          "data": "synthetic (seeded R-MAT graph, Poisson arrivals)",
                          "config": {"workload": args.workload, "V": g.V, "E": g.E},
                          "cpu_baseline": {"value": value, "unit": "queries/s", "cores": O.lib().oracle_get_threads(),
                                           "kind": "port", "cpu_model": cpu_model(), "sample": f"queries {idx} of the trace, one at a time"},
                          "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    import torch
    import vertexsurge_gb300 as vs
    from vertexsurge_gb300 import build as b
    b.build_all()
    torch.cuda.set_device(local_rank)
    vs.init(local_rank)
    t0 = time.time()
    g = graphgen.rmat(w["scale"], 16, 0.57, 0.19, 0.19, seed=27)
    log(f"graph {g.V} vertices {g.E} edges in {time.time() - t0:.1f}s")
    dg = vs.DeviceGraph.from_host(g)
    trace = serve.make_trace(g, w["queries"], w["rate"], s_range=(64, w["s_max"]), l_max=w["l_max"])
    budget = int(w["budget_gb"] * (1 << 30))
    pickers = {"plain": None}
    if picker_train.WEIGHTS_FILE.exists():
        pk = vs.Picker()
        pk.set_params(np.load(picker_train.WEIGHTS_FILE))
        pickers["learned"] = pk
    # warm-up: the first queries alone (kernels loaded, hub indexes built)
    solo_srv = serve.Server(dg, budget_bytes=1 << 62, slots=1)
    wstream = torch.cuda.Stream()
    for r in trace[: max(3, args.warmup)]:
        solo_srv.run_query(r, wstream)
    torch.cuda.synchronize()
    launches0 = vs.kernel_launches()
    clocks = ClockSampler(local_rank)
    reports, results = {}, {}
    for name, pk in pickers.items():
        for r in trace:
            r.result = ()
        reports[name] = serve.Server(dg, budget, slots=w["slots"], picker=pk).serve(trace)
        results[name] = [r.result for r in trace]
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = vs.kernel_launches() - launches0
    solo = serve.solo_results(dg, trace[: w["check"]])
    same_mix = all(results["plain"][i] == solo[i] for i in range(len(solo)))
    same_picker = all(res == results["plain"] for res in results.values())
    assert same_mix and same_picker, "served answers differ alone / in the mix / under the picker"
    parity = None
    if rank == 0 and not args.no_cpu:
        idx, want, dt = serving_oracle(g, trace, w["oracle_queries"])
        got = [results["plain"][i] for i in idx]
        parity = {"queries": len(idx), "equal": got == want,
                  "against": f"queries {idx}: oracle VExpand bit count, numpy join and triangle counts",
                  "oracle_s": dt}
        if got != want:
            print(json.dumps({"parity": parity, "got": got, "want": want}), flush=True)
            raise SystemExit("parity: served counts differ from the oracle's")
    rep = reports["plain"]
    h2d = sum(r.sources.nbytes + r.keys.nbytes + r.payload.nbytes for r in trace)
    line = {"metric": "served queries/s", "value": rep["queries_per_s"], "unit": "queries/s", "n_gpus": world,
            "steps": 1, "warmup": max(3, args.warmup), "ms_per_step": 1000 * rep["wall_s"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded R-MAT graph a=0.57, Poisson arrivals, Zipf join keys)",
            "config": {"workload": args.workload, "V": g.V, "E": g.E, "queries": w["queries"],
                       "rate_qps": w["rate"], "budget_gb": w["budget_gb"], "slots": w["slots"],
                       "s_range": [64, w["s_max"]], "l_max": w["l_max"], "l2": "inputs larger than L2",
                       "parallelism": f"replicas{world}"},
            "latency": {name: {k: rep_[k] for k in ("p50_ms", "p99_ms", "service_p50_ms", "queries_per_s",
                                                    "peak_bytes", "peak_concurrent")}
                        for name, rep_ in reports.items()},
            "queries_per_s": {name: rep_["queries_per_s"] for name, rep_ in reports.items()},
            "check": {"same_alone_and_in_mix": same_mix, "queries": len(solo), "same_under_picker": same_picker},
            "roofline": None, "cpu_baseline": None, "parity": parity,
            "e2e": {"value": rep["queries_per_s"], "unit": "queries/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 3 * 8 * len(trace)},
            "gpu_launches": launches, "clocks": clk}
    if rank == 0:  # every rank serves its own replica of the trace; rank 0 reports
        print(json.dumps(line), flush=True)


def run_reference(args, w, rank, world):
    """--impl reference: the oracle (CPU restatement of the reference) on host cores."""
    if rank != 0:
        return
    from vertexsurge_gb300 import build as b
    b.build_gen()
    b.build_oracle()
    if "batched" in w:
        return run_reference_batched(args, w)
    from oracle import pyoracle as O
    t0 = time.time()
    g = make_graph(w)
    sa, _ = sources(g, w)
    log(f"graph {g.V} vertices {g.E} edges in {time.time() - t0:.1f}s")
    S = w["cpu_S"]
    src = sa[:S]
    k0, k1 = w["hops_a"]
    blk = cpu_blocks(g)
    _, _, st = O.vexpand(g, src, k0, k1, "shortest", "forward", want_matrix=False, hop_stats=True, blocks=blk)
    src_edges = S * sum(st["active_edges"][1:])
    for _ in range(min(args.warmup, 1)):
        O.vexpand(g, src, k0, k1, "shortest", "forward", want_matrix=False, blocks=blk)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        O.vexpand(g, src, k0, k1, "shortest", "forward", want_matrix=False, blocks=blk)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = src_edges * args.steps / total / 1e9
    cores = O.lib().oracle_get_threads()
    sample = (f"VExpand(Shortest, [{k0},{k1}], Forward) from {S} of the A sources on the full graph "
              f"per step ({src_edges / 1e9:.2f} Gsrc-edges), the reference's BlockHilbert hop over "
              f"{CPU_BLOCKS} target blocks")
    line = {"impl": "reference", "metric": "multi-source expand Gsrc-edges/s", "value": value,
            "unit": "Gsrc-edges/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": min(args.warmup, 1),
            "ms_per_step": 1000 * total / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded power-law graph, uniform sources)",
            "config": pattern_config(args, g, w, args.gpus),
            "cpu_baseline": {"value": value, "unit": "Gsrc-edges/s", "cores": cores, "kind": "port", "cpu_model": cpu_model(),
                             "sample": sample},
            "e2e": {"value": value, "unit": "Gsrc-edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args, w, rank, world, local_rank):
    import torch
    import vertexsurge_gb300 as vs
    from vertexsurge_gb300 import build as b
    b.build_all()
    torch.cuda.set_device(local_rank)
    vs.init(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    t0 = time.time()
    g = make_graph(w)
    sa, sb = sources(g, w)
    log(f"[rank {rank}] graph {g.V} vertices {g.E} edges in {time.time() - t0:.1f}s")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dg = vs.DeviceGraph.from_host(g, stream=stream)
    ka, kb = w["hops_a"], w["hops_b"]
    Sa, Sb = len(sa), len(sb)
    # autotuned PULL kernel shape, SPARSE threshold and hub bin per expand (untimed)
    from vertexsurge_gb300 import autotune
    t0 = time.time()
    tc = args.tune_cache or None
    tA = autotune.tune(dg, sa, ka[0], ka[1], "shortest", "forward", stream=stream, cache_file=tc)
    if args.expand_a:
        tA = dict(tA, **json.loads(args.expand_a))
    tB = autotune.tune(dg, sb, kb[0], kb[1], "shortest", "forward", stream=stream, cache_file=tc)
    tP = autotune.tune(dg, sa, 1, 1, "any", "forward", stream=stream, cache_file=tc)
    tuned = {k: {x: t.get(x, 0.0) for x in ("pull_kind", "sparse_frac", "hub_threshold", "slice_words",
                                           "short_share", "ms")}
             for k, t in (("A", tA), ("B", tB), ("P", tP))}
    log(f"[rank {rank}] autotune {time.time() - t0:.1f}s: {tuned}")
    for name, t in (("A", tA), ("B", tB), ("P", tP)):
        for row in sorted(t["table"], key=lambda r: r["ms"])[:6]:
            log(f"[rank {rank}]   tune {name}: {row}")
    pA = autotune.make_plan(dg, Sa, ka[0], ka[1], "shortest", "forward", tA)
    pB = autotune.make_plan(dg, Sb, kb[0], kb[1], "shortest", "forward", tB)
    pP = autotune.make_plan(dg, Sa, 1, 1, "any", "forward", tP)
    dA = torch.from_numpy(sa.view(np.int32)).to("cuda")
    dB = torch.from_numpy(sb.view(np.int32)).to("cuda")
    adj = [dict(graph=dg, direction="forward", base_col=0), dict(graph=dg, direction="forward", base_col=1)]

    def step(timing=False):
        pA.run(dA, stream=stream)
        pB.run(dB, stream=stream)
        A, B = pA.result(), pB.result()
        _, jc, _ = vs.hash_join(A, B, 1, 1, only_count=True, stream=stream)
        pP.run(dA, stream=stream)
        _, tc, _ = vs.mintersect(pP.result(), adj, g.V, only_count=True, stream=stream)
        return jc, tc

    # exact E_active of every hop (stats pass, untimed)
    for p in (pA, pB, pP):
        p.set_tuning(collect_stats=True)
    jc, tc = step()
    stA, stB, stP = pA.stats(stream), pB.stats(stream), pP.stats(stream)
    src_edges = (Sa * sum(stA["active_edges"][1:]) + Sb * sum(stB["active_edges"][1:])
                 + Sa * sum(stP["active_edges"][1:]))
    log(f"[rank {rank}] A hops {stA['hops_run']} strat {stA['strategy'][1:]} e_act {stA['active_edges'][1:]}")
    log(f"[rank {rank}] B strat {stB['strategy'][1:]} e_act {stB['active_edges'][1:]} join={jc} tri={tc}")
    for p in (pA, pB, pP):
        p.set_tuning(collect_stats=False)
    pA.set_tuning(timing=True)  # per-hop CUDA events around the dominant pull kernel
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local_rank)
    launches0 = vs.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pull_ms, pull_comp, pull_launches = 0.0, 0.0, 0
    pull_hop_ms = {}
    W = (Sa + 63) // 64
    W += W & 1
    torch.cuda.nvtx.range_push("timed")
    ev0.record(stream)
    for _ in range(args.steps):
        step()
        st = pA.stats(stream)
        for h in range(1, st["hops_run"] + 1):
            if st["strategy"][h] == vs.STRAT_PULL:
                pull_ms += st["pull_ms"][h]
                pull_hop_ms[h] = pull_hop_ms.get(h, 0.0) + st["pull_ms"][h]
                pull_launches += 1
                # compulsory bytes of the hop: CSR offsets, the
                # active in-list entries and P = 4 passes over the V x S
                # matrices (frontier read, next layer write, visited read + write)
                pull_comp += expand_bytes(g.V, W, stA["active_edges"][h], True, False, gathers=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    launches = vs.kernel_launches() - launches0
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = world * src_edges * args.steps / (ms / 1e3) / 1e9

    # expand A alone with each short-mode kernel (the next target's visited
    # words and flag loaded ahead, and not: pull kernel bit 2), per-hop
    # CUDA-event times of the PULL hops
    short_kernels = None
    if any(stA["short_pull"][1:]):
        short_kernels = {}
        kind0 = int(tA.get("pull_kind", 0))
        for name, kind in (("preload", kind0 & 3), ("no_preload", (kind0 & 3) | 4)):
            pA.set_pull_kernel(kind)
            per_hop = {}
            for _ in range(3):
                pA.run(dA, stream=stream)
            for _ in range(5):
                pA.run(dA, stream=stream)
                sth = pA.stats(stream)
                for h in range(1, sth["hops_run"] + 1):
                    if sth["strategy"][h] == vs.STRAT_PULL:
                        per_hop[str(h)] = per_hop.get(str(h), 0.0) + sth["pull_ms"][h] / 5
            short_kernels[name] = per_hop
        pA.set_pull_kernel(kind0)
        pA.run(dA, stream=stream)  # the result the parity check reads comes from the tuned kernel

    # e2e: one-shot C-ABI calls, sources from pinned host memory, counts read back
    pA.set_tuning(timing=False)
    hA = torch.from_numpy(sa.view(np.int32)).pin_memory()
    hB = torch.from_numpy(sb.view(np.int32)).pin_memory()

    def step_e2e():
        A, _, _ = vs.expand(dg, hA, ka[0], ka[1], "shortest", "forward", stream=stream, **autotune.params_kw(tA))
        B, _, _ = vs.expand(dg, hB, kb[0], kb[1], "shortest", "forward", stream=stream, **autotune.params_kw(tB))
        _, jc2, _ = vs.hash_join(A, B, 1, 1, only_count=True, stream=stream)
        A.free()
        B.free()
        P, _, _ = vs.expand(dg, hA, 1, 1, "any", "forward", stream=stream, **autotune.params_kw(tP))
        _, tc2, _ = vs.mintersect(P, adj, g.V, only_count=True, stream=stream)
        P.free()
        return jc2, tc2

    for _ in range(max(1, min(args.warmup, 3))):
        step_e2e()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        jc2, tc2 = step_e2e()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1)
    assert (jc2, tc2) == (jc, tc), "e2e results differ from the plan path"
    e2e = {"value": world * src_edges * args.steps / (ms_e2e / 1e3) / 1e9, "unit": "Gsrc-edges/s",
           "h2d_bytes_per_step": int(4 * (2 * Sa + Sb)), "d2h_bytes_per_step": 16,
           "ms_per_step": ms_e2e / args.steps}

    # learned picker: the same query with the trained network choosing each hop
    learned = None
    from vertexsurge_gb300 import picker_train
    if picker_train.WEIGHTS_FILE.exists():
        pk = vs.Picker()
        pk.set_params(np.load(picker_train.WEIGHTS_FILE))
        lp = [autotune.make_plan(dg, n, k0, k1, path, "forward", t, use_picker=True)
              for n, (k0, k1), path, t in ((Sa, ka, "shortest", tA), (Sb, kb, "shortest", tB),
                                           (Sa, (1, 1), "any", tP))]
        for p in lp:
            p.set_picker(pk)
        # the intersection's membership method, chosen by its own trained network
        from vertexsurge_gb300 import isect_train
        ipk = None
        if isect_train.WEIGHTS_FILE.exists():
            ipk = vs.Picker()
            ipk.set_params(np.load(isect_train.WEIGHTS_FILE))

        def step_learned():
            lp[0].run(dA, stream=stream)
            lp[1].run(dB, stream=stream)
            _, jc3, _ = vs.hash_join(lp[0].result(), lp[1].result(), 1, 1, only_count=True, stream=stream)
            lp[2].run(dA, stream=stream)
            _, tc3, _ = vs.mintersect(lp[2].result(), adj, g.V, only_count=True, stream=stream, method_picker=ipk)
            return jc3, tc3

        for _ in range(max(1, min(args.warmup, 3))):
            step_learned()
        torch.cuda.synchronize()
        l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("learned")
        l0.record(stream)
        for _ in range(args.steps):
            jc3, tc3 = step_learned()
        l1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        assert (jc3, tc3) == (jc, tc), "learned-picker results differ from the fixed planner"
        ms_l = l0.elapsed_time(l1) / args.steps
        learned = {"queries_per_s": 1000.0 / ms_l, "ms_per_step": ms_l,
                   "value": world * src_edges / (ms_l / 1e3) / 1e9,
                   "strategies_a": lp[0].stats(stream)["strategy"][1:]}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak, peak_kind = peaks()
    achieved = pull_comp / (pull_ms / 1e3) / 1e9 if pull_ms else None
    short_hops = [h for h in range(1, len(stA["short_pull"])) if stA["short_pull"][h]]
    rl_kernel = "k_pull_short" if short_hops else "k_pull"
    traffic = profiled_traffic(args.workload, rl_kernel)
    per_launch_ms = pull_ms / max(1, pull_launches)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved else None,
                "frac_nominal": achieved / NOMINAL_HBM_GBS if achieved else None,
                "bytes": "compulsory bytes per PULL hop, 8(V+1) + 4 E_act + 4 * 8W V (CSR offsets, active "
                         "in-list entries, frontier read, next-layer write, visited read + write), E_act exact "
                         "from the stats pass",
                "bytes_per_launch": pull_comp / max(1, pull_launches),
                "traffic": traffic,
                "dram_frac": (traffic / (per_launch_ms / 1e3) / 1e9) / peak if traffic and per_launch_ms else None,
                "traffic_source": (f"profiles/{rl_kernel}_{args.workload}.md (ncu dram__bytes_read.sum + "
                                   "dram__bytes_write.sum per working launch)") if traffic else
                                  ("not captured at this size (a DRAM-counter capture of a full-size launch holds "
                                   "too much device memory); the 1M-vertex instance's layers are several times "
                                   "denser per row, so its traffic does not scale to these hops by units processed"),
                "kernel": (f"{rl_kernel} (expand A, PULL hops {sorted(pull_hop_ms)}, short mode on "
                           f"{ {h: ('words', 'slots')[stA['short_pull'][h] - 1] for h in short_hops} })"),
                "peak_source": peak_kind,
                "per_launch_ms": per_launch_ms,
                "per_hop_ms": {str(h): t / args.steps for h, t in sorted(pull_hop_ms.items())}}
    cpu = None
    parity = None
    if world == 1 and not args.no_cpu:
        cpu, ow = cpu_baseline(g, w, sa)
        # the oracle's sample (the first cpu_S A sources) against the same rows
        # of the GPU's A result from the timed plan: rows are independent BFSs,
        # so the sample's matrix is words [0, cpu_S/64) of every GPU column
        gw = pA.result().download(stream)
        nw = ow.shape[1]
        equal = bool(np.array_equal(gw[:, :nw], ow))
        parity = {"rows": int(w["cpu_S"]), "equal": equal,
                  "against": f"oracle VExpand(Shortest, {list(ka)}, Forward) from the first {w['cpu_S']} A "
                             "sources, whole bit matrix (rows x V) compared bit for bit"}
        del gw
        if not equal:
            raise SystemExit("parity: the GPU's A rows differ from the oracle's")
    line = {"metric": "multi-source expand Gsrc-edges/s", "value": value, "unit": "Gsrc-edges/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded power-law graph, uniform sources)",
            "config": pattern_config(args, g, w, world),
            "queries_per_s": {"plain": 1000.0 / ms_per_step,
                              "learned": learned["queries_per_s"] if learned else None},
            "learned_picker": learned, "autotune": tuned,
            "results": {"join_count": jc, "triangles": tc, "visited_a": stA["visit_count"],
                        "hops_run_a": stA["hops_run"], "strategies_a": stA["strategy"][1:],
                        "src_edges_per_step": src_edges},
            "roofline": roofline, "cpu_baseline": cpu, "parity": parity, "e2e": e2e, "gpu_launches": launches,
            "clocks": clk, "short_kernels_ms": short_kernels}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="zipf10M_pattern")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--tune-cache", default="", help="JSON file of autotuner results (read if present, "
                    "written otherwise)")
    ap.add_argument("--expand-a", default="", help="JSON object overriding tuned knobs of expand A "
                    "(pull_kind, sparse_frac, hub_threshold, slice_words, short_share), e.g. for profiling")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    w = WORKLOADS[args.workload]
    if w.get("kind") == "join":
        if rank == 0 or args.impl != "reference":
            run_join(args, w, rank, world, local_rank, reference=args.impl == "reference")
    elif w.get("kind") == "serving":
        if rank == 0 or args.impl != "reference":
            run_serving(args, w, rank, world, local_rank)
    elif args.impl == "reference":
        run_reference(args, w, rank, world)
    elif "batched" in w:
        run_gpu_batched(args, w, rank, world, local_rank)
    else:
        run_gpu(args, w, rank, world, local_rank)


if __name__ == "__main__":
    main()
