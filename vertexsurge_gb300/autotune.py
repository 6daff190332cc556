"""Autotuner for expand plans.

For one query shape (graph, source count, hop range, path type, direction) it
times the expand under candidate settings and keeps the fastest:
  * the PULL kernel shape (vs_expand_plan_set_pull_kernel: occupancy bound and
    L2 cache policies),
  * the SPARSE threshold of the fixed planner (pair-list edge work below this
    fraction of E runs as SPARSE),
  * the hub degree bin (in-degree above which a vertex gets a whole CTA),
  * the source-word group width (words per PULL pass) for very wide rows,
  * whether PULL hops over sparse frontier rows gather the rows' source lists.
Timing uses CUDA events around whole plan runs on the plan's stream; every
candidate gives the same result, so only time decides.  Results are cached
per shape in memory and, when a path is given, in a JSON file.
"""
from __future__ import annotations

import json
import statistics
from pathlib import Path

from . import _abi as vs

_CACHE: dict = {}


def _key(dg, S, k_min, k_max, path, direction):
    # source counts in power-of-two buckets share a setting
    b = 1 << max(0, (int(S) - 1).bit_length())
    return f"V{dg.V}-E{dg.E}-d{int(dg.directed)}|S{b}|{k_min}-{k_max}|{path}|{direction}"


def _time_runs(plan, src, repeats, stream):
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(repeats)]
    plan.run(src, stream=stream)  # warm
    for a, b in ev:
        a.record(stream)
        plan.run(src, stream=stream)
        b.record(stream)
    torch.cuda.synchronize()
    return statistics.median(a.elapsed_time(b) for a, b in ev)


def tune(dg, src, k_min, k_max, path="shortest", direction="forward", stream=None, repeats=3,
         pull_kinds=(0, 1, 2, 3), sparse_fracs=(0.0005, 0.002, 0.005, 0.02), hub_thresholds=(0, 256),
         slice_words=(0,), short_shares=(0.0, -1.0), cache_file: str | None = None) -> dict:
    """Time the candidates; returns {'pull_kind', 'sparse_frac', 'hub_threshold', 'slice_words',
    'short_share', 'ms', 'table'} and caches it."""
    import torch
    key = _key(dg, len(src), k_min, k_max, path, direction)
    if key in _CACHE:
        return _CACHE[key]
    if cache_file and Path(cache_file).exists():
        disk = json.loads(Path(cache_file).read_text())
        if key in disk:
            _CACHE[key] = disk[key]
            return disk[key]
    stream = stream or torch.cuda.current_stream()
    dsrc = torch.from_numpy(src.view("int32")).to("cuda") if hasattr(src, "view") else src
    table = []
    for hub in hub_thresholds:
        for sw in slice_words:
            for rb in short_shares:
                plan = vs.ExpandPlan(dg, len(src), vs.make_params(k_min, k_max, path, direction,
                                                                  hub_threshold=hub, slice_words=sw,
                                                                  short_share=rb))
                try:
                    for pk in pull_kinds:
                        plan.set_pull_kernel(pk)
                        for sf in sparse_fracs:
                            plan.set_tuning(sparse_frac=sf)
                            ms = _time_runs(plan, dsrc, repeats, stream)
                            table.append({"pull_kind": pk, "sparse_frac": sf, "hub_threshold": hub,
                                          "slice_words": sw, "short_share": rb, "ms": ms})
                finally:
                    plan.free()
    best = min(table, key=lambda r: r["ms"])
    out = dict(best)
    out["table"] = table
    _CACHE[key] = out
    if cache_file:
        disk = json.loads(Path(cache_file).read_text()) if Path(cache_file).exists() else {}
        disk[key] = out
        Path(cache_file).write_text(json.dumps(disk, indent=1))
    return out


def apply(plan, setting: dict):
    """Apply the runtime knobs of a tuned setting to a plan created with its
    hub_threshold and slice_words."""
    plan.set_pull_kernel(setting["pull_kind"])
    plan.set_tuning(sparse_frac=setting["sparse_frac"])


def params_kw(setting: dict | None) -> dict:
    """Keyword arguments of make_params / expand for a tuned setting."""
    s = setting or {}
    return {"hub_threshold": s.get("hub_threshold", 0), "slice_words": s.get("slice_words", 0),
            "pull_kernel": s.get("pull_kind", 0), "sparse_frac": s.get("sparse_frac", 0.0),
            "short_share": s.get("short_share", 0.0)}


def make_plan(dg, S, k_min, k_max, path, direction, setting: dict | None, **kw):
    """An expand plan built with a tuned setting (or the defaults)."""
    return vs.ExpandPlan(dg, S, vs.make_params(k_min, k_max, path, direction, **params_kw(setting), **kw))
