"""Source sharding of the pattern query over ranks, one GPU per rank.

The S sources of a VExpand are S independent BFSs (one bit per source in
every row), so with the graph replicated on every GPU, rank r of G expands
only its slice of the sources and no data moves between ranks while the hops
run.  Slices are whole 64-source words: rank r takes words
[r*W/G, (r+1)*W/G) of the W = ceil(S/64) words, so the ranks' result
matrices, side by side, are the full result word for word.

The pattern query shards by the sources of its first expand A; the second
expand B is small and replicated.  Every count of the query is then a sum of
per-rank counts:
  |A|          = sum_r |A_r|
  |A join B|   = sum_v popc(A col v) * popc(B col v) = sum_r |A_r join B|
  triangles    = sum over base pairs (a, b) of P, and P's rows are A's sources
so the only exchange is one all-reduce of a few int64 counts at the end (or a
gather of the matrices when the caller wants them).  The engine is the
library's GPU path; it is passed in so the sharding logic can be exercised
with any engine that offers the same calls.
"""
from __future__ import annotations

import numpy as np


def shard_range(S: int, world: int, rank: int, align: int = 64) -> tuple:
    """[lo, hi) of the sources rank `rank` expands (multiples of `align`
    except at S); some ranks get none when there are fewer words than ranks."""
    words = (S + align - 1) // align
    w0, w1 = words * rank // world, words * (rank + 1) // world
    return min(S, w0 * align), min(S, w1 * align)


class GpuEngine:
    """The library's operators on this rank's GPU."""

    def __init__(self, dg, graph_V: int, adj=None, stream=None):
        from . import _abi as vs
        self.vs, self.dg, self.V, self.stream = vs, dg, graph_V, stream
        self.adj = adj or [dict(graph=dg, direction="forward", base_col=0),
                           dict(graph=dg, direction="forward", base_col=1)]

    def expand(self, sources, k_min, k_max, path, direction):
        m, _, _ = self.vs.expand(self.dg, np.ascontiguousarray(sources, np.uint32), k_min, k_max, path,
                                 direction, stream=self.stream)
        return m

    def count(self, m) -> int:
        return int(m.count(stream=self.stream))

    def join_count(self, a, b) -> int:
        return int(self.vs.hash_join(a, b, 1, 1, only_count=True, stream=self.stream)[1])

    def triangles(self, p) -> int:
        return int(self.vs.mintersect(p, self.adj, self.V, only_count=True, stream=self.stream)[1])

    def words(self, m) -> np.ndarray:
        return m.download(self.stream)

    def free(self, m):
        m.free()


def _allreduce_sum(vals, group=None):
    import torch
    import torch.distributed as dist
    backend = dist.get_backend(group)
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.tensor(vals, dtype=torch.int64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return [int(x) for x in t.cpu().tolist()]


def local_counts(engine, sa, sb, hops_a, hops_b, rank: int, world: int, triangles: bool = True) -> list:
    """This rank's share [|A_r|, |A_r join B|, triangles of P_r] of the pattern
    query (A's and P's sources sharded, B replicated)."""
    lo, hi = shard_range(len(sa), world, rank)
    local = [0, 0, 0]
    if hi <= lo:
        return local
    B = engine.expand(sb, hops_b[0], hops_b[1], "shortest", "forward")
    A = engine.expand(sa[lo:hi], hops_a[0], hops_a[1], "shortest", "forward")
    local[0] = engine.count(A)
    local[1] = engine.join_count(A, B)
    engine.free(A)
    engine.free(B)
    if triangles:
        P = engine.expand(sa[lo:hi], 1, 1, "any", "forward")
        local[2] = engine.triangles(P)
        engine.free(P)
    return local


def sharded_pattern(engine, sa, sb, hops_a, hops_b, rank: int, world: int, group=None,
                    triangles: bool = True) -> dict:
    """The pattern query with A's (and P's) sources sharded over the ranks and
    B replicated; every rank returns the global counts (one all-reduce)."""
    local = local_counts(engine, sa, sb, hops_a, hops_b, rank, world, triangles)
    tot = _allreduce_sum(local, group) if world > 1 else local
    return {"visited_a": tot[0], "join_count": tot[1], "triangles": tot[2] if triangles else None,
            "rows": shard_range(len(sa), world, rank)}


def gather_expand(engine, sources, k_min, k_max, path, direction, rank: int, world: int,
                  group=None) -> np.ndarray:
    """A sharded expand whose logical words (V, ceil(S/64)) are gathered on every rank."""
    import torch.distributed as dist
    lo, hi = shard_range(len(sources), world, rank)
    if hi > lo:
        m = engine.expand(sources[lo:hi], k_min, k_max, path, direction)
        w = engine.words(m)
        engine.free(m)
    else:
        w = None
    parts = [None] * world
    if world > 1:
        dist.all_gather_object(parts, w, group=group)
    else:
        parts = [w]
    parts = [p for p in parts if p is not None]
    full = np.concatenate(parts, axis=1) if parts else np.zeros((0, 0), np.uint64)
    return full[:, : (len(sources) + 63) // 64]
