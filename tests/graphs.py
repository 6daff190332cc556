"""Small test graphs and an independent reachability reference (scipy),
used to pin the expand oracle, which no reference test pins."""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
from scipy.sparse.csgraph import shortest_path

from vertexsurge_gb300 import graphgen


def adjacency(g, direction: str) -> sp.csr_matrix:
    """Boolean adjacency A[u, v] = 1 when one expand step moves u -> v."""
    V = g.V
    rows = np.repeat(np.arange(V, dtype=np.int64), np.diff(g.fwd_off))
    A = sp.csr_matrix((np.ones(g.E, dtype=np.int8), (rows, g.fwd_dst.astype(np.int64))), shape=(V, V))
    if not g.directed or direction == "forward":
        return A
    if direction == "backward":
        return A.T.tocsr()
    return ((A + A.T) > 0).astype(np.int8).tocsr()


def reach_any(g, sources, k_min, k_max, direction="forward") -> np.ndarray:
    """R[i, v] = exists a walk of length in [k_min, k_max] from sources[i] to v."""
    A = adjacency(g, direction).astype(np.float32)
    S = len(sources)
    cur = sp.csr_matrix((np.ones(S, np.float32), (np.arange(S), np.asarray(sources, np.int64))),
                        shape=(S, g.V))
    R = np.zeros((S, g.V), dtype=bool)
    if k_min == 0:
        R |= cur.toarray() > 0
    for h in range(1, k_max + 1):
        cur = (cur @ A)
        cur.data[:] = 1
        cur.eliminate_zeros()
        if h >= k_min:
            R |= cur.toarray() > 0
    return R


def bfs_dist(g, sources, direction="forward") -> np.ndarray:
    A = adjacency(g, direction)
    d = shortest_path(A, unweighted=True, directed=True, indices=np.asarray(sources, np.int64))
    return d


def reach_shortest(g, sources, k_min, k_max, direction="forward") -> np.ndarray:
    d = bfs_dist(g, sources, direction)
    return (d >= k_min) & (d <= k_max)


def find_shortest(g, sources, targets, cap=50, direction="forward") -> np.ndarray:
    d = bfs_dist(g, sources, direction)
    out = d[np.arange(len(sources)), np.asarray(targets, np.int64)]
    return np.where(np.isfinite(out) & (out <= cap), out, -1).astype(np.int32)


def small_graphs():
    """A spread of small cleaned graphs (directed and undirected, skewed and flat)."""
    return {
        "rmat10": graphgen.rmat(10, 16, 0.57, 0.19, 0.19, seed=11),
        "rmat11_skew": graphgen.rmat(11, 8, 0.65, 0.15, 0.15, seed=12),
        "rmat9_undirected": graphgen.rmat(9, 8, 0.57, 0.19, 0.19, seed=13, undirected=True),
        "zipf3000": graphgen.zipf(3000, 60000, 2.1, 2000, seed=14),
    }
