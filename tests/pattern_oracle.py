"""Oracle side of the pattern query (test infrastructure only).

The pattern query of the benchmark, evaluated on the CPU:
  A = VExpand(sources_a, Shortest, [ka0, ka1], Forward)
  B = VExpand(sources_b, Shortest, [kb0, kb1], Forward)
  J = HashJoin(A, B) on the vertex id, count only: the reference's plan
      converts both results to ColMain (TableConvert, big_operators2.cpp:28-86)
      and joins the matrices (join.cpp:406-430), which counts
      sum_v popc(A column v) * popc(B column v)
  T = Mintersect(Any [1,1] from sources_a; out-list of a, out-list of b):
      sum over edges a -> b with a a source of |N+(a) & N+(b)|
The expands and the join run through the oracle restatement.  The oracle's
Mintersect scans flat dependencies linearly per base tuple
(mintersect.cpp:149-165), which is quadratic at these sizes, so the triangle
count is computed by an independent sparse-matrix product instead.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from oracle import pyoracle as O


def expand(g, src, k0, k1, path="shortest"):
    words, _, st = O.vexpand(g, src, k0, k1, path, "forward", hop_stats=True)
    return words, st


def join_count(g, wa, sa, wb, sb) -> int:
    """HashJoin(A, B) on the vertex column, count only, through the oracle."""
    A_, B_, K = 1, 2, 3
    ca = O.table_convert(wa, len(sa), g.V, False)
    cb = O.table_convert(wb, len(sb), g.V, False)
    ta = O.Table(O.COLMAIN, [A_, K], words=ca, mrows=len(sa), mcols=g.V, row_map=sa)
    tb = O.Table(O.COLMAIN, [B_, K], words=cb, mrows=len(sb), mcols=g.V, row_map=sb)
    return O.hash_join(ta, tb, K, only_count=True)[2]


def triangle_count(g, sa) -> int:
    """sum over edges a -> b (a in sa) of |N+(a) & N+(b)| (scipy, independent)."""
    V = g.V
    rows = np.repeat(np.arange(V, dtype=np.int64), np.diff(g.fwd_off))
    A = sp.csr_matrix((np.ones(g.E, dtype=np.int64), (rows, g.fwd_dst.astype(np.int64))), shape=(V, V))
    M = A[np.asarray(sa, dtype=np.int64)]
    X = M @ A.T
    return int(M.multiply(X).sum())


def pattern(g, sa, sb, ka, kb):
    """(A words, A stats, B words, B stats, join count, triangle count)."""
    wa, sta = expand(g, sa, *ka)
    wb, stb = expand(g, sb, *kb)
    return wa, sta, wb, stb, join_count(g, wa, sa, wb, sb), triangle_count(g, sa)
