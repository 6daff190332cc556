"""An engine for the sharding logic built on the oracle (CPU), so the
multi-rank path runs as gloo ranks without a GPU.  Test infrastructure only."""
import numpy as np

from oracle import pyoracle as O


class _Mat:
    def __init__(self, words, sources):
        self.words, self.sources = words, np.ascontiguousarray(sources, np.uint32)


class OracleEngine:
    def __init__(self, g):
        self.g = g

    def expand(self, sources, k_min, k_max, path, direction):
        w, _, _ = O.vexpand(self.g, sources, k_min, k_max, path, direction)
        return _Mat(w, sources)

    def count(self, m):
        return O.matrix_count(m.words, len(m.sources), self.g.V)

    def join_count(self, a, b):
        ta = O.Table(O.COLMAIN, [0, 1], words=a.words, mrows=len(a.sources), mcols=self.g.V,
                     row_map=a.sources)
        tb = O.Table(O.COLMAIN, [2, 1], words=b.words, mrows=len(b.sources), mcols=self.g.V,
                     row_map=b.sources)
        return O.hash_join(ta, tb, 1, only_count=True)[2]

    def triangles(self, p):
        g = self.g
        base = O.Table(O.VARROW, [0, 1], words=p.words, mrows=len(p.sources), mcols=g.V, row_map=p.sources)
        src = np.repeat(np.arange(g.V, dtype=np.uint32), np.diff(g.fwd_off))
        e1 = O.Table(O.FLAT, [0, 2], cols=[src, g.fwd_dst])
        e2 = O.Table(O.FLAT, [1, 2], cols=[src, g.fwd_dst])
        return O.mintersect(base, [e1, e2], 2, g.V, only_count=True)[2]

    def words(self, m):
        return m.words

    def free(self, m):
        pass
