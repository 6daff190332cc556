"""The small plain-method configuration end to end on the GPU against the
oracle: a directed R-MAT graph at scale 16 (65,536 vertices, average
out-degree 16, a=0.57 b=0.19 c=0.19, self-loops and duplicate edges removed),
512 uniformly sampled sources, hop range [1,3]: the 65,536 x 512 reachability
bit matrix bit-exact, its population count, and the self-ring count (sources
that reach themselves in 1..3 hops)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import words_to_bool
from vertexsurge_gb300 import graphgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rmat16(vs):
    g = graphgen.rmat(16, 16, 0.57, 0.19, 0.19, seed=1)
    return g, vs.DeviceGraph.from_host(g)


@pytest.mark.parametrize("path", ["any", "shortest"])
def test_rmat16_512_sources_hops_1_3(vs, rmat16, path):
    g, dg = rmat16
    assert g.V == 65536 and 0.9e6 < g.E <= 16 * 65536
    src = graphgen.sample_sources(g.V, 512, seed=2)
    m, _, _ = vs.expand(dg, src, 1, 3, path, "forward")
    got = m.download()
    exp, _, _ = O.vexpand(g, src, 1, 3, path, "forward")
    assert np.array_equal(got, exp)
    assert m.count() == O.matrix_count(exp, len(src), g.V)
    R = words_to_bool(got, len(src))
    ring = int(R[np.arange(len(src)), src].sum())
    Ro = words_to_bool(exp, len(src))
    assert ring == int(Ro[np.arange(len(src)), src].sum())
    # the ring count through MatrixTableSelect on the sources (S x S) and its diagonal
    sel = m.select(src)
    d = words_to_bool(sel.download(), len(src))
    assert int(d[np.arange(len(src)), np.arange(len(src))].sum()) == ring
    m.free()


def test_rmat16_e1_self_ring_count(vs, rmat16):
    """e1-style count: Count(MatrixTableSelect(VExpand(S, Both, Shortest, [0,3]), T=S))
    = #{(a, b) in S x S : dist(a, b) <= 3}, a = b included."""
    g, dg = rmat16
    src = graphgen.sample_sources(g.V, 512, seed=2)
    m, _, _ = vs.expand(dg, src, 0, 3, "shortest", "both")
    sel = m.select(src)
    got = sel.count()
    exp_w, _, _ = O.vexpand(g, src, 0, 3, "shortest", "both")
    exp = O.matrix_count(O.matrix_select(exp_w, len(src), g.V, src), len(src), len(src))
    assert got == exp >= len(src)
    sel.free()
    m.free()
