"""Serving loop: continuous batching under a byte budget, queries overlapping
on separate streams, and every answer identical alone and in the mix (exact
integer counts, so the tolerance is zero) and, for the first queries, equal to
the oracle's."""
import numpy as np
import pytest

from vertexsurge_gb300 import graphgen

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix(vs):
    from vertexsurge_gb300 import serve
    g = graphgen.rmat(14, 16, seed=3)
    dg = vs.DeviceGraph.from_host(g)
    trace = serve.make_trace(g, 24, rate_qps=1e6, s_range=(16, 700), l_max=5, join_rows=(100, 5000), seed=9)
    solo = serve.solo_results(dg, trace)
    srv0 = serve.Server(dg, budget_bytes=1 << 62, slots=1)
    budget = 3 * max(srv0.footprint(r) for r in trace)
    srv = serve.Server(dg, budget_bytes=budget, slots=6)
    rep = srv.serve(trace)
    assert [r.result for r in trace] == solo
    # and the first queries against the oracle: visited count, join count, triangles
    from oracle import pyoracle as O
    from tests import pattern_oracle as P
    for r in trace[:3]:
        words, _, _ = O.vexpand(g, r.sources, 1, r.k_max, "shortest", "forward")
        visited = O.matrix_count(words, len(r.sources), g.V)
        cm = O.table_convert(words, len(r.sources), g.V, False)
        a = O.Table(O.COLMAIN, [0, 1], words=cm, mrows=len(r.sources), mcols=g.V, row_map=r.sources)
        k = O.Table(O.FLAT, [2, 1], cols=[r.payload, r.keys])
        jc = O.hash_join(k, a, 1, only_count=True)[2]
        assert r.result == (visited, jc, P.triangle_count(g, r.sources)), r.result
    assert rep["peak_bytes"] <= budget
    assert rep["peak_concurrent"] >= 2          # work of several queries was in flight together
    assert rep["queries"] == 24 and rep["p99_ms"] >= rep["p50_ms"] > 0


def test_admission_rejects_a_query_above_the_budget(vs):
    from vertexsurge_gb300 import serve
    g = graphgen.rmat(12, 8, seed=4)
    dg = vs.DeviceGraph.from_host(g)
    trace = serve.make_trace(g, 2, rate_qps=1e6, s_range=(500, 600), seed=2)
    srv = serve.Server(dg, budget_bytes=1024, slots=2)
    with pytest.raises(ValueError):
        srv.serve(trace)
