"""The pattern query of the benchmark on a GPU-scale power-law graph against
the oracle, with the planner's own per-hop choices (no forced strategy, no
forced short mode): 1M vertices, ~30M edges (out-degree ~ Zipf(2.1) capped at
50k, uniform targets, uint32 CSR), the benchmark's query shape:
  A = VExpand(4,096 sources, Shortest, [1,4]),  B = VExpand(4,096, Shortest, [1,2]),
  A x B vertex-id join count, triangle count over out-lists.
Bit matrices are compared bit-exactly, counts exactly.  The test also asserts
that the planner took the paths the 10M-vertex benchmark takes: SPARSE hops
from the sources and short-mode PULL hops (the whole frontier is larger than
half of L2 here, so short mode is chosen by the real rule)."""
import numpy as np
import pytest

from tests import pattern_oracle as P
from vertexsurge_gb300 import graphgen

pytestmark = pytest.mark.gpu

STRAT_PULL, STRAT_SPARSE = 1, 3


@pytest.fixture(scope="module")
def zipf1m(vs):
    g = graphgen.zipf(1_000_000, 30_000_000, 2.1, 50_000, seed=3)
    sa = graphgen.sample_sources(g.V, 4096, seed=101)
    sb = graphgen.sample_sources(g.V, 4096, seed=102)
    return g, vs.DeviceGraph.from_host(g), sa, sb


@pytest.fixture(scope="module")
def oracle_pattern(zipf1m):
    g, _, sa, sb = zipf1m
    return P.pattern(g, sa, sb, (1, 4), (1, 2))


def test_pattern_query_matches_oracle(vs, zipf1m, oracle_pattern):
    g, dg, sa, sb = zipf1m
    wa, sta, wb, stb, jc, tc = oracle_pattern
    A, _, st_a = vs.expand(dg, sa, 1, 4, "shortest", "forward", stats=True)
    B, _, st_b = vs.expand(dg, sb, 1, 2, "shortest", "forward", stats=True)
    assert np.array_equal(A.download(), wa)
    assert np.array_equal(B.download(), wb)
    _, gj, _ = vs.hash_join(A, B, 1, 1, only_count=True)
    assert gj == jc > 0
    A.free()
    B.free()
    Pm, _, _ = vs.expand(dg, sa, 1, 1, "any", "forward")
    adj = [dict(graph=dg, direction="forward", base_col=0), dict(graph=dg, direction="forward", base_col=1)]
    _, gt, _ = vs.mintersect(Pm, adj, g.V, only_count=True)
    assert gt == tc > 0
    Pm.free()
    # the hop counts and E_active agree with the oracle's layer loop
    assert st_a["hops_run"] == sta["hops_run"] == 4
    assert st_a["active_edges"][1:5] == sta["active_edges"][1:5]
    # the planner's paths at this scale: SPARSE from the sources, then short-mode PULL
    assert st_a["strategy"][1] == STRAT_SPARSE
    short_hops = [h for h in range(1, 5) if st_a["short_pull"][h]]
    assert short_hops and all(st_a["strategy"][h] == STRAT_PULL for h in short_hops), st_a
    print("A strategies", st_a["strategy"][1:5], "short modes", st_a["short_pull"][1:5],
          "B strategies", st_b["strategy"][1:3])


def test_short_modes_at_scale_match_oracle(vs, zipf1m, oracle_pattern):
    """Short mode forced on every PULL hop (share above 1), with SPARSE hops
    at the planner's threshold and at a tenth of it, so that PULL hops follow
    both SPARSE and PULL layers: word mode (a frontier of mostly one-id rows)
    and slot mode (mostly 2..15-id rows) both run on the 1M-vertex graph, and
    the matrix is the oracle's bit for bit each time."""
    g, dg, sa, _ = zipf1m
    wa = oracle_pattern[0]
    seen = set()
    for sparse_frac in (0.02, 0.002):
        plan = vs.ExpandPlan(dg, len(sa), vs.make_params(1, 4, "shortest", "forward", short_share=2.0,
                                                         sparse_frac=sparse_frac))
        plan.set_tuning(collect_stats=True)
        plan.run(sa)
        st = plan.stats()
        assert np.array_equal(plan.result().download(), wa), (sparse_frac, st)
        seen |= {st["short_pull"][h] for h in range(1, 5) if st["strategy"][h] == STRAT_PULL}
        print("sparse_frac", sparse_frac, "strategies", st["strategy"][1:5], "short modes", st["short_pull"][1:5])
        plan.free()
    assert seen == {1, 2}, seen
