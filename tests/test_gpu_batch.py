"""Batched queries (many expand + join queries in one CUDA-graph launch):
row-block join counts against numpy on the downloaded matrix, and every
query's count in the batch against the same query run alone through the
one-query operators (VExpand + HashJoin)."""
import numpy as np
import pytest

from tests.conftest import words_to_bool
from tests import graphs as G
from vertexsurge_gb300 import graphgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graphs(vs):
    hg = G.small_graphs()
    return {k: (g, vs.DeviceGraph.from_host(g)) for k, g in hg.items()}


def test_row_block_counts_match_numpy(vs, graphs):
    import torch
    g, dg = graphs["zipf3000"]
    S = 333
    src = graphgen.sample_sources(g.V, S, seed=41)
    m, _, _ = vs.expand(dg, src, 1, 3, "shortest", "forward")
    bits = words_to_bool(m.download(), S)  # S x V
    rng = np.random.default_rng(5)
    # unaligned, empty, one-row and full blocks; keys with ids >= V (no match)
    blocks_rows = [(0, 1), (3, 70), (70, 200), (130, 130), (64, 128), (200, 333), (0, 333)]
    keys, blocks = [], []
    k0 = 0
    for r0, r1 in blocks_rows:
        k = rng.integers(0, g.V + 50, int(rng.integers(0, 3000)), dtype=np.uint32)
        keys.append(k)
        blocks.append((r0, r1, k0, k0 + len(k)))
        k0 += len(k)
    allk = np.concatenate(keys)
    dk = torch.from_numpy(allk.view(np.int32)).cuda()
    cnt = torch.full((len(blocks),), -1, dtype=torch.int64, device="cuda")
    vs.join_count_row_blocks(m, dk, blocks, cnt)
    got = cnt.cpu().numpy()
    colsum = lambda r0, r1: bits[r0:r1].sum(axis=0)  # noqa: E731
    for q, ((r0, r1), k) in enumerate(zip(blocks_rows, keys)):
        cs = colsum(r0, r1)
        kk = k[k < g.V]
        assert got[q] == int(cs[kk].sum()), (q, r0, r1)
    # the same counts through the one-query HashJoin on a matrix of those rows alone
    for q, ((r0, r1), k) in enumerate(zip(blocks_rows, keys)):
        if r1 - r0 == 0 or len(k) == 0:
            continue
        a, _, _ = vs.expand(dg, src[r0:r1], 1, 3, "shortest", "forward")
        kt = vs.FlatTable.from_columns([k])
        _, c, _ = vs.hash_join(kt, a, 0, 1, only_count=True)
        assert c == got[q], q
        kt.free()
        a.free()
    m.free()


def test_row_block_counts_reject_bad_blocks(vs, graphs):
    import torch
    g, dg = graphs["zipf3000"]
    m, _, _ = vs.expand(dg, graphgen.sample_sources(g.V, 64, seed=1), 1, 2, "shortest", "forward")
    dk = torch.zeros(10, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    with pytest.raises(vs.VsError):
        vs.join_count_row_blocks(m, dk, [(0, 65, 0, 10)], cnt)  # rows past the matrix
    with pytest.raises(vs.VsError):
        vs.join_count_row_blocks(m, dk.cpu(), [(0, 64, 0, 10)], cnt)  # host keys
    m.free()


@pytest.mark.parametrize("wave_rows,lanes", [(256, 1), (400, 1), (256, 3)])
def test_batch_counts_equal_solo(vs, graphs, wave_rows, lanes):
    """Every query's count in the batch (eager and replayed as one graph,
    waves on one or several concurrent lanes) equals the query run alone, and
    a few equal the oracle's VExpand + TableConvert + HashJoin count."""
    import torch
    from oracle import pyoracle as O
    from vertexsurge_gb300 import batch
    g, dg = graphs["rmat11_skew"]
    qs = batch.make_queries(g, 14, s_range=(3, 250), l_range=(1, 4), join_rows=(10, 4000), seed=3)
    solo = batch.solo_counts(dg, qs)
    for i in (0, 5, 13):
        q = qs[i]
        words, _, _ = O.vexpand(g, q.sources, 1, q.k_max, "shortest", "forward")
        cm = O.table_convert(words, len(q.sources), g.V, False)
        a = O.Table(O.COLMAIN, [0, 1], words=cm, mrows=len(q.sources), mcols=g.V, row_map=q.sources)
        k = O.Table(O.FLAT, [1], cols=[q.keys])
        assert O.hash_join(k, a, 1, only_count=True)[2] == solo[i], i
    stream = torch.cuda.Stream()
    b = batch.Batch(dg, qs, wave_rows, stream, lanes=lanes)
    assert b.lanes == min(lanes, len(b.waves))
    assert len(b.waves) >= 2, [len(q.sources) for q in qs]
    b.run_eager()
    assert np.array_equal(b.counts(), solo)
    b.d_counts.zero_()
    cg = b.capture()
    assert cg.kernels > 0
    for _ in range(2):
        b.d_counts.fill_(-1)
        b.launch()
        assert np.array_equal(b.counts(), solo)
    b.free()


def test_source_sharding_local_counts_sum_to_whole(vs, graphs):
    """Per-rank shares of the pattern query, computed one rank after another
    on this GPU (independent launches), sum to the unsharded counts, which
    equal the oracle engine's."""
    from tests.shard_oracle_engine import OracleEngine
    from vertexsurge_gb300 import shard
    g, dg = graphs["zipf3000"]
    eng = shard.GpuEngine(dg, g.V)
    sa = graphgen.sample_sources(g.V, 300, seed=21)
    sb = graphgen.sample_sources(g.V, 120, seed=22)
    whole = shard.local_counts(eng, sa, sb, (1, 3), (1, 2), 0, 1)
    assert whole == shard.local_counts(OracleEngine(g), sa, sb, (1, 3), (1, 2), 0, 1)
    for world in (2, 3, 8):
        parts = [shard.local_counts(eng, sa, sb, (1, 3), (1, 2), r, world) for r in range(world)]
        assert [sum(x) for x in zip(*parts)] == whole, world
