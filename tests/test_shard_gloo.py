"""Source sharding over ranks (world size 2, gloo, CPU): the sharded pattern
query gives the unsharded counts, and gathered expand matrices equal the full
matrix, including ranks that get no source word.  The per-rank engine is the
oracle, so no GPU is needed; the GPU engine offers the same calls."""
import json
import os
import socket

import numpy as np
import pytest

from vertexsurge_gb300 import shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir, cases):
    import torch.distributed as dist
    from tests import graphs as G
    from tests.shard_oracle_engine import OracleEngine
    from vertexsurge_gb300 import graphgen
    from vertexsurge_gb300 import shard as sh
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    g = G.small_graphs()["rmat10"]
    eng = OracleEngine(g)
    res = {}
    for name, Sa, Sb in cases:
        sa = graphgen.sample_sources(g.V, Sa, seed=11)
        sb = graphgen.sample_sources(g.V, Sb, seed=12)
        r = sh.sharded_pattern(eng, sa, sb, (1, 3), (1, 2), rank, world)
        full = sh.gather_expand(eng, sa, 1, 3, "any", "forward", rank, world)
        res[name] = {"counts": [r["visited_a"], r["join_count"], r["triangles"]], "rows": list(r["rows"]),
                     "full_sum": int(np.bitwise_count(full).sum()), "full_shape": list(full.shape),
                     "full_hash": int(np.bitwise_xor.reduce(full.ravel() * np.uint64(0x9E3779B97F4A7C15)
                                                            + np.arange(full.size, dtype=np.uint64)))}
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)
    dist.barrier()
    dist.destroy_process_group()


CASES = [("even", 256, 100), ("ragged", 150, 70), ("one_word", 40, 30)]


def test_shard_ranges_cover_sources_once():
    for S in (1, 40, 63, 64, 65, 150, 4096, 4097):
        for world in (1, 2, 3, 8):
            rs = [shard.shard_range(S, world, r) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == S
            for (a, b), (c, d) in zip(rs, rs[1:]):
                assert b == c and a <= b
            assert all(lo % 64 == 0 for lo, hi in rs if hi > lo)


def test_sharded_pattern_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    from oracle import pyoracle as O
    from tests import graphs as G
    from tests.shard_oracle_engine import OracleEngine
    from vertexsurge_gb300 import graphgen
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path), CASES), nprocs=2, join=True,
                       start_method="spawn")
    r0 = json.loads((tmp_path / "rank0.json").read_text())
    r1 = json.loads((tmp_path / "rank1.json").read_text())
    g = G.small_graphs()["rmat10"]
    eng = OracleEngine(g)
    for name, Sa, Sb in CASES:
        sa = graphgen.sample_sources(g.V, Sa, seed=11)
        sb = graphgen.sample_sources(g.V, Sb, seed=12)
        one = shard.sharded_pattern(eng, sa, sb, (1, 3), (1, 2), 0, 1)
        exp = [one["visited_a"], one["join_count"], one["triangles"]]
        assert r0[name]["counts"] == exp == r1[name]["counts"], name
        assert r0[name]["rows"][1] == r1[name]["rows"][0]
        w, _, _ = O.vexpand(g, sa, 1, 3, "any", "forward")
        assert r0[name]["full_shape"] == list(w.shape) == r1[name]["full_shape"]
        assert r0[name]["full_sum"] == int(np.bitwise_count(w).sum()) == r1[name]["full_sum"]
        h = int(np.bitwise_xor.reduce(w.ravel() * np.uint64(0x9E3779B97F4A7C15)
                                      + np.arange(w.size, dtype=np.uint64)))
        assert r0[name]["full_hash"] == h == r1[name]["full_hash"], name
