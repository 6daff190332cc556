"""The bench's JSON line (CPU only): the reference arm runs the CPU
restatement of the path on the small R-MAT pattern and prints one line with
every key of the contract; without a GPU the default arm is not run."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config"}


def test_reference_arm_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload",
                          "rmat16_pattern", "--steps", "1", "--warmup", "1"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert KEYS <= set(d) and d["impl"] == "reference"
    assert d["metric"] == "multi-source expand Gsrc-edges/s" and d["unit"] == "Gsrc-edges/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["config"]["workload"] == "rmat16_pattern"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert "BlockHilbert" in cb["sample"] and cb["cpu_model"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_serving_oracle_counts():
    """The serving workload's CPU check (bench.serving_oracle): its visited
    count, its numpy join count (sum of the key columns' popcounts) and its
    triangle count over sorted lists equal the oracle's VExpand count, the
    oracle's HashJoin through TableConvert, and an independent sparse-matrix
    triangle count, on a small trace."""
    sys.path.insert(0, str(ROOT))
    import bench
    from oracle import pyoracle as O
    from tests import pattern_oracle as P
    from vertexsurge_gb300 import graphgen, serve
    g = graphgen.rmat(12, 16, seed=3)
    trace = serve.make_trace(g, 6, 1e6, s_range=(16, 200), l_max=4, join_rows=(100, 2000), seed=9)
    idx, out, _ = bench.serving_oracle(g, trace, 3)
    assert len(idx) == 3 and idx == sorted(range(6), key=lambda i: (len(trace[i].sources) * trace[i].k_max, i))[:3]
    for i, got in zip(idx, out):
        r = trace[i]
        words, _, _ = O.vexpand(g, r.sources, 1, r.k_max, "shortest", "forward")
        cm = O.table_convert(words, len(r.sources), g.V, False)
        a = O.Table(O.COLMAIN, [0, 1], words=cm, mrows=len(r.sources), mcols=g.V, row_map=r.sources)
        k = O.Table(O.FLAT, [2, 1], cols=[r.payload, r.keys])
        want = (O.matrix_count(words, len(r.sources), g.V), O.hash_join(k, a, 1, only_count=True)[2],
                P.triangle_count(g, r.sources))
        assert got == want and got[1] > 0 and got[2] > 0


def test_batched_cpu_leg_counts():
    """The batched workload's CPU leg (bench.cpu_batched, the BlockHilbert hop
    over the bench's block layout) gives, per query, the join count of the
    CSR-pull oracle and of numpy (sum of the key columns' popcounts)."""
    import numpy as np
    sys.path.insert(0, str(ROOT))
    import bench
    from oracle import pyoracle as O
    from vertexsurge_gb300 import batch, graphgen
    g = graphgen.zipf(5000, 60000, 2.1, 2000, seed=14)
    queries = batch.make_queries(g, 5, (16, 300), (2, 5), (50, 5000), seed=4)
    idx, counts, dt = bench.cpu_batched(g, {"batched": {"cpu_queries": 4}}, queries, bench.cpu_blocks(g))
    assert idx == [0, 1, 2, 3] and dt > 0
    for i, got in zip(idx, counts):
        q = queries[i]
        words, _, _ = O.vexpand(g, q.sources, 1, q.k_max, "shortest", "forward")
        colcnt = np.bitwise_count(words).sum(axis=1, dtype=np.int64)
        assert got == int(colcnt[q.keys].sum()) and got > 0


def test_cpu_baseline_leg():
    """The default workload's CPU leg (bench.cpu_baseline) on a small graph:
    its matrix is the oracle's VExpand of the sample, and its record carries
    the keys of the line's cpu_baseline."""
    import numpy as np
    sys.path.insert(0, str(ROOT))
    import bench
    from oracle import pyoracle as O
    from vertexsurge_gb300 import graphgen
    g = graphgen.zipf(4000, 50000, 2.1, 1000, seed=14)
    sa = graphgen.sample_sources(g.V, 300, seed=2)
    w = {"cpu_S": 128, "hops_a": (1, 4)}
    rec, words = bench.cpu_baseline(g, w, sa)
    want, _, _ = O.vexpand(g, sa[:128], 1, 4, "shortest", "forward")
    assert np.array_equal(words, want)
    assert rec["value"] > 0 and rec["unit"] == "Gsrc-edges/s" and rec["kind"] == "port"
    assert rec["cores"] >= 1 and rec["cpu_model"] and "BlockHilbert" in rec["sample"]
