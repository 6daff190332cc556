"""The C++ operator layer (VExpand, HashJoin, Mintersect, TableConvert,
MatrixTableSelect, Count over the C ABI) runs the reference's own unit-test
cases and three query-plan shapes on the GPU (vertexsurge_gb300/cpp/vs_ops_test.cpp)."""
import subprocess

import numpy as np
import pytest

from vertexsurge_gb300 import build

pytestmark = pytest.mark.gpu


def test_cpp_operator_suite():
    r = subprocess.run([str(build.OPS_TEST)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    print(r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout


def _undirected(g):
    from vertexsurge_gb300 import graphgen
    src = np.repeat(np.arange(g.V, dtype=np.uint32), np.diff(g.fwd_off))
    s = np.concatenate([src, g.fwd_dst])
    d = np.concatenate([g.fwd_dst, src])
    key = np.unique(s.astype(np.uint64) << np.uint64(32) | d.astype(np.uint64))
    s, d = (key >> np.uint64(32)).astype(np.uint32), (key & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    off = np.zeros(g.V + 1, np.int64)
    np.add.at(off, s.astype(np.int64) + 1, 1)
    off = np.cumsum(off)
    return graphgen.HostGraph(g.V, len(d), off, d, off, d, directed=False)


@pytest.mark.parametrize("undirected", [False, True])
@pytest.mark.parametrize("layout", ["csr", "flat", "blocks", "imported"])
def test_graph_directory_through_cpp_loader(tmp_path, undirected, layout):
    """Graph(dir).load() reads the reference's directory layout (CSR files,
    or only a flat edge list, one file or target blocks, from which it builds
    the CSR, or what the social-network importer wrote from a SNAP edge list);
    the count of an expand over it equals the oracle's on the same arrays."""
    from oracle import pyoracle as O
    from tests import graphs as G
    from vertexsurge_gb300 import graph_dir, importer
    g = G.small_graphs()["rmat10"]
    if undirected:
        g = _undirected(g)
    if layout == "csr":
        graph_dir.save(tmp_path, g)
    elif layout == "flat":
        graph_dir.save(tmp_path, g, csr=False, flats=("random",))
    elif layout == "blocks":
        graph_dir.save(tmp_path, g, csr=False, partitioned={"hilbert": 6})
    else:  # the edges as a SNAP file with relabelled raw ids, imported (knows is undirected)
        rows = np.repeat(np.arange(g.V, dtype=np.uint64), np.diff(g.fwd_off))
        raw = lambda v: np.uint64(1_000_003) * (np.uint64(g.V) - np.asarray(v, np.uint64)) + np.uint64(7)
        importer.output_vlgpm(tmp_path, raw(rows), raw(g.fwd_dst))
        g = graph_dir.load(tmp_path)["Person_knows_Person"]
    r = subprocess.run([str(build.OPS_TEST), "--graph-dir", str(tmp_path)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = int(r.stdout.split("count")[1].split()[0])
    src = np.array([(i * 7) % g.V for i in range(min(g.V, 100))], np.uint32)
    w, _, _ = O.vexpand(g, src, 1, 3, "shortest", "forward")
    assert got == O.matrix_count(w, len(src), g.V) > 0
