"""VQL queries end to end on the GPU: a graph directory in the reference's
layout with a Person.community property, queries parsed and built into the
reference's plan shape (scans, VExpand + MatrixTableSelect, Mintersect) by
the C++ front end, results against brute-force evaluation of the pattern."""
import subprocess

import numpy as np
import pytest

from tests import graphs as G
from vertexsurge_gb300 import build, graph_dir, graphgen

pytestmark = pytest.mark.gpu


def undirected(g):
    src = np.repeat(np.arange(g.V, dtype=np.uint32), np.diff(g.fwd_off))
    s = np.concatenate([src, g.fwd_dst])
    d = np.concatenate([g.fwd_dst, src])
    keep = s != d
    key = np.unique(s[keep].astype(np.uint64) << np.uint64(32) | d[keep].astype(np.uint64))
    s, d = (key >> np.uint64(32)).astype(np.uint32), (key & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    off = np.zeros(g.V + 1, np.int64)
    np.add.at(off, s.astype(np.int64) + 1, 1)
    off = np.cumsum(off)
    return graphgen.HostGraph(g.V, len(d), off, d, off, d, directed=False)


@pytest.fixture(scope="module")
def gdir(tmp_path_factory):
    g = undirected(graphgen.rmat(9, 8, seed=21))
    tag = np.random.default_rng(4).integers(0, 4, g.V).astype(np.uint8)
    d = tmp_path_factory.mktemp("vqlgraph")
    graph_dir.save(d, g, properties={"community": tag})
    return d, g, tag


def run(d, q):
    r = subprocess.run([str(build.OPS_TEST), "--vql", str(d), q], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.split("\n")
    if lines[0].startswith("count"):
        return int(lines[0].split()[1])
    return sorted(tuple(int(x) for x in ln.split()[1:]) for ln in lines[1:] if ln.startswith("r:"))


def walks(g, k0, k1):
    A = G.adjacency(g, "forward").astype(bool).toarray()
    R, P = np.zeros_like(A), np.eye(g.V, dtype=bool)
    for h in range(1, k1 + 1):
        P = (P.astype(np.int32) @ A.astype(np.int32)) > 0
        if h >= k0:
            R |= P
    return R


def test_two_vertex_any(gdir):
    d, g, tag = gdir
    got = run(d, "vmatch (a{tag:1-1})-[1..2]-(b{tag:2-2}) return a, b;")
    R = walks(g, 1, 2)
    A, B = np.nonzero(tag == 1)[0], np.nonzero(tag == 2)[0]
    exp = sorted((int(a), int(b)) for a in A for b in B if R[a, b])
    assert got == exp and len(exp) > 0


def test_two_vertex_shortest_count(gdir):
    d, g, tag = gdir
    got = run(d, "vmatch (a{tag:0-1})-[2..3]s-(b{tag:3-3}) return count of a, b;")
    A, B = np.nonzero(tag <= 1)[0], np.nonzero(tag == 3)[0]
    D = G.bfs_dist(g, A, "forward")
    assert got == int(((D[:, B] >= 2) & (D[:, B] <= 3)).sum()) > 0


def test_triangle_query(gdir):
    d, g, tag = gdir
    A1 = G.adjacency(g, "forward").astype(bool).toarray()
    for q, mult in (("vmatch (a{tag:1-1})-(b{tag:2-2})-(c)-(a) return count of a, b, c;", 1),
                    ("vmatch (a{tag:1-2})-(b)-(c{tag:0-0}), (c)-(a) return count of a, b, c;", 1)):
        got = run(d, q)
        ta = (tag == 1) if "a{tag:1-1}" in q else (tag >= 1) & (tag <= 2)
        tb = (tag == 2) if "b{tag:2-2}" in q else np.ones(g.V, bool)
        tc = (tag == 0) if "c{tag:0-0}" in q else np.ones(g.V, bool)
        M = A1.astype(np.int64)
        T = (M * tb[None, :]) @ (M * tc[None, :])  # T[a, c] = sum_b M[a,b] tb[b] M[b,c] tc[c]
        exp = int((ta[:, None] * T * M.T).sum())
        assert got == exp * mult > 0, q


def test_triangle_tuples(gdir):
    d, g, tag = gdir
    got = run(d, "vmatch (a{tag:3-3})-(b)-(c{tag:1-1})-(a) return a, b, c;")
    A1 = G.adjacency(g, "forward").astype(bool).toarray()
    exp = sorted((int(a), int(b), int(c)) for a in np.nonzero(tag == 3)[0] for b in range(g.V)
                 if A1[a, b] for c in np.nonzero(tag == 1)[0] if A1[b, c] and A1[c, a])
    assert got == exp and len(exp) > 0
