"""The reference's on-disk graph directory (schema.json + DiskArray files):
file names, the DiskArray header, and a save/load round trip (host only)."""
import json

import numpy as np
import pytest

from tests import graphs as G
from vertexsurge_gb300 import graph_dir


def test_csr_file_names_follow_the_reference():
    # EdgeSchema::get_*_csr_*_name (meta/schema.cpp:36-66)
    d = graph_dir.csr_names("Account", "transfer", "Account", True)
    assert d == {"fwd_data": "Account-transfer->Account_csr_src_dst",
                 "fwd_index": "Account-transfer->Account_csr_src_dst_index",
                 "bwd_data": "Account<-transfer-Account_csr_dst_src",
                 "bwd_index": "Account<-transfer-Account_csr_dst_src_index"}
    u = graph_dir.csr_names("Person", "knows", "Person", False)
    assert u == {"fwd_data": "Person-knows-Person_csr_src_dst",
                 "fwd_index": "Person-knows-Person_csr_src_dst_index"}


def test_disk_array_header_and_round_trip(tmp_path):
    a = np.arange(1000, dtype=np.int64) * 3
    graph_dir.write_disk_array(tmp_path / "x", a)
    raw = (tmp_path / "x").read_bytes()
    assert len(raw) == 64 + 8000
    assert np.frombuffer(raw[:16], np.int64).tolist() == [1000, 8]
    assert np.array_equal(graph_dir.read_disk_array(tmp_path / "x", np.int64), a)
    with pytest.raises(ValueError):
        graph_dir.read_disk_array(tmp_path / "x", np.uint32)  # element size mismatch
    # a file with spare capacity after the elements (as the reference's arrays grow)
    graph_dir.write_disk_array(tmp_path / "y", np.arange(10, dtype=np.uint32))
    with open(tmp_path / "y", "ab") as f:
        f.write(b"\0" * 4096)
    assert np.array_equal(graph_dir.read_disk_array(tmp_path / "y", np.uint32), np.arange(10))


@pytest.mark.parametrize("name", ["rmat10", "zipf3000"])
def test_graph_save_load_round_trip(tmp_path, name):
    g = G.small_graphs()[name]
    graph_dir.save(tmp_path, g)
    schema = json.loads((tmp_path / "schema.json").read_text())
    assert schema["vertex"][0]["statistics"]["count"] == g.V
    assert schema["edge"][0]["statistics"]["count"] == g.E
    h = graph_dir.load(tmp_path)["Person_knows_Person"]
    for f in ("fwd_off", "fwd_dst", "rev_off", "rev_src"):
        assert np.array_equal(getattr(h, f), getattr(g, f)), f
    assert (h.V, h.E, h.directed) == (g.V, g.E, g.directed)


def test_flat_edge_file_names_follow_the_reference():
    # EdgeSchema::get_flat_edges_name (meta/schema.cpp:69-97, orders :391-408)
    assert graph_dir.flat_edges_name("A", "t", "A", True, "forward", "hilbert") == "A-t->A_hilbert"
    assert graph_dir.flat_edges_name("A", "t", "A", True, "backward", "src_dst", 3) == "A<-t-A_src_dst_3"
    assert graph_dir.flat_edges_name("P", "k", "P", False, "forward", "dst_src", 0) == "P-k-P_dst_src_0"


def test_partition_by_dst_blocks():
    """graph_loader.hh:112-138: blocks of about n/count edges that end only
    where the target changes."""
    dst = np.array([0, 0, 0, 1, 1, 2, 3, 3, 3, 3, 4, 5], np.uint32)
    blocks = graph_dir.partition_by_dst(dst, 3)
    assert blocks == [(0, 5), (5, 10), (10, 12)]
    assert graph_dir.partition_by_dst(np.array([7, 7, 7], np.uint32), 2) == [(0, 3), (3, 3)]


def test_partition_by_dst_matches_the_edge_walk():
    """The block search (first target change at or after the expected end)
    equals walking the edges one by one as graph_loader.hh:112-138 does."""
    def walk(d, count):
        n, pos, out = len(d), 0, []
        for i in range(count):
            if pos >= n:
                out.append((n, n))
                continue
            expected = pos + (n - pos) // (count - i)
            end = pos + 1
            while end < n and not (end >= expected and d[end] != d[end - 1]):
                end += 1
            out.append((pos, end))
            pos = end
        return out
    rng = np.random.default_rng(3)
    for _ in range(500):
        n = int(rng.integers(0, 300))
        d = np.sort(rng.integers(0, int(rng.integers(1, 60)), n)).astype(np.uint32)
        c = int(rng.integers(1, 12))
        assert graph_dir.partition_by_dst(d, c) == walk(d, c)


@pytest.mark.parametrize("name", ["rmat10", "rmat9_undirected"])
def test_flat_edge_lists(tmp_path, name):
    """Every flat list holds the edge set (backward lists as (dst, src)), in
    its order; the partitioned blocks are target-disjoint and concatenate to
    the (dst, src)-sorted edges; a directory with flat lists only loads to the
    same CSR."""
    g = G.small_graphs()[name]
    graph_dir.save(tmp_path, g, flats=("hilbert", "src_dst", "dst_src", "random"),
                   partitioned={"hilbert": 5, "src_dst": 3})
    info = json.loads((tmp_path / "schema.json").read_text())["edge"][0]["store_info"]
    assert info == {"flats": ["hilbert", "src_dst", "dst_src", "random"], "partitioned_flats": ["hilbert", "src_dst"],
                    "partition_counts": [5, 3]}
    rows = np.repeat(np.arange(g.V, dtype=np.uint32), np.diff(g.fwd_off))
    fwd = set(zip(rows.tolist(), g.fwd_dst.tolist()))
    n = 1
    while n < g.V:
        n *= 2
    for direction in ["forward"] + (["backward"] if g.directed else []):
        for order in ("hilbert", "src_dst", "dst_src", "random"):
            p = graph_dir.read_flat_edges(tmp_path, "Person", "knows", "Person", g.directed, direction, order)
            s, d = (p[:, 0], p[:, 1]) if direction == "forward" else (p[:, 1], p[:, 0])
            assert len(p) == g.E and set(zip(s.tolist(), d.tolist())) == fwd, (direction, order)
            if order == "src_dst":
                assert np.all(np.diff(s.astype(np.int64) * g.V + d) > 0)
            if order == "dst_src":
                assert np.all(np.diff(d.astype(np.int64) * g.V + s) > 0)
            if order == "hilbert":
                assert np.all(np.diff(graph_dir.curve_index(n, s, d).astype(np.int64)) > 0)
        for order, count in (("hilbert", 5), ("src_dst", 3)):
            parts = []
            for i in range(count):
                name_i = graph_dir.flat_edges_name("Person", "knows", "Person", g.directed, direction, order, i)
                q = np.asarray(graph_dir.read_disk_array(tmp_path / name_i, np.uint64)).view(np.uint32).reshape(-1, 2)
                parts.append(q if direction == "forward" else q[:, ::-1])
            dsts = [set(q[:, 1].tolist()) for q in parts]
            assert all(not (dsts[i] & dsts[j]) for i in range(count) for j in range(i + 1, count))
            assert sum(len(q) for q in parts) == g.E
            assert [min(x) for x in dsts if x] == sorted(min(x) for x in dsts if x)
    # flat lists only: load rebuilds the CSR
    flat_only = tmp_path / "flat_only"
    graph_dir.save(flat_only, g, csr=False, partitioned={"hilbert": 4})
    h = graph_dir.load(flat_only)["Person_knows_Person"]
    for f in ("fwd_off", "fwd_dst", "rev_off", "rev_src"):
        assert np.array_equal(getattr(h, f), getattr(g, f)), f
