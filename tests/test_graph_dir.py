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
