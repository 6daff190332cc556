"""The social-network importer (host only): a SNAP edge list into the
reference's graph directory, with the reference importer's numbering,
communities, reverse edges and neighbour-only de-duplication
(src/objects/meta/graph_loader.cpp:151-305, include/meta/graph_loader.hh:59-79)."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from vertexsurge_gb300 import graph_dir, importer

ROOT = Path(__file__).resolve().parent.parent

SNAP = """# a SNAP edge list
# FromNodeId ToNodeId
900 17
17 900
42 900
42 42
5000000000 17
900 42
42 900
"""


def expected_edges(lines):
    """The reference importer's edge list written out by hand: raw ids
    numbered in ascending order, the list then its reverse, equal neighbouring
    pairs dropped, then sorted by (src, dst)."""
    pairs = [tuple(int(x) for x in l.split()) for l in lines if l.strip() and not l.startswith("#")]
    ids = sorted({v for p in pairs for v in p})
    rank = {v: i for i, v in enumerate(ids)}
    e = [(rank[a], rank[b]) for a, b in pairs]
    e = e + [(b, a) for a, b in e]
    kept = [p for i, p in enumerate(e) if i == 0 or p != e[i - 1]]
    return ids, sorted(kept)


def csr_pairs(g):
    rows = np.repeat(np.arange(g.V), np.diff(g.fwd_off))
    return list(zip(rows.tolist(), np.asarray(g.fwd_dst).tolist()))


def test_snap_text_import(tmp_path):
    src = tmp_path / "edges.txt"
    src.write_text(SNAP)
    rs, rd = importer.load_snap_txt(src)
    g = importer.output_vlgpm(tmp_path / "db", rs, rd)
    ids, want = expected_edges(SNAP.splitlines())
    assert g.V == len(ids) == 4
    assert csr_pairs(g) == want
    # 42-900 occurs three times (twice as given, once reversed from 900 42), never
    # next to itself in the list: all three copies stay, as the reference keeps them
    assert want.count((1, 2)) == 3 and want.count((2, 1)) == 3
    assert want.count((1, 1)) == 2  # the self loop and its reverse copy
    d = tmp_path / "db"
    schema = json.loads((d / "schema.json").read_text())
    assert schema["graph_type"] == "Social Network"
    assert schema["vertex"][0]["statistics"]["count"] == 4
    e = schema["edge"][0]
    assert e["directed"] is False and e["statistics"]["count"] == len(want)
    assert e["store_info"]["flats"] == ["src_dst", "hilbert"] and e["store_info"]["partitioned_flats"] == []
    assert np.array_equal(graph_dir.read_disk_array(d / "Person.id", np.uint32), np.arange(4))
    assert np.array_equal(graph_dir.read_disk_array(d / "Person.community", np.uint8), importer.communities(4))
    h = graph_dir.load(d)["Person_knows_Person"]
    assert csr_pairs(h) == want
    for order in ("src_dst", "hilbert"):
        p = graph_dir.read_flat_edges(d, "Person", "knows", "Person", False, "forward", order)
        assert sorted(map(tuple, p.tolist())) == want, order


def test_communities_follow_the_reference_blocks():
    n = 30000
    c = importer.communities(n)
    counts = np.bincount(c, minlength=13)
    assert counts[:3].tolist() == [2048] * 3 and counts[3] == 20480 and counts[4] == n - 3 * 2048 - 20480
    assert counts[5:].sum() == 0
    assert np.array_equal(c, importer.communities(n))  # seeded
    assert not np.array_equal(c, np.sort(c))         # shuffled


def test_snap_csv_and_blocks(tmp_path):
    src = tmp_path / "edges.csv"
    src.write_text("node_1,node_2\n3,1\n1,2\n2,3\n3,1\n")
    rs, rd = importer.load_snap_csv(src)
    g = importer.output_vlgpm(tmp_path / "db", rs, rd, partitions=2)
    _, want = expected_edges(["3 1", "1 2", "2 3", "3 1"])
    assert csr_pairs(g) == want
    info = json.loads((tmp_path / "db" / "schema.json").read_text())["edge"][0]["store_info"]
    assert info["partitioned_flats"] == ["src_dst", "hilbert"] and info["partition_counts"] == [2, 2]
    bad = tmp_path / "bad.csv"
    bad.write_text("a,b\n1,2\n")
    with pytest.raises(ValueError):
        importer.load_snap_csv(bad)


def test_command_line(tmp_path):
    src = tmp_path / "edges.txt"
    src.write_text(SNAP)
    out = subprocess.run([sys.executable, "-m", "vertexsurge_gb300.importer", "-s", str(src), "-d",
                          str(tmp_path / "db"), "-i", "snap-txt"], capture_output=True, text=True, cwd=ROOT,
                         timeout=120)
    assert out.returncode == 0, out.stderr
    assert "4 Person" in out.stdout
    assert (tmp_path / "db" / "schema.json").exists()


def test_ldbc_interactive_and_bi(tmp_path):
    """LDBC inputs: the vertices are the person files' ids (an isolated person
    is a vertex), the knows files give the edges; an edge naming an unknown
    person is refused."""
    ic = tmp_path / "ic" / "social_network" / "dynamic"
    ic.mkdir(parents=True)
    (ic / "person_0_0.csv").write_text("id|firstName|lastName|place\n933|Ann|A|1\n4139|Bo|B|2\n10995|Cy|C|3\n77|Di|D|4\n")
    (ic / "person_knows_person_0_0.csv").write_text(
        "Person.id|Person.id|creationDate\n933|4139|2010\n933|10995|2011\n4139|10995|2012\n")
    persons, rs, rd = importer.load_ldbc_ic(tmp_path / "ic")
    g = importer.output_vlgpm(tmp_path / "db_ic", rs, rd, persons=persons)
    assert g.V == 4  # 77 has no edge but is a person
    ids = [77, 933, 4139, 10995]
    rank = {v: i for i, v in enumerate(ids)}
    e = [(rank[a], rank[b]) for a, b in [(933, 4139), (933, 10995), (4139, 10995)]]
    assert csr_pairs(g) == sorted(e + [(b, a) for a, b in e])
    bi = tmp_path / "bi" / "graphs" / "csv" / "bi" / "composite-merged-fk" / "initial_snapshot" / "dynamic"
    (bi / "Person").mkdir(parents=True)
    (bi / "Person_knows_Person").mkdir(parents=True)
    (bi / "Person" / "part-0.csv").write_text("creationDate|id|firstName|LocationCityId\n1|933|Ann|5\n2|4139|Bo|6\n")
    (bi / "Person" / "part-1.csv").write_text("creationDate|id|firstName|LocationCityId\n3|10995|Cy|7\n4|77|Di|8\n")
    (bi / "Person_knows_Person" / "part-0.csv").write_text(
        "creationDate|Person1Id|Person2Id\n1|933|4139\n2|933|10995\n")
    (bi / "Person_knows_Person" / "part-1.csv").write_text("creationDate|Person1Id|Person2Id\n3|4139|10995\n")
    persons, rs, rd = importer.load_ldbc_bi(tmp_path / "bi")
    g2 = importer.output_vlgpm(tmp_path / "db_bi", rs, rd, persons=persons)
    assert g2.V == 4 and csr_pairs(g2) == csr_pairs(g)
    with pytest.raises(ValueError):
        importer.rearrange(np.array([933], np.uint64), np.array([5], np.uint64), persons=persons)
    with pytest.raises(ValueError):
        importer.rearrange(rs, rd, persons=np.array([933, 933], np.uint64))
