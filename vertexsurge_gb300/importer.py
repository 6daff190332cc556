"""Importer: a social-network edge list (SNAP text or CSV) into the
reference's graph directory, as the reference's importer writes it for the
"sn" graph type (src/objects/importer.cpp:120-152; SocialNetworkImporter,
src/objects/meta/graph_loader.cpp:151-305), so the same input feeds both sides.

Steps, each as the reference takes it:
  * parse: SNAP text, one "src dst" pair of 64-bit raw ids per line, lines
    starting with '#' skipped (:151-186); SNAP CSV, a "node_1,node_2" header
    then one pair per line (:107-117,188-209); LDBC SNB interactive, '|'
    separated social_network/dynamic/person_0_0.csv (column "id") and
    person_knows_person_0_0.csv (the first two columns) (:44-69,93-105,
    138-149); LDBC SNB BI, every .csv of the initial snapshot's
    dynamic/Person (column "id") and dynamic/Person_knows_Person (columns
    Person1Id, Person2Id) (:17-42,71-91,121-136), files in name order (the
    reference takes them in directory order);
  * vertices: the distinct raw ids of the edge list (SNAP) or of the person
    files (LDBC, which must hold every edge endpoint and no id twice),
    numbered in ascending raw-id order (rearrange, :262-278;
    unify_vertex_and_collect_statistics, include/meta/graph_loader.hh:11-23);
  * communities: set_random_community (:229-260), through the host library's
    vsg_sn_communities (the standard library's mt19937 and shuffle);
  * edges: raw ids mapped to the new ids; knows is undirected, so every edge
    is appended reversed (add_reverse_edges, storage/graph_concepts.hh:100-107),
    then equal NEIGHBOURING pairs are dropped before the sort by (src, dst) —
    the reference runs std::unique on the unsorted list
    (deduplicate_edges, :109-112; unify_edge_and_collect_statistics,
    graph_loader.hh:59-79), so a pair repeated far apart stays repeated, and
    this importer keeps that multiset;
  * output: Person.id and Person.community DiskArrays, the src_dst CSR, the
    flat lists in src_dst and hilbert order (init_graph_schema, :211-227; with
    no block count the partitioned forms collapse into the single files),
    schema.json with graph_type "Social Network".
Not written: Person.name (random letters drawn in the reference's hash-set
order, not a value any operator of the path reads).  The reference's CSV path
collects the vertex set from edge fields that are not yet filled
(:197-200); here it is the raw ids, as in the text path.
"""
from __future__ import annotations

import argparse
from pathlib import Path

import numpy as np

from . import graph_dir, graphgen

COMMUNITY_SEED = 1234


def _pairs(a: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    a = np.asarray(a, np.uint64).reshape(-1, 2)
    return a[:, 0].copy(), a[:, 1].copy()


def load_snap_txt(path) -> tuple[np.ndarray, np.ndarray]:
    """(raw src, raw dst) uint64 arrays of a SNAP edge-list text file:
    whitespace-separated pairs, '#' lines skipped."""
    try:
        a = np.loadtxt(path, dtype=np.uint64, comments="#", usecols=(0, 1), ndmin=2)
    except ValueError as e:
        raise ValueError(f"{path}: expected two vertex ids per line ({e})") from None
    return _pairs(a)


def load_snap_csv(path) -> tuple[np.ndarray, np.ndarray]:
    """(raw src, raw dst) of a CSV with the header node_1,node_2."""
    with open(path) as f:
        header = f.readline().strip().split(",")
    if header != ["node_1", "node_2"]:
        raise ValueError(f"{path}: header must be node_1,node_2, got {header}")
    try:
        a = np.loadtxt(path, dtype=np.uint64, delimiter=",", skiprows=1, ndmin=2)
    except ValueError as e:
        raise ValueError(f"{path}: every row holds two vertex ids ({e})") from None
    if a.size and a.shape[1] != 2:
        raise ValueError(f"{path}: every row holds two vertex ids")
    return _pairs(a)


def _psv_columns(path, names) -> list:
    """The named columns (uint64) of a '|'-separated file with a header line."""
    with open(path) as f:
        titles = f.readline().rstrip("\n").split("|")
    idx = []
    for name in names:
        if name not in titles:
            raise ValueError(f"{path}: no column {name}")
        idx.append(titles.index(name))
    a = np.loadtxt(path, dtype=np.uint64, delimiter="|", skiprows=1, usecols=idx, ndmin=2)
    return [a[:, k].copy() for k in range(len(idx))]


def load_ldbc_ic(root) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(raw person ids, raw src, raw dst) of an LDBC SNB interactive dataset."""
    dyn = Path(root) / "social_network" / "dynamic"
    (persons,) = _psv_columns(dyn / "person_0_0.csv", ["id"])
    kp = dyn / "person_knows_person_0_0.csv"
    with open(kp) as f:
        kt = f.readline().rstrip("\n").split("|")
    if kt[:2] != ["Person.id", "Person.id"]:
        raise ValueError(f"{kp}: header must start with Person.id|Person.id, got {kt}")
    a = np.loadtxt(kp, dtype=np.uint64, delimiter="|", skiprows=1, usecols=(0, 1), ndmin=2)
    return (persons, *_pairs(a))


def load_ldbc_bi(root) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(raw person ids, raw src, raw dst) of an LDBC SNB BI dataset (every .csv
    of the initial snapshot's Person and Person_knows_Person folders, in name
    order)."""
    dyn = Path(root) / "graphs" / "csv" / "bi" / "composite-merged-fk" / "initial_snapshot" / "dynamic"
    persons = [_psv_columns(p, ["id"])[0] for p in sorted((dyn / "Person").glob("*.csv"))]
    knows = [_psv_columns(p, ["Person1Id", "Person2Id"]) for p in sorted((dyn / "Person_knows_Person").glob("*.csv"))]
    cat = lambda xs: np.concatenate(xs) if xs else np.zeros(0, np.uint64)
    return cat(persons), cat([k[0] for k in knows]), cat([k[1] for k in knows])


def communities(n: int, seed: int = COMMUNITY_SEED) -> np.ndarray:
    out = np.zeros(n, np.uint8)
    if graphgen._lib().vsg_sn_communities(n, seed, out.ctypes.data if n else None):
        raise ValueError("community assignment failed")
    return out


def _sorted_unique(x: np.ndarray) -> np.ndarray:
    """Distinct values ascending (a sort and a neighbour mask: several times
    faster than np.unique on large uint64 arrays)."""
    y = np.sort(x)
    if len(y) < 2:
        return y
    keep = np.empty(len(y), bool)
    keep[0] = True
    keep[1:] = y[1:] != y[:-1]
    return y[keep]


def rearrange(raw_src: np.ndarray, raw_dst: np.ndarray, persons: np.ndarray | None = None):
    """(raw ids in vertex order, community per vertex, HostGraph of knows);
    the vertices are `persons` when given, else the edge endpoints."""
    raw_src = np.asarray(raw_src, np.uint64)
    raw_dst = np.asarray(raw_dst, np.uint64)
    if persons is None:
        raw_ids = _sorted_unique(np.concatenate([raw_src, raw_dst]))  # vertex i has the i-th smallest raw id
    else:
        raw_ids = _sorted_unique(np.asarray(persons, np.uint64))
        if len(raw_ids) != len(persons):
            raise ValueError("a person id occurs twice")
    V = len(raw_ids)
    if V >= 1 << 32:
        raise ValueError("more vertices than 32-bit ids hold")
    s = np.searchsorted(raw_ids, raw_src)
    d = np.searchsorted(raw_ids, raw_dst)
    if persons is not None and len(s) and (s.max() >= V or d.max() >= V or np.any(raw_ids[np.minimum(s, V - 1)] != raw_src)
                                           or np.any(raw_ids[np.minimum(d, V - 1)] != raw_dst)):
        raise ValueError("an edge names a person the person files do not hold")
    s = s.astype(np.uint32)
    d = d.astype(np.uint32)
    # undirected: the list and its reverse, neighbouring duplicates dropped, then sorted
    es = np.concatenate([s, d])
    ed = np.concatenate([d, s])
    keep = np.ones(len(es), bool)
    if len(es) > 1:
        keep[1:] = (es[1:] != es[:-1]) | (ed[1:] != ed[:-1])
    # sorted by (src, dst): one sort of the pairs packed as src << 32 | dst
    key = np.sort((es[keep].astype(np.uint64) << np.uint64(32)) | ed[keep].astype(np.uint64))
    es = (key >> np.uint64(32)).astype(np.uint32)
    ed = (key & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    off = np.zeros(V + 1, np.int64)
    off[1:] = np.cumsum(np.bincount(es, minlength=V))
    g = graphgen.HostGraph(V, len(ed), off, ed, off, ed, directed=False)
    return raw_ids, communities(V), g


def output_vlgpm(out_dir, raw_src, raw_dst, partitions: int | None = None,
                 persons: np.ndarray | None = None) -> graphgen.HostGraph:
    """Write the directory; partitions: block count of the partitioned flat
    lists (the reference's -b), none by default; persons: the vertex raw ids
    (LDBC inputs), else the edge endpoints."""
    raw_ids, comm, g = rearrange(raw_src, raw_dst, persons)
    props = {"id": np.arange(g.V, dtype=np.uint32), "community": comm}
    part = {"src_dst": partitions, "hilbert": partitions} if partitions else None
    graph_dir.save(out_dir, g, properties=props, flats=("src_dst", "hilbert"), partitioned=part,
                   graph_name="Social Network", graph_type="Social Network")
    return g


def main():
    ap = argparse.ArgumentParser(description="import a social-network edge list into a graph directory")
    ap.add_argument("-s", "--source", required=True, help="edge list file, or the LDBC dataset directory")
    ap.add_argument("-d", "--dir", required=True, help="graph directory to write")
    ap.add_argument("-i", "--input", choices=["snap-txt", "snap-csv", "ldbc-ic", "ldbc-bi"], default="snap-txt")
    ap.add_argument("-b", "--blocks", type=int, default=None, help="partitioned flat lists in this many blocks")
    args = ap.parse_args()
    persons = None
    if args.input == "snap-txt":
        raw_src, raw_dst = load_snap_txt(args.source)
    elif args.input == "snap-csv":
        raw_src, raw_dst = load_snap_csv(args.source)
    else:
        persons, raw_src, raw_dst = (load_ldbc_ic if args.input == "ldbc-ic" else load_ldbc_bi)(args.source)
    g = output_vlgpm(Path(args.dir), raw_src, raw_dst, args.blocks, persons)
    print(f"{g.V} Person, {g.E} knows (both directions) -> {args.dir}")


if __name__ == "__main__":
    main()
