"""The reference's on-disk graph directory, read and written from Python.

A graph directory holds `schema.json` (the GraphSchema: vertex types with
their counts, edge types with direction and edge count) and one file per
variable, named as the reference names them (meta/schema.cpp:36-66,
:160-205):

  forward CSR   "{src}-{type}->{dst}_csr_src_dst"  (+ "_index")   directed
                "{src}-{type}-{dst}_csr_src_dst"   (+ "_index")   undirected
  backward CSR  "{dst}<-{type}-{src}_csr_dst_src"  (+ "_index")   directed only

Every variable file is a DiskArray (storage/disk_array.hh:53, :330-352): a
64-byte header whose first two int64 are the element count and the element
size, then the elements (Offset = int64 for CSR indexes, VID = uint32 for CSR
targets).  An undirected edge type stores both directions of every edge in its
one forward CSR (meta/graph_loader.hh:64-66), so its backward lists are the
forward lists.

`load` gives HostGraph objects that DeviceGraph.from_host uploads; `save`
writes a HostGraph in the same layout, so the reference's Graph::load
(storage/graph_store.cpp:48-73) reads graphs generated here and the C++
operator layer's Graph(dir).load() reads graphs the reference imported.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from .graphgen import HostGraph

HEADER_BYTES = 64


def forward_edge_name(src: str, etype: str, dst: str, directed: bool) -> str:
    return f"{src}-{etype}->{dst}" if directed else f"{src}-{etype}-{dst}"


def backward_edge_name(src: str, etype: str, dst: str, directed: bool) -> str:
    return f"{dst}<-{etype}-{src}" if directed else f"{dst}-{etype}-{src}"


def csr_names(src: str, etype: str, dst: str, directed: bool) -> dict:
    """File names of the CSR variables of one edge type (index, data per direction)."""
    f = forward_edge_name(src, etype, dst, directed) + "_csr_src_dst"
    out = {"fwd_data": f, "fwd_index": f + "_index"}
    if directed:
        b = backward_edge_name(src, etype, dst, directed) + "_csr_dst_src"
        out.update({"bwd_data": b, "bwd_index": b + "_index"})
    return out


def read_disk_array(path, dtype) -> np.ndarray:
    """A DiskArray file as a read-only memory map of `dtype` elements."""
    path = Path(path)
    hdr = np.fromfile(path, dtype=np.int64, count=2)
    if len(hdr) < 2:
        raise ValueError(f"{path}: shorter than the DiskArray header")
    n, size = int(hdr[0]), int(hdr[1])
    dt = np.dtype(dtype)
    if size != dt.itemsize:
        raise ValueError(f"{path}: element size {size}, expected {dt.itemsize}")
    if path.stat().st_size < HEADER_BYTES + n * size:
        raise ValueError(f"{path}: {n} elements of {size} B do not fit the file")
    if n == 0:
        return np.zeros(0, dt)
    return np.memmap(path, dtype=dt, mode="r", offset=HEADER_BYTES, shape=(n,))


def write_disk_array(path, arr: np.ndarray) -> None:
    arr = np.ascontiguousarray(arr)
    hdr = np.zeros(HEADER_BYTES // 8, np.int64)
    hdr[0], hdr[1] = len(arr), arr.dtype.itemsize
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(arr.tobytes())


PROPERTY_TYPES = {np.dtype(np.uint8): "TagValue8", np.dtype(np.uint16): "TagValue16",
                  np.dtype(np.uint32): "VID", np.dtype(np.int32): "Int32", np.dtype(np.int64): "Int64"}


def save(dir_, g: HostGraph, vertex_type="Person", edge_type="knows", graph_name="synthetic",
         properties: dict | None = None) -> None:
    """Write one vertex type (with optional properties: name -> per-vertex
    array, stored as "Type.name") and one self edge type (src = dst)."""
    d = Path(dir_)
    d.mkdir(parents=True, exist_ok=True)
    props = {}
    for name, arr in (properties or {}).items():
        arr = np.ascontiguousarray(arr)
        if len(arr) != g.V or arr.dtype not in PROPERTY_TYPES:
            raise ValueError(f"property {name}: one value per vertex of a supported type")
        write_disk_array(d / f"{vertex_type}.{name}", arr)
        props[name] = {"name": name, "type": PROPERTY_TYPES[arr.dtype]}
    names = csr_names(vertex_type, edge_type, vertex_type, g.directed)
    write_disk_array(d / names["fwd_index"], g.fwd_off.astype(np.int64))
    write_disk_array(d / names["fwd_data"], g.fwd_dst.astype(np.uint32))
    if g.directed:
        write_disk_array(d / names["bwd_index"], g.rev_off.astype(np.int64))
        write_disk_array(d / names["bwd_data"], g.rev_src.astype(np.uint32))
    schema = {
        "graph_name": graph_name, "graph_type": "synthetic",
        "vertex": [{"type": vertex_type, "statistics": {"count": int(g.V)}, "properties": props}],
        "edge": [{"type": edge_type, "directed": bool(g.directed), "allow_multiple_edge": False,
                  "src": vertex_type, "dst": vertex_type, "properties": {},
                  "statistics": {"count": int(g.E)},
                  "store_info": {"flats": [], "partitioned_flats": [], "partition_counts": []}}],
    }
    (d / "schema.json").write_text(json.dumps(schema, indent=4))


def load(dir_) -> dict:
    """{"{src}_{type}_{dst}": HostGraph} for every edge type with CSR files whose
    source and target vertex types are the same (the expand's graphs)."""
    d = Path(dir_)
    schema = json.loads((d / "schema.json").read_text())
    counts = {v["type"]: int(v["statistics"]["count"]) for v in schema["vertex"]}
    out = {}
    for e in schema["edge"]:
        src, dst, et, directed = e["src"], e["dst"], e["type"], bool(e["directed"])
        if src != dst:
            continue
        V, E = counts[src], int(e["statistics"]["count"])
        names = csr_names(src, et, dst, directed)
        fo = np.asarray(read_disk_array(d / names["fwd_index"], np.int64))
        fd = np.asarray(read_disk_array(d / names["fwd_data"], np.uint32))
        if directed:
            ro = np.asarray(read_disk_array(d / names["bwd_index"], np.int64))
            rs = np.asarray(read_disk_array(d / names["bwd_data"], np.uint32))
        else:
            ro, rs = fo, fd
        if len(fo) != V + 1 or int(fo[-1]) != len(fd) or len(fd) != E:
            raise ValueError(f"edge type {src}_{et}_{dst}: CSR sizes do not match the schema")
        out[f"{src}_{et}_{dst}"] = HostGraph(V=V, E=E, fwd_off=fo, fwd_dst=fd, rev_off=ro, rev_src=rs,
                                             directed=directed)
    return out
