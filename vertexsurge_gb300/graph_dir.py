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

Flat edge lists (meta/graph_loader.hh:202-276, names meta/schema.cpp:69-97):
VIDPair files (two uint32 per edge; the backward direction stores each edge
as (dst, src)) named "{edge name}_{order}" for one file and
"{edge name}_{order}_{i}" for the blocks of a partitioned list, order one of
hilbert, src_dst, dst_src, random.  A partitioned list cuts the edges, sorted
by (dst, src), into blocks of about equal size that never split one target's
edges (partition_by_dst, graph_loader.hh:112-138), then orders every block.
`save` writes them on request and `load` rebuilds the CSR from a flat list
when an edge type has no CSR files.
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


FLAT_ORDERS = ("hilbert", "src_dst", "dst_src", "random")


def flat_edges_name(src: str, etype: str, dst: str, directed: bool, direction: str, order: str,
                    index: int | None = None) -> str:
    """EdgeSchema::get_flat_edges_name (meta/schema.cpp:69-97)."""
    if order not in FLAT_ORDERS:
        raise ValueError(f"unknown flat edge order {order}")
    base = (forward_edge_name if direction == "forward" else backward_edge_name)(src, etype, dst, directed)
    return f"{base}_{order}" + ("" if index is None else f"_{index}")


# The space-filling curve of the "hilbert" flat order (utils/peano.hh:20-89):
# per level the quadrant q = 2 * x_bit + y_bit is visited at the position its
# state's order gives, and the state of the sub-square follows a table.
_CURVE_ORDER = np.array([[0, 1, 3, 2], [3, 2, 0, 1], [0, 2, 3, 1], [3, 1, 0, 2]])  # states RA, RD, CA, CD
_CURVE_POS = np.argsort(_CURVE_ORDER, axis=1)       # quadrant -> position in the state's order
_CURVE_SUB = np.array([[2, 0, 0, 3], [3, 1, 1, 2], [0, 2, 2, 1], [1, 3, 3, 0]])  # state of the sub-square


def curve_index(n: int, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Curve position of the cells (x, y) in an n x n grid (n a power of two),
    the order of XYToIndex(n, x, y, RA)."""
    x = np.asarray(x, np.int64).copy()
    y = np.asarray(y, np.int64).copy()
    idx = np.zeros(len(x), np.uint64)
    state = np.zeros(len(x), np.int64)
    half = n // 2
    while half >= 1:
        q = (x // half) * 2 + (y // half)
        pos = _CURVE_POS[state, q]
        idx = idx * np.uint64(4) + pos.astype(np.uint64)
        state = _CURVE_SUB[state, pos]
        x %= half
        y %= half
        half //= 2
    return idx


def _pow2_at_least(x: int) -> int:
    p = 1
    while p < x:
        p <<= 1
    return p


def _pair_order(major: np.ndarray, minor: np.ndarray) -> np.ndarray:
    """Permutation sorting uint32 pairs by (major, minor): one stable argsort of
    the pairs packed into uint64 keys (several times faster than lexsort)."""
    key = (np.asarray(major, np.uint64) << np.uint64(32)) | np.asarray(minor, np.uint64)
    return np.argsort(key, kind="stable")


def order_edges(src: np.ndarray, dst: np.ndarray, order: str, n_src: int, n_dst: int, seed: int = 0) -> np.ndarray:
    """Permutation putting the edges (src, dst) in a flat order."""
    if order == "src_dst":
        return _pair_order(src, dst)
    if order == "dst_src":
        return _pair_order(dst, src)
    if order == "hilbert":
        return np.argsort(curve_index(_pow2_at_least(max(n_src, n_dst)), src, dst), kind="stable")
    return np.random.default_rng(seed).permutation(len(src))


def partition_by_dst(dst_sorted: np.ndarray, count: int) -> list:
    """Block bounds [(b, e)] of edges sorted by (dst, src): block i ends at the
    first target change at or after pos + (n - pos) / (count - i)
    (graph_loader.hh:112-138); blocks after the last edge are empty."""
    n, pos, out = len(dst_sorted), 0, []
    d = np.asarray(dst_sorted)
    changes = np.flatnonzero(d[1:] != d[:-1]) + 1 if n > 1 else np.zeros(0, np.int64)  # i: d[i] != d[i-1]
    for i in range(count):
        if pos >= n:
            out.append((n, n))
            continue
        expected = pos + (n - pos) // (count - i)
        # the first target change at or after max(pos + 1, expected), else the end
        k = int(np.searchsorted(changes, max(pos + 1, expected)))
        end = int(changes[k]) if k < len(changes) else n
        out.append((pos, end))
        pos = end
    return out


def write_flat_edges(dir_, g: HostGraph, src_type: str, etype: str, dst_type: str, flats=(), partitioned=None):
    """The flat edge lists of one edge type for both stored directions: one
    file per order in `flats`, and `partitioned` ({order: block count}) lists
    cut by target; returns the schema's store_info."""
    d = Path(dir_)
    rows = np.repeat(np.arange(g.V, dtype=np.uint32), np.diff(g.fwd_off).astype(np.int64))
    src, dst = rows, np.asarray(g.fwd_dst, np.uint32)
    dirs = ["forward"] + (["backward"] if g.directed else [])

    def pairs(a, b, direction):
        out = np.empty((len(a), 2), np.uint32)
        out[:, 0], out[:, 1] = (a, b) if direction == "forward" else (b, a)
        return out.view(np.uint64).reshape(-1)

    for direction in dirs:
        for order in flats:
            perm = order_edges(src, dst, order, g.V, g.V)
            write_disk_array(d / flat_edges_name(src_type, etype, dst_type, g.directed, direction, order),
                             pairs(src[perm], dst[perm], direction))
        for order, count in (partitioned or {}).items():
            by_dst = _pair_order(dst, src)
            s_, t_ = src[by_dst], dst[by_dst]
            for i, (b, e) in enumerate(partition_by_dst(t_, count)):
                perm = order_edges(s_[b:e], t_[b:e], order, g.V, g.V)
                write_disk_array(d / flat_edges_name(src_type, etype, dst_type, g.directed, direction, order, i),
                                 pairs(s_[b:e][perm], t_[b:e][perm], direction))
    return {"flats": list(flats), "partitioned_flats": list((partitioned or {}).keys()),
            "partition_counts": [int(c) for c in (partitioned or {}).values()]}


def read_flat_edges(dir_, src_type: str, etype: str, dst_type: str, directed: bool, direction: str, order: str,
                    count: int | None = None) -> np.ndarray:
    """A flat edge list (blocks concatenated when partitioned) as (n, 2) uint32
    pairs, as stored (the backward direction holds (dst, src))."""
    d = Path(dir_)
    names = [flat_edges_name(src_type, etype, dst_type, directed, direction, order, i)
             for i in (range(count) if count is not None else [None])]
    parts = [np.asarray(read_disk_array(d / n, np.uint64)) for n in names]
    flat = np.concatenate(parts) if parts else np.zeros(0, np.uint64)
    return flat.view(np.uint32).reshape(-1, 2)


def csr_from_pairs(V: int, src: np.ndarray, dst: np.ndarray):
    """(offsets, targets) of the lists of src -> dst, targets sorted per list."""
    order = _pair_order(src, dst)
    off = np.zeros(V + 1, np.int64)
    np.cumsum(np.bincount(src, minlength=V), out=off[1:])
    return off, np.ascontiguousarray(dst[order], np.uint32)


PROPERTY_TYPES = {np.dtype(np.uint8): "TagValue8", np.dtype(np.uint16): "TagValue16",
                  np.dtype(np.uint32): "VID", np.dtype(np.int32): "Int32", np.dtype(np.int64): "Int64"}


def save(dir_, g: HostGraph, vertex_type="Person", edge_type="knows", graph_name="synthetic",
         properties: dict | None = None, flats=(), partitioned=None, csr=True, graph_type="synthetic") -> None:
    """Write one vertex type (with optional properties: name -> per-vertex
    array, stored as "Type.name") and one self edge type (src = dst): its CSR
    files (unless csr is False) and the flat edge lists asked for (`flats`:
    orders written as one file, `partitioned`: {order: block count})."""
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
    if csr:
        write_disk_array(d / names["fwd_index"], g.fwd_off.astype(np.int64))
        write_disk_array(d / names["fwd_data"], g.fwd_dst.astype(np.uint32))
        if g.directed:
            write_disk_array(d / names["bwd_index"], g.rev_off.astype(np.int64))
            write_disk_array(d / names["bwd_data"], g.rev_src.astype(np.uint32))
    store_info = write_flat_edges(d, g, vertex_type, edge_type, vertex_type, flats, partitioned)
    schema = {
        "graph_name": graph_name, "graph_type": graph_type,
        "vertex": [{"type": vertex_type, "statistics": {"count": int(g.V)}, "properties": props}],
        "edge": [{"type": edge_type, "directed": bool(g.directed), "allow_multiple_edge": False,
                  "src": vertex_type, "dst": vertex_type, "properties": {},
                  "statistics": {"count": int(g.E)},
                  "store_info": store_info}],
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
        if not (d / names["fwd_index"]).exists():  # no CSR files: rebuild them from a flat edge list
            info = e.get("store_info", {})
            if info.get("flats"):
                pr = read_flat_edges(d, src, et, dst, directed, "forward", info["flats"][0])
            elif info.get("partitioned_flats"):
                pr = read_flat_edges(d, src, et, dst, directed, "forward", info["partitioned_flats"][0],
                                     int(info["partition_counts"][0]))
            else:
                raise ValueError(f"edge type {src}_{et}_{dst}: neither CSR files nor flat edge lists")
            fo, fd = csr_from_pairs(V, pr[:, 0], pr[:, 1])
            ro, rs = csr_from_pairs(V, pr[:, 1], pr[:, 0]) if directed else (fo, fd)
            out[f"{src}_{et}_{dst}"] = HostGraph(V=V, E=E, fwd_off=fo, fwd_dst=fd, rev_off=ro, rev_src=rs,
                                                 directed=directed)
            continue
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
