"""Synthetic graphs in CSR form (wraps libvsgen.so, csrc/host/graphgen.cpp).

R-MAT and power-law (Zipf out-degree) generators producing cleaned,
sorted uint32 CSR with int64 offsets and the matching reverse CSR, as the
reference's importer does for its graphs (src/include/meta/graph_loader.hh:163-200).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
GEN_PATH = PKG / "libvsgen.so"


class _VsgGraph(C.Structure):
    _fields_ = [("V", C.c_uint32), ("E", C.c_uint64), ("fwd_off", C.POINTER(C.c_int64)),
                ("fwd_dst", C.POINTER(C.c_uint32)), ("rev_off", C.POINTER(C.c_int64)),
                ("rev_src", C.POINTER(C.c_uint32))]


_gen = None


def _lib():
    global _gen
    if _gen is None:
        if not GEN_PATH.exists():
            raise RuntimeError(f"{GEN_PATH} missing: run vertexsurge_gb300.build.build_all()")
        L = C.CDLL(str(GEN_PATH))
        L.vsg_rmat.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                               C.c_int, C.POINTER(_VsgGraph)]
        L.vsg_zipf.argtypes = [C.c_uint32, C.c_uint64, C.c_double, C.c_uint32, C.c_uint64,
                               C.POINTER(_VsgGraph)]
        L.vsg_from_edges.argtypes = [C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int,
                                     C.POINTER(_VsgGraph)]
        L.vsg_free.argtypes = [C.POINTER(_VsgGraph)]
        L.vsg_sample_sources.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64, C.c_void_p]
        L.vsg_hash.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.vsg_hash.restype = C.c_uint64
        L.vsg_sn_communities.argtypes = [C.c_uint64, C.c_uint32, C.c_void_p]
        _gen = L
    return _gen


@dataclass
class HostGraph:
    V: int
    E: int
    fwd_off: np.ndarray  # int64 [V+1]
    fwd_dst: np.ndarray  # uint32 [E]
    rev_off: np.ndarray  # int64 [V+1]
    rev_src: np.ndarray  # uint32 [E]
    directed: bool = True
    name: str = ""

    def out_degree(self) -> np.ndarray:
        return np.diff(self.fwd_off)

    def in_degree(self) -> np.ndarray:
        return np.diff(self.rev_off)


def _take(g: _VsgGraph, directed: bool, name: str) -> HostGraph:
    V, E = int(g.V), int(g.E)
    fo = np.ctypeslib.as_array(g.fwd_off, shape=(V + 1,)).copy()
    ro = np.ctypeslib.as_array(g.rev_off, shape=(V + 1,)).copy()
    if E:
        fd = np.ctypeslib.as_array(g.fwd_dst, shape=(E,)).copy()
        rs = np.ctypeslib.as_array(g.rev_src, shape=(E,)).copy()
    else:
        fd = np.zeros(0, np.uint32)
        rs = np.zeros(0, np.uint32)
    _lib().vsg_free(C.byref(g))
    return HostGraph(V, E, fo, fd, ro, rs, directed, name)


def rmat(scale: int, edge_factor: int = 16, a=0.57, b=0.19, c=0.19, seed: int = 1,
         undirected: bool = False) -> HostGraph:
    g = _VsgGraph()
    rc = _lib().vsg_rmat(scale, edge_factor, a, b, c, seed, 1 if undirected else 0, C.byref(g))
    if rc:
        raise ValueError("vsg_rmat rejected its arguments")
    return _take(g, not undirected, f"rmat{scale}_a{a}")


def zipf(V: int, target_edges: int, alpha: float = 2.1, max_deg: int = 50000, seed: int = 3) -> HostGraph:
    g = _VsgGraph()
    rc = _lib().vsg_zipf(V, target_edges, alpha, max_deg, seed, C.byref(g))
    if rc:
        raise ValueError("vsg_zipf rejected its arguments")
    return _take(g, True, f"zipf{V}")


def from_edges(V: int, src, dst, undirected: bool = False) -> HostGraph:
    s = np.ascontiguousarray(src, dtype=np.uint32)
    d = np.ascontiguousarray(dst, dtype=np.uint32)
    g = _VsgGraph()
    rc = _lib().vsg_from_edges(V, len(s), s.ctypes.data, d.ctypes.data, 1 if undirected else 0, C.byref(g))
    if rc:
        raise ValueError("vsg_from_edges rejected its arguments")
    return _take(g, not undirected, "edges")


def sample_sources(V: int, n: int, seed: int = 2) -> np.ndarray:
    out = np.zeros(n, dtype=np.uint32)
    if _lib().vsg_sample_sources(V, n, seed, out.ctypes.data):
        raise ValueError("n > V")
    return out


def hash64(seed: int, a: int, b: int) -> int:
    return int(_lib().vsg_hash(seed, a, b))
