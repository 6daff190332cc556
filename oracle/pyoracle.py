"""ORACLE — test infrastructure only.

ctypes binding of oracle/build/liboracle.so (oracle.cpp), the CPU
restatement of VertexSurge's operators.  Only tests, the smoke check and the
benchmark's CPU-baseline leg use it.  Matrices are exchanged in logical form:
numpy uint64 arrays of shape (cols, ceil(rows/64)).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle.so"

FLAT, VARROW, COLMAIN = 0, 1, 2
T_VID, T_I64 = 0, 1


class OrTable(C.Structure):
    _fields_ = [("kind", C.c_int), ("ncols", C.c_uint32), ("var", C.POINTER(C.c_int32)),
                ("type", C.POINTER(C.c_int32)), ("cols", C.POINTER(C.c_void_p)), ("nrows", C.c_uint64),
                ("mrows", C.c_uint32), ("mcols", C.c_uint32), ("words", C.c_void_p),
                ("row_map", C.c_void_p), ("col_map", C.c_void_p)]


class OrResult(C.Structure):
    _fields_ = [("ncols", C.c_uint32), ("nrows", C.c_uint64), ("var", C.c_int32 * 16),
                ("type", C.c_int32 * 16), ("cols", C.c_void_p * 16), ("count", C.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} missing: run vertexsurge_gb300.build.build_all()")
        L = C.CDLL(str(LIB))
        L.oracle_vexpand.argtypes = [C.c_uint32] + [C.c_void_p] * 4 + [C.c_int, C.c_void_p, C.c_uint32,
                                     C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_uint32, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_flat_blocks.argtypes = [C.c_uint32] + [C.c_void_p] * 4 + [C.c_int, C.c_int, C.c_uint32]
        L.oracle_flat_blocks.restype = C.c_void_p
        L.oracle_flat_blocks_free.argtypes = [C.c_void_p]
        L.oracle_flat_blocks_export.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_flat_blocks_export.restype = C.c_uint64
        L.oracle_vexpand_blocks.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                            C.c_int, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p]
        L.oracle_hash_join.argtypes = [C.POINTER(OrTable), C.POINTER(OrTable), C.c_int32, C.c_int,
                                       C.POINTER(OrResult)]
        L.oracle_mintersect.argtypes = [C.POINTER(OrTable), C.POINTER(OrTable), C.c_uint32, C.c_int32,
                                        C.c_uint32, C.c_int, C.POINTER(OrResult)]
        L.oracle_free_result.argtypes = [C.POINTER(OrResult)]
        L.oracle_matrix_select.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                           C.c_uint32, C.c_void_p]
        L.oracle_table_convert.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_int,
                                           C.c_void_p]
        L.oracle_matrix_count.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32]
        L.oracle_matrix_count.restype = C.c_uint64
        L.oracle_matrix_iterate.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_matrix_iterate.restype = C.c_uint64
        L.oracle_matrix_column_count.argtypes = [C.POINTER(OrTable), C.c_int, C.c_void_p, C.c_void_p]
        L.oracle_matrix_row_or_sum.argtypes = [C.POINTER(OrTable), C.c_void_p]
        L.oracle_matrix_row_or_sum.restype = C.c_uint64
        L.oracle_semi_join.argtypes = [C.POINTER(OrTable), C.POINTER(OrTable), C.c_void_p, C.c_uint32, C.c_int,
                                       C.POINTER(OrResult), C.c_void_p]
        L.oracle_matrix_filter.argtypes = [C.POINTER(OrTable), C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                           C.c_void_p, C.c_uint64, C.c_int]
        L.oracle_matrix_filter.restype = C.c_uint64
        L.oracle_vertex_mask_any_neighbor.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint8,
                                                      C.c_void_p]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_get_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


_PATHS = {"any": 0, "shortest": 1, "find_shortest": 2}
_DIRS = {"forward": 0, "backward": 1, "both": 2}


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


class FlatBlocks:
    """The reference's BlockHilbert edge layout of one expand direction:
    n_blocks target-disjoint blocks of (u, v) pairs, each in curve order."""

    def __init__(self, g, direction="forward", n_blocks=64):
        self.V = g.V
        self.direction = direction
        self.n_blocks = int(n_blocks)
        self._h = lib().oracle_flat_blocks(g.V, _p(g.fwd_off), _p(g.fwd_dst), _p(g.rev_off), _p(g.rev_src),
                                           1 if g.directed else 0, _DIRS[direction], self.n_blocks)
        if not self._h:
            raise ValueError("oracle_flat_blocks rejected its arguments")

    def export(self):
        """(block offsets (n_blocks + 1,), pairs (n, 2) of (u, v))."""
        n = lib().oracle_flat_blocks_export(self._h, None, None)
        off = np.zeros(self.n_blocks + 1, np.uint64)
        pairs = np.zeros((n, 2), np.uint32)
        lib().oracle_flat_blocks_export(self._h, _p(off), _p(pairs))
        return off, pairs

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_flat_blocks_free(self._h)
            self._h = None


def vexpand(g, sources, k_min, k_max, path="any", direction="forward", targets=None,
            stack_row_count=1024, want_matrix=True, hop_stats=False, blocks=None):
    """VExpand(Dense) on the CPU. Returns (logical words (V, ceil(S/64)) or None,
    distances or None, hop stats dict or None).  With `blocks` (a FlatBlocks of
    this graph and direction) the hops run the reference's BlockHilbert loop
    over that layout; otherwise a pull over the CSR in-lists."""
    src = np.ascontiguousarray(sources, dtype=np.uint32)
    S = len(src)
    W = (S + 63) // 64
    out = np.zeros((g.V, W), dtype=np.uint64) if (want_matrix and path != "find_shortest") else None
    tg = None if targets is None else np.ascontiguousarray(targets, dtype=np.uint32)
    dist = np.zeros(S, dtype=np.int32) if path == "find_shortest" else None
    hs = np.zeros(4 * 64, dtype=np.uint64) if hop_stats else None
    if blocks is not None:
        if blocks.V != g.V or blocks.direction != direction:
            raise ValueError("blocks were built for another graph or direction")
        rc = lib().oracle_vexpand_blocks(blocks._h, _p(src), S, k_min, k_max, _PATHS[path], stack_row_count,
                                         _p(tg), _p(dist), _p(out), _p(hs))
    else:
        rc = lib().oracle_vexpand(g.V, _p(g.fwd_off), _p(g.fwd_dst), _p(g.rev_off), _p(g.rev_src),
                                  1 if g.directed else 0, _p(src), S, k_min, k_max, _PATHS[path],
                                  _DIRS[direction], stack_row_count, _p(tg), _p(dist), _p(out), _p(hs))
    if rc:
        raise ValueError("oracle_vexpand rejected its arguments")
    st = None
    if hs is not None:
        hs = hs.reshape(4, 64)
        n = int(hs[3, 0])
        st = {"hops_run": n, "visit_count": [int(x) for x in hs[0, : n + 1]],
              "layer_count": [int(x) for x in hs[1, : n + 1]],
              "active_edges": [int(x) for x in hs[2, : n + 1]]}
    return out, dist, st


class Table:
    """A table for the join / intersection oracles (keeps its buffers alive)."""

    def __init__(self, kind, var, cols=None, types=None, words=None, mrows=0, mcols=0,
                 row_map=None, col_map=None):
        self.kind = kind
        self.var = np.ascontiguousarray(var, dtype=np.int32)
        self.keep = []
        t = OrTable()
        t.kind = kind
        t.ncols = len(var)
        t.var = self.var.ctypes.data_as(C.POINTER(C.c_int32))
        if kind == FLAT:
            arrs = []
            tys = []
            for c in cols:
                c = np.ascontiguousarray(c)
                if c.dtype == np.int64:
                    tys.append(T_I64)
                else:
                    c = np.ascontiguousarray(c.astype(np.uint32))
                    tys.append(T_VID)
                arrs.append(c)
            self.types = np.asarray(tys if types is None else types, dtype=np.int32)
            self.cols = arrs
            self.ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
            t.type = self.types.ctypes.data_as(C.POINTER(C.c_int32))
            t.cols = C.cast(self.ptrs, C.POINTER(C.c_void_p))
            t.nrows = len(arrs[0]) if arrs else 0
        else:
            self.words = np.ascontiguousarray(words, dtype=np.uint64)
            t.mrows, t.mcols = mrows, mcols
            t.words = self.words.ctypes.data
            if row_map is not None:
                self.row_map = np.ascontiguousarray(row_map, dtype=np.uint32)
                t.row_map = self.row_map.ctypes.data
            if col_map is not None:
                self.col_map = np.ascontiguousarray(col_map, dtype=np.uint32)
                t.col_map = self.col_map.ctypes.data
        self.t = t


def _result(r: OrResult):
    cols = []
    for i in range(r.ncols):
        if r.type[i] == T_I64:
            a = np.ctypeslib.as_array(C.cast(r.cols[i], C.POINTER(C.c_int64)), shape=(r.nrows,)).copy() \
                if r.nrows else np.zeros(0, np.int64)
        else:
            a = np.ctypeslib.as_array(C.cast(r.cols[i], C.POINTER(C.c_uint32)), shape=(r.nrows,)).copy() \
                if r.nrows else np.zeros(0, np.uint32)
        cols.append(a)
    var = [r.var[i] for i in range(r.ncols)]
    count = int(r.count)
    lib().oracle_free_result(C.byref(r))
    return var, cols, count


def hash_join(a: Table, b: Table, key_var: int, only_count=False):
    r = OrResult()
    if lib().oracle_hash_join(C.byref(a.t), C.byref(b.t), key_var, 1 if only_count else 0, C.byref(r)):
        raise ValueError("oracle_hash_join rejected its arguments")
    return _result(r)


def mintersect(base: Table, deps: list, new_var: int, new_type_count: int, only_count=False):
    arr = (OrTable * len(deps))(*[d.t for d in deps])
    r = OrResult()
    if lib().oracle_mintersect(C.byref(base.t), arr, len(deps), new_var, new_type_count,
                               1 if only_count else 0, C.byref(r)):
        raise ValueError("oracle_mintersect rejected its arguments")
    return _result(r)


def matrix_select(words, rows, cols, targets, stack_row_count=1024):
    t = np.ascontiguousarray(targets, dtype=np.uint32)
    out = np.zeros((len(t), (rows + 63) // 64), dtype=np.uint64)
    w = np.ascontiguousarray(words, dtype=np.uint64)
    if lib().oracle_matrix_select(rows, cols, _p(w), stack_row_count, _p(t), len(t), _p(out)):
        raise ValueError("target out of range")
    return out


def table_convert(words, rows, cols, transpose, stack_row_count=1024):
    w = np.ascontiguousarray(words, dtype=np.uint64)
    if transpose:
        out = np.zeros((rows, (cols + 63) // 64), dtype=np.uint64)
    else:
        out = np.zeros((cols, (rows + 63) // 64), dtype=np.uint64)
    lib().oracle_table_convert(rows, cols, _p(w), stack_row_count, 1 if transpose else 0, _p(out))
    return out


def matrix_count(words, rows, cols, stack_row_count=1024) -> int:
    w = np.ascontiguousarray(words, dtype=np.uint64)
    return int(lib().oracle_matrix_count(rows, cols, _p(w), stack_row_count))


def matrix_iterate(words, rows, cols, row_map=None, col_map=None, stack_row_count=1024):
    w = np.ascontiguousarray(words, dtype=np.uint64)
    rm = None if row_map is None else np.ascontiguousarray(row_map, dtype=np.uint32)
    cm = None if col_map is None else np.ascontiguousarray(col_map, dtype=np.uint32)
    n = int(lib().oracle_matrix_iterate(rows, cols, _p(w), stack_row_count, _p(rm), _p(cm), None, None))
    r = np.zeros(n, np.uint32)
    c = np.zeros(n, np.uint32)
    lib().oracle_matrix_iterate(rows, cols, _p(w), stack_row_count, _p(rm), _p(cm), _p(r), _p(c))
    return r, c


def matrix_column_count(m: Table, order: int = 0):
    """MatrixColumnCount: (column values, counts); order 0 none, 1 ascending, 2 descending."""
    n = m.t.mcols
    cols = np.zeros(n, np.uint32)
    cnt = np.zeros(n, np.int64)
    if lib().oracle_matrix_column_count(C.byref(m.t), order, _p(cols), _p(cnt)):
        raise ValueError("oracle_matrix_column_count rejected its arguments")
    return cols, cnt


def matrix_row_or_sum(m: Table) -> np.ndarray:
    """MatrixRowOrSum: values of the columns holding any bit, in column order."""
    out = np.zeros(m.t.mcols, np.uint32)
    n = lib().oracle_matrix_row_or_sum(C.byref(m.t), _p(out))
    return out[:n]


def semi_join(a: Table, b: Table, key_vars, only_count=False):
    """SemiJoin<N>: (var, cols, count) for a flat a; (masked words or None, count) for a VarRow a."""
    kv = np.ascontiguousarray(key_vars, dtype=np.int32)
    r = OrResult()
    words = None
    if a.kind != FLAT and not only_count:
        words = np.zeros_like(a.words)
    if lib().oracle_semi_join(C.byref(a.t), C.byref(b.t), _p(kv), len(kv), 1 if only_count else 0,
                              C.byref(r), _p(words)):
        raise ValueError("oracle_semi_join rejected its arguments")
    if a.kind != FLAT:
        return words, int(r.count)
    if only_count:
        return None, None, int(r.count)
    count = int(r.count)
    var, cols, _ = _result(r)
    return var, cols, count


def matrix_filter(m: Table, row_keep=None, row_values=0, col_keep=None, col_values=0, pairs=None, pairs_mode=0):
    """MatrixTableFilter in place on m.words; returns the number of bits cleared."""
    rk = None if row_keep is None else np.ascontiguousarray(row_keep, dtype=np.uint64)
    ck = None if col_keep is None else np.ascontiguousarray(col_keep, dtype=np.uint64)
    pk = None if pairs is None else np.ascontiguousarray(pairs, dtype=np.uint64)
    return int(lib().oracle_matrix_filter(C.byref(m.t), _p(rk), int(row_values), _p(ck), int(col_values), _p(pk),
                                          0 if pk is None else len(pk), int(pairs_mode)))


def vertex_mask_any_neighbor(off, adj, V, prop, value):
    mask = np.zeros((V + 63) // 64, np.uint64)
    o = np.ascontiguousarray(off, dtype=np.int64)
    a = np.ascontiguousarray(adj, dtype=np.uint32)
    pr = np.ascontiguousarray(prop, dtype=np.uint8)
    lib().oracle_vertex_mask_any_neighbor(_p(o), _p(a), int(V), _p(pr), int(value), _p(mask))
    return mask
