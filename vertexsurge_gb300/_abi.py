"""ctypes binding of the C ABI in include/vertexsurge_gb300.h.

This is the Python-side view of the drop-in boundary: every call goes to
libvsgb300.so (hand-written sm_103a CUDA).  There is no fallback: if the
library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libvsgb300.so"

VS_OK, VS_ERR_ARG, VS_ERR_OOM, VS_ERR_CUDA, VS_ERR_TIMEOUT, VS_ERR_UNSUPPORTED, VS_ERR_CAPACITY = range(7)
DIR_FORWARD, DIR_BACKWARD, DIR_BOTH = 0, 1, 2
PATH_ANY, PATH_SHORTEST, PATH_FIND_SHORTEST = 0, 1, 2
STRAT_AUTO, STRAT_PULL, STRAT_PUSH, STRAT_SPARSE = 0, 1, 2, 3
KIND_VARROW, KIND_COLMAIN = 1, 2
T_VID, T_I64 = 0, 1
MAX_HOPS = 64

_DIRS = {"forward": DIR_FORWARD, "backward": DIR_BACKWARD, "both": DIR_BOTH}
_PATHS = {"any": PATH_ANY, "shortest": PATH_SHORTEST, "find_shortest": PATH_FIND_SHORTEST}
_STRATS = {"auto": STRAT_AUTO, "pull": STRAT_PULL, "push": STRAT_PUSH, "sparse": STRAT_SPARSE}


class VsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"vertexsurge_gb300 error {code}: {msg}")
        self.code = code


class ExpandParams(C.Structure):
    _fields_ = [("k_min", C.c_uint32), ("k_max", C.c_uint32), ("path_type", C.c_int32),
                ("direction", C.c_int32), ("strategy", C.c_int32), ("use_picker", C.c_int32),
                ("hub_threshold", C.c_uint32), ("slice_words", C.c_uint32),
                ("pair_capacity", C.c_uint64), ("pull_kernel", C.c_int32), ("reserved", C.c_int32),
                ("sparse_frac", C.c_double), ("short_share", C.c_double)]


class ExpandStats(C.Structure):
    _fields_ = [("hops_run", C.c_uint32), ("found", C.c_uint32), ("visit_count", C.c_uint64),
                ("new_bits", C.c_uint64 * (MAX_HOPS + 1)),
                ("active_vertices", C.c_uint64 * (MAX_HOPS + 1)),
                ("active_edges", C.c_uint64 * (MAX_HOPS + 1)),
                ("pairs", C.c_uint64 * (MAX_HOPS + 1)),
                ("strategy", C.c_int32 * (MAX_HOPS + 1)),
                ("hop_ms", C.c_float * (MAX_HOPS + 1)),
                ("pull_ms", C.c_float * (MAX_HOPS + 1)),
                ("short_pull", C.c_int32 * (MAX_HOPS + 1)),
                ("short_rows", C.c_uint64 * (MAX_HOPS + 1)),
                ("short_edges", C.c_uint64 * (MAX_HOPS + 1)),
                ("tiny_rows", C.c_uint64 * (MAX_HOPS + 1))]

    def as_dict(self) -> dict:
        n = self.hops_run + 1
        return {"hops_run": self.hops_run, "found": self.found, "visit_count": self.visit_count,
                "new_bits": list(self.new_bits[:n]), "active_vertices": list(self.active_vertices[:n]),
                "active_edges": list(self.active_edges[:n]), "pairs": list(self.pairs[:n]),
                "strategy": list(self.strategy[:n]), "hop_ms": list(self.hop_ms[:n]),
                "pull_ms": list(self.pull_ms[:n]), "short_pull": list(self.short_pull[:n]),
                "short_rows": list(self.short_rows[:n]), "short_edges": list(self.short_edges[:n]),
                "tiny_rows": list(self.tiny_rows[:n])}


class BitmatInfo(C.Structure):
    _fields_ = [("rows", C.c_uint32), ("cols", C.c_uint32), ("wpc", C.c_uint32), ("kind", C.c_int32),
                ("has_row_map", C.c_int32), ("has_col_map", C.c_int32), ("words", C.c_void_p)]


class TableRef(C.Structure):
    _fields_ = [("flat", C.c_void_p), ("mat", C.c_void_p), ("key_col", C.c_uint32)]


class IsectDep(C.Structure):
    _fields_ = [("mat", C.c_void_p), ("flat", C.c_void_p), ("graph", C.c_void_p),
                ("direction", C.c_int32), ("u_col", C.c_uint32), ("nv_col", C.c_uint32),
                ("base_col", C.c_uint32), ("algo", C.c_int32)]


ISECT_ALGOS = {"auto": 0, "binary": 1, "merge": 2, "bitmap": 3}


_lib = None

# (name, restype, argtypes) for every entry point of the header
_SIGS = [
    ("vs_last_error", C.c_char_p, []),
    ("vs_version", C.c_char_p, []),
    ("vs_kernel_launches", C.c_uint64, []),
    ("vs_expand_plan_set_tuning", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_int]),
    ("vs_init", C.c_int, [C.c_int]),
    ("vs_graph_upload", C.c_int, [C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("vs_graph_info", C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64),
                                C.POINTER(C.c_int)]),
    ("vs_graph_free", C.c_int, [C.c_void_p]),
    ("vs_bitmat_create", C.c_int, [C.c_uint32, C.c_uint32, C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("vs_bitmat_upload", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("vs_bitmat_download", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("vs_bitmat_set_maps", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("vs_bitmat_get_maps", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("vs_bitmat_get_info", C.c_int, [C.c_void_p, C.POINTER(BitmatInfo)]),
    ("vs_bitmat_free", C.c_int, [C.c_void_p]),
    ("vs_bitmat_count", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.c_void_p]),
    ("vs_matrix_select", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p), C.c_void_p]),
    ("vs_table_convert", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.c_void_p]),
    ("vs_bitmat_to_flat", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p]),
    ("vs_flat_create", C.c_int, [C.c_uint32, C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    ("vs_flat_upload", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("vs_flat_download", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("vs_flat_info", C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.c_void_p]),
    ("vs_flat_free", C.c_int, [C.c_void_p]),
    ("vs_expand_plan_create", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(ExpandParams),
                                        C.POINTER(C.c_void_p)]),
    ("vs_expand_plan_run", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("vs_expand_plan_result", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("vs_expand_plan_stats", C.c_int, [C.c_void_p, C.POINTER(ExpandStats), C.c_void_p]),
    ("vs_expand_plan_free", C.c_int, [C.c_void_p]),
    ("vs_expand_plan_footprint", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(ExpandParams),
                                           C.POINTER(C.c_uint64)]),
    ("vs_expand", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(ExpandParams), C.c_void_p,
                            C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(ExpandStats), C.c_void_p]),
    ("vs_hash_join", C.c_int, [TableRef, TableRef, C.c_int, C.c_uint64, C.POINTER(C.c_void_p),
                               C.POINTER(C.c_uint64), C.c_void_p]),
    ("vs_mintersect", C.c_int, [TableRef, C.POINTER(IsectDep), C.c_uint32, C.c_uint32, C.c_int,
                                C.c_uint64, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.c_void_p]),
    ("vs_hash_join_count_noalloc", C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_int,
                                             C.c_void_p, C.c_void_p]),
]

_SIGS += [
    ("vs_picker_create", C.c_int, [C.c_uint64, C.POINTER(C.c_void_p)]),
    ("vs_picker_free", C.c_int, [C.c_void_p]),
    ("vs_picker_num_params", C.c_int, []),
    ("vs_picker_set_params", C.c_int, [C.c_void_p, C.c_void_p]),
    ("vs_picker_get_params", C.c_int, [C.c_void_p, C.c_void_p]),
    ("vs_picker_forward", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    ("vs_picker_backward", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                                     C.POINTER(C.c_float), C.c_void_p]),
    ("vs_picker_train", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32,
                                  C.c_float, C.c_uint64, C.POINTER(C.c_float), C.c_void_p]),
    ("vs_picker_predict", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    ("vs_expand_plan_set_picker", C.c_int, [C.c_void_p, C.c_void_p]),
    ("vs_expand_plan_set_hop_strategies", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    ("vs_expand_plan_log_features", C.c_int, [C.c_void_p, C.c_int]),
    ("vs_expand_plan_set_row_limits", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    ("vs_expand_plan_set_pull_kernel", C.c_int, [C.c_void_p, C.c_int]),
    ("vs_expand_plan_set_row_limits_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    ("vs_capture_begin", C.c_int, [C.c_void_p]),
    ("vs_capture_end", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("vs_captured_launch", C.c_int, [C.c_void_p, C.c_void_p]),
    ("vs_captured_kernels", C.c_uint64, [C.c_void_p]),
    ("vs_captured_free", C.c_int, [C.c_void_p]),
    ("vs_hash_join_count_row_blocks", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                                C.c_void_p]),
    ("vs_matrix_column_count", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.c_void_p]),
    ("vs_select_ids_in_range", C.c_int, [C.c_void_p, C.c_int, C.c_uint32, C.c_int64, C.c_int64,
                                         C.POINTER(C.c_void_p), C.c_void_p]),
    ("vs_flat_column", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p)]),
    ("vs_mintersect_ex", C.c_int, [TableRef, C.POINTER(IsectDep), C.c_uint32, C.c_uint32, C.c_int, C.c_uint64,
                                   C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64),
                                   C.c_void_p]),
    ("vs_expand_layers", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(ExpandParams),
                                   C.POINTER(C.c_void_p), C.POINTER(C.c_uint32), C.c_void_p]),
    ("vs_layers_to_flat", C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p),
                                    C.c_void_p]),
    ("vs_layers_to_flat_first", C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.c_uint32,
                                          C.POINTER(C.c_void_p), C.c_void_p]),
    ("vs_matrix_row_or_sum", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p]),
    ("vs_semi_join", C.c_int, [TableRef, TableRef, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int,
                               C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.c_void_p]),
    ("vs_expand_plan_features", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("vs_release_cached", C.c_int, []),
    ("vs_matrix_filter", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                   C.c_uint64, C.c_int, C.c_void_p]),
    ("vs_vertex_mask_any_neighbor", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_uint32, C.c_uint8,
                                              C.c_void_p, C.c_void_p]),
]

# internal entry points (not part of the header)
_EXTRA_SIGS = []

HEADER_SYMBOLS = [s[0] for s in _SIGS]


def lib() -> C.CDLL:
    """Load libvsgb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run vertexsurge_gb300.build.build_all() "
                               "(the CUDA extension is required; there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in _SIGS + _EXTRA_SIGS:
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> int:
    if rc not in (VS_OK,):
        raise VsError(rc, lib().vs_last_error().decode())
    return rc


def init(device: int = 0) -> None:
    check(lib().vs_init(device))


def kernel_launches() -> int:
    return int(lib().vs_kernel_launches())


def release_cached() -> None:
    """Free the idle expand plans the library keeps for one-shot expands."""
    check(lib().vs_release_cached())


def _ptr(a) -> C.c_void_p:
    """Pointer of a numpy array (host) or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return C.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if isinstance(a, int):
        return C.c_void_p(a)
    raise TypeError(type(a))


def _stream(s) -> C.c_void_p:
    if s is None:
        return None
    if hasattr(s, "cuda_stream"):
        return C.c_void_p(s.cuda_stream)
    return C.c_void_p(int(s))


class DeviceGraph:
    """A CSR graph resident in HBM (vs_graph)."""

    def __init__(self, V, E, fwd_off, fwd_dst, rev_off, rev_src, directed=True, stream=None):
        self.h = None
        h = C.c_void_p()
        check(lib().vs_graph_upload(V, E, _ptr(fwd_off), _ptr(fwd_dst), _ptr(rev_off), _ptr(rev_src),
                                    1 if directed else 0, _stream(stream), C.byref(h)))
        self.h = h
        self.V, self.E, self.directed = int(V), int(E), bool(directed)

    @classmethod
    def from_host(cls, g, stream=None) -> "DeviceGraph":
        return cls(g.V, g.E, g.fwd_off, g.fwd_dst, g.rev_off, g.rev_src, g.directed, stream)

    def free(self):
        if self.h:
            lib().vs_graph_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class BitMatrix:
    """A device bit matrix handle (vs_bitmat)."""

    def __init__(self, h: C.c_void_p, owner=None):
        self.h = h
        self._owner = owner  # keeps a plan alive for borrowed views

    @classmethod
    def create(cls, rows, cols, kind=KIND_VARROW, stream=None):
        h = C.c_void_p()
        check(lib().vs_bitmat_create(rows, cols, kind, _stream(stream), C.byref(h)))
        return cls(h)

    @classmethod
    def from_logical(cls, words: np.ndarray, rows: int, cols: int, kind=KIND_VARROW,
                     row_map=None, col_map=None, stream=None):
        m = cls.create(rows, cols, kind, stream)
        words = np.ascontiguousarray(words, dtype=np.uint64)
        assert words.size == cols * ((rows + 63) // 64)
        check(lib().vs_bitmat_upload(m.h, _ptr(words), _stream(stream)))
        if row_map is not None or col_map is not None:
            rm = None if row_map is None else np.ascontiguousarray(row_map, dtype=np.uint32)
            cm = None if col_map is None else np.ascontiguousarray(col_map, dtype=np.uint32)
            check(lib().vs_bitmat_set_maps(m.h, _ptr(rm), _ptr(cm), _stream(stream)))
        return m

    def info(self) -> BitmatInfo:
        inf = BitmatInfo()
        check(lib().vs_bitmat_get_info(self.h, C.byref(inf)))
        return inf

    @property
    def shape(self):
        i = self.info()
        return i.rows, i.cols

    def download(self, stream=None) -> np.ndarray:
        """Logical words, shape (cols, ceil(rows/64))."""
        i = self.info()
        out = np.zeros((i.cols, (i.rows + 63) // 64), dtype=np.uint64)
        check(lib().vs_bitmat_download(self.h, _ptr(out), _stream(stream)))
        return out

    def maps(self, stream=None):
        i = self.info()
        rm = np.zeros(i.rows, np.uint32) if i.has_row_map else None
        cm = np.zeros(i.cols, np.uint32) if i.has_col_map else None
        check(lib().vs_bitmat_get_maps(self.h, _ptr(rm), _ptr(cm), _stream(stream)))
        return rm, cm

    def count(self, stream=None) -> int:
        c = C.c_uint64()
        check(lib().vs_bitmat_count(self.h, C.byref(c), _stream(stream)))
        return int(c.value)

    def select(self, targets: np.ndarray, stream=None) -> "BitMatrix":
        t = np.ascontiguousarray(targets, dtype=np.uint32)
        h = C.c_void_p()
        check(lib().vs_matrix_select(self.h, _ptr(t), len(t), C.byref(h), _stream(stream)))
        return BitMatrix(h)

    def convert(self, transpose: bool, stream=None) -> "BitMatrix":
        h = C.c_void_p()
        check(lib().vs_table_convert(self.h, 1 if transpose else 0, C.byref(h), _stream(stream)))
        return BitMatrix(h)

    def to_flat(self, stream=None) -> "FlatTable":
        h = C.c_void_p()
        check(lib().vs_bitmat_to_flat(self.h, C.byref(h), _stream(stream)))
        return FlatTable(h)

    def free(self):
        if self.h:
            lib().vs_bitmat_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class FlatTable:
    """A device flat table handle (vs_flat): columns of uint32 (VID) or int64."""

    def __init__(self, h: C.c_void_p):
        self.h = h

    @classmethod
    def from_columns(cls, cols, stream=None) -> "FlatTable":
        types = []
        arrs = []
        for c in cols:
            c = np.ascontiguousarray(c)
            if c.dtype == np.int64:
                types.append(T_I64)
            else:
                c = c.astype(np.uint32)
                types.append(T_VID)
            arrs.append(np.ascontiguousarray(c))
        n = len(arrs[0])
        assert all(len(a) == n for a in arrs)
        t = (C.c_int32 * len(types))(*types)
        h = C.c_void_p()
        check(lib().vs_flat_create(len(arrs), t, n, C.byref(h)))
        f = cls(h)
        for i, a in enumerate(arrs):
            check(lib().vs_flat_upload(h, i, _ptr(a), _stream(stream)))
        return f

    def info(self):
        nc = C.c_uint32()
        nr = C.c_uint64()
        types = (C.c_int32 * 16)()
        check(lib().vs_flat_info(self.h, C.byref(nc), C.byref(nr), types))
        return int(nc.value), int(nr.value), list(types[: nc.value])

    def columns(self, stream=None) -> list:
        nc, nr, types = self.info()
        out = []
        for i, t in enumerate(types):
            a = np.zeros(nr, dtype=np.int64 if t == T_I64 else np.uint32)
            check(lib().vs_flat_download(self.h, i, _ptr(a), _stream(stream)))
            out.append(a)
        return out

    def free(self):
        if self.h:
            lib().vs_flat_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def make_params(k_min, k_max, path="any", direction="forward", strategy="auto", use_picker=False,
                hub_threshold=0, slice_words=0, pair_capacity=0, pull_kernel=0, sparse_frac=0.0,
                short_share=0.0) -> ExpandParams:
    p = ExpandParams()
    p.k_min, p.k_max = int(k_min), int(k_max)
    p.path_type = _PATHS[path] if isinstance(path, str) else int(path)
    p.direction = _DIRS[direction] if isinstance(direction, str) else int(direction)
    p.strategy = _STRATS[strategy] if isinstance(strategy, str) else int(strategy)
    p.use_picker = 1 if use_picker else 0
    p.hub_threshold = int(hub_threshold)
    p.slice_words = int(slice_words)
    p.pair_capacity = int(pair_capacity)
    p.pull_kernel = int(pull_kernel)
    p.sparse_frac = float(sparse_frac)
    p.short_share = float(short_share)
    return p


class Captured:
    """A CUDA graph recorded from library calls on one stream (vs_capture_*).

    Use as a context manager around the calls to record:
        with vs.Captured(stream) as cg: plan.run(dsrc, stream=stream); ...
        cg.launch(stream)
    Objects the recorded calls use (plans, tensors) must outlive it: pass them
    as `keep`."""

    def __init__(self, stream, keep=()):
        self.stream, self.h, self._keep = stream, None, list(keep)

    def __enter__(self):
        check(lib().vs_capture_begin(_stream(self.stream)))
        return self

    def __exit__(self, et, ev, tb):
        h = C.c_void_p()
        rc = lib().vs_capture_end(_stream(self.stream), C.byref(h))
        if et is None:
            check(rc)
            self.h = h
        elif rc == 0 and h.value:  # the recorded calls raised: drop the partial graph
            lib().vs_captured_free(h)
        return False

    def keep(self, *objs):
        self._keep.extend(objs)

    @property
    def kernels(self) -> int:
        return int(lib().vs_captured_kernels(self.h)) if self.h else 0

    def launch(self, stream=None):
        check(lib().vs_captured_launch(self.h, _stream(stream if stream is not None else self.stream)))

    def free(self):
        if self.h:
            lib().vs_captured_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


MAX_ROW_BLOCKS = 512  # VS_MAX_ROW_BLOCKS


class RowBlock(C.Structure):
    _fields_ = [("row_begin", C.c_uint32), ("row_end", C.c_uint32),
                ("key_begin", C.c_uint64), ("key_end", C.c_uint64)]


def join_count_row_blocks(m: "BitMatrix", keys, blocks, counts, stream=None):
    """Per row block q: count of HashJoin(rows of q of m, keys[key_begin:key_end]) on
    the vertex id (vs_hash_join_count_row_blocks).  keys: device int32/uint32 tensor;
    counts: device int64 tensor of len(blocks), overwritten in stream order;
    blocks: [(row_begin, row_end, key_begin, key_end)]."""
    arr = (RowBlock * len(blocks))(*[RowBlock(*map(int, b)) for b in blocks])
    check(lib().vs_hash_join_count_row_blocks(m.h, _ptr(keys), arr, len(blocks), _ptr(counts),
                                              _stream(stream)))


def plan_footprint(graph: "DeviceGraph", S: int, params: ExpandParams) -> int:
    """Device bytes an expand plan for S sources allocates."""
    b = C.c_uint64()
    check(lib().vs_expand_plan_footprint(graph.h, S, C.byref(params), C.byref(b)))
    return int(b.value)


class ExpandPlan:
    """Reusable expand workspace (vs_expand_plan)."""

    def __init__(self, graph: DeviceGraph, S: int, params: ExpandParams):
        h = C.c_void_p()
        check(lib().vs_expand_plan_create(graph.h, S, C.byref(params), C.byref(h)))
        self.h = h
        self.graph = graph
        self.S = S
        self.params = params

    def set_tuning(self, sparse_frac=-1.0, push_frac=-1.0, collect_stats=False, timing=False):
        check(lib().vs_expand_plan_set_tuning(self.h, sparse_frac, push_frac, 1 if collect_stats else 0,
                                              1 if timing else 0))

    def run(self, sources, targets=None, distances=None, stream=None):
        check(lib().vs_expand_plan_run(self.h, _ptr(sources), _ptr(targets), _ptr(distances),
                                       _stream(stream)))

    def result(self) -> BitMatrix:
        h = C.c_void_p()
        check(lib().vs_expand_plan_result(self.h, C.byref(h)))
        return BitMatrix(h, owner=self)

    def set_picker(self, picker):
        check(lib().vs_expand_plan_set_picker(self.h, picker.h if picker is not None else None))
        self._picker = picker

    def set_hop_strategies(self, strategies):
        """strategies[h] for h = 1..k_max ('auto'/'pull'/'push'/'sparse' or codes); None clears."""
        if strategies is None:
            check(lib().vs_expand_plan_set_hop_strategies(self.h, None, 0))
            return
        arr = np.zeros(len(strategies), dtype=np.int32)
        for i, x in enumerate(strategies):
            arr[i] = _STRATS[x] if isinstance(x, str) else int(x)
        check(lib().vs_expand_plan_set_hop_strategies(self.h, _ptr(arr), len(arr)))

    def set_row_limits_device(self, row_kmax, n: int, stream=None):
        """Row limits from a device uint8 tensor (stream-ordered, capturable)."""
        check(lib().vs_expand_plan_set_row_limits_device(self.h, _ptr(row_kmax), int(n), _stream(stream)))

    def set_pull_kernel(self, kind: int):
        """PULL kernel variant 0..3 (bit 0: 8 blocks/SM, bit 1: L2 cache policies)."""
        check(lib().vs_expand_plan_set_pull_kernel(self.h, int(kind)))

    def set_row_limits(self, row_kmax):
        """Per-row last hop (batched queries); None removes the limits."""
        if row_kmax is None:
            check(lib().vs_expand_plan_set_row_limits(self.h, None, 0))
            return
        a = np.ascontiguousarray(row_kmax, dtype=np.uint8)
        check(lib().vs_expand_plan_set_row_limits(self.h, _ptr(a), len(a)))

    def log_features(self, on=True):
        check(lib().vs_expand_plan_log_features(self.h, 1 if on else 0))

    def features(self, stream=None) -> np.ndarray:
        out = np.zeros((MAX_HOPS + 1, 32), dtype=np.float32)
        check(lib().vs_expand_plan_features(self.h, _ptr(out), _stream(stream)))
        return out

    def stats(self, stream=None) -> dict:
        s = ExpandStats()
        check(lib().vs_expand_plan_stats(self.h, C.byref(s), _stream(stream)))
        return s.as_dict()

    def free(self):
        if self.h:
            lib().vs_expand_plan_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def expand(graph: DeviceGraph, sources, k_min, k_max, path="any", direction="forward",
           strategy="auto", targets=None, stream=None, stats=False, **kw):
    """One-shot VExpand. Returns (BitMatrix or None, distances or None, stats dict or None).
    sources: numpy array, or a torch tensor (host, pinned or device) of 32-bit ids."""
    if hasattr(sources, "data_ptr"):
        src = sources
        S = int(sources.numel())
    else:
        src = np.ascontiguousarray(sources, dtype=np.uint32)
        S = len(src)
    p = make_params(k_min, k_max, path, direction, strategy, **kw)
    dist = None
    tg = None
    if p.path_type == PATH_FIND_SHORTEST:
        tg = np.ascontiguousarray(targets, dtype=np.uint32)
        dist = np.zeros(S, dtype=np.int32)
    out = C.c_void_p()
    st = ExpandStats() if stats else None
    check(lib().vs_expand(graph.h, _ptr(src), S, C.byref(p), _ptr(tg), _ptr(dist),
                          None if p.path_type == PATH_FIND_SHORTEST else C.byref(out),
                          C.byref(st) if st is not None else None, _stream(stream)))
    m = BitMatrix(out) if out.value else None
    return m, dist, (st.as_dict() if st is not None else None)


def hash_join(a, b, key_a=0, key_b=0, only_count=False, max_rows=1 << 62, stream=None):
    """HashJoin over two operands (FlatTable with key column, or a ColMain BitMatrix).
    Returns (FlatTable or None, exact count, truncated flag)."""
    ra, rb = TableRef(), TableRef()
    for r, t, k in ((ra, a, key_a), (rb, b, key_b)):
        if isinstance(t, FlatTable):
            r.flat = t.h
        else:
            r.mat = t.h
        r.key_col = k
    out = C.c_void_p()
    cnt = C.c_uint64()
    rc = lib().vs_hash_join(ra, rb, 1 if only_count else 0, max_rows,
                            None if only_count else C.byref(out), C.byref(cnt), _stream(stream))
    truncated = rc == VS_ERR_CAPACITY
    if not truncated:
        check(rc)
    return (FlatTable(out) if out.value else None), int(cnt.value), truncated


def mintersect(base, deps, new_vertex_count=0, only_count=False, max_rows=1 << 62, stream=None,
               method_picker=None, features=False):
    """Mintersect. deps: list of dicts with keys mat/flat/graph, direction, u_col, nv_col, base_col
    and, for graph adjacency, algo ('auto', 'binary', 'merge', 'bitmap').  method_picker: a Picker
    trained on intersection timings that chooses the method of 'auto' adjacency deps on the device;
    features=True appends the call's 32 features to the returned tuple."""
    rb = TableRef()
    if isinstance(base, FlatTable):
        rb.flat = base.h
    else:
        rb.mat = base.h
    arr = (IsectDep * len(deps))()
    for i, d in enumerate(deps):
        arr[i].mat = d["mat"].h if d.get("mat") is not None else None
        arr[i].flat = d["flat"].h if d.get("flat") is not None else None
        arr[i].graph = d["graph"].h if d.get("graph") is not None else None
        arr[i].direction = _DIRS.get(d.get("direction", "forward"), 0) if isinstance(
            d.get("direction", "forward"), str) else int(d["direction"])
        arr[i].u_col = d.get("u_col", 0)
        arr[i].nv_col = d.get("nv_col", 1)
        arr[i].base_col = d.get("base_col", 0)
        al = d.get("algo", "auto")
        arr[i].algo = ISECT_ALGOS[al] if isinstance(al, str) else int(al)
    out = C.c_void_p()
    cnt = C.c_uint64()
    feat = np.zeros(32, np.float32) if features else None
    if method_picker is not None or features:
        rc = lib().vs_mintersect_ex(rb, arr, len(deps), new_vertex_count, 1 if only_count else 0, max_rows,
                                    method_picker.h if method_picker is not None else None, _ptr(feat),
                                    None if only_count else C.byref(out), C.byref(cnt), _stream(stream))
    else:
        rc = lib().vs_mintersect(rb, arr, len(deps), new_vertex_count, 1 if only_count else 0, max_rows,
                                 None if only_count else C.byref(out), C.byref(cnt), _stream(stream))
    truncated = rc == VS_ERR_CAPACITY
    if not truncated:
        check(rc)
    res = (FlatTable(out) if out.value else None), int(cnt.value), truncated
    return res + (feat,) if features else res


def expand_layers(graph: "DeviceGraph", sources, k_min, k_max, path="shortest", direction="forward",
                  stream=None, **kw) -> list:
    """VExpand with distances (Dense): [(h, BitMatrix of layer h)] for h = k_min..k_actual."""
    src = np.ascontiguousarray(sources, dtype=np.uint32)
    p = make_params(k_min, k_max, path, direction, **kw)
    n = k_max - k_min + 1
    arr = (C.c_void_p * n)()
    got = C.c_uint32()
    check(lib().vs_expand_layers(graph.h, _ptr(src), len(src), C.byref(p), arr, C.byref(got), _stream(stream)))
    return [(k_min + i, BitMatrix(C.c_void_p(arr[i]))) for i in range(got.value)]


def layers_to_flat(layers: list, stream=None, first=False) -> "FlatTable":
    """(row value, column value, distance) tuples of [(distance, BitMatrix)];
    first=True keeps each (row, column) pair once, at its smallest distance."""
    hs = (C.c_void_p * max(1, len(layers)))(*[m.h for _, m in layers])
    d = np.ascontiguousarray([h for h, _ in layers], dtype=np.int32)
    out = C.c_void_p()
    fn = lib().vs_layers_to_flat_first if first else lib().vs_layers_to_flat
    check(fn(hs, _ptr(d), len(layers), C.byref(out), _stream(stream)))
    return FlatTable(out)


def select_ids_in_range(values, lo, hi, stream=None) -> "FlatTable":
    """Scan filter: ids i with lo <= values[i] <= hi; values a device torch tensor of
    uint8/int16/int32/int64 (or None with an int n meaning every id < n)."""
    if isinstance(values, int):
        ptr, nbytes, n = None, 0, values
    else:
        ptr, nbytes, n = _ptr(values), values.element_size(), values.numel()
    out = C.c_void_p()
    check(lib().vs_select_ids_in_range(ptr, nbytes, n, int(lo), int(hi), C.byref(out), _stream(stream)))
    return FlatTable(out)


def matrix_column_count(m: "BitMatrix", order=0, stream=None) -> "FlatTable":
    """MatrixColumnCount: (column value VID, count I64) per column; order 0/1/2 or
    None/'asc'/'desc'."""
    o = {None: 0, "asc": 1, "desc": 2}.get(order, order)
    out = C.c_void_p()
    check(lib().vs_matrix_column_count(m.h, int(o), C.byref(out), _stream(stream)))
    return FlatTable(out)


def matrix_row_or_sum(m: "BitMatrix", stream=None) -> "FlatTable":
    """MatrixRowOrSum: the values of the columns holding any bit."""
    out = C.c_void_p()
    check(lib().vs_matrix_row_or_sum(m.h, C.byref(out), _stream(stream)))
    return FlatTable(out)


def matrix_filter(m: "BitMatrix", row_keep=None, row_values=0, col_keep=None, col_values=0, pairs=None,
                  pairs_mode=0, stream=None):
    """MatrixTableFilter in place: keep bit (r, c) when row value r is in the row_keep
    bitset, column value c in the col_keep bitset and (r, c) passes the pair list
    (pairs_mode 1: listed pairs only, 2: all but listed; keys r << 32 | c, sorted).
    Arrays: numpy uint64 (host, copied in by the call) or torch device tensors."""
    def arr(x):
        return None if x is None or hasattr(x, "data_ptr") else np.ascontiguousarray(x, dtype=np.uint64)

    rk = row_keep if hasattr(row_keep, "data_ptr") else arr(row_keep)
    ck = col_keep if hasattr(col_keep, "data_ptr") else arr(col_keep)
    pk = pairs if hasattr(pairs, "data_ptr") else arr(pairs)
    npairs = 0 if pk is None else (int(pk.numel()) if hasattr(pk, "numel") else len(pk))
    check(lib().vs_matrix_filter(m.h, _ptr(rk), int(row_values), _ptr(ck), int(col_values), _ptr(pk), npairs,
                                 int(pairs_mode), _stream(stream)))


def vertex_mask_any_neighbor(graph: "DeviceGraph", prop, value: int, direction="forward", stream=None):
    """Bitset (numpy uint64, ceil(V/64) words): bit v set when a neighbour u of v in the
    graph has prop[u] == value (prop: uint8 numpy array or device tensor)."""
    p = prop if hasattr(prop, "data_ptr") else np.ascontiguousarray(prop, dtype=np.uint8)
    n = int(p.numel()) if hasattr(p, "numel") else len(p)
    mask = np.zeros((graph.V + 63) // 64, np.uint64)
    check(lib().vs_vertex_mask_any_neighbor(graph.h, _DIRS[direction], _ptr(p), n, int(value), _ptr(mask),
                                            _stream(stream)))
    return mask


def semi_join(a, b, a_keys, b_keys, only_count=False, stream=None):
    """SemiJoin over key columns a_keys / b_keys (matrix: 0 row, 1 column).
    Returns (FlatTable or BitMatrix or None, count)."""
    ra, rb = TableRef(), TableRef()
    for r, t in ((ra, a), (rb, b)):
        if isinstance(t, FlatTable):
            r.flat = t.h
        else:
            r.mat = t.h
    ak = np.ascontiguousarray(a_keys, dtype=np.uint32)
    bk = np.ascontiguousarray(b_keys, dtype=np.uint32)
    assert len(ak) == len(bk)
    of, om, cnt = C.c_void_p(), C.c_void_p(), C.c_uint64()
    check(lib().vs_semi_join(ra, rb, len(ak), _ptr(ak), _ptr(bk), 1 if only_count else 0, C.byref(of),
                             C.byref(om), C.byref(cnt), _stream(stream)))
    res = FlatTable(of) if of.value else (BitMatrix(om) if om.value else None)
    return res, int(cnt.value)


class Picker:
    """The learned per-hop strategy picker (vs_picker): 32-64-64-3 MLP,
    bf16 weights, trained by the library's CUDA kernels."""

    def __init__(self, seed: int = 1):
        h = C.c_void_p()
        check(lib().vs_picker_create(seed, C.byref(h)))
        self.h = h
        self.nparam = int(lib().vs_picker_num_params())

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparam, dtype=np.float32)
        check(lib().vs_picker_get_params(self.h, _ptr(out)))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparam
        check(lib().vs_picker_set_params(self.h, _ptr(p)))

    def forward(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros((X.shape[0], 3), dtype=np.float32)
        check(lib().vs_picker_forward(self.h, _ptr(X), X.shape[0], _ptr(out), None))
        return out

    def backward(self, X: np.ndarray, y: np.ndarray):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.int32)
        g = np.zeros(self.nparam, dtype=np.float32)
        loss = C.c_float()
        check(lib().vs_picker_backward(self.h, _ptr(X), _ptr(y), X.shape[0], _ptr(g), C.byref(loss), None))
        return g, float(loss.value)

    def train(self, X, y, epochs=30, batch=512, lr=3e-3, seed=7) -> float:
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.int32)
        loss = C.c_float()
        check(lib().vs_picker_train(self.h, _ptr(X), _ptr(y), X.shape[0], epochs, batch, lr, seed,
                                    C.byref(loss), None))
        return float(loss.value)

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros(X.shape[0], dtype=np.int32)
        check(lib().vs_picker_predict(self.h, _ptr(X), X.shape[0], _ptr(out), None))
        return out

    def free(self):
        if self.h:
            lib().vs_picker_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
