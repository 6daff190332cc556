"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import re
from pathlib import Path

from vertexsurge_gb300 import _abi

ROOT = Path(__file__).resolve().parents[1]


def header_symbols():
    syms = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(vs_[a-z_0-9]+)\s*\(", text, re.M):
            syms.add(m.group(1))
    return syms


def test_header_declares_the_operator_set():
    syms = header_symbols()
    for needed in ("vs_expand", "vs_hash_join", "vs_mintersect", "vs_matrix_select", "vs_table_convert",
                   "vs_bitmat_count", "vs_graph_upload", "vs_expand_plan_run"):
        assert needed in syms


def test_library_exports_every_header_symbol():
    lib = ctypes.CDLL(str(_abi.LIB_PATH))
    missing = [s for s in sorted(header_symbols()) if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert header_symbols() <= set(_abi.HEADER_SYMBOLS)


def test_version_string_without_gpu():
    assert b"sm_103a" in _abi.lib().vs_version()
