import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built():
    from vertexsurge_gb300 import build
    build.build_all()
    return True


@pytest.fixture(scope="session")
def vs():
    import vertexsurge_gb300 as vs
    vs.init(0)
    return vs


def words_to_bool(words: np.ndarray, rows: int) -> np.ndarray:
    """Logical words (cols, ceil(rows/64)) -> dense bool matrix (rows, cols)."""
    w = np.ascontiguousarray(words, dtype=np.uint64)
    cols = w.shape[0]
    bits = np.unpackbits(w.view(np.uint8).reshape(cols, -1), axis=1, bitorder="little")
    return bits[:, :rows].T.astype(bool)


def bool_to_words(m: np.ndarray) -> np.ndarray:
    """Dense bool (rows, cols) -> logical words (cols, ceil(rows/64))."""
    rows, cols = m.shape
    W = (rows + 63) // 64
    pad = np.zeros((cols, W * 64), dtype=np.uint8)
    pad[:, :rows] = m.T
    return np.packbits(pad, axis=1, bitorder="little").view(np.uint64).reshape(cols, W).copy()
