"""GPU glue operators against the oracle: Count, MatrixTableSelect,
TableConvert (copy and bit transpose, maps swapped), TableConvert(Flat) /
the matrix iterators — including the reference's own test shapes
(big_operators2.cpp:215-296, bit_matrix_table.cpp:363-483)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import bool_to_words, words_to_bool

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rows,cols", [(1000, 10000), (2000, 10000), (1, 1), (63, 65), (64, 64), (130, 7)])
def test_convert_and_count(vs, rows, cols):
    rng = np.random.default_rng(rows * 31 + cols)
    m = rng.random((rows, cols)) < 0.5
    w = bool_to_words(m)
    rm = rng.integers(0, 1 << 30, rows).astype(np.uint32)
    cm = rng.integers(0, 1 << 30, cols).astype(np.uint32)
    gm = vs.BitMatrix.from_logical(w, rows, cols, kind=1, row_map=rm, col_map=cm)
    assert gm.count() == int(m.sum()) == O.matrix_count(w, rows, cols)
    for transpose in (False, True):
        t = gm.convert(transpose)
        got = t.download()
        exp = O.table_convert(w, rows, cols, transpose)
        assert np.array_equal(got, exp)
        r2, c2 = t.maps()
        assert np.array_equal(r2, cm if transpose else rm)
        assert np.array_equal(c2, rm if transpose else cm)
        assert t.info().kind == 2


def test_select(vs):
    rng = np.random.default_rng(3)
    rows, cols = 700, 3000
    m = rng.random((rows, cols)) < 0.1
    w = bool_to_words(m)
    rm = np.arange(rows, dtype=np.uint32) * 3
    gm = vs.BitMatrix.from_logical(w, rows, cols, kind=1, row_map=rm)
    t = rng.integers(0, cols, 555).astype(np.uint32)
    t[:10] = t[0]  # duplicates are kept
    s = gm.select(t)
    assert np.array_equal(s.download(), O.matrix_select(w, rows, cols, t))
    r2, c2 = s.maps()
    assert np.array_equal(c2, t) and np.array_equal(r2, rm)
    with pytest.raises(vs.VsError):
        gm.select(np.array([cols], np.uint32))
    with pytest.raises(vs.VsError):
        s.select(np.array([0], np.uint32))  # a matrix with a col_map (reference asserts)


def test_iterator_round_trip(vs):
    rng = np.random.default_rng(123)
    rows, cols = 2000, 10000
    m = rng.random((rows, cols)) < 0.5
    w = bool_to_words(m)
    rm = rng.permutation(1 << 20)[:rows].astype(np.uint32)
    gm = vs.BitMatrix.from_logical(w, rows, cols, kind=1, row_map=rm)
    r, c = gm.to_flat().columns()
    orr, occ = O.matrix_iterate(w, rows, cols, row_map=rm)
    assert len(r) == len(orr) == int(m.sum())
    a = np.sort(r.astype(np.uint64) << 32 | c)
    b = np.sort(orr.astype(np.uint64) << 32 | occ)
    assert np.array_equal(a, b)


def test_upload_masks_padding_bits(vs):
    rows, cols = 10, 3
    w = np.full((cols, 1), ~np.uint64(0), dtype=np.uint64)
    gm = vs.BitMatrix.from_logical(w, rows, cols)
    assert gm.count() == rows * cols
    assert np.array_equal(words_to_bool(gm.download(), rows), np.ones((rows, cols), bool))
