"""Packing of batched queries into waves (host logic, no GPU)."""
import numpy as np
import pytest

from vertexsurge_gb300 import batch


def _q(n, k):
    return batch.Query(np.arange(n, dtype=np.uint32), k, np.zeros(1, np.uint32))


def test_pack_respects_width_and_groups_by_last_hop():
    qs = [_q(100, 2), _q(300, 6), _q(50, 6), _q(400, 3), _q(10, 2), _q(500, 4)]
    waves = batch.pack(qs, 512)
    assert sorted(i for w in waves for i in w) == list(range(len(qs)))
    for w in waves:
        assert sum(len(qs[i].sources) for i in w) <= 512
    order = [i for w in waves for i in w]
    ks = [qs[i].k_max for i in order]
    assert ks == sorted(ks, reverse=True)


def test_pack_rejects_oversize_query():
    with pytest.raises(ValueError):
        batch.pack([_q(600, 2)], 512)
