"""The allocation-free count-only join (vs_hash_join_count_noalloc) against
the allocating entry point (vs_hash_join with only_count = 1), through the C
ABI, on two calls in a row.

Its callers are engines that cannot call cudaMalloc while answering a query
(all device memory is handed to their own allocator up front), so the hash
table lives in a fixed device array of the library; the second call checks
that the table left behind by the first is cleared before reuse.  This file
is collected last so that a failure here never hides another test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def noalloc_count(vs, ka, kb, key_type):
    import torch
    da = torch.from_numpy(ka.view(np.int32 if key_type == vs.T_VID else np.int64)).cuda()
    db = torch.from_numpy(kb.view(np.int32 if key_type == vs.T_VID else np.int64)).cuda()
    out = np.zeros(1, dtype=np.uint64)
    torch.cuda.synchronize()
    rc = vs.lib().vs_hash_join_count_noalloc(ctypes.c_void_p(da.data_ptr()), len(ka),
                                             ctypes.c_void_p(db.data_ptr()), len(kb), key_type,
                                             ctypes.c_void_p(out.ctypes.data), None)
    return rc, int(out[0])


def numpy_count(ka, kb):
    """Sum over keys of multiplicity_a(k) * multiplicity_b(k), computed on the
    host without any of the library's hash code."""
    ua, ca = np.unique(ka, return_counts=True)
    ub, cb = np.unique(kb, return_counts=True)
    _, ia, ib = np.intersect1d(ua, ub, assume_unique=True, return_indices=True)
    return int(np.sum(ca[ia].astype(np.int64) * cb[ib].astype(np.int64)))


def allocating_count(vs, ka, kb):
    a = vs.FlatTable.from_columns([ka])
    b = vs.FlatTable.from_columns([kb])
    _, count, _ = vs.hash_join(a, b, 0, 0, only_count=True)
    return count


def test_no_alloc_join_matches_allocating_join_twice(vs):
    rng = np.random.default_rng(2024)
    # call 1: skewed uint32 keys, larger table
    ka = (rng.zipf(1.5, 200_000) % 50_000).astype(np.uint32)
    kb = rng.integers(0, 50_000, 150_000).astype(np.uint32)
    rc, c1 = noalloc_count(vs, ka, kb, vs.T_VID)
    assert rc == 0, vs.lib().vs_last_error()
    assert c1 == numpy_count(ka, kb) > 0
    assert c1 == allocating_count(vs, ka, kb)
    # call 2: int64 keys including the all-ones value, a smaller table: stale
    # slots of call 1 must not leak into this count
    ka2 = rng.integers(-5, 3000, 40_000).astype(np.int64)
    ka2[:17] = -1
    kb2 = rng.integers(-5, 3000, 90_000).astype(np.int64)
    kb2[:5] = -1
    rc, c2 = noalloc_count(vs, ka2, kb2, vs.T_I64)
    assert rc == 0, vs.lib().vs_last_error()
    assert c2 == numpy_count(ka2, kb2) > 0
    assert c2 == allocating_count(vs, ka2, kb2)


def test_no_alloc_join_rejects_tables_above_its_limit(vs):
    big = np.zeros(262_145, dtype=np.uint32)
    rc, _ = noalloc_count(vs, big, big, vs.T_VID)
    assert rc == 6  # VS_ERR_CAPACITY
    assert b"262144" in vs.lib().vs_last_error()


def test_no_alloc_join_rejects_host_keys(vs):
    """Host arrays are refused with VS_ERR_ARG before any kernel is queued."""
    import torch
    ka = np.arange(1000, dtype=np.uint32)
    db = torch.from_numpy(ka.view(np.int32)).cuda()
    out = np.zeros(1, dtype=np.uint64)
    torch.cuda.synchronize()
    n0 = vs.kernel_launches()
    for a_ptr, b_ptr in ((ka.ctypes.data, db.data_ptr()), (db.data_ptr(), ka.ctypes.data)):
        rc = vs.lib().vs_hash_join_count_noalloc(ctypes.c_void_p(a_ptr), len(ka), ctypes.c_void_p(b_ptr),
                                                 len(ka), vs.T_VID, ctypes.c_void_p(out.ctypes.data), None)
        assert rc == 1  # VS_ERR_ARG
        assert b"device memory" in vs.lib().vs_last_error()
    assert vs.kernel_launches() == n0
