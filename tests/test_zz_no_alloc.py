"""nlm_neighbor_search_noalloc (static device scratch, no allocation)
against nlm_neighbor_search, both called through the C ABI.

The file name sorts last so that the test runs after every other GPU test as
well as alone.  Each case calls the no-allocation entry twice in a row (the
second call reuses the scratch the first one left behind) and requires
integer-exact agreement with the allocating entry point.
"""
import ctypes as C

import numpy as np
import pytest

from nlmech_gb300 import abi, configs

pytestmark = pytest.mark.gpu

NLM_ERR_INVALID = 1


def _call(L, name, x, horizon, dim):
    fn = getattr(L, name)
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
    n = x.shape[0]
    rowptr = np.zeros(n + 1, dtype=np.int64)
    rc = fn(C.c_int(dim), C.c_int64(n), abi.dptr(x), C.c_double(horizon),
            abi.ptr(rowptr, C.c_int64), C.POINTER(C.c_int32)())
    if rc != 0:
        return rc, None, None
    cols = np.zeros(int(rowptr[-1]), dtype=np.int32)
    rc = fn(C.c_int(dim), C.c_int64(n), abi.dptr(x), C.c_double(horizon),
            abi.ptr(rowptr, C.c_int64), abi.ptr(cols, C.c_int32))
    return rc, rowptr, cols


def _cases():
    x2, _ = configs.grid2d(150, 120, 1e-3, seed=3)
    yield x2, 3.0e-3, 2
    x3, _ = configs.grid3d(24, 22, 20, 1e-3, seed=4)
    yield x3, 2.0e-3, 3
    rng = np.random.default_rng(6)
    xr = np.zeros((4000, 3))
    xr[:, :2] = rng.uniform(0, 1e-2, size=(4000, 2))
    xr[17] = xr[18]  # coincident pair
    yield xr, 4.0e-4, 2
    yield np.array([[0., 0, 0], [1., 0, 0], [0., 0.5, 0]]), 1.0, 2
    yield np.zeros((1, 3)), 1.0, 2


def test_noalloc_matches_allocating_search(gpu):
    L = gpu.load()
    for x, hz, dim in _cases():
        rc, rp_ref, cc_ref = _call(L, "nlm_neighbor_search", x, hz, dim)
        assert rc == 0
        for _ in range(2):
            rc, rp, cc = _call(L, "nlm_neighbor_search_noalloc", x, hz, dim)
            assert rc == 0, L.nlm_last_error().decode()
            assert np.array_equal(rp, rp_ref)
            assert np.array_equal(cc, cc_ref)


def test_noalloc_empty_and_limits(gpu):
    L = gpu.load()
    rc, rp, cc = _call(L, "nlm_neighbor_search_noalloc", np.zeros((0, 3)), 1.0, 2)
    assert rc == 0 and list(rp) == [0] and len(cc) == 0
    # above the node limit: rejected on the host before any launch
    x = np.zeros((65537, 3))
    x[:, 0] = np.arange(65537) * 1e-3
    rc, _, _ = _call(L, "nlm_neighbor_search_noalloc", x, 1.5e-3, 2)
    assert rc == NLM_ERR_INVALID
    assert b"65536" in L.nlm_last_error()
    # a sparse cloud whose search grid needs more cells than the scratch holds
    x = np.array([[0., 0, 0], [1., 1., 0]])
    rc, _, _ = _call(L, "nlm_neighbor_search_noalloc", x, 1e-3, 2)
    assert rc == NLM_ERR_INVALID
    assert b"262144" in L.nlm_last_error()
    # more than 4,194,304 bonds from at most 65,536 nodes (about 73 per row):
    # found after the counting pass, before any bond is written
    x3, _ = configs.grid3d(40, 40, 40, 1e-3, seed=8)
    rc, _, _ = _call(L, "nlm_neighbor_search_noalloc", x3, 2.6e-3, 3)
    assert rc == NLM_ERR_INVALID
    assert b"4194304" in L.nlm_last_error()
    # a cluster of 600 nodes inside one horizon: rows of 599 entries
    rng = np.random.default_rng(10)
    xc = np.zeros((600, 3))
    xc[:, :2] = rng.uniform(0, 1e-4, size=(600, 2))
    rc, _, _ = _call(L, "nlm_neighbor_search_noalloc", xc, 1e-3, 2)
    assert rc == NLM_ERR_INVALID
    assert b"512" in L.nlm_last_error()
    # the next call in range still works after the rejections
    x2, _ = configs.grid2d(40, 30, 1e-3, seed=9)
    rc, rp_ref, cc_ref = _call(L, "nlm_neighbor_search", x2, 3e-3, 2)
    rc2, rp, cc = _call(L, "nlm_neighbor_search_noalloc", x2, 3e-3, 2)
    assert rc == 0 and rc2 == 0
    assert np.array_equal(rp, rp_ref) and np.array_equal(cc, cc_ref)
