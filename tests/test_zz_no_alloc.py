"""rg_bfs_depth_noalloc, the entry point for callers that cannot allocate
device memory (a framework that owns the device memory pool, or a serving loop
that must not synchronize on cudaMalloc).  It is checked against the regular
rg_bfs on the same CSR, through the C ABI, on two calls in a row: the second
call starts from the first call's leftovers in the shared scratch array, so it
shows that the entry point clears what it must.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test."""

import ctypes as C

import numpy as np
import pytest

import radar_graph as rg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as b
    b.build()


def _dev_copy(L, arr):
    p = C.c_void_p()
    rg._check(L.rg_device_alloc(max(arr.nbytes, 4), C.byref(p)))
    if arr.nbytes:
        rg._check(L.rg_copy_to_device(p, arr.ctypes.data, arr.nbytes))
    return p


def test_noalloc_bfs_matches_rg_bfs_on_two_calls():
    L = rg.lib()
    off, adj = rg.rmat_csr(14, 8, seed=7)
    n, m = len(off) - 1, len(adj)
    deg = np.diff(off.astype(np.int64))
    nz = np.nonzero(deg)[0]
    roots = [int(nz[0]), int(nz[len(nz) // 2])]
    with rg.Graph.from_csr(off, adj) as g:
        want = [g.bfs("push", r)[1:3] for r in roots]  # (depth, rounds)
    d_off, d_adj = _dev_copy(L, off), _dev_copy(L, adj)
    d_depth = _dev_copy(L, np.zeros(n, np.int32))
    try:
        for (depth_want, rounds_want), root in zip(want, roots):
            rounds = C.c_int64()
            rg._check(L.rg_bfs_depth_noalloc(d_off, d_adj, n, m, root, d_depth, None, C.byref(rounds)))
            got = np.empty(n, np.int32)
            rg._check(L.rg_copy_to_host(got.ctypes.data, d_depth, got.nbytes))
            assert np.array_equal(got, depth_want)
            assert rounds.value == rounds_want
    finally:
        for p in (d_off, d_adj, d_depth):
            L.rg_device_free(p)


def test_noalloc_rejects_graphs_beyond_the_scratch_limit():
    L = rg.lib()
    tiny = _dev_copy(L, np.zeros(8, np.uint32))
    try:
        rounds = C.c_int64()
        too_big = 2097152 + 1  # RG_NOALLOC_MAX_VERTICES + 1
        st = L.rg_bfs_depth_noalloc(tiny, tiny, too_big, 0, 0, tiny, None, C.byref(rounds))
        assert st == 1  # RG_EINVAL, before any device access
        assert b"scratch limit" in L.rg_last_error()
    finally:
        L.rg_device_free(tiny)


def test_noalloc_skips_neighbour_ids_beyond_n():
    """A CSR passed as device pointers cannot be validated on the host: a
    neighbour id >= n is skipped by the kernel instead of indexing past the
    caller's depth array (path 0-1-2 with a stray id 7 in vertex 0's list)."""
    L = rg.lib()
    off = np.array([0, 2, 4, 5], np.uint32)
    adj = np.array([1, 7, 0, 2, 1], np.uint32)
    d_off, d_adj = _dev_copy(L, off), _dev_copy(L, adj)
    d_depth = _dev_copy(L, np.zeros(3, np.int32))
    try:
        rounds = C.c_int64()
        rg._check(L.rg_bfs_depth_noalloc(d_off, d_adj, 3, 5, 0, d_depth, None, C.byref(rounds)))
        got = np.empty(3, np.int32)
        rg._check(L.rg_copy_to_host(got.ctypes.data, d_depth, got.nbytes))
        assert got.tolist() == [0, 1, 2]
        assert rounds.value == 3
    finally:
        for p in (d_off, d_adj, d_depth):
            L.rg_device_free(p)
