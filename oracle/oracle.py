"""ctypes binding of the oracle (oracle.cc): the CPU restatement of the
reference's frontier engine and apps.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker or as the timed CPU reference.
The product path never imports it.
"""

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
VARIANTS = {"push": 0, "push-pull": 1, "degree-sorting": 2, "hubdup": 3, "radar": 4}

_lib = None
_P = C.POINTER


def build():
    """Compiles liboracle.so (g++ only)."""
    src = os.path.join(HERE, "oracle.cc")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["g++", "-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared", "-Wall", "-o", LIB, src],
                       check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        u32p, i32p, i64p, f64p = _P(C.c_uint32), _P(C.c_int32), _P(C.c_int64), _P(C.c_double)
        L.orc_dedup_symmetric.argtypes = [C.c_int64, C.c_int64, u32p, u32p, u32p, u32p]
        L.orc_dedup_symmetric.restype = C.c_int64
        L.orc_degree_sort.argtypes = [C.c_int64, u32p, u32p, u32p, u32p, u32p]
        L.orc_degree_sort.restype = None
        L.orc_pagerank.argtypes = [C.c_int64, u32p, u32p, C.c_int, C.c_int64, C.c_int, f64p, i64p, f64p]
        L.orc_bfs.argtypes = [C.c_int64, u32p, u32p, C.c_int, C.c_uint32, C.c_int, u32p, i64p]
        L.orc_bc.argtypes = [C.c_int64, u32p, u32p, C.c_int, u32p, C.c_int, C.c_int, f64p, i64p]
        L.orc_radii.argtypes = [C.c_int64, u32p, u32p, C.c_int, u32p, C.c_int, C.c_int, i32p, i64p]
        L.orc_bc_sources.argtypes = [C.c_int64, u32p, C.c_int, u32p]
        L.orc_bc_sources.restype = None
        L.orc_radii_seeds.argtypes = [C.c_int64, u32p]
        L.orc_depths_from_parents.argtypes = [C.c_int64, u32p, i32p]
        L.orc_depths_from_parents.restype = None
        L.orc_bfs_depths.argtypes = [C.c_int64, u32p, u32p, C.c_uint32, i32p]
        L.orc_bfs_depths.restype = None
        L.orc_generate_edges.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_int, u32p, u32p]
        L.orc_csr_from_edges.argtypes = [C.c_int64, C.c_int64, u32p, u32p, u32p, u32p]
        L.orc_csr_from_edges.restype = C.c_int64
        L.orc_source_picker.argtypes = [C.c_int64, u32p, C.c_int, u32p]
        L.orc_source_picker.restype = None
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(_P(t))


def _u32(a):
    return np.ascontiguousarray(a, np.uint32)


def generate_edges(scale, edge_factor, seed=1, uniform=False):
    """The GAP generator's seeded edge list (generator.h:52-114)."""
    ne = edge_factor << scale
    src, dst = np.empty(ne, np.uint32), np.empty(ne, np.uint32)
    if lib().orc_generate_edges(scale, edge_factor, seed, 1 if uniform else 0, _p(src, C.c_uint32),
                                _p(dst, C.c_uint32)):
        raise ValueError("bad scale or edge factor")
    return src, dst


def csr_from_edges(n, src, dst):
    """Symmetric CSR of an edge list with the loader's clean-up (IO.h:429-474)."""
    src, dst = _u32(src), _u32(dst)
    off = np.empty(n + 1, np.uint32)
    adj = np.empty(max(2 * len(src), 1), np.uint32)
    m = lib().orc_csr_from_edges(n, len(src), _p(src, C.c_uint32), _p(dst, C.c_uint32), _p(off, C.c_uint32),
                                 _p(adj, C.c_uint32))
    if m < 0:
        raise ValueError("edge id out of range or too many edges")
    return off, adj[:m].copy()


def rmat_csr(scale, edge_factor, seed=1, uniform=False):
    """Symmetric R-MAT (or Erdos-Renyi) CSR built by the oracle alone."""
    src, dst = generate_edges(scale, edge_factor, seed, uniform)
    return csr_from_edges(1 << scale, src, dst)


def source_picker(deg, k):
    """GAP SourcePicker (benchmark.h:47-64): k roots with nonzero degree."""
    deg = _u32(deg)
    out = np.empty(k, np.uint32)
    lib().orc_source_picker(len(deg), _p(deg, C.c_uint32), k, _p(out, C.c_uint32))
    return out


def dedup_symmetric(n, off_n, adj):
    """IO.h:429-474 clean-up.  off_n has n start offsets (file form)."""
    off_n, adj = _u32(off_n), _u32(adj)
    oo = np.empty(n + 1, np.uint32)
    oa = np.empty(max(len(adj), 1), np.uint32)
    m = lib().orc_dedup_symmetric(n, len(adj), _p(off_n, C.c_uint32), _p(adj, C.c_uint32), _p(oo, C.c_uint32),
                                  _p(oa, C.c_uint32))
    return oo, oa[:m].copy()


def degree_sort(off, adj):
    off, adj = _u32(off), _u32(adj)
    n = len(off) - 1
    ids = np.empty(n, np.uint32)
    no = np.empty(n + 1, np.uint32)
    na = np.empty(max(len(adj), 1), np.uint32)
    lib().orc_degree_sort(n, _p(off, C.c_uint32), _p(adj, C.c_uint32), _p(ids, C.c_uint32), _p(no, C.c_uint32),
                          _p(na, C.c_uint32))
    return ids, no, na[:len(adj)].copy()


class _InEdges:
    """In-edges of a directed graph for the calls inside the block."""

    def __init__(self, in_off, in_adj):
        self.arrays = (_u32(in_off), _u32(in_adj)) if in_off is not None else None

    def __enter__(self):
        if self.arrays:
            lib().orc_set_in_edges(_p(self.arrays[0], C.c_uint32), _p(self.arrays[1], C.c_uint32))

    def __exit__(self, *a):
        lib().orc_set_in_edges(None, None)


def transpose(off, adj):
    """In-edges (in_off, in_adj) of a CSR, sources ascending per vertex."""
    off, adj = _u32(off), _u32(adj)
    n = len(off) - 1
    io, ia = np.empty(n + 1, np.uint32), np.empty(len(adj), np.uint32)
    lib().orc_transpose(n, _p(off, C.c_uint32), _p(adj, C.c_uint32), _p(io, C.c_uint32), _p(ia, C.c_uint32))
    return io, ia


def dedup_directed(n, off_n, adj):
    """Directed clean-up of the text loader: sorted out-lists, no repeats or
    self loops (off_n: n start offsets)."""
    return dedup_symmetric(n, off_n, adj)


def bc_sources_directed(outdeg, indeg, k):
    outdeg, indeg = _u32(outdeg), _u32(indeg)
    out = np.empty(k, np.uint32)
    lib().orc_bc_sources_directed(len(outdeg), _p(outdeg, C.c_uint32), _p(indeg, C.c_uint32), k, _p(out, C.c_uint32))
    return out


def pagerank(off, adj, variant="push", max_iters=20, threads=0, in_off=None, in_adj=None):
    off, adj = _u32(off), _u32(adj)
    n = len(off) - 1
    r = np.empty(n, np.float64)
    it, l1 = C.c_int64(), C.c_double()
    with _InEdges(in_off, in_adj):
        lib().orc_pagerank(n, _p(off, C.c_uint32), _p(adj, C.c_uint32), VARIANTS[variant], max_iters, threads,
                           _p(r, C.c_double), C.byref(it), C.byref(l1))
    return r, it.value, l1.value


def pagerank_delta(off, adj, variant="push", max_iters=20, threads=0, in_off=None, in_adj=None):
    """PageRankDelta (PageRankDelta.C): (ranks, printed round count, L1)."""
    off, adj = _u32(off), _u32(adj)
    n = len(off) - 1
    r = np.empty(n, np.float64)
    it, l1 = C.c_int64(), C.c_double()
    with _InEdges(in_off, in_adj):
        lib().orc_pagerank_delta(n, _p(off, C.c_uint32), _p(adj, C.c_uint32), VARIANTS[variant], max_iters, threads,
                                 _p(r, C.c_double), C.byref(it), C.byref(l1))
    return r, it.value, l1.value


def bfs(off, adj, root, variant="push", threads=0, in_off=None, in_adj=None):
    off, adj = _u32(off), _u32(adj)
    n = len(off) - 1
    par = np.empty(n, np.uint32)
    rounds = C.c_int64()
    with _InEdges(in_off, in_adj):
        lib().orc_bfs(n, _p(off, C.c_uint32), _p(adj, C.c_uint32), VARIANTS[variant], root, threads,
                      _p(par, C.c_uint32), C.byref(rounds))
    return par, rounds.value


def bc(off, adj, sources, variant="push", threads=0, in_off=None, in_adj=None):
    off, adj, s = _u32(off), _u32(adj), _u32(sources)
    n = len(off) - 1
    d = np.empty(n, np.float64)
    lv = C.c_int64()
    with _InEdges(in_off, in_adj):
        lib().orc_bc(n, _p(off, C.c_uint32), _p(adj, C.c_uint32), VARIANTS[variant], _p(s, C.c_uint32), len(s),
                     threads, _p(d, C.c_double), C.byref(lv))
    return d, lv.value


def radii(off, adj, seeds, variant="push", threads=0, in_off=None, in_adj=None):
    off, adj, s = _u32(off), _u32(adj), _u32(seeds)
    n = len(off) - 1
    r = np.empty(n, np.int32)
    rounds = C.c_int64()
    with _InEdges(in_off, in_adj):
        lib().orc_radii(n, _p(off, C.c_uint32), _p(adj, C.c_uint32), VARIANTS[variant], _p(s, C.c_uint32), len(s),
                        threads, _p(r, C.c_int32), C.byref(rounds))
    return r, rounds.value


def bc_sources(deg_orig, k):
    deg_orig = _u32(deg_orig)
    out = np.empty(k, np.uint32)
    lib().orc_bc_sources(len(deg_orig), _p(deg_orig, C.c_uint32), k, _p(out, C.c_uint32))
    return out


def triangles(off, adj, threads=0):
    """GAP tc_local: (per-vertex triangle counts by original id, total)."""
    off, adj = _u32(off), _u32(adj)
    n = len(off) - 1
    c = np.empty(n, np.uint64)
    tot = C.c_uint64()
    lib().orc_triangles(n, _p(off, C.c_uint32), _p(adj, C.c_uint32), threads, _p(c, C.c_uint64), C.byref(tot))
    return c, tot.value


def take_edges():
    """Edges the oracle's edgeMap calls traversed since the last call."""
    f = lib().orc_take_edges
    f.restype = C.c_int64
    return int(f())


def radii_seeds(n):
    out = np.empty(64, np.uint32)
    k = lib().orc_radii_seeds(n, _p(out, C.c_uint32))
    return out[:k].copy()


def bfs_depths(off, adj, root):
    off, adj = _u32(off), _u32(adj)
    n = len(off) - 1
    d = np.empty(n, np.int32)
    lib().orc_bfs_depths(n, _p(off, C.c_uint32), _p(adj, C.c_uint32), root, _p(d, C.c_int32))
    return d


def depths_from_parents(parents):
    parents = _u32(parents)
    d = np.empty(len(parents), np.int32)
    lib().orc_depths_from_parents(len(parents), _p(parents, C.c_uint32), _p(d, C.c_int32))
    return d


def check_bfs_tree(off, adj, root, parents, depth):
    """Property check: root is its own parent; every reached v's parent is a
    neighbour one level up; unreached vertices have no parent."""
    off, adj = _u32(off), _u32(adj)
    n = len(off) - 1
    none = np.uint32(0xFFFFFFFF)
    if parents[root] != root or depth[root] != 0:
        return False
    reached = parents != none
    if not np.array_equal(reached, depth >= 0):
        return False
    for v in np.nonzero(reached)[0]:
        if v == root:
            continue
        p = parents[v]
        if depth[p] != depth[v] - 1:
            return False
        nb = adj[off[v]:off[v + 1]]
        if p not in nb:
            return False
    return True


def degree_sort_directed(off, adj, in_off, in_adj, by_in=True):
    """Directed preprocessGraph (IO.h:739-842): rank by in-degree (-preprocess
    1) or out-degree (0), descending, ties by descending id; out- and in-lists
    relabelled, their order kept.  Returns (new_ids, off, adj, in_off, in_adj)."""
    off, adj, in_off, in_adj = (np.asarray(a, np.int64) for a in (off, adj, in_off, in_adj))
    n = len(off) - 1
    outdeg, indeg = np.diff(off), np.diff(in_off)
    key = (indeg if by_in else outdeg) * n + np.arange(n)
    order = np.argsort(-key, kind="stable")
    new_ids = np.empty(n, np.int64)
    new_ids[order] = np.arange(n)

    def relabel(o, a, deg):
        no = np.zeros(n + 1, np.int64)
        no[1:] = np.cumsum(deg[order])
        starts = o[order]
        idx = np.repeat(starts - no[:-1], deg[order]) + np.arange(no[-1])
        return no.astype(np.uint32), new_ids[a[idx]].astype(np.uint32)

    so, sa = relabel(off, adj, outdeg)
    sio, sia = relabel(in_off, in_adj, indeg)
    return new_ids.astype(np.uint32), so, sa, sio, sia
