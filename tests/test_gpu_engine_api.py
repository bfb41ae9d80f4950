"""The engine-level C ABI (rg_edgemap / rg_vertexmap), driven the way the
reference apps drive Ligra's edgeMap and vertexMap.

Each test writes one app's Compute loop against the ABI alone -- frontiers,
operators and caller-owned device arrays -- and compares the result with the
golden vectors the reference's own binaries produced:

  PageRank  PageRank.C:163-176      (PR_F + PR_Vertex_F, L1 break, reset, swap)
  BC        BC-manyiter-v2.C:180-232 (BC_F + BC_Vertex_F per level, inverse
                                      path counts, BC_Back_F + BC_Back_Vertex_F
                                      back through the saved levels)
  Radii     Radii.C:162-196          (Radii_Vertex_F sync, Radii_F per round)

Both dense directions are run: RG_DENSE_FORWARD (dense rounds push, as the
push variants call edgeMap) and without it (dense rounds pull, ligra.h:302-307).
"""

import ctypes as C

import numpy as np
import pytest

import radar_graph as rg
from conftest import assert_close

pytestmark = pytest.mark.gpu

NAMES = ["rmat12", "er10"]
FLAGS = {"dense-push": rg.DENSE_FORWARD, "dense-pull": 0}


class Dev:
    """A caller-owned device array (rg_device_alloc) with host copies."""

    def __init__(self, L, arr):
        self.L = L
        self.dtype, self.n = arr.dtype, arr.size
        self.p = C.c_void_p()
        rg._check(L.rg_device_alloc(max(arr.nbytes, 8), C.byref(self.p)))
        self.put(arr)

    def put(self, arr):
        arr = np.ascontiguousarray(arr, self.dtype)
        if arr.nbytes:
            rg._check(self.L.rg_copy_to_device(self.p, arr.ctypes.data, arr.nbytes))

    def get(self):
        out = np.empty(self.n, self.dtype)
        if out.nbytes:
            rg._check(self.L.rg_copy_to_host(out.ctypes.data, self.p, out.nbytes))
        return out

    def free(self):
        self.L.rg_device_free(self.p)


class Frontiers:
    """rg_frontier handles of one graph, freed together."""

    def __init__(self, L, G):
        self.L, self.G, self.hs = L, G, []

    def new(self, ids=None):
        f = C.c_void_p()
        rg._check(self.L.rg_frontier_create(self.G.handle, C.byref(f)))
        self.hs.append(f)
        if ids is not None:
            ids = np.ascontiguousarray(ids, np.uint32)
            rg._check(self.L.rg_frontier_set(f, ids.ctypes.data_as(C.POINTER(C.c_uint32)), len(ids)))
        return f

    def count(self, f):
        c = C.c_int64()
        rg._check(self.L.rg_frontier_count(f, C.byref(c)))
        return c.value

    def free(self):
        for f in self.hs:
            self.L.rg_frontier_free(f)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("mode", FLAGS)
def test_pagerank_loop_through_edgemap(golden, name, mode):
    g = golden[name]
    L = rg.lib()
    with rg.Graph.from_csr(g["off"], g["adj"]) as G:
        n = G.n
        fr = Frontiers(L, G)
        pc, pn = Dev(L, np.full(n, 1.0 / n)), Dev(L, np.zeros(n))
        try:
            everyone = fr.new()
            rg._check(L.rg_frontier_set_all(everyone))
            args = rg.OpArgs()
            ranks = None
            for _ in range(20):
                args.p_curr, args.p_next = pc.p.value, pn.p.value
                # edgeMap(GA, Frontier, PR_F, 0, no_output | dense_forward): threshold 0 -> dense
                rg._check(L.rg_edgemap(G.handle, everyone, rg.OPS["pagerank"], C.byref(args), None,
                                       rg.NO_OUTPUT | FLAGS[mode], 0, None))
                rg._check(L.rg_vertexmap(G.handle, everyone, rg.VOPS["pr_damp"], C.byref(args), None))
                cur, nxt = pc.get(), pn.get()
                if np.abs(cur - nxt).sum() < 1e-7:  # L1 < epsilon: the ranks are p_next
                    ranks = nxt
                    break
                pc.put(np.zeros(n))  # PR_Vertex_Reset, then swap
                pc, pn = pn, pc
            if ranks is None:
                ranks = pc.get()
            assert_close(ranks, g["pr_push"], what=f"PageRank via rg_edgemap {name} {mode}")
        finally:
            pc.free()
            pn.free()
            fr.free()


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("mode", FLAGS)
def test_bc_loop_through_edgemap(golden, name, mode):
    g = golden[name]
    L = rg.lib()
    with rg.Graph.from_csr(g["off"], g["adj"]) as G:
        n = G.n
        src = int(G.bc_pick_sources(1)[0])
        fr = Frontiers(L, G)
        paths = np.zeros(n)
        paths[src] = 1.0
        visited = np.zeros((n + 31) // 32, np.uint32)
        visited[src >> 5] = np.uint32(1 << (src & 31))
        d_paths, d_deps, d_vis = Dev(L, paths), Dev(L, np.zeros(n)), Dev(L, visited)
        try:
            args = rg.OpArgs()
            args.num_paths, args.deps, args.visited_bits = d_paths.p.value, d_deps.p.value, d_vis.p.value
            levels = [fr.new([src])]
            while fr.count(levels[-1]) > 0:  # forward phase
                out = fr.new()
                rg._check(L.rg_edgemap(G.handle, levels[-1], rg.OPS["bc_fwd"], C.byref(args), out, FLAGS[mode], -1,
                                       None))
                rg._check(L.rg_vertexmap(G.handle, out, rg.VOPS["bc_visit"], C.byref(args), None))
                levels.append(out)
            rounds = len(levels) - 1
            with np.errstate(divide="ignore"):
                inv = 1.0 / d_paths.get()  # inverseNumPaths (inf where no path)
            d_paths.put(inv)
            d_vis.put(np.zeros_like(visited))
            rg._check(L.rg_vertexmap(G.handle, levels[rounds - 1], rg.VOPS["bc_back"], C.byref(args), None))
            for r in range(rounds - 2, -1, -1):  # backward phase (symmetric: the transpose is the graph)
                rg._check(L.rg_edgemap(G.handle, levels[r + 1], rg.OPS["bc_bwd"], C.byref(args), None,
                                       rg.NO_OUTPUT | FLAGS[mode], -1, None))
                rg._check(L.rg_vertexmap(G.handle, levels[r], rg.VOPS["bc_back"], C.byref(args), None))
            with np.errstate(invalid="ignore"):
                deps = (d_deps.get() - inv) / inv
            assert_close(deps, g["bc1_push"], what=f"BC via rg_edgemap {name} {mode}")
        finally:
            for d in (d_paths, d_deps, d_vis):
                d.free()
            fr.free()


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("mode", FLAGS)
def test_radii_loop_through_edgemap(golden, name, mode):
    g = golden[name]
    L = rg.lib()
    with rg.Graph.from_csr(g["off"], g["adj"]) as G:
        n = G.n
        seeds = rg.radii_seeds_orig(n)
        radii = np.full(n, -1, np.int32)
        nxt = np.zeros(n, np.uint64)
        for i, v in enumerate(seeds):
            radii[v] = 0
            nxt[v] = np.uint64(1) << np.uint64(i)
        fr = Frontiers(L, G)
        d_vis, d_next, d_radii = Dev(L, np.zeros(n, np.int64)), Dev(L, nxt.view(np.int64)), Dev(L, radii)
        try:
            args = rg.OpArgs()
            args.visited, args.next_visited, args.radii = d_vis.p.value, d_next.p.value, d_radii.p.value
            frontier = fr.new(seeds)
            rnd = 0
            while fr.count(frontier) > 0:
                rnd += 1
                rg._check(L.rg_vertexmap(G.handle, frontier, rg.VOPS["radii_sync"], C.byref(args), None))
                args.round = rnd
                out = fr.new()
                rg._check(L.rg_edgemap(G.handle, frontier, rg.OPS["radii"], C.byref(args), out, FLAGS[mode], -1, None))
                frontier = out
            assert np.array_equal(d_radii.get(), g["radii_push"]), f"Radii via rg_edgemap {name} {mode}"
        finally:
            for d in (d_vis, d_next, d_radii):
                d.free()
            fr.free()


def test_level_trace_records_every_edgemap(golden):
    """rg_set_trace: one record per edgeMap, as Ligra's frontierStats prints
    PUSH/PULL and the frontier size per iteration -- BFS on rmat12 goes sparse,
    dense, then sparse again, and every dense level passes the m/20 test."""
    g = golden["rmat12"]
    with rg.Graph.from_csr(g["off"], g["adj"]) as G:
        rg.set_trace(True)
        try:
            _, _, rounds, _ = G.bfs("push-pull", int(g["bfs_roots"][0]))
            tr = rg.take_trace()
        finally:
            rg.set_trace(False)
        assert len(tr) == rounds or len(tr) == rounds - 1
        assert {t["mode"] for t in tr} >= {"sparse-push", "pull"}
        for t in tr:
            dense = t["frontier"] + t["degsum"] > t["threshold"]
            assert (t["mode"] != "sparse-push") == dense
            assert t["threshold"] == G.m // 20
        assert rg.take_trace() == []  # taken and cleared
