"""GPU parity: the CUDA engine (through the C ABI) against the golden vectors
of the reference's own apps and against the oracle on larger seeded graphs.

Tolerances: PageRank ranks and BC dependencies within 1e-9 relative (RTOL in
conftest.py); BFS depths, Radii and the degree-sort permutation bit-exact;
BFS parents must form a valid BFS tree (parents themselves may differ, as they
do between reference runs)."""

import numpy as np
import pytest

import oracle as orc
import radar_graph as rg
from conftest import GOLDEN_NAMES, assert_close

pytestmark = pytest.mark.gpu

VARIANTS = ["push", "push-pull", "degree-sorting", "hubdup", "radar"]
SORTED = rg.SORTED_VARIANTS


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as b
    b.build()


class Dev:
    """Unsorted and degree-sorted device images of one CSR."""

    def __init__(self, off, adj):
        self.off, self.adj = off, adj
        self.g = rg.Graph.from_csr(off, adj)
        self.gs = self.g.degree_sort()

    def pick(self, variant):
        return self.gs if variant in SORTED else self.g


@pytest.fixture(scope="module")
def dev(golden):
    return {name: Dev(g["off"], g["adj"]) for name, g in golden.items()}


def _gold(g, prefix, variant):
    key = f"{prefix}_{variant}"
    return g[key] if key in g else g[f"{prefix}_push"]


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_degree_sort_bit_exact(golden, dev, name):
    g, D = golden[name], dev[name]
    assert np.array_equal(D.gs.new_ids, g["new_ids"])
    off, adj, ids = D.gs.download()
    ids2, o2, a2 = orc.degree_sort(g["off"], g["adj"])
    assert np.array_equal(ids, ids2) and np.array_equal(off, o2) and np.array_equal(adj, a2)


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", VARIANTS)
def test_pagerank(golden, dev, name, variant):
    r, it, l1 = dev[name].pick(variant).pagerank(variant, 20)
    assert_close(r, _gold(golden[name], "pr", variant), what=f"pr {name} {variant}")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "radar"])
def test_pagerank_l1_break(golden, dev, name, variant):
    g = golden[name]
    r, it, l1 = dev[name].pick(variant).pagerank(variant, 200)
    assert it == int(g["pr200_iters"][0])
    assert l1 < 1e-7
    assert_close(r, g["pr200_push"], what="pr200")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", VARIANTS)
def test_bfs(golden, dev, name, variant):
    g, D = golden[name], dev[name]
    G = D.pick(variant)
    off, adj, _ = G.download()
    for ri, root in enumerate(g["bfs_roots"]):
        par, depth, rounds, reached = G.bfs(variant, int(root))
        assert np.array_equal(depth, _gold(g, f"bfs{ri}", variant)), f"bfs {name} {variant} root {root}"
        assert reached == int((depth >= 0).sum())
        rr = G.new_ids[root] if variant in SORTED else root
        inner_depth = orc.depths_from_parents(par[np.argsort(G.new_ids)] if variant in SORTED else par)
        # parents are internal ids; check the tree on the internal graph
        par_int = np.empty_like(par)
        if variant in SORTED:
            par_int[G.new_ids] = par
        else:
            par_int = par
        assert orc.check_bfs_tree(off, adj, rr, par_int, orc.depths_from_parents(par_int))
        del inner_depth


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", VARIANTS)
def test_pagerank_delta(golden, dev, name, variant):
    g = golden[name]
    r, it, l1 = dev[name].pick(variant).pagerank_delta(variant, 20)
    key = f"prd_{variant}" if f"prd_{variant}" in g else "prd_push"
    assert it == int(g[f"prd_iters_{variant}" if f"prd_iters_{variant}" in g else "prd_iters_push"][0])
    assert_close(r, g[key], what=f"prd {name} {variant}")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_pagerank_delta_maxiters_cutoff(golden, dev, name):
    g = golden[name]
    r, it, _ = dev[name].g.pagerank_delta("push", 5)
    assert it == int(g["prd5_iters"][0])
    assert_close(r, g["prd5_push"], what=f"prd5 {name}")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("k", [1, 4])
def test_bc(golden, dev, name, variant, k):
    g = golden[name]
    d, levels = dev[name].pick(variant).bc(variant, k)
    assert_close(d, _gold(g, f"bc{k}", variant), what=f"bc{k} {name} {variant}")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", VARIANTS)
def test_radii(golden, dev, name, variant):
    r, rounds = dev[name].pick(variant).radii(variant)
    assert np.array_equal(r, golden[name]["radii_push"]), f"radii {name} {variant}"


def test_bc_sources_match_reference_selector(golden, dev):
    for name, g in golden.items():
        deg = np.diff(g["off"].astype(np.int64)).astype(np.uint32)
        if deg.max() == 0:
            continue
        want = orc.bc_sources(deg, 16)
        assert np.array_equal(dev[name].g.bc_pick_sources(16), want)
        assert np.array_equal(dev[name].gs.bc_pick_sources(16), want)


# ---------------------------------------------------------------------------
# larger seeded graphs against the oracle (sizes the oracle finishes in seconds)
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def s16():
    off, adj = rg.rmat_csr(16, 16, seed=1)  # the configuration PageRank is quoted on
    return Dev(off, adj)


@pytest.mark.parametrize("variant", VARIANTS)
def test_s16_pagerank_vs_oracle(s16, variant):
    r, it, _ = s16.pick(variant).pagerank(variant, 20)
    ro, ito, _ = orc.pagerank(s16.off, s16.adj, "push", 20, 0)
    assert it == ito
    assert_close(r, ro, what=f"s16 pr {variant}")


@pytest.mark.parametrize("variant", VARIANTS)
def test_s16_pagerank_delta_vs_oracle(s16, variant):
    G = s16.pick(variant)
    r, it, l1 = G.pagerank_delta(variant, 100)
    ro, ito, l1o = orc.pagerank_delta(s16.off, s16.adj, "push", 100, 0)
    assert it == ito
    assert_close(r, ro, what=f"s16 prd {variant}")
    assert abs(l1 - l1o) <= 1e-9 * l1o


@pytest.mark.parametrize("variant", VARIANTS)
def test_s16_bfs_bc_radii_vs_oracle(s16, variant):
    G = s16.pick(variant)
    deg = np.diff(s16.off.astype(np.int64))
    roots = orc.bc_sources(deg.astype(np.uint32), 3)
    for root in roots:
        _, depth, _, _ = G.bfs(variant, int(root))
        assert np.array_equal(depth, orc.bfs_depths(s16.off, s16.adj, int(root)))
    d, _ = G.bc(variant, 2)
    do, _ = orc.bc(s16.off, s16.adj, orc.bc_sources(deg.astype(np.uint32), 2), "push", 0)
    assert_close(d, do, what=f"s16 bc {variant}")
    r, _ = G.radii(variant)
    ro, _ = orc.radii(s16.off, s16.adj, orc.radii_seeds(len(deg)), "push", 1)
    assert np.array_equal(r, ro)


def test_s16_er_contrast_vs_oracle():
    off, adj = rg.rmat_csr(16, 16, seed=1, uniform=True)
    D = Dev(off, adj)
    r, _, _ = D.gs.pagerank("radar", 20)
    ro, _, _ = orc.pagerank(off, adj, "push", 20, 0)
    assert_close(r, ro, what="er pr")
    rr, _ = D.gs.radii("radar")
    ro2, _ = orc.radii(off, adj, orc.radii_seeds(len(off) - 1), "push", 1)
    assert np.array_equal(rr, ro2)


# ---------------------------------------------------------------------------
# edge cases
# ---------------------------------------------------------------------------

def test_isolated_root_and_empty_graph_parts():
    # vertex 5 isolated; n = 37 (not a multiple of 32)
    src = np.array([0, 1, 2, 3, 30, 36], np.uint32)
    dst = np.array([1, 2, 3, 0, 31, 35], np.uint32)
    off, adj = rg.csr_from_edges(37, src, dst)
    with rg.Graph.from_csr(off, adj) as g:
        par, depth, rounds, reached = g.bfs("push", 5)
        assert reached == 1 and rounds == 1 and depth[5] == 0 and (depth >= 0).sum() == 1
        for v in VARIANTS:
            G = g.degree_sort() if v in SORTED else g
            r, _, _ = G.pagerank(v, 20)
            ro, _, _ = orc.pagerank(off, adj, "push", 20, 1)
            assert_close(r, ro, what=f"tiny pr {v}")
            rad, _ = G.radii(v)
            ro2, _ = orc.radii(off, adj, orc.radii_seeds(37), "push", 1)
            assert np.array_equal(rad, ro2)


def test_graph_without_edges():
    off = np.zeros(9, np.uint32)
    adj = np.zeros(0, np.uint32)
    with rg.Graph.from_csr(off, adj) as g:
        r, it, l1 = g.pagerank("push", 5)
        assert np.allclose(r, 0.15 / 8 * 0 + (0.85 * 0 + 0.15 / 8))
        _, depth, rounds, reached = g.bfs("push", 3)
        assert reached == 1 and rounds == 1
        with pytest.raises(rg.RgError):
            g.bc("push", 1)  # no vertex with out-degree > 0 can be drawn


def test_bad_arguments_are_errors(dev):
    g = dev["tiny"].g
    with pytest.raises(rg.RgError) as e:
        g.bfs("push", 10**6)
    assert e.value.status == 1
    with pytest.raises(rg.RgError):
        g.radii_seeds(np.arange(65, dtype=np.uint32) % 12)
    with pytest.raises(ValueError):
        g.pagerank("nope", 1)


# ---------------------------------------------------------------------------
# engine-level API: a BFS written against rg_edgemap, like BFS.C's loop
# ---------------------------------------------------------------------------

def test_edgemap_api_bfs_loop(golden):
    import ctypes as C
    g = golden["rmat12"]
    L = rg.lib()
    with rg.Graph.from_csr(g["off"], g["adj"]) as G:
        n = G.n
        root = int(g["bfs_roots"][0])
        parents = np.full(n, 0xFFFFFFFF, np.uint32)
        parents[root] = root
        dp = C.c_void_p()
        rg._check(L.rg_device_alloc(4 * n, C.byref(dp)))
        rg._check(L.rg_copy_to_device(dp, parents.ctypes.data, 4 * n))
        fa, fb = C.c_void_p(), C.c_void_p()
        rg._check(L.rg_frontier_create(G.handle, C.byref(fa)))
        rg._check(L.rg_frontier_create(G.handle, C.byref(fb)))
        ids = np.array([root], np.uint32)
        rg._check(L.rg_frontier_set(fa, ids.ctypes.data_as(C.POINTER(C.c_uint32)), 1))
        args = rg.OpArgs()
        args.parents = dp.value
        depth = np.full(n, -1, np.int32)
        depth[root] = 0
        level = 0
        cnt = C.c_int64(1)
        for mode in range(2):
            pass
        while cnt.value > 0:
            level += 1
            rg._check(L.rg_edgemap(G.handle, fa, rg.OPS["bfs"], C.byref(args), fb, rg.DENSE_FORWARD, -1, None))
            rg._check(L.rg_frontier_count(fb, C.byref(cnt)))
            mem = np.empty(n, np.uint8)
            rg._check(L.rg_frontier_get(fb, mem.ctypes.data_as(C.POINTER(C.c_uint8))))
            depth[mem.astype(bool)] = level
            fa, fb = fb, fa
        assert np.array_equal(depth, g["bfs0_push"])
        L.rg_frontier_free(fa)
        L.rg_frontier_free(fb)
        L.rg_device_free(dp)


def test_recreated_graphs_do_not_reuse_stale_launches():
    """Graphs freed and re-created with the same sizes get the same pooled
    device addresses; cached PageRank launches must still follow the new
    graph (a cache keyed by addresses alone replayed a freed graph's sweep
    partition)."""
    for rep in range(3):
        for seed in (1, 2):
            off, adj = rg.rmat_csr(13, 8, seed=seed)
            with rg.Graph.from_csr(off, adj) as g, g.degree_sort() as gs:
                for opts in ({"direction": 1, "hub_smem_kb": 0}, {"direction": 0, "hub_smem_kb": 48}):
                    old = {k: rg.get_option(k) for k in opts}
                    for k, v in opts.items():
                        rg.set_option(k, v)
                    try:
                        r, it, _ = gs.pagerank("radar", 20)
                    finally:
                        for k, v in old.items():
                            rg.set_option(k, v)
                    ro, ito, _ = orc.pagerank(off, adj, "push", 20, 0)
                    assert it == ito
                    assert_close(r, ro, what=f"recreated graph seed {seed} rep {rep} {opts}")
