"""Batched execution on the GPU: 64-source bitmask BFS on one resident graph
and the persistent many-graph launch.  Every batched result must equal the
corresponding single-query result (and the oracle): BFS depths bit-exact,
PageRank ranks identical to rg_pagerank (same exact-sum arithmetic) and within
1e-9 relative of the oracle."""

import numpy as np
import pytest

import oracle as orc
import radar_graph as rg
from conftest import assert_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as b
    b.build()


def _sources(off, k, seed):
    deg = np.diff(off.astype(np.int64))
    rng = np.random.default_rng(seed)
    nz = np.nonzero(deg)[0]
    if len(nz) == 0:
        return np.zeros(k, np.uint32)
    s = rng.choice(nz, size=k, replace=True)
    s[0] = int(np.argmin(deg))  # include a low-degree (possibly isolated) vertex
    return s.astype(np.uint32)


@pytest.mark.parametrize("k", [1, 7, 64])
@pytest.mark.parametrize("sorted_graph", [False, True])
def test_bfs_multi_equals_single_source(golden, k, sorted_graph):
    g = golden["rmat12"]
    src = _sources(g["off"], k, seed=k)
    src[-1] = src[0]  # a duplicate source
    with rg.Graph.from_csr(g["off"], g["adj"]) as G:
        H = G.degree_sort() if sorted_graph else G
        depths, rounds = H.bfs_multi(src)
        for q, s in enumerate(src):
            assert np.array_equal(depths[q], orc.bfs_depths(g["off"], g["adj"], int(s))), q
            _, d1, _, _ = H.bfs("push", int(s))
            assert np.array_equal(depths[q], d1)
        if H is not G:
            H.free()


def test_bfs_multi_s16_dense_levels():
    off, adj = rg.rmat_csr(16, 16, seed=1)
    src = _sources(off, 64, seed=3)
    with rg.Graph.from_csr(off, adj) as G, G.degree_sort() as H:
        depths, _ = H.bfs_multi(src)
        for q in (0, 1, 31, 63):
            assert np.array_equal(depths[q], orc.bfs_depths(off, adj, int(src[q])))


@pytest.mark.parametrize("unsorted", [False, True], ids=["sorted", "unsorted"])
def test_bitmask_sweep_widths_agree(unsorted):
    """The dense bitmask rounds take 16 edges per lane with the 16x sweep
    shapes and 8 otherwise; Radii (64 samples), 64-source BFS and the oracle's
    depths must not depend on it, on a graph with several dense rounds and,
    unsorted, with empty rows between nonempty ones."""
    off, adj = rg.rmat_csr(16, 16, seed=1)
    src = _sources(off, 64, seed=3)
    with rg.Graph.from_csr(off, adj) as G, G.degree_sort() as S:
        H = G if unsorted else S
        got = {}
        for shape in (81, 161):
            old_shape, old_dir = rg.get_option("sweep_shape"), rg.get_option("direction")
            try:
                rg.set_option("sweep_shape", shape)
                rg.set_option("direction", 1)  # pulled dense rounds
                got[shape] = (H.radii("radar")[0], H.bfs_multi(src)[0])
            finally:
                rg.set_option("sweep_shape", old_shape)
                rg.set_option("direction", old_dir)
        assert np.array_equal(got[81][0], got[161][0])
        assert np.array_equal(got[81][1], got[161][1])
        for q in (0, 5, 63):
            assert np.array_equal(got[161][1][q], orc.bfs_depths(off, adj, int(src[q])))


def test_bfs_multi_rejects_bad_input(golden):
    g = golden["tiny"]
    with rg.Graph.from_csr(g["off"], g["adj"]) as G:
        with pytest.raises(rg.RgError):
            G.bfs_multi(np.arange(65, dtype=np.uint32) % 12)
        with pytest.raises(rg.RgError):
            G.bfs_multi(np.array([99], np.uint32))


def test_batch_persistent_matches_single_queries():
    rng = np.random.default_rng(11)
    csrs = []
    for i in range(12):
        scale = int(rng.integers(6, 12))
        ef = int(rng.integers(4, 20))
        csrs.append(rg.rmat_csr(scale, ef, seed=100 + i))
    csrs.append((np.zeros(5, np.uint32), np.zeros(0, np.uint32)))  # a graph without edges
    k = 64
    sources = np.stack([_sources(o, k, seed=i) for i, (o, _) in enumerate(csrs)])
    B = rg.Batch(csrs)
    depths, ranks, iters, ms = B.run(sources, pr_iters=10)
    assert ms > 0
    for i, (off, adj) in enumerate(csrs):
        for q in (0, 5, 63):
            assert np.array_equal(depths[i][q], orc.bfs_depths(off, adj, int(sources[i, q]))), (i, q)
        ro, ito, _ = orc.pagerank(off, adj, "push", 10, 1)
        assert iters[i] == ito, i
        assert_close(ranks[i], ro, what=f"batch pr {i}")
        if len(adj):
            with rg.Graph.from_csr(off, adj) as G:
                r1, it1, _ = G.pagerank("push-pull", 10)
                assert np.array_equal(ranks[i], r1)  # same exact sums, bit for bit
    B.free()
