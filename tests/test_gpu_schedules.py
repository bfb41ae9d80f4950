"""Schedules never change results: every scheduling option (direction, dense
threshold, hub shared-memory budget, PageRank sweep shape) gives the oracle's
results -- bit-exact for BFS depths and Radii, 1e-9 relative for PageRank and
BC -- on a skewed R-MAT graph and a uniform (Erdos-Renyi) one."""

import contextlib

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


@contextlib.contextmanager
def options(**kw):
    old = {k: rg.get_option(k) for k in kw}
    try:
        for k, v in kw.items():
            rg.set_option(k, v)
        yield
    finally:
        for k, v in old.items():
            rg.set_option(k, v)


class G:
    def __init__(self, uniform):
        self.off, self.adj = rg.rmat_csr(15, 16, seed=3, uniform=uniform)
        g = rg.Graph.from_csr(self.off, self.adj)
        self.gs = g.degree_sort()
        self.g = g
        self.deg = np.diff(self.off.astype(np.int64)).astype(np.uint32)
        self.pr = orc.pagerank(self.off, self.adj, "push", 20, 0)
        self.prd = orc.pagerank_delta(self.off, self.adj, "push", 30, 0)
        self.root = int(orc.bc_sources(self.deg, 1)[0])
        self.depth = orc.bfs_depths(self.off, self.adj, self.root)
        self.bc_src = orc.bc_sources(self.deg, 2)
        self.bc = orc.bc(self.off, self.adj, self.bc_src, "push", 0)[0]
        self.radii = orc.radii(self.off, self.adj, orc.radii_seeds(len(self.deg)), "push", 1)[0]


@pytest.fixture(scope="module", params=[False, True], ids=["rmat", "er"])
def graph(request):
    return G(request.param)


@pytest.mark.parametrize("shape", [40, 41, 42, 80, 81, 82, 160, 161, 162])
@pytest.mark.parametrize("direction,kb", [(0, 0), (0, 16), (0, 48), (1, 0), (1, 16), (1, 64)])
@pytest.mark.parametrize("variant", ["radar", "hubdup", "push-pull"])
def test_pagerank_schedules(graph, shape, direction, kb, variant):
    G_ = graph.gs if variant == "radar" else graph.g
    with options(sweep_shape=shape, direction=direction, hub_smem_kb=kb):
        r, it, _ = G_.pagerank(variant, 20)
    assert it == graph.pr[1]
    assert_close(r, graph.pr[0], what=f"pr {variant} shape {shape} dir {direction} kb {kb}")


@pytest.mark.parametrize("div", [1, 2, 5, 20, 1000])
@pytest.mark.parametrize("direction", [0, 1])
@pytest.mark.parametrize("variant", ["radar", "push", "push-pull", "hubdup"])
def test_radii_and_bfs_schedules(graph, div, direction, variant):
    G_ = graph.gs if variant == "radar" else graph.g
    with options(dense_div=div, direction=direction):
        r, _ = G_.radii(variant)
        _, depth, _, _ = G_.bfs(variant, graph.root)
    assert np.array_equal(r, graph.radii)
    assert np.array_equal(depth, graph.depth)


@pytest.mark.parametrize("div", [2, 20, 80])
@pytest.mark.parametrize("direction,kb", [(0, 0), (0, 16), (1, 0)])
@pytest.mark.parametrize("variant", ["radar", "hubdup", "push-pull", "push"])
def test_pagerank_delta_schedules(graph, div, direction, kb, variant):
    G_ = graph.gs if variant == "radar" else graph.g
    with options(dense_div=div, direction=direction, hub_smem_kb=kb):
        r, it, _ = G_.pagerank_delta(variant, 30)
    assert it == graph.prd[1]
    assert_close(r, graph.prd[0], what=f"prd {variant} div {div} dir {direction} kb {kb}")


@pytest.mark.parametrize("div", [5, 20, 80])
@pytest.mark.parametrize("kb", [0, 4, 16, 48])
@pytest.mark.parametrize("fwd_hubs", [1, 0])
@pytest.mark.parametrize("variant", ["radar", "hubdup", "push-pull"])
def test_bc_schedules(graph, div, kb, fwd_hubs, variant):
    G_ = graph.gs if variant == "radar" else graph.g
    with options(dense_div=div, hub_smem_kb=kb, bc_fwd_hubs=fwd_hubs):
        d, _ = G_.bc_sources(graph.bc_src, variant)
    assert_close(d, graph.bc, what=f"bc {variant} div {div} kb {kb} fwd_hubs {fwd_hubs}")


def test_autotune_keeps_results(graph):
    G_ = graph.gs
    before = (G_.pagerank("radar", 20)[0], G_.radii("radar")[0], G_.bfs("radar", graph.root)[1])
    G_.autotune("radar")
    after = (G_.pagerank("radar", 20)[0], G_.radii("radar")[0], G_.bfs("radar", graph.root)[1])
    # the untuned RADAR schedule pushes with FP64 atomics (the reference's
    # arbitrary addition order); the tuned one may pull (exact sums)
    assert_close(before[0], after[0], what="PageRank before/after tuning")
    assert np.array_equal(before[1], after[1]) and np.array_equal(before[2], after[2])
    assert np.array_equal(after[1], graph.radii)


def test_pull_schedules_are_bit_identical(graph):
    """Every pull sweep shape, with and without the shared-memory hub cache,
    forms each vertex's sum exactly and rounds it once: the ranks are
    identical bit for bit, whatever the order of the additions."""
    G_ = graph.gs
    G_.clear_tuning()  # the thread's options below, not an earlier test's tuning
    ref = None
    for shape in (40, 41, 42, 80, 81, 82, 160, 161, 162):
        for kb in (0, 48):
            with options(direction=1, sweep_shape=shape, hub_smem_kb=kb):
                r, it, _ = G_.pagerank("radar", 20)
            if ref is None:
                ref = r
            assert np.array_equal(r, ref), f"pull shape {shape} kb {kb}"
    with options(direction=1):
        r2, _, _ = graph.g.pagerank("push-pull", 20)
    assert np.array_equal(r2, ref)  # the unsorted graph, mapped back to original ids
