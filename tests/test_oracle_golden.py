"""Pins the oracle (the CPU restatement in oracle/oracle.cc) against golden
vectors produced by the reference's own OpenMP apps (tests/golden/make_golden.py).
CPU only."""

import numpy as np
import pytest

import oracle as orc
from conftest import GOLDEN_NAMES, assert_close

SORTED = ("degree-sorting", "radar")


@pytest.fixture(scope="module")
def graphs(golden):
    out = {}
    for name, g in golden.items():
        n = len(g["raw_off"])
        off, adj = orc.dedup_symmetric(n, g["raw_off"], g["raw_adj"])
        ids, so, sa = orc.degree_sort(off, adj)
        out[name] = dict(g=g, off=off, adj=adj, ids=ids, so=so, sa=sa)
    return out


def _pick(G, variant):
    return (G["so"], G["sa"]) if variant in SORTED else (G["off"], G["adj"])


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_loader_cleanup(graphs, name):
    G = graphs[name]
    assert np.array_equal(G["off"], G["g"]["off"])
    assert np.array_equal(G["adj"], G["g"]["adj"])


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_degree_sort_permutation(graphs, name):
    G = graphs[name]
    assert np.array_equal(G["ids"], G["g"]["new_ids"])
    # relabelled lists keep their order (IO.h:877-895)
    inv = np.argsort(G["ids"])
    for r in range(0, len(G["ids"]), max(1, len(G["ids"]) // 50)):
        v = inv[r]
        assert np.array_equal(G["sa"][G["so"][r]:G["so"][r + 1]], G["ids"][G["adj"][G["off"][v]:G["off"][v + 1]]])


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting", "hubdup", "radar"])
def test_pagerank(graphs, name, variant):
    G = graphs[name]
    key = f"pr_{variant}"
    if key not in G["g"]:
        pytest.skip("no golden for this variant on this graph")
    o, a = _pick(G, variant)
    r, it, _ = orc.pagerank(o, a, variant, 20, 4)
    if variant in SORTED:
        r = r[G["ids"]]
    assert 1 <= it <= 21
    assert_close(r, G["g"][key], what=key)


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_pagerank_l1_break(graphs, name):
    G = graphs[name]
    r, it, l1 = orc.pagerank(G["off"], G["adj"], "push", 200, 4)
    assert it == int(G["g"]["pr200_iters"][0])
    assert l1 < 1e-7
    assert_close(r, G["g"]["pr200_push"], what="pr200")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting", "hubdup", "radar"])
def test_pagerank_delta(graphs, name, variant):
    G = graphs[name]
    key = f"prd_{variant}"
    if key not in G["g"]:
        pytest.skip("no golden for this variant on this graph")
    o, a = _pick(G, variant)
    r, it, l1 = orc.pagerank_delta(o, a, variant, 20, 4)
    if variant in SORTED:
        r = r[G["ids"]]
    assert it == int(G["g"][f"prd_iters_{variant}"][0])
    assert_close(r, G["g"][key], what=key)


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_pagerank_delta_maxiters_cutoff(graphs, name):
    G = graphs[name]
    r, it, _ = orc.pagerank_delta(G["off"], G["adj"], "push", 5, 4)
    assert it == int(G["g"]["prd5_iters"][0])
    assert_close(r, G["g"]["prd5_push"], what="prd5")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting", "radar"])
def test_bfs_depths(graphs, name, variant):
    G = graphs[name]
    for ri, root in enumerate(G["g"]["bfs_roots"]):
        key = f"bfs{ri}_{variant}"
        if key not in G["g"]:
            pytest.skip("no golden")
        o, a = _pick(G, variant)
        rr = G["ids"][root] if variant in SORTED else root
        par, _ = orc.bfs(o, a, rr, variant, 4)
        d = orc.depths_from_parents(par)
        assert orc.check_bfs_tree(o, a, rr, par, d)
        if variant in SORTED:
            d = d[G["ids"]]
        assert np.array_equal(d, G["g"][key]), key
        assert np.array_equal(d, orc.bfs_depths(G["off"], G["adj"], root))


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting", "radar"])
@pytest.mark.parametrize("k", [1, 4])
def test_bc(graphs, name, variant, k):
    G = graphs[name]
    key = f"bc{k}_{variant}"
    if key not in G["g"]:
        pytest.skip("no golden")
    deg = np.diff(G["off"].astype(np.int64)).astype(np.uint32)
    src = orc.bc_sources(deg, k)
    o, a = _pick(G, variant)
    s2 = G["ids"][src] if variant in SORTED else src
    d, _ = orc.bc(o, a, s2, variant, 4)
    if variant in SORTED:
        d = d[G["ids"]]
    assert_close(d, G["g"][key], what=key)


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting"])
def test_radii(graphs, name, variant):
    G = graphs[name]
    n = len(G["off"]) - 1
    seeds = orc.radii_seeds(n)
    o, a = _pick(G, variant)
    s2 = G["ids"][seeds] if variant in SORTED else seeds
    r, _ = orc.radii(o, a, s2, variant, 4)
    if variant in SORTED:
        r = r[G["ids"]]
    assert np.array_equal(r, G["g"][f"radii_{variant}"])


def test_radii_seed_hash_matches_python():
    import radar_graph as rg
    for n in (12, 1000, 1 << 20):
        assert np.array_equal(orc.radii_seeds(n), rg.radii_seeds_orig(n))


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_triangles(graphs, name):
    """GAP tc_local's total (the reference binary) and the per-vertex counts'
    invariant (tc_local.cc:119-126: they sum to three times the total)."""
    G = graphs[name]
    counts, total = orc.triangles(G["off"], G["adj"], 4)
    assert total == int(G["g"]["tc_total"][0])
    assert int(counts.sum()) == 3 * total


def test_triangles_brute_force():
    import radar_graph as rg
    off, adj = rg.rmat_csr(9, 8, seed=5)
    counts, total = orc.triangles(off, adj, 2)
    n = len(off) - 1
    nb = [set(adj[off[v]:off[v + 1]].tolist()) for v in range(n)]
    want = np.zeros(n, np.uint64)
    t = 0
    for u in range(n):
        for v in nb[u]:
            if v > u:
                for w in nb[u] & nb[v]:
                    if w > v:
                        t += 1
                        want[[u, v, w]] += 1
    assert total == t and np.array_equal(counts, want)
