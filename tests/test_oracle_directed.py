"""Pins the oracle on DIRECTED graphs against the reference's own apps run
without -s (tests/golden/make_golden.py): the loader's clean-up and CSC, the
in-degree sort, and PageRank, PageRankDelta, BFS, BC (whose graph the
reference transposes once per source) and Radii.  CPU only."""

import numpy as np
import pytest

import oracle as orc
from conftest import DIRECTED_NAMES, assert_close

SORTED = ("degree-sorting", "radar")


@pytest.fixture(scope="module")
def dgraphs(golden_directed):
    out = {}
    for name, g in golden_directed.items():
        n = len(g["raw_off"])
        off, adj = orc.dedup_directed(n, g["raw_off"], g["raw_adj"])
        io, ia = orc.transpose(off, adj)
        ids, so, sa, sio, sia = orc.degree_sort_directed(off, adj, io, ia)
        out[name] = dict(g=g, n=n, plain=(off, adj, io, ia), sorted=(so, sa, sio, sia), ids=ids)
    return out


def _run(G, variant):
    o, a, io, ia = G["sorted"] if variant in SORTED else G["plain"]
    return o, a, dict(in_off=io, in_adj=ia)


def _orig(G, variant, arr):
    return arr[G["ids"]] if variant in SORTED else arr


@pytest.mark.parametrize("name", DIRECTED_NAMES)
def test_loader_and_transpose(dgraphs, name):
    G = dgraphs[name]
    off, adj, io, ia = G["plain"]
    assert np.array_equal(off, G["g"]["off"]) and np.array_equal(adj, G["g"]["adj"])
    assert np.array_equal(io, G["g"]["in_off"]) and np.array_equal(ia, G["g"]["in_adj"])


@pytest.mark.parametrize("name", DIRECTED_NAMES)
def test_in_degree_sort(dgraphs, name):
    assert np.array_equal(dgraphs[name]["ids"], dgraphs[name]["g"]["new_ids"])


@pytest.mark.parametrize("name", DIRECTED_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting", "hubdup", "radar"])
def test_pagerank(dgraphs, name, variant):
    G = dgraphs[name]
    key = f"pr_{variant}"
    if key not in G["g"]:
        pytest.skip("no golden for this variant on this graph")
    o, a, kw = _run(G, variant)
    r, it, _ = orc.pagerank(o, a, variant, 20, 4, **kw)
    assert_close(_orig(G, variant, r), G["g"][key], what=key)


@pytest.mark.parametrize("name", DIRECTED_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting"])
def test_pagerank_delta(dgraphs, name, variant):
    G = dgraphs[name]
    o, a, kw = _run(G, variant)
    r, it, _ = orc.pagerank_delta(o, a, variant, 20, 4, **kw)
    assert it == int(G["g"][f"prd_iters_{variant}"][0])
    assert_close(_orig(G, variant, r), G["g"][f"prd_{variant}"], what=f"prd {variant}")


@pytest.mark.parametrize("name", DIRECTED_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting"])
def test_bfs_bc_radii(dgraphs, name, variant):
    G = dgraphs[name]
    g = G["g"]
    o, a, kw = _run(G, variant)
    ids = G["ids"] if variant in SORTED else np.arange(G["n"], dtype=np.uint32)
    for ri, root in enumerate(g["bfs_roots"]):
        par, _ = orc.bfs(o, a, int(ids[root]), variant, 4, **kw)
        assert np.array_equal(_orig(G, variant, orc.depths_from_parents(par)), g[f"bfs{ri}_{variant}"])
    off, _, io, _ = G["plain"]
    outdeg, indeg = np.diff(off.astype(np.int64)), np.diff(io.astype(np.int64))
    for k in (1, 2, 3):
        src = orc.bc_sources_directed(outdeg, indeg, k)
        d, _ = orc.bc(o, a, ids[src], variant, 4, **kw)
        assert_close(_orig(G, variant, d), g[f"bc{k}_{variant}"], what=f"bc{k} {variant}")
    seeds = orc.radii_seeds(G["n"])
    r, _ = orc.radii(o, a, ids[seeds], variant, 1, **kw)
    assert np.array_equal(_orig(G, variant, r), g[f"radii_{variant}"])
