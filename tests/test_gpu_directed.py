"""Directed graphs on the GPU against the reference's own apps run without -s
(tests/golden/make_golden.py): the loader and in-degree sort, PageRank (all
variants), PageRankDelta, BFS, BC with 1-3 sources (the reference transposes
the graph once per source) and Radii, under both directions of the dense
iterations."""

import contextlib
import os
import subprocess

import numpy as np
import pytest

import radar_graph as rg
from conftest import DIRECTED_NAMES, ROOT, assert_close

pytestmark = pytest.mark.gpu

SORTED = rg.SORTED_VARIANTS


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


class D:
    def __init__(self, g):
        self.g = rg.Graph.from_csr_directed(g["off"], g["adj"])
        self.gs = self.g.degree_sort()  # in-degree order (-preprocess 1)

    def pick(self, variant):
        return self.gs if variant in SORTED else self.g


@pytest.fixture(scope="module")
def dev(golden_directed):
    return {name: D(g) for name, g in golden_directed.items()}


def _write_raw(g, path):
    raw_off = np.append(g["raw_off"], np.uint32(len(g["raw_adj"])))
    rg.write_adjacency(path, raw_off, g["raw_adj"])


@pytest.mark.parametrize("name", DIRECTED_NAMES)
def test_loader_and_sort(golden_directed, dev, tmp_path, name):
    g = golden_directed[name]
    path = tmp_path / "d.adj"
    _write_raw(g, path)
    off, adj = rg.read_graph(path, symmetric=False)
    assert np.array_equal(off, g["off"]) and np.array_equal(adj, g["adj"])
    assert dev[name].g.directed and dev[name].gs.directed
    assert np.array_equal(dev[name].gs.new_ids, g["new_ids"])


@pytest.mark.parametrize("name", DIRECTED_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting", "hubdup", "radar"])
@pytest.mark.parametrize("direction", [0, 1])
def test_pagerank(golden_directed, dev, name, variant, direction):
    g = golden_directed[name]
    key = f"pr_{variant}" if f"pr_{variant}" in g else "pr_push"
    with options(direction=direction):
        r, it, _ = dev[name].pick(variant).pagerank(variant, 20)
    assert_close(r, g[key], what=f"{name} pr {variant} dir {direction}")


@pytest.mark.parametrize("name", DIRECTED_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting"])
@pytest.mark.parametrize("direction", [0, 1])
def test_pagerank_delta(golden_directed, dev, name, variant, direction):
    g = golden_directed[name]
    with options(direction=direction):
        r, it, _ = dev[name].pick(variant).pagerank_delta(variant, 20)
    assert it == int(g[f"prd_iters_{variant}"][0])
    assert_close(r, g[f"prd_{variant}"], what=f"{name} prd {variant} dir {direction}")


@pytest.mark.parametrize("name", DIRECTED_NAMES)
@pytest.mark.parametrize("variant", ["push", "push-pull", "degree-sorting", "radar"])
@pytest.mark.parametrize("direction,div", [(0, 20), (1, 20), (1, 2)])
def test_bfs_bc_radii(golden_directed, dev, name, variant, direction, div):
    g = golden_directed[name]
    gv = "degree-sorting" if variant == "radar" else variant  # results are the same in every variant
    G = dev[name].pick(variant)
    with options(direction=direction, dense_div=div):
        for ri, root in enumerate(g["bfs_roots"]):
            _, depth, _, _ = G.bfs(variant, int(root))
            assert np.array_equal(depth, g[f"bfs{ri}_{gv}"]), (name, variant, ri)
        for k in (1, 2, 3):
            d, _ = G.bc(variant, k)
            assert_close(d, g[f"bc{k}_{gv}"], what=f"{name} bc{k} {variant}")
        r, _ = G.radii(variant)
    assert np.array_equal(r, g[f"radii_{gv}"])


def test_directed_refusals(golden_directed):
    g = golden_directed[DIRECTED_NAMES[0]]
    with rg.Graph.from_csr_directed(g["off"], g["adj"]) as G:
        with pytest.raises(rg.RgError, match="undirected"):
            G.triangles()


def test_served_directed_queries(golden_directed):
    """Directed graphs served with coalescing: every result equals the query
    run alone (BC within 1e-9 relative)."""
    g = golden_directed["drmat13"]
    with rg.Graph.from_csr_directed(g["off"], g["adj"]) as G0, G0.degree_sort() as G:
        n = G.n
        deg = np.diff(g["off"].astype(np.int64))
        srcs = [int(v) for v in np.nonzero(deg)[0][::97][:30]]
        qs = [("bfs", s) for s in srcs] + [("bc", s) for s in srcs[:20]] + [("radii", i) for i in range(12)]
        with rg.Server([G], workers=1, max_batch=64) as S:
            ts = [S.submit(0, kind, s) for kind, s in qs]
            outs = [S.wait(t, 0, kind)[0] for t, (kind, _) in zip(ts, qs)]
            st = S.stats()
        assert st["batched"] > 0
        for (kind, s), got in zip(qs, outs):
            if kind == "bfs":
                assert np.array_equal(got, G.bfs("push", s)[1]), (kind, s)
            elif kind == "bc":
                assert_close(got, G.bc_sources(np.array([s], np.uint32), "push")[0], what=f"bc {s}")
            else:
                assert np.array_equal(got, G.radii_seeds(rg.radii_query_seeds(s, n), "push")[0]), (kind, s)


def test_cli_directed(golden_directed, tmp_path):
    g = golden_directed["drmat10"]
    path = tmp_path / "d.adj"
    _write_raw(g, path)
    out = tmp_path / "pr.txt"
    exe = os.path.join(ROOT, "radar-graph_gb300", "bin", "PageRank")
    r = subprocess.run([exe, "-rounds", "0", "-maxiters", "20", "-variant", "degree-sorting", "-out", str(out),
                        str(path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert_close(np.loadtxt(out), g["pr_degree-sorting"], what="directed PageRank via CLI")
