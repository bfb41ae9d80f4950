"""Batched Radii (rg_radii_multi): every query's row equals the same query
run alone (rg_radii_seeds), bit for bit, on symmetric and directed, unsorted
and degree-sorted graphs, for 1..16 queries, including colliding samples."""

import numpy as np
import pytest

import radar_graph as rg
from conftest import DIRECTED_NAMES, GOLDEN_NAMES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as b
    b.build()


def _check(G, seeds, what):
    rows, rounds = G.radii_multi(seeds)
    assert rows.shape == (len(seeds), G.n)
    for q in range(len(seeds)):
        want, _ = G.radii_seeds(seeds[q], "push")
        assert np.array_equal(rows[q], want), f"{what} query {q}"
    return rounds


def _query_seeds(n, nq, k=64, base=0):
    return np.stack([rg.radii_query_seeds(base + q, n)[:k] for q in range(nq)])


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_golden_graphs(golden, name):
    g = golden[name]
    with rg.Graph.from_csr(g["off"], g["adj"]) as G, G.degree_sort() as S:
        n = G.n
        seeds = _query_seeds(n, 5, k=min(n, 64))
        _check(G, seeds, name)
        _check(S, seeds, name + " sorted")
        # the reference's own sample set as query 0
        ref = np.stack([rg.radii_query_seeds(0, n)[: min(n, 64)]])
        rows, _ = G.radii_multi(ref)
        assert np.array_equal(rows[0], G.radii_seeds(ref[0], "push")[0])


@pytest.mark.parametrize("nq", [1, 2, 3, 4, 5, 8, 9, 16])
@pytest.mark.parametrize("uniform", [False, True], ids=["rmat", "er"])
def test_many_queries(nq, uniform):
    off, adj = rg.rmat_csr(14, 16, seed=5, uniform=uniform)
    with rg.Graph.from_csr(off, adj) as G0, G0.degree_sort() as G:
        seeds = _query_seeds(G.n, nq, base=11)
        if nq >= 3:
            seeds[1, 5] = seeds[1, 9]  # a collision inside one query: the larger sample index wins
            seeds[2, :] = seeds[0, :]  # two identical queries
        _check(G, seeds, f"s14 nq={nq}")


@pytest.mark.parametrize("name", DIRECTED_NAMES)
def test_directed(golden_directed, name):
    g = golden_directed[name]
    with rg.Graph.from_csr_directed(g["off"], g["adj"]) as G:
        _check(G, _query_seeds(G.n, 6, k=min(G.n, 64), base=3), name)


def test_errors():
    off, adj = rg.rmat_csr(8, 4, seed=1)
    with rg.Graph.from_csr(off, adj) as G:
        with pytest.raises(rg.RgError):
            G.radii_multi(np.zeros((17, 4), np.uint32))
        with pytest.raises(rg.RgError):
            G.radii_multi(np.zeros((2, 65), np.uint32))
        with pytest.raises(rg.RgError):
            G.radii_multi(np.full((2, 4), G.n, np.uint32))


@pytest.mark.parametrize("n", [1, 6])
def test_no_edges(n):
    off = np.zeros(n + 1, np.uint32)
    with rg.Graph.from_csr(off, np.zeros(0, np.uint32)) as G:
        seeds = np.stack([rg.radii_query_seeds(q, n) for q in range(3)])
        _check(G, seeds, f"no edges n={n}")
