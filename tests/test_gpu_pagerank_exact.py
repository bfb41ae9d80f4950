"""PageRank's arithmetic, checked bit for bit.

A pure-Python model computes what the pull sweeps promise: per iteration the
reference's terms p[s]/deg(s) (IEEE double division, PageRank.C:48), each
vertex's sum of them exact (Python integers on the terms scaled by 2^124) and
rounded to the nearest double once, p' = fma(0.85, sum, 0.15/n) (exact
rational arithmetic, rounded once) and the L1 break on the exact sum of the
double |p - p'| (PageRank.C:163-176).  Every pull schedule must equal the
model exactly; the model itself is checked against the oracle (the reference's
order of FP64 additions) to 1e-12 on the CPU."""

from fractions import Fraction

import numpy as np
import pytest

import oracle as orc
import radar_graph as rg

SCALE = 2 ** 124


def model_pagerank(off, adj, max_iters, in_off=None, in_adj=None):
    """(ranks, iteration count as the reference prints it) of the exact-sum
    PageRank; in_off/in_adj: in-lists of a directed graph (else symmetric)."""
    n = len(off) - 1
    io, ia = (off, adj) if in_off is None else (in_off, in_adj)
    deg = np.diff(off.astype(np.int64))
    p = [1.0 / n] * n
    added = (1 - 0.85) * (1.0 / n)
    fa, fd = Fraction(added), Fraction(0.85)
    iters = max_iters + 1
    for it in range(max_iters):
        c = [int(Fraction(p[s] / float(deg[s])) * SCALE) if deg[s] else 0 for s in range(n)]
        pn, l1 = [], 0
        for v in range(n):
            s = sum(c[u] for u in ia[io[v]:io[v + 1]])
            total = float(Fraction(s, SCALE))
            x = float(fd * Fraction(total) + fa)  # fma: one rounding
            l1 += int(Fraction(abs(p[v] - x)) * SCALE)
            pn.append(x)
        p = pn
        if Fraction(l1, SCALE) < Fraction(1e-7):
            iters = it + 1
            break
    return np.array(p), iters


@pytest.fixture(scope="module")
def small():
    return orc.rmat_csr(9, 8, 4)


def test_model_agrees_with_the_oracle(small):
    off, adj = small
    r, it = model_pagerank(off, adj, 20)
    ro, ito, _ = orc.pagerank(off, adj, "push", 20, 1)
    assert it == ito
    assert np.max(np.abs(r - ro) / ro) < 1e-12


@pytest.mark.gpu
def test_pull_ranks_equal_the_exact_model_bit_for_bit(small):
    off, adj = small
    want, it_want = model_pagerank(off, adj, 20)
    with rg.Graph.from_csr(off, adj) as g, g.degree_sort() as gs:
        r, it, _ = g.pagerank("push-pull", 20)
        assert it == it_want and np.array_equal(r, want)
        old = rg.get_option("direction")
        rg.set_option("direction", 1)
        try:
            r2, it2, _ = gs.pagerank("radar", 20)
        finally:
            rg.set_option("direction", old)
        assert it2 == it_want and np.array_equal(r2, want)


@pytest.mark.gpu
def test_l1_break_iteration_equals_the_model(small):
    off, adj = small
    want, it_want = model_pagerank(off, adj, 200)
    assert it_want < 201  # the run stops on L1 < 1e-7
    with rg.Graph.from_csr(off, adj) as g:
        r, it, l1 = g.pagerank("push-pull", 200)
    assert it == it_want and np.array_equal(r, want) and l1 < 1e-7


@pytest.mark.gpu
def test_directed_pull_equals_the_model():
    off, adj = orc.rmat_csr(9, 8, 6)
    # a directed graph: each symmetric edge kept one way (u < v), every third also the other way
    src = np.repeat(np.arange(len(off) - 1), np.diff(off.astype(np.int64))).astype(np.uint32)
    keep = (src < adj) | (np.arange(len(adj)) % 3 == 0)
    n = len(off) - 1
    with rg.Graph.from_edges(n, src[keep], adj[keep], directed=True) as g:
        o, a, _ = g.download()
        io, ia = orc.transpose(o, a)
        want, it_want = model_pagerank(o, a, 20, io, ia)
        r, it, _ = g.pagerank("push-pull", 20)
    assert it == it_want and np.array_equal(r, want)
