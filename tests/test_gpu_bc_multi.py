"""Multi-source BC (rg_bc_multi): every row equals the single-source BC from
that source (rg_bc_sources with one source, itself pinned to the reference's
BC-manyiter-v2 output), within 1e-9 relative and with identical NaN
positions, on symmetric and directed, unsorted and degree-sorted graphs, for
1..64 sources including repeats and isolated vertices."""

import numpy as np
import pytest

import radar_graph as rg
from conftest import DIRECTED_NAMES, GOLDEN_NAMES, assert_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as b
    b.build()


def _check_rows(G, sources, what):
    rows, levels = G.bc_multi(sources)
    assert rows.shape == (len(sources), G.n) and levels >= 1
    for q, s in enumerate(sources):
        want, _ = G.bc_sources(np.array([s], np.uint32), "push")
        assert_close(rows[q], want, what=f"{what} source {s} (row {q})")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("sorted_handle", [False, True])
def test_golden_first_source(golden, name, sorted_handle):
    """Row 0 for the reference's first drawn source is the golden 1-source BC."""
    g = golden[name]
    with rg.Graph.from_csr(g["off"], g["adj"]) as G0:
        G = G0.degree_sort() if sorted_handle else G0
        src = G.bc_pick_sources(3)
        rows, _ = G.bc_multi(src)
        assert_close(rows[0], g["bc1_push"], what=f"{name} golden bc1")
        _check_rows(G, src, name)
        if sorted_handle:
            G.free()


@pytest.mark.parametrize("k", [1, 5, 32, 33, 64])
@pytest.mark.parametrize("uniform", [False, True], ids=["rmat", "er"])
def test_rmat_many_sources(k, uniform):
    off, adj = rg.rmat_csr(14, 16, seed=3, uniform=uniform)
    deg = np.diff(off.astype(np.int64))
    rng = np.random.default_rng(k)
    src = rng.integers(0, len(deg), size=k).astype(np.uint32)
    if k >= 5:
        src[1] = src[0]  # a repeated source
        iso = np.nonzero(deg == 0)[0]
        if len(iso):
            src[2] = iso[0]  # an isolated source: its row is NaN except itself (0)
    with rg.Graph.from_csr(off, adj) as G, G.degree_sort() as S:
        _check_rows(S, src, f"s14 k={k}")
        if k in (1, 33):
            _check_rows(G, src, f"s14 unsorted k={k}")


@pytest.mark.parametrize("name", DIRECTED_NAMES)
def test_directed(golden_directed, name):
    g = golden_directed[name]
    with rg.Graph.from_csr_directed(g["off"], g["adj"]) as G, G.degree_sort() as S:
        deg = np.diff(g["off"].astype(np.int64))
        src = np.nonzero(deg)[0][:: max(1, len(deg) // 40)][:40].astype(np.uint32)
        _check_rows(G, src, f"{name} directed")
        _check_rows(S, src[:7], f"{name} directed sorted")


def test_star_hub_split_over_tiles():
    """A hub whose edges span many warp tiles (atomics merge its row)."""
    n = 5000
    src = np.zeros(n - 1, np.uint32)
    dst = np.arange(1, n, dtype=np.uint32)
    ring_s = np.arange(1, n - 1, dtype=np.uint32)
    off, adj = rg.csr_from_edges(n, np.concatenate([src, ring_s]), np.concatenate([dst, ring_s + 1]))
    with rg.Graph.from_csr(off, adj) as G:
        _check_rows(G, np.array([1, 7, 2500, 4999, 0], np.uint32), "star+path")


def test_errors():
    off, adj = rg.rmat_csr(8, 4, seed=1)
    with rg.Graph.from_csr(off, adj) as G:
        with pytest.raises(rg.RgError):
            G.bc_multi(np.zeros(0, np.uint32))
        with pytest.raises(rg.RgError):
            G.bc_multi(np.zeros(65, np.uint32))
        with pytest.raises(rg.RgError):
            G.bc_multi(np.array([G.n], np.uint32))


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_rows_equal_the_oracle(golden, name):
    """Independent of the GPU single-source path: each row against the CPU
    oracle's single-source BC (oracle/oracle.cc, BC-manyiter-v2.C)."""
    import oracle as orc
    g = golden[name]
    with rg.Graph.from_csr(g["off"], g["adj"]) as G:
        src = G.bc_pick_sources(4)
        rows, _ = G.bc_multi(src)
    for q, s in enumerate(src):
        want, _ = orc.bc(g["off"], g["adj"], np.array([s], np.uint32), "push", 0)
        assert_close(rows[q], want, what=f"{name} oracle source {s}")


def _layered(width, layers):
    """Vertex 0, then `layers` layers of `width` vertices, complete bipartite
    between consecutive layers: vertex 0 reaches layer k by width^(k-1) paths."""
    src, dst = [], []
    prev = [0]
    nxt_id = 1
    for _ in range(layers):
        cur = list(range(nxt_id, nxt_id + width))
        nxt_id += width
        for a in prev:
            for b in cur:
                src.append(a)
                dst.append(b)
        prev = cur
    return rg.csr_from_edges(nxt_id, np.array(src, np.uint32), np.array(dst, np.uint32))


def test_path_counts_past_64_bits_fall_back():
    """16^17 = 2^68 shortest paths reach the last layer: the 64-bit counts
    would wrap, so the call must answer through single-source passes."""
    off, adj = _layered(16, 18)
    with rg.Graph.from_csr(off, adj) as G:
        _check_rows(G, np.array([0, 3, 200], np.uint32), "layered 16x18")


def test_path_counts_below_64_bits():
    off, adj = _layered(8, 12)  # 8^11 = 2^33 paths: exact in 64 bits
    with rg.Graph.from_csr(off, adj) as G:
        _check_rows(G, np.array([0, 1, 50, 96], np.uint32), "layered 8x12")


@pytest.mark.parametrize("n", [1, 6])
def test_no_edges(n):
    off = np.zeros(n + 1, np.uint32)
    with rg.Graph.from_csr(off, np.zeros(0, np.uint32)) as G:
        src = np.arange(min(n, 3), dtype=np.uint32)
        rows, levels = G.bc_multi(src)
        for q, s in enumerate(src):
            want = np.full(n, np.nan)
            want[s] = 0.0
            assert_close(rows[q], want, what=f"isolated source {s}")
