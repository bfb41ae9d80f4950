"""Parity at a large size: R-MAT scale 20, edge factor 16, seed 1 (1,048,576
vertices, 31,404,780 directed edges), every app on the GPU against the
oracle on the same graph.

The graph is generated and cleaned by the oracle (its restatement of the GAP
generator and of the loader's clean-up), so nothing of the product goes into
the input.  Checks, with the tolerances of the small-graph tests:
  - the degree-sort permutation, bit-exact (IO.h:843-895);
  - RADAR PageRank, 20 iterations, and push-pull PageRank on the unsorted
    graph, 1e-9 relative (PageRank.C:163-176);
  - 16 search roots by GAP's SourcePicker (benchmark.h:47-64), identical
    roots; BFS depths from each, bit-exact, for RADAR on the sorted graph and
    push-pull on the unsorted one (BFS.C:122-188); the 16 roots as one
    multi-source traversal, the same rows;
  - BC from 4 reference-picked sources, chained, 1e-9 relative with NaN
    positions equal (BC-manyiter-v2.C:205-367);
  - Radii with the 64 hashInt samples, bit-exact (Radii.C:140-218).
"""

import numpy as np
import pytest

import oracle as orc
import radar_graph as rg
from conftest import assert_close

pytestmark = pytest.mark.gpu

SCALE = 20


@pytest.fixture(scope="module")
def s20():
    off, adj = orc.rmat_csr(SCALE, 16, 1)
    ids, so, sa = orc.degree_sort(off, adj)
    g = rg.Graph.from_csr(off, adj)
    gs = g.degree_sort()
    deg = np.diff(off.astype(np.int64)).astype(np.uint32)
    yield {"off": off, "adj": adj, "ids": ids, "so": so, "sa": sa, "g": g, "gs": gs, "deg": deg}
    gs.free()
    g.free()


def test_s20_degree_sort_permutation(s20):
    assert len(s20["adj"]) == 31404780
    assert np.array_equal(s20["gs"].new_ids, s20["ids"])


@pytest.mark.parametrize("variant", ["radar", "push-pull"])
def test_s20_pagerank_20_iterations(s20, variant):
    G = s20["gs"] if variant == "radar" else s20["g"]
    r, it, _ = G.pagerank(variant, 20)
    if variant == "radar":
        want, ito, _ = orc.pagerank(s20["so"], s20["sa"], "radar", 20)
        want = want[s20["ids"]]
    else:
        want, ito, _ = orc.pagerank(s20["off"], s20["adj"], "push-pull", 20)
    assert it == ito
    assert_close(r, want, what=f"s20 PageRank {variant}")


def test_s20_bfs_16_source_picker_roots(s20):
    roots = s20["g"].pick_roots(16)
    assert np.array_equal(roots, orc.source_picker(s20["deg"], 16))
    assert np.array_equal(s20["gs"].pick_roots(16), roots)
    rows, _ = s20["g"].bfs_multi(roots)
    for q, r in enumerate(roots):
        want = orc.bfs_depths(s20["off"], s20["adj"], int(r))
        assert np.array_equal(s20["gs"].bfs("radar", int(r))[1], want), f"RADAR BFS root {r}"
        assert np.array_equal(s20["g"].bfs("push-pull", int(r))[1], want), f"push-pull BFS root {r}"
        assert np.array_equal(rows[q], want), f"multi-source row {q}"


def test_s20_bc_4_sources(s20):
    src = s20["gs"].bc_pick_sources(4)
    assert np.array_equal(src, orc.bc_sources(s20["deg"], 4))
    got, _ = s20["gs"].bc_sources(src, "radar")
    want, _ = orc.bc(s20["so"], s20["sa"], s20["ids"][src], "radar")
    assert_close(got, want[s20["ids"]], what="s20 BC 4 sources")


def test_s20_radii(s20):
    got, _ = s20["gs"].radii("radar")
    seeds = orc.radii_seeds(len(s20["off"]) - 1)
    want, _ = orc.radii(s20["so"], s20["sa"], s20["ids"][seeds], "radar")
    assert np.array_equal(got, want[s20["ids"]])
