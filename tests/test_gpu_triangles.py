"""Triangle counting (GAP tc_local) on the GPU: totals equal the reference
binary's (golden) and the oracle's, per-vertex counts equal the oracle's,
for unsorted and degree-sorted handles and every hub budget."""

import contextlib
import os
import subprocess

import numpy as np
import pytest

import oracle as orc
import radar_graph as rg
from conftest import GOLDEN_NAMES, ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as b
    b.build()


@contextlib.contextmanager
def hub_kb(kb):
    old = rg.get_option("hub_smem_kb")
    rg.set_option("hub_smem_kb", kb)
    try:
        yield
    finally:
        rg.set_option("hub_smem_kb", old)


@pytest.mark.parametrize("name", GOLDEN_NAMES)
@pytest.mark.parametrize("sorted_handle", [False, True])
def test_golden_totals(golden, name, sorted_handle):
    g = golden[name]
    with rg.Graph.from_csr(g["off"], g["adj"]) as G:
        H = G.degree_sort() if sorted_handle else G
        counts, total = H.triangles()
        assert total == int(g["tc_total"][0])
        want, _ = orc.triangles(g["off"], g["adj"], 0)
        assert np.array_equal(counts, want)
        if sorted_handle:
            H.free()


@pytest.mark.parametrize("kb", [0, 16, 48, 200])
@pytest.mark.parametrize("uniform", [False, True], ids=["rmat", "er"])
def test_s16_vs_oracle(kb, uniform):
    off, adj = rg.rmat_csr(16, 16, seed=1, uniform=uniform)
    want, wt = orc.triangles(off, adj, 0)
    with rg.Graph.from_csr(off, adj) as G, hub_kb(kb):
        counts, total = G.triangles()
    assert total == wt
    assert np.array_equal(counts, want)


def test_no_edges_and_isolated():
    off = np.zeros(6, np.uint32)
    with rg.Graph.from_csr(off, np.zeros(0, np.uint32)) as G:
        counts, total = G.triangles()
    assert total == 0 and not counts.any()


def test_cli_triangle_count(golden, tmp_path):
    g = golden["rmat12"]
    raw_off = np.append(g["raw_off"], np.uint32(len(g["raw_adj"])))
    path = tmp_path / "g.adj"
    rg.write_adjacency(path, raw_off, g["raw_adj"])
    out = tmp_path / "tri.txt"
    exe = os.path.join(ROOT, "radar-graph_gb300", "bin", "TriangleCount")
    r = subprocess.run([exe, "-s", "-rounds", "0", "-out", str(out), str(path)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert f"{int(g['tc_total'][0])} triangles" in r.stdout
    want, _ = orc.triangles(g["off"], g["adj"], 0)
    assert np.array_equal(np.loadtxt(out, dtype=np.uint64), want)


@pytest.mark.parametrize("fmt", ["el", "wel", "gr", "graph", "mtx", "sym.mtx"])
def test_cli_reads_gap_edge_lists(tmp_path, fmt):
    """TriangleCount -s on each GAP text format counts what GAP's tc_local
    counted on the same file (golden)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_gap_formats as mg
    gold = np.load(os.path.join(ROOT, "tests", "golden", "gap_formats.npz"))
    want = dict(zip(gold["formats"].tolist(), gold["totals"].tolist()))[fmt]
    path = mg.write_formats(gold["src"], gold["dst"], str(tmp_path / "g"))[fmt]
    exe = os.path.join(ROOT, "radar-graph_gb300", "bin", "TriangleCount")
    r = subprocess.run([exe, "-s", "-rounds", "0", path], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert f"{want} triangles" in r.stdout
