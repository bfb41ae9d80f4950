"""Host-side input path of the product (librg.so, no GPU needed): Ligra text
and binary readers with the reference loader's clean-up, the seeded
generator, the edge-list -> CSR builder, and the C-ABI export list."""

import os
import re

import numpy as np
import pytest

import oracle as orc
import radar_graph as rg
from conftest import GOLDEN_NAMES, ROOT


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as b  # radar-graph_gb300/build.py
    b.build()


def _write_raw(path, off_n, adj):
    with open(path, "w") as f:
        f.write("AdjacencyGraph\n%d\n%d\n" % (len(off_n), len(adj)))
        f.write("".join(f"{int(x)}\n" for x in off_n))
        f.write("".join(f"{int(x)}\n" for x in adj))


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_text_reader_matches_reference_loader(golden, tmp_path, name):
    g = golden[name]
    p = tmp_path / "g.adj"
    _write_raw(p, g["raw_off"], g["raw_adj"])
    off, adj = rg.read_graph(p)
    assert np.array_equal(off, g["off"])
    assert np.array_equal(adj, g["adj"])


def test_writer_reader_roundtrip(tmp_path):
    off, adj = rg.rmat_csr(9, 8, seed=5)
    p = tmp_path / "w.adj"
    rg.write_adjacency(p, off, adj)
    o2, a2 = rg.read_graph(p)
    assert np.array_equal(off, o2) and np.array_equal(adj, a2)


def test_binary_reader(tmp_path):
    off, adj = rg.rmat_csr(9, 8, seed=6)
    base = tmp_path / "b"
    (tmp_path / "b.config").write_text(f"{len(off) - 1}\n")
    adj.astype(np.uint32).tofile(str(base) + ".adj")
    off[:-1].astype(np.uint32).tofile(str(base) + ".idx")
    o2, a2 = rg.read_graph(base, binary=True)
    assert np.array_equal(off, o2) and np.array_equal(adj, a2)


@pytest.mark.parametrize("text,what", [
    ("NotAGraph\n2\n1\n0\n1\n0\n", "header"),
    ("AdjacencyGraph\n2\n2\n0\n1\n1\n", "short"),
    ("AdjacencyGraph\n2\n1\n0\n1\n7\n", "edge id >= n"),
    ("AdjacencyGraph\n2\n1\n1\n0\n1\n", "non-monotone offsets"),
    ("AdjacencyGraph\n2\n1\n0\n1\n1\n5\n", "trailing"),
])
def test_bad_text_files_are_errors(tmp_path, text, what):
    p = tmp_path / "bad.adj"
    p.write_text(text)
    with pytest.raises(rg.RgError) as e:
        rg.read_graph(p)
    assert e.value.status == 5, what  # RG_EFORMAT, where the reference abort()s


def test_missing_file_is_io_error(tmp_path):
    with pytest.raises(rg.RgError) as e:
        rg.read_graph(tmp_path / "nope.adj")
    assert e.value.status == 4


def test_generator_is_deterministic_and_in_range():
    s1, d1 = rg.generate_edges(10, 8, seed=1)
    s2, d2 = rg.generate_edges(10, 8, seed=1)
    s3, _ = rg.generate_edges(10, 8, seed=2)
    assert np.array_equal(s1, s2) and np.array_equal(d1, d2)
    assert not np.array_equal(s1, s3)
    assert s1.max() < 1024 and d1.max() < 1024 and len(s1) == 8 << 10
    # R-MAT skew: the most popular endpoint is far above the mean degree
    deg = np.bincount(np.concatenate([s1, d1]), minlength=1024)
    assert deg.max() > 10 * deg.mean()
    su, du = rg.generate_edges(10, 8, seed=1, uniform=True)
    degu = np.bincount(np.concatenate([su, du]), minlength=1024)
    assert degu.max() < 4 * degu.mean()


@pytest.mark.parametrize("scale,ef,seed,uniform", [(8, 4, 1, False), (10, 16, 3, False), (9, 8, 2, True)])
def test_csr_from_edges_matches_text_loader_semantics(scale, ef, seed, uniform):
    s, d = rg.generate_edges(scale, ef, seed, uniform)
    n = 1 << scale
    off, adj = rg.csr_from_edges(n, s, d)
    # the same edge list through the oracle's restatement of IO.h:429-474
    ss = np.concatenate([s, d]).astype(np.int64)
    dd = np.concatenate([d, s]).astype(np.uint32)
    order = np.argsort(ss, kind="stable")
    raw_off = np.searchsorted(ss[order], np.arange(n)).astype(np.uint32)
    o2, a2 = orc.dedup_symmetric(n, raw_off, dd[order])
    assert np.array_equal(off, o2) and np.array_equal(adj, a2)


def test_csr_from_edges_rejects_out_of_range():
    with pytest.raises(rg.RgError) as e:
        rg.csr_from_edges(4, np.array([0, 9], np.uint32), np.array([1, 2], np.uint32))
    assert e.value.status == 1


def test_library_exports_every_declared_symbol():
    """librg.so loads and exports every function include/*.h declares."""
    decl = set()
    inc = os.path.join(ROOT, "include")
    for h in os.listdir(inc):
        if h.endswith(".h"):
            txt = open(os.path.join(inc, h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            decl |= set(re.findall(r"\b(rg_[a-z0-9_]+)\s*\(", txt))
    assert decl, "no declarations found"
    L = rg.lib()
    missing = [s for s in decl if not hasattr(L, s)]
    assert not missing, missing
    assert set(rg.exported_symbols()) <= decl
    assert rg.version().startswith("radar-graph-gb300")


def test_engine_options_round_trip_and_validate():
    """Scheduling options are host state of the calling thread: each reads
    back what was set, out-of-range values are RG_EINVAL and leave the old
    value, and another thread starts from the defaults."""
    import threading
    valid = {"direction": [0, 1], "hub_slots": [0, 512], "hub_smem_kb": [0, 4, 227],
             "dense_div": [1, 1000, 20], "sweep_shape": [40, 42, 80, 82, 160, 162], "bc_fwd_hubs": [0, 1],
             "async_results": [1, 0]}
    bad = {"direction": [2, -1], "hub_slots": [-1], "hub_smem_kb": [-1, 228], "dense_div": [0],
           "sweep_shape": [43, 50, 91, 163, 120], "bc_fwd_hubs": [2, -1],
           "async_results": [2, -1]}
    assert set(valid) == set(rg.OPTIONS)
    for name in valid:
        old = rg.get_option(name)
        try:
            for v in valid[name]:
                rg.set_option(name, v)
                assert rg.get_option(name) == v, name
            for v in bad[name]:
                with pytest.raises(rg.RgError) as e:
                    rg.set_option(name, v)
                assert e.value.status == 1, (name, v)
                assert rg.get_option(name) == valid[name][-1], name
        finally:
            rg.set_option(name, old)
    rg.set_option("dense_div", 7)
    try:
        seen = []
        t = threading.Thread(target=lambda: seen.append(rg.get_option("dense_div")))
        t.start()
        t.join()
        assert seen == [20] and rg.get_option("dense_div") == 7
    finally:
        rg.set_option("dense_div", 20)


def test_no_cuda_device_is_a_clean_error():
    """Without a GPU the device entry points fail with a status, not a crash."""
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    off, adj = rg.rmat_csr(6, 4)
    with pytest.raises(rg.RgError) as e:
        rg.Graph.from_csr(off, adj)
    assert e.value.status in (3, 8)


# ---- GAP text edge lists (rg_read_edges) -----------------------------------

def _gap_golden():
    import os
    from conftest import GOLDEN
    return np.load(os.path.join(GOLDEN, "gap_formats.npz"))


def test_gap_formats_match_the_reference_triangle_totals(tmp_path):
    """The same edges in every GAP format: read, symmetric clean-up, and the
    triangle total equals GAP tc_local's on that file (golden)."""
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_gap_formats as mg
    import oracle as orc
    gold = _gap_golden()
    paths = mg.write_formats(gold["src"], gold["dst"], str(tmp_path / "g"))
    want = dict(zip(gold["formats"].tolist(), gold["totals"].tolist()))
    assert set(want) == set(mg.FORMATS)
    ref_off, ref_adj = rg.csr_from_edges(int(max(gold["src"].max(), gold["dst"].max())) + 1, gold["src"], gold["dst"])
    for fmt, path in paths.items():
        n, s, d = rg.read_edges(path)
        off, adj = rg.csr_from_edges(n, s, d)
        assert np.array_equal(off, ref_off) and np.array_equal(adj, ref_adj), fmt
        _, total = orc.triangles(off, adj, 0)
        assert total == want[fmt], fmt


def test_gap_formats_parse_details(tmp_path):
    p = tmp_path / "a.el"
    p.write_text("0 1\n1 2\n\n2 2\n5 3\n")
    n, s, d = rg.read_edges(p)
    assert n == 6 and s.tolist() == [0, 1, 2, 5] and d.tolist() == [1, 2, 2, 3]
    p = tmp_path / "a.gr"  # only 'a' lines; ids as written
    p.write_text("c comment\np sp 4 2\na 1 2 7\na 3 1 2.5\n")
    n, s, d = rg.read_edges(p)
    assert n == 4 and s.tolist() == [1, 3] and d.tolist() == [2, 1]
    p = tmp_path / "a.graph"  # weighted METIS (fmt 1), an empty list, comments
    p.write_text("% c\n3 2 1\n2 5 3 1\n% between lists\n\n1 9\n")
    n, s, d = rg.read_edges(p)
    assert n == 3 and s.tolist() == [0, 0, 2] and d.tolist() == [1, 2, 0]
    p = tmp_path / "a.mtx"
    p.write_text("%%MatrixMarket matrix coordinate integer symmetric\n%x\n3 3 2\n2 1 4\n3 3 1\n")
    n, s, d = rg.read_edges(p)
    assert n == 3 and s.tolist() == [1, 0, 2, 2] and d.tolist() == [0, 1, 2, 2]


@pytest.mark.parametrize("name,text,match", [
    ("a.txt", "0 1\n", "suffix"),
    ("b.el", "0 x\n", "malformed"),
    ("c.el", "0 -1\n", "range"),
    ("d.mtx", "%%MatrixMarket matrix array real general\n2 2\n1\n", "coordinate"),
    ("e.mtx", "%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1 1\n", "field"),
    ("f.mtx", "%%MatrixMarket matrix coordinate pattern general\n2 3 1\n1 1\n", "square"),
    ("g.graph", "3 2 11\n2\n", "fmt"),
    ("h.mtx", "hello\n", "MatrixMarket"),
])
def test_gap_format_errors(tmp_path, name, text, match):
    p = tmp_path / name
    p.write_text(text)
    with pytest.raises(rg.RgError, match=match):
        rg.read_edges(p)
    with pytest.raises(rg.RgError):
        rg.read_edges(tmp_path / "missing.el")
