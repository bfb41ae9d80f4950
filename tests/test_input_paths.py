"""Fast input paths: GAP serialized graphs (.sg) on the host, and the CSR
built on the device from an edge list, which must equal the host clean-up
(rg_csr_from_edges, the symmetric loader's IO.h:429-474) bit for bit."""

import struct

import numpy as np
import pytest

import radar_graph as rg
from conftest import assert_close


def _write_sg(path, off, adj, directed=False, bad_size=False, inverse=None):
    """GAP's layout (writer.h): bool directed, int64 edges, int64 nodes,
    int64 offsets[n+1], int32 neighbours[m]; a directed graph may follow
    with its in-lists (inverse = (in_off, in_adj))."""
    n, m = len(off) - 1, len(adj)
    with open(path, "wb") as f:
        f.write(struct.pack("<?qq", directed, m, n))
        f.write(np.asarray(off, np.int64).tobytes())
        f.write(np.asarray(adj, np.int32).tobytes()[: (4 * m - 4) if bad_size else None])
        if inverse is not None:
            f.write(np.asarray(inverse[0], np.int64).tobytes())
            f.write(np.asarray(inverse[1], np.int32).tobytes())


@pytest.mark.parametrize("with_inverse", [False, True])
def test_sg_directed(tmp_path, with_inverse):
    import oracle as orc
    off = np.array([0, 2, 3, 3, 4], np.uint32)
    adj = np.array([1, 3, 2, 0], np.uint32)
    inv = orc.transpose(off, adj) if with_inverse else None
    p = tmp_path / "d.sg"
    _write_sg(p, off, adj, directed=True, inverse=inv)
    o2, a2, directed = rg.read_sg(p, allow_directed=True)
    assert directed and np.array_equal(o2, off) and np.array_equal(a2, adj)
    with pytest.raises(rg.RgError, match="directed"):
        rg.read_sg(p)
    _write_sg(p, off, adj)
    assert rg.read_sg(p, allow_directed=True)[2] is False


def test_sg_round_trip(tmp_path):
    off, adj = rg.rmat_csr(10, 8, seed=4)
    p = tmp_path / "g.sg"
    _write_sg(p, off, adj)
    o2, a2 = rg.read_sg(p)
    assert np.array_equal(o2, off) and np.array_equal(a2, adj)


def test_sg_errors(tmp_path):
    off, adj = rg.rmat_csr(8, 4, seed=1)
    p = tmp_path / "d.sg"
    _write_sg(p, off, adj, directed=True)
    with pytest.raises(rg.RgError, match="directed"):
        rg.read_sg(p)
    _write_sg(p, off, adj, bad_size=True)
    with pytest.raises(rg.RgError, match="size"):
        rg.read_sg(p)
    bad = np.array(adj, copy=True)
    bad[3] = len(off) + 5  # neighbour id >= n
    _write_sg(p, off, bad)
    with pytest.raises(rg.RgError, match="range"):
        rg.read_sg(p)
    with pytest.raises(rg.RgError):
        rg.read_sg(tmp_path / "missing.sg")


def test_device_build_rejects_bad_arguments():
    with pytest.raises(rg.RgError):
        rg.Graph.from_edges(0, np.zeros(1, np.uint32), np.zeros(1, np.uint32))
    with pytest.raises(ValueError):
        rg.Graph.from_edges(4, np.zeros(2, np.uint32), np.zeros(1, np.uint32))


def _cases():
    yield "tiny", 12, np.array([0, 0, 1, 2, 2, 3, 4, 5, 5, 6, 7, 8, 1, 0, 4], np.uint32), \
        np.array([1, 1, 2, 0, 2, 4, 5, 3, 6, 7, 8, 6, 3, 0, 4], np.uint32)
    yield "loops_only", 5, np.array([0, 1, 1, 4], np.uint32), np.array([0, 1, 1, 4], np.uint32)
    yield "no_edges", 7, np.zeros(0, np.uint32), np.zeros(0, np.uint32)
    yield "one_vertex", 1, np.zeros(3, np.uint32), np.zeros(3, np.uint32)
    yield "isolated_tail", 100, np.array([0, 1, 2], np.uint32), np.array([1, 2, 0], np.uint32)
    for sc, ef, seed, uni in ((10, 16, 1, False), (12, 8, 2, True), (14, 16, 3, False), (16, 16, 1, False)):
        s, d = rg.generate_edges(sc, ef, seed, uni)
        yield f"{'er' if uni else 'rmat'}{sc}", 1 << sc, s, d


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(_cases()), ids=lambda c: c[0])
def test_device_build_equals_host_cleanup(case):
    _, n, s, d = case
    off, adj = rg.csr_from_edges(n, s, d)
    with rg.Graph.from_edges(n, s, d) as g:
        assert (g.n, g.m) == (n, len(adj))
        o2, a2, _ = g.download()
        assert np.array_equal(o2, off)
        assert np.array_equal(a2, adj)
        if len(adj):  # and the apps run on it like on an uploaded graph
            with rg.Graph.from_csr(off, adj) as g2:
                # pulls sum exactly: identical; pushes add with FP64 atomics in
                # any order, as the reference does: within rounding
                r, it, _ = g.pagerank("push-pull", 5)
                r2, it2, _ = g2.pagerank("push-pull", 5)
                assert it == it2 and np.array_equal(r, r2)
                r, it, _ = g.pagerank("push", 5)
                r2, it2, _ = g2.pagerank("push", 5)
                assert it == it2
                assert_close(r, r2, what="push PageRank on the device-built graph")


@pytest.mark.gpu
def test_device_build_rejects_ids_out_of_range():
    with pytest.raises(rg.RgError, match="endpoint"):
        rg.Graph.from_edges(4, np.array([0, 1], np.uint32), np.array([2, 9], np.uint32))


def _directed_cleanup(n, s, d):
    """Directed per-list clean-up in numpy: out-lists sorted, repeats and
    self loops dropped."""
    s, d = np.asarray(s, np.uint64), np.asarray(d, np.uint64)
    keys = np.unique(((s << np.uint64(32)) | d)[s != d])
    src = (keys >> np.uint64(32)).astype(np.int64)
    off = np.searchsorted(src, np.arange(n + 1), side="left").astype(np.uint32)
    return off, (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(_cases()), ids=lambda c: c[0])
def test_directed_device_build_equals_cleanup(case):
    _, n, s, d = case
    off, adj = _directed_cleanup(n, s, d)
    with rg.Graph.from_edges(n, s, d, directed=True) as g:
        assert g.directed and (g.n, g.m) == (n, len(adj))
        o2, a2, _ = g.download()
        assert np.array_equal(o2, off)
        assert np.array_equal(a2, adj)
        if len(adj):  # in-lists: pulls over them equal the uploaded graph's
            with rg.Graph.from_csr_directed(off, adj) as g2:
                for v in ("push", "push-pull"):
                    r, it, _ = g.pagerank(v, 5)
                    r2, it2, _ = g2.pagerank(v, 5)
                    assert it == it2
                    if v == "push-pull":  # exact sums
                        assert np.array_equal(r, r2)
                    else:  # FP64 atomics in any order
                        assert_close(r, r2, what="directed push PageRank")


@pytest.mark.gpu
@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
@pytest.mark.parametrize("case", [(10, 8, 1), (14, 16, 2), (16, 16, 3)], ids=["s10", "s14", "s16"])
def test_create_sorted_equals_upload_then_sort(case, pinned):
    scale, ef, seed = case
    off, adj = rg.rmat_csr(scale, ef, seed=seed)
    if len(adj) % 4 == 0:  # exercise the relabel's exact tail: drop the last vertex's last edge
        last = int(np.nonzero(np.diff(off.astype(np.int64)))[0][-1])
        keep = np.ones(len(adj), bool)
        keep[int(off[last + 1]) - 1] = False
        adj = adj[keep]
        off = off.copy()
        off[last + 1:] -= 1
    a = rg.pinned_empty(len(adj), np.uint32) if pinned else np.array(adj, copy=True)
    a[:] = adj
    with rg.Graph.from_csr(off, adj) as g0, g0.degree_sort() as want, rg.Graph.from_csr_sorted(off, a) as got:
        wo, wa, wi = want.download()
        go, ga, gi = got.download()
        assert np.array_equal(wo, go) and np.array_equal(wa, ga) and np.array_equal(wi, gi)
        r1, _, _ = want.pagerank("push-pull", 10)
        r2, _, _ = got.pagerank("push-pull", 10)
        assert np.array_equal(r1, r2)  # exact sums: identical
        r1, _, _ = want.pagerank("radar", 10)
        r2, _, _ = got.pagerank("radar", 10)
        assert_close(r1, r2, what="RADAR PageRank on the fused create+sort graph")


@pytest.mark.gpu
@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
def test_create_sorted_rejects_bad_input(pinned):
    off = np.array([0, 2, 3, 4], np.uint32)
    adj = np.array([1, 2, 0, 0], np.uint32)
    a = rg.pinned_empty(4, np.uint32) if pinned else np.array(adj, copy=True)
    a[:] = adj
    a[3] = 7  # neighbour id >= n
    with pytest.raises(rg.RgError):
        rg.Graph.from_csr_sorted(off, a)
    a[3] = 0
    bad_off = np.array([0, 3, 2, 4], np.uint32)  # not monotone
    with pytest.raises(rg.RgError):
        rg.Graph.from_csr_sorted(bad_off, a)
