"""Serving: queries submitted concurrently to the request loop must return
exactly what the same query returns alone through the single-query entry
points -- BFS depths and Radii bit-exact, BC within 1e-9 relative -- whether
they were coalesced into a multi-source batch or not."""

import threading
import time

import numpy as np
import pytest

import radar_graph as rg
from conftest import assert_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import build as b
    b.build()


@pytest.fixture(scope="module")
def graphs():
    a = rg.Graph.from_csr(*rg.rmat_csr(12, 16, seed=1))
    b0 = rg.Graph.from_csr(*rg.rmat_csr(13, 8, seed=2))
    b = b0.degree_sort()
    b0.free()
    yield [a, b]
    a.free()
    b.free()


def _alone(G, kind, src):
    if kind == "bfs":
        return G.bfs("push", int(src))[1]
    if kind == "bc":
        return G.bc_sources(np.array([src], np.uint32), "push")[0]
    return G.radii_seeds(rg.radii_query_seeds(int(src), G.n), "push")[0]


def test_mixed_queries_alone_equal_in_the_mix(graphs):
    rng = np.random.default_rng(5)
    queries = []
    for _ in range(90):
        gi = int(rng.integers(0, 2))
        kind = rng.choice(["bfs", "bfs", "bfs", "bc", "radii"])
        n = graphs[gi].n
        queries.append((gi, str(kind), int(rng.integers(0, n)) if kind != "radii" else int(rng.integers(0, 1000))))
    results = [None] * len(queries)
    with rg.Server(graphs, workers=3, max_batch=64) as S:
        def client(idx):
            for i in idx:
                gi, kind, src = queries[i]
                t = S.submit(gi, kind, src)
                results[i] = S.wait(t, gi, kind)[0]
        # submit from several threads at once so queries arrive while others run
        th = [threading.Thread(target=client, args=(list(range(j, len(queries), 4)),)) for j in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        st = S.stats()
    assert st["completed"] == len(queries)
    assert st["launches"] <= len(queries)
    for (gi, kind, src), got in zip(queries, results):
        want = _alone(graphs[gi], kind, src)
        if kind == "bc":
            assert_close(got, want, what=f"bc g{gi} s{src}")
        else:
            assert np.array_equal(got, want), (gi, kind, src)


def test_bfs_queries_are_coalesced(graphs):
    with rg.Server(graphs[:1], workers=1, max_batch=64) as S:
        # a burst: one worker, so later arrivals wait and are coalesced
        tickets = [S.submit(0, "bfs", s) for s in range(0, 4000, 40)]
        outs = [S.wait(t, 0, "bfs")[0] for t in tickets]
        st = S.stats()
    assert st["launches"] < len(tickets)
    assert st["batched"] > 0
    for s, got in zip(range(0, 4000, 40), outs):
        assert np.array_equal(got, graphs[0].bfs("push", s)[1])


def test_bad_queries_are_errors(graphs):
    with rg.Server(graphs, workers=1) as S:
        with pytest.raises(rg.RgError):
            S.submit(5, "bfs", 0)
        with pytest.raises(rg.RgError):
            S.submit(0, "bfs", 10**9)


def test_bc_queries_are_coalesced(graphs):
    G = graphs[1]
    srcs = list(range(3, 3 + 40 * 97, 97))
    with rg.Server([G], workers=1, max_batch=64) as S:
        tickets = [S.submit(0, "bc", s) for s in srcs]
        outs = [S.wait(t, 0, "bc")[0] for t in tickets]
        st = S.stats()
    assert st["launches"] < len(tickets) and st["batched"] > 0
    for s, got in zip(srcs, outs):
        assert_close(got, _alone(G, "bc", s), what=f"bc s{s}")


def test_radii_queries_are_coalesced(graphs):
    G = graphs[0]
    seeds = list(range(40))
    with rg.Server([G], workers=1, max_batch=64) as S:
        tickets = [S.submit(0, "radii", s) for s in seeds]
        outs = [S.wait(t, 0, "radii")[0] for t in tickets]
        st = S.stats()
    assert st["launches"] < len(tickets) and st["batched"] > 0
    for s, got in zip(seeds, outs):
        assert np.array_equal(got, _alone(G, "radii", s)), s


def test_tiny_hbm_budget_admits_one_batch_at_a_time(graphs):
    """Admission by free HBM: with a budget far below any batch's working set,
    every batch waits until nothing else holds device memory and then runs
    alone (never two on the device at once), and every result is still the
    query's result alone."""
    rng = np.random.default_rng(9)
    queries = [(int(rng.integers(0, 2)), str(rng.choice(["bfs", "bc", "radii"])), int(rng.integers(0, 4096)))
               for _ in range(24)]
    with rg.Server(graphs, workers=4, max_batch=8, hbm_fraction=1e-9) as S:
        tickets = [S.submit(gi, kind, src) for gi, kind, src in queries]
        # fetched in submission order, not batch order: unfetched results of
        # one batch must not hold back another forever
        outs = [S.wait(t, gi, kind, timeout_ms=120000)[0] for t, (gi, kind, _) in zip(tickets, queries)]
        st = S.stats()
    assert st["completed"] == len(queries)
    assert st["admission_waits"] > 0
    assert st["peak_running"] == 1
    for (gi, kind, src), got in zip(queries, outs):
        want = _alone(graphs[gi], kind, src)
        if kind == "bc":
            assert_close(got, want, what=f"bc g{gi} s{src}")
        else:
            assert np.array_equal(got, want), (gi, kind, src)


def test_wait_times_out_and_cancel_drops_the_query(graphs):
    """A query the paused workers never take: the bounded wait returns
    RG_ETIMEOUT (the ticket stays valid), a cancelled query never runs and its
    wait returns RG_ECANCELED, and the server serves normally once resumed."""
    G = graphs[0]
    with rg.Server([G], workers=2) as S:
        S.pause(True)
        t1 = S.submit(0, "bfs", 7)
        t2 = S.submit(0, "bc", 9)
        with pytest.raises(rg.RgError) as e:
            S.wait(t1, 0, "bfs", timeout_ms=50)
        assert e.value.status == 7  # RG_ETIMEOUT
        S.cancel(t2)
        with pytest.raises(rg.RgError) as e:
            S.wait(t2, 0, "bc", timeout_ms=50)
        assert e.value.status == 9  # RG_ECANCELED
        S.pause(False)
        got = S.wait(t1, 0, "bfs", timeout_ms=60000)[0]  # the same ticket, served after the resume
        assert np.array_equal(got, _alone(G, "bfs", 7))
        st = S.stats()
        assert st["completed"] == 1 and st["cancelled"] == 1
        # a finished, unfetched result can be cancelled too; its memory is released
        t3 = S.submit(0, "radii", 3)
        deadline = time.time() + 60
        while S.stats()["completed"] < 2 and time.time() < deadline:
            time.sleep(0.01)
        S.cancel(t3)
        with pytest.raises(rg.RgError) as e:
            S.wait(t3, 0, "radii", timeout_ms=1000)
        assert e.value.status == 9
        with pytest.raises(rg.RgError):
            S.cancel(12345)  # unknown ticket
