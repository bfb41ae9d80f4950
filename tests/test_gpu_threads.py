"""Several host threads querying one resident graph at once.

Each calling thread has its own stream and scratch (the library's
per-thread context), so PageRank, PageRankDelta, BFS, BC and Radii calls --
single-query and batched -- made from four threads at the same time on one
graph handle return what the same calls return one at a time: BFS depths,
Radii and pulled PageRank ranks (exact sums) bit-exact; pushed PageRank, BC
and PageRankDelta within 1e-9 relative (their FP64 atomics add in a
different order).
"""

import threading

import numpy as np
import pytest

import radar_graph as rg
from conftest import assert_close

pytestmark = pytest.mark.gpu


def _jobs(g, off):
    n = len(off) - 1
    deg_nz = np.nonzero(np.diff(off.astype(np.int64)))[0]  # roots in original ids
    rng = np.random.default_rng(7)
    roots = rng.choice(deg_nz, 6, replace=False)
    src = g.bc_pick_sources(6)
    seeds = np.stack([rg.radii_query_seeds(q, n) for q in range(3)])
    jobs = []
    for v in ("radar", "push"):
        jobs.append(("pagerank", v, lambda v=v: g.pagerank(v, 20)[0]))
    jobs.append(("pagerank_pull", "push-pull", lambda: g.pagerank("push-pull", 20)[0]))
    jobs.append(("pagerank_delta", "radar", lambda: g.pagerank_delta("radar", 30)[0]))
    for r in roots:
        jobs.append(("bfs", int(r), lambda r=r: g.bfs("radar", int(r), parents=False)[1]))
    for s in src:
        jobs.append(("bc", int(s), lambda s=s: g.bc_sources(np.array([s], np.uint32), "radar")[0]))
    jobs.append(("bc_multi", 6, lambda: g.bc_multi(src)[0]))
    for q in range(3):
        jobs.append(("radii", q, lambda q=q: g.radii_seeds(seeds[q], "radar")[0]))
    jobs.append(("radii_multi", 3, lambda: g.radii_multi(seeds)[0]))
    return jobs


def _same(kind, got, want, what):
    if kind in ("bc", "bc_multi", "pagerank_delta", "pagerank"):
        assert_close(got, want, what=what)
    else:
        assert np.array_equal(got, want), what


def test_four_threads_one_graph():
    off, adj = rg.rmat_csr(14, 16, seed=5)
    with rg.Graph.from_csr(off, adj) as g0, g0.degree_sort() as g:
        jobs = _jobs(g, off)
        want = [fn() for _, _, fn in jobs]
        got = [[None] * len(jobs) for _ in range(2)]
        errors = []

        def worker(rep, idx):
            try:
                for i in idx:
                    got[rep][i] = jobs[i][2]()
            except Exception as e:  # surfaced after join
                errors.append(e)

        # two passes, each job list dealt round-robin to four threads (the
        # second pass in the reverse order, so different calls overlap)
        for rep in range(2):
            order = list(range(len(jobs)))[:: 1 if rep == 0 else -1]
            th = [threading.Thread(target=worker, args=(rep, order[t::4])) for t in range(4)]
            for t in th:
                t.start()
            for t in th:
                t.join()
        assert not errors, errors
        for rep in range(2):
            for i, (kind, arg, _) in enumerate(jobs):
                _same(kind, got[rep][i], want[i], f"pass {rep} {kind} {arg}")
