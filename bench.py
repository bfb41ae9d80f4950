"""Benchmark of the GB300 frontier engine against the reference's CPU path.

Headline workload: RADAR (degree-sorted graph, hub duplication where the
autotuner finds it pays) PageRank / BFS / BC / Radii on a symmetric R-MAT
scale-24 graph (edge factor 16, a=0.57 b=0.19 c=0.19, seed 1) on one GB300.
A step is one pass of the four apps over the resident graph: PageRank 20
iterations, BFS from one root, BC from one source, Radii with 64 samples.
`value` = edges traversed / device time (GTEPS) with the graph resident in HBM;
the graph (about 2 GB of edges) is far larger than L2, so no flush is needed
between steps.  `e2e` = the same through the public C ABI from host buffers:
each step uploads the CSR, degree-sorts it on the device and copies every
app's result back.

The same JSON line also carries the batched launch (512 uneven R-MAT graphs,
64-source BFS + 10-iteration PageRank each, one persistent launch) and the
served stream (3 resident graphs, Poisson arrivals of a BFS/BC/Radii mix),
each against the plain one-query-per-launch GPU path, and the next rows:
PageRankDelta, the device CSR build, triangle counting and the directed path
(the same four apps on a directed R-MAT graph, in-degree sorted).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--scale S] [--impl reference]

Under torchrun each rank runs an independent replica on its own GPU (replicas
only: the engine has no cross-GPU exchange); rank 0 prints the whole-job line.
"""

import argparse
import concurrent.futures as cf
import ctypes
import json
import os
import queue
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "radar-graph_gb300"))

METRIC = "GTEPS + % HBM roofline per app (RMAT s24); batched queries/s, p50/p99 vs plain"
APPS = ("pagerank", "bfs", "bc", "radii")
EXTRA_LEGS = ("er_contrast", "config2", "graph_build", "triangles", "directed", "batched", "batched_sources",
              "serving")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for i, nm in enumerate(names):
                    if r[5 + i].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cuda_profiler(on):
    """Marks the profiled ranges -- the timed step, the gather probe and the
    extra legs -- for
    a profiler started with --profile-from-start off (cudaProfilerStart/Stop
    of the CUDA runtime the library loaded); a profiler started from the
    start stops at the end of the timed step unless the extra legs reopen
    it.  A no-op when no profiler is attached."""
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        (rt.cudaProfilerStart if on else rt.cudaProfilerStop)()
        return


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def replica_rate(pg, ms_per_step, edges_per_step):
    """Whole-job GTEPS over replicas: every rank's edges / the slowest rank's
    step time (max over ranks), and that step time."""
    ms = allreduce(pg, ms_per_step, "MAX")
    edges = allreduce(pg, edges_per_step, "SUM")
    return edges / (ms / 1e3) / 1e9, ms


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allreduce(pg, x, op):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=getattr(pg.ReduceOp, op))
    return float(t.item())


def gather_ceiling_ms(gs, reps=5):
    """Best time (ms) to stream gs's edge array and gather 8 bytes per edge,
    the ceiling of any pull over that graph, from the benchmark's measurement
    library (librg_probe.so, built beside librg.so; not in the product ABI)."""
    L = ctypes.CDLL(os.path.join(ROOT, "radar-graph_gb300", "librg_probe.so"))
    L.rg_probe_gather_ceiling.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    L.rg_probe_gather_ceiling.restype = ctypes.c_int
    ms = ctypes.c_double()
    st = L.rg_probe_gather_ceiling(gs.handle, reps, ctypes.byref(ms))
    if st != 0:
        raise RuntimeError(f"gather probe failed: status {st}")
    return ms.value


def measured_traffic(kernel, scale):
    """DRAM bytes (read + write) of one launch of `kernel` (its template
    instance) on the RMAT graph of this scale, from the ncu capture recorded in
    profiles/traffic.json (None when no capture of that kernel and workload is
    recorded)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    rec = json.load(open(p)).get(kernel, {})
    return rec.get("dram_bytes_per_launch") if rec.get("scale") == scale else None


def bench_input(rg, scale, ef=16, seed=1, reps=3):
    """The symmetric loader's clean-up (both directions, sort, drop repeats
    and self loops) on the host (the oracle-equivalent rg_csr_from_edges,
    OpenMP) against the device build (rg_graph_create_from_edges), on the
    same edge list, with the results compared."""
    src, dst = rg.generate_edges(scale, ef, seed, False)
    n = 1 << scale
    t0 = time.perf_counter()
    off, adj = rg.csr_from_edges(n, src, dst)
    host_s = time.perf_counter() - t0
    src_p, dst_p = rg.pinned_empty(len(src), np.uint32), rg.pinned_empty(len(dst), np.uint32)
    src_p[:], dst_p[:] = src, dst
    dev_ms = []
    for i in range(reps + 1):
        rg.lib().rg_synchronize()
        t0 = time.perf_counter()
        g = rg.Graph.from_edges(n, src_p, dst_p)
        rg.lib().rg_synchronize()
        if i:
            dev_ms.append((time.perf_counter() - t0) * 1e3)
        if i == reps:
            o2, a2, _ = g.download()
            identical = bool(np.array_equal(o2, off) and np.array_equal(a2, adj))
        g.free()
    return {"edges_in": int(len(src)), "n": n, "m": int(len(adj)), "host_cleanup_s": round(host_s, 3),
            "host_threads": os.cpu_count(), "device_build_ms": round(min(dev_ms), 2),
            "speedup": round(host_s * 1e3 / min(dev_ms), 1), "identical": identical,
            "input": "edge list in pinned host memory (upload included)"}


def bench_triangles(rg, gs, with_cpu, small_scale=20):
    """Triangle counting (GAP tc_local): the GPU on the bench graph, and GPU
    against the oracle port (all host cores) on a smaller RMAT graph."""
    out = {}
    ms = []
    for i in range(3):
        _, total = gs.triangles()
        if i:
            ms.append(rg.last_timing()["total_ms"])
    out["s_bench"] = {"triangles": int(total), "ms": round(min(ms), 2)}
    off, adj = make_graph(rg, small_scale, 16, 1)
    with rg.Graph.from_csr(off, adj) as g:
        g.triangles()
        t0 = time.perf_counter()
        _, tg = g.triangles()
        gpu_s = time.perf_counter() - t0
    small = {"scale": small_scale, "triangles": int(tg), "gpu_ms": round(gpu_s * 1e3, 2)}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        t0 = time.perf_counter()
        _, tc = orc.triangles(off, adj, os.cpu_count() or 1)
        small["cpu_port_s"] = round(time.perf_counter() - t0, 3)
        small["cpu_threads"] = os.cpu_count()
        small["identical"] = int(tc) == int(tg)
    out["s_small"] = small
    return out


def bench_directed(rg, scale, with_cpu, ef=16, seed=1, reps=3):
    """The directed path: RMAT edges kept one way (src -> dst), built on the
    device (out-lists cleaned, in-lists), in-degree sorted, then the four
    RADAR apps (PageRank pulls over in-edges, BC transposes per source), with
    the oracle port on the same sorted graph (PageRank 2 iterations, BFS, BC,
    Radii) and the BFS depths and radii compared."""
    src, dst = rg.generate_edges(scale, ef, seed, False)
    n = 1 << scale
    src_p, dst_p = rg.pinned_empty(len(src), np.uint32), rg.pinned_empty(len(dst), np.uint32)
    src_p[:], dst_p[:] = src, dst
    build_ms = []
    for i in range(reps + 1):
        rg.lib().rg_synchronize()
        t0 = time.perf_counter()
        g = rg.Graph.from_edges(n, src_p, dst_p, directed=True)
        rg.lib().rg_synchronize()
        if i:
            build_ms.append((time.perf_counter() - t0) * 1e3)
        if i < reps:
            g.free()
    root = int(g.pick_roots(1)[0])
    gs = g.degree_sort()  # in-degree order (-preprocess 1)
    g.free()
    bc_src = gs.bc_pick_sources(1)
    gs.autotune("radar")
    stats = {}
    for i in range(reps + 1):
        run_step(rg, gs, root, bc_src, stats if i else {})
    apps = {k: {"gteps": round(s["edges"] / (s["ms"] / 1e3) / 1e9, 3), "ms": round(s["ms"] / reps, 3)}
            for k, s in stats.items()}
    tot_e = sum(s["edges"] for s in stats.values())
    tot_ms = sum(s["ms"] for s in stats.values())
    out = {"n": n, "m": int(gs.m), "edges_in": int(len(src)), "device_build_ms": round(min(build_ms), 2),
           "gteps": round(tot_e / (tot_ms / 1e3) / 1e9, 3), "ms_per_step": round(tot_ms / reps, 3), "apps": apps,
           "workload": f"RADAR PageRank(20 it)+BFS+BC(1 src)+Radii(64) on directed RMAT s{scale} ef{ef} seed {seed}, "
                       "in-degree sorted, autotuned schedule"}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        cores = os.cpu_count() or 1
        so, sa, ids = gs.download()
        io, ia = orc.transpose(so, sa)
        kw = {"in_off": io, "in_adj": ia}
        _, depth, _, _ = gs.bfs("radar", root)
        r_gpu, _ = gs.radii("radar")
        seeds = orc.radii_seeds(n)
        t, e, res = {}, {}, {}
        runs = {
            "pagerank": lambda: orc.pagerank(so, sa, "radar", 2, cores, **kw),
            "bfs": lambda: orc.bfs(so, sa, int(ids[root]), "radar", cores, **kw),
            "bc": lambda: orc.bc(so, sa, ids[bc_src], "radar", cores, **kw),
            "radii": lambda: orc.radii(so, sa, ids[seeds], "radar", cores, **kw),
        }
        for k, fn in runs.items():
            orc.take_edges()
            t0 = time.time()
            res[k] = fn()
            t[k] = time.time() - t0
            e[k] = orc.take_edges()
        par = res["bfs"][0]
        d_cpu = orc.depths_from_parents(par)[ids]
        out["cpu_port"] = {"gteps": round(sum(e.values()) / sum(t.values()) / 1e9, 4), "cores": cores,
                           "sample": "PageRank 2 iterations + BFS + BC 1 source + Radii 64 on the same sorted graph",
                           "seconds": {k: round(v, 3) for k, v in t.items()},
                           "identical_bfs_depths_and_radii": bool(np.array_equal(depth, d_cpu) and
                                                                  np.array_equal(r_gpu, res["radii"][0][ids]))}
    gs.free()
    return out


def bench_batched_sources(rg, gs, reps=2, plain_sample=8):
    """Many sources on one resident graph per traversal (rg_bfs_multi,
    rg_bc_multi, rg_radii_multi) against one query per launch: queries/s of
    each, the plain side timed on `plain_sample` queries, results compared."""
    n = gs.n
    out = {}
    cases = {
        "bfs": (64, lambda s: gs.bfs_multi(s), lambda s: gs.bfs("radar", int(s))[1]),
        "bc": (64, lambda s: gs.bc_multi(s), lambda s: gs.bc_sources(np.array([s], np.uint32), "radar")[0]),
        "radii": (16, lambda s: gs.radii_multi(s), lambda s: gs.radii_seeds(s, "radar")[0]),
    }
    for kind, (k, multi, single) in cases.items():
        if kind == "radii":
            src = np.stack([rg.radii_query_seeds(q, n) for q in range(k)])
        else:
            src = gs.bc_pick_sources(k)
        multi(src)
        ms = []
        for _ in range(reps):
            rows = multi(src)[0]
            ms.append(rg.last_timing()["total_ms"])
        single(src[0])
        t_plain, ok = 0.0, True
        for q in range(plain_sample):
            want = single(src[q])
            t_plain += rg.last_timing()["total_ms"]
            if kind == "bc":
                ok &= bool(np.array_equal(np.isnan(rows[q]), np.isnan(want)) and np.allclose(
                    rows[q][~np.isnan(want)], want[~np.isnan(want)], rtol=1e-9, atol=0))
            else:
                ok &= bool(np.array_equal(rows[q], want))
        qps, plain_qps = k / (min(ms) / 1e3), plain_sample / (t_plain / 1e3)
        out[kind] = {"per_traversal": k, "ms": round(min(ms), 2), "queries_per_s": round(qps, 1),
                     "plain_queries_per_s": round(plain_qps, 1), "speedup_vs_plain": round(qps / plain_qps, 2),
                     "identical_results": ok}
    return out


def make_graph(rg, scale, ef, seed, uniform=False):
    src, dst = rg.generate_edges(scale, ef, seed, uniform)
    return rg.csr_from_edges(1 << scale, src, dst)


def run_step(rg, gs, root, bc_src, stats):
    """One pass of the four RADAR apps over the resident graph."""
    ms, edges, launches = 0.0, 0, 0
    per = {}
    gs.pagerank("radar", 20)
    per["pagerank"] = rg.last_timing()
    gs.bfs("radar", root)
    per["bfs"] = rg.last_timing()
    gs.bc_sources(bc_src, "radar")
    per["bc"] = rg.last_timing()
    gs.radii("radar")
    per["radii"] = rg.last_timing()
    for k, t in per.items():
        ms += t["total_ms"]
        edges += t["edges_traversed"]
        launches += t["kernel_launches"]
        s = stats.setdefault(k, {"ms": 0.0, "edges": 0, "bytes": 0, "edge_ms": 0.0, "edge_launches": 0})
        s["ms"] += t["total_ms"]
        s["edges"] += t["edges_traversed"]
        s["bytes"] += t["algorithmic_bytes"]
        s["edge_ms"] += t["edge_ms"]
        s["edge_launches"] += t["edge_launches"]
    return ms, edges, launches


def app_rates(stats, reps, hbm):
    return {k: {"gteps": round(s["edges"] / (s["ms"] / 1e3) / 1e9, 3), "ms": round(s["ms"] / reps, 3),
                "hbm_frac_of_measured": round(s["bytes"] / (s["ms"] / 1e3) / 1e9 / hbm, 4)}
            for k, s in stats.items()}


def bench_er_contrast(rg, scale, with_cpu, hbm, reps=3, pr_iters_cpu=5):
    """The low-skew contrast: an Erdos-Renyi graph with the bench graph's
    vertex count and generated edge count (GAP MakeUniformEL,
    generator.h:64-79), degree-sorted, the same four RADAR apps (autotuned),
    and the oracle port on it with every result compared."""
    off, adj = make_graph(rg, scale, 16, 1, uniform=True)
    with rg.Graph.from_csr(off, adj) as g:
        gs = g.degree_sort()
    root = int(gs.pick_roots(1)[0])
    bc_src = gs.bc_pick_sources(1)
    gs.autotune("radar")
    stats = {}
    for i in range(reps + 1):
        run_step(rg, gs, root, bc_src, stats if i else {})
    tot_e = sum(s["edges"] for s in stats.values())
    tot_ms = sum(s["ms"] for s in stats.values())
    out = {"n": gs.n, "m": int(gs.m), "gteps": round(tot_e / (tot_ms / 1e3) / 1e9, 3),
           "ms_per_step": round(tot_ms / reps, 3), "apps": app_rates(stats, reps, hbm),
           "workload": f"RADAR PageRank(20 it)+BFS+BC(1 src)+Radii(64) on Erdos-Renyi s{scale}, "
                       f"{16 << scale} generated edges, seed 1, symmetric, degree-sorted"}
    if with_cpu:
        t, e, port = port_run(off, adj, root, bc_src, pr_iters_cpu)
        out["parity"] = parity(gpu_results(gs, root, bc_src, pr_iters_cpu), port)
        out["parity"]["pagerank"]["iterations"] = pr_iters_cpu
        out["cpu_port"] = {"gteps": round(sum(e.values()) / sum(t.values()) / 1e9, 4), "cores": os.cpu_count(),
                           "seconds": {k: round(v, 3) for k, v in t.items()},
                           "sample": f"PageRank {pr_iters_cpu} iterations + BFS + BC 1 source + Radii 64"}
    gs.free()
    return out


def bench_config2(rg, with_cpu, scale=22, nroots=16, reps=3):
    """RADAR PageRank (20 iterations, degree-sorted, autotuned) and push-pull
    BFS from 16 GAP SourcePicker roots (benchmark.h:47-64) on R-MAT s22 ef16
    seed 1.  The push-pull variant does not degree-sort, so its BFS runs on
    the graph as loaded; the 16 roots also run as one 16-source traversal
    (rg_bfs_multi).  The oracle port runs the same apps and every result is
    compared (ranks 1e-9 relative, depths bit-exact)."""
    off, adj = make_graph(rg, scale, 16, 1)
    g = rg.Graph.from_csr(off, adj)
    gs = g.degree_sort()
    roots = g.pick_roots(nroots)
    gs.autotune("radar")
    pr_ms, pr_e, bfs_ms, bfs_e, multi_ms = [], 0, [], 0, []
    for i in range(reps + 1):
        ranks, pr_it, _ = gs.pagerank("radar", 20)
        t = rg.last_timing()
        if i:
            pr_ms.append(t["total_ms"])
            pr_e = t["edges_traversed"]
        ms, e, depths = 0.0, 0, []
        for r in roots:
            depths.append(g.bfs("push-pull", int(r), parents=False)[1].copy())
            t = rg.last_timing()
            ms += t["total_ms"]
            e += t["edges_traversed"]
        if i:
            bfs_ms.append(ms)
            bfs_e = e
        rows, _ = g.bfs_multi(roots)
        if i:
            multi_ms.append(rg.last_timing()["total_ms"])
    out = {"n": g.n, "m": int(g.m), "roots": [int(r) for r in roots],
           "pagerank": {"gteps": round(pr_e / (min(pr_ms) / 1e3) / 1e9, 3), "ms": round(min(pr_ms), 3),
                        "iterations": pr_it},
           "bfs_push_pull_16_roots": {"gteps": round(bfs_e / (min(bfs_ms) / 1e3) / 1e9, 3),
                                      "ms_all_roots": round(min(bfs_ms), 3),
                                      "one_16_source_traversal_ms": round(min(multi_ms), 3),
                                      "multi_equals_single": bool(all(np.array_equal(rows[q], depths[q])
                                                                      for q in range(nroots)))},
           "workload": f"RADAR PageRank 20 it + push-pull BFS from {nroots} SourcePicker roots, RMAT s{scale} ef16"}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        cores = os.cpu_count() or 1
        ids, so, sa = orc.degree_sort(off, adj)
        orc.take_edges()
        t0 = time.time()
        pr_port = orc.pagerank(so, sa, "radar", 20, cores)[0][ids]
        t_pr, e_pr = time.time() - t0, orc.take_edges()
        t0 = time.time()
        d_port = [orc.depths_from_parents(orc.bfs(off, adj, int(r), "push-pull", cores)[0]) for r in roots]
        t_bfs, e_bfs = time.time() - t0, orc.take_edges()
        r, same_nan = max_rel(ranks, pr_port)
        same = [bool(np.array_equal(d, dp)) for d, dp in zip(depths, d_port)]
        out["parity"] = {"pagerank": {"max_rel": float(f"{r:.3e}"), "ok": bool(same_nan and r <= 1e-9)},
                         "bfs_depths_identical_roots": int(sum(same)), "all_ok": bool(same_nan and r <= 1e-9 and all(same))}
        out["cpu_port"] = {"pagerank_gteps": round(e_pr / t_pr / 1e9, 4), "bfs_gteps": round(e_bfs / t_bfs / 1e9, 4),
                           "seconds": {"pagerank": round(t_pr, 3), "bfs_16_roots": round(t_bfs, 3)}, "cores": cores}
    gs.free()
    g.free()
    return out


# ---------------------------------------------------------------------------
# batched launch: 512 uneven graphs, one persistent launch vs one query per launch
# ---------------------------------------------------------------------------

def bench_batched(rg, ngraphs=512, k=64, pr_iters=10, plain_graphs=24, seed=7):
    rng = np.random.default_rng(seed)
    specs = [(int(rng.integers(10, 17)), int(rng.integers(8, 33)), 1000 + i) for i in range(ngraphs)]
    t0 = time.time()
    with cf.ThreadPoolExecutor(max_workers=4) as ex:  # ctypes releases the GIL; each call is OpenMP inside
        csrs = list(ex.map(lambda s: make_graph(rg, *s), specs))
    gen_s = time.time() - t0
    srcs = []
    for i, (off, _) in enumerate(csrs):
        deg = np.diff(off.astype(np.int64))
        nz = np.nonzero(deg)[0]
        srcs.append(np.random.default_rng(i).choice(nz, size=k).astype(np.uint32))
    sources = np.stack(srcs)
    B = rg.Batch(csrs)
    B.run(sources, pr_iters)  # warm
    dev, wall = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        depths, ranks, iters, ms = B.run(sources, pr_iters)
        wall.append((time.perf_counter() - t0) * 1e3)
        dev.append(ms)
    nq = ngraphs * (k + 1)
    # plain: every query alone through the single-query entry points, timed
    # in the same two scopes as the batched launch: device time (CUDA events
    # around the call's kernels, as rg_batch_run's device_ms) and wall-clock
    # (the call through ctypes including its result copy to the host)
    plain_dev, plain_wall, plain_q, identical = 0.0, 0.0, 0, True
    for i in range(plain_graphs):
        off, adj = csrs[i]
        with rg.Graph.from_csr(off, adj) as G:
            G.bfs("push", int(sources[i, 0]))  # warm this graph's buffers
            for q in range(k):
                t0 = time.perf_counter()
                _, d, _, _ = G.bfs("push", int(sources[i, q]))
                plain_wall += (time.perf_counter() - t0) * 1e3
                plain_dev += rg.last_timing()["total_ms"]
                identical &= bool(np.array_equal(d, depths[i][q]))
            t0 = time.perf_counter()
            r, _, _ = G.pagerank("push-pull", pr_iters)
            plain_wall += (time.perf_counter() - t0) * 1e3
            plain_dev += rg.last_timing()["total_ms"]
            identical &= bool(np.array_equal(r, ranks[i]))
            plain_q += k + 1
    B.free()
    total_e = int(sum(len(a) for _, a in csrs))
    qps_dev, qps_wall = nq / (min(dev) / 1e3), nq / (min(wall) / 1e3)
    plain_qps_dev, plain_qps_wall = plain_q / (plain_dev / 1e3), plain_q / (plain_wall / 1e3)
    return {"graphs": ngraphs, "scales": "U[10,16]", "edge_factor": "U[8,32]", "sources_per_graph": k,
            "pr_iters": pr_iters, "total_directed_edges": total_e, "queries": nq,
            "launch_ms": round(min(dev), 3), "call_wall_ms": round(min(wall), 3),
            "queries_per_s": round(qps_dev, 1), "plain_queries_per_s": round(plain_qps_dev, 1),
            "speedup_vs_plain": round(qps_dev / plain_qps_dev, 2),
            "timing_scope": "device time on both sides (CUDA events around the kernels, result copies excluded)",
            "wall": {"queries_per_s": round(qps_wall, 1), "plain_queries_per_s": round(plain_qps_wall, 1),
                     "speedup_vs_plain": round(qps_wall / plain_qps_wall, 2),
                     "scope": "wall-clock of the API call on both sides, result copies to the host included"},
            "plain_sample_queries": plain_q, "identical_results": identical, "graph_build_s": round(gen_s, 1)}


# ---------------------------------------------------------------------------
# served stream: 3 resident graphs, Poisson arrivals, BFS 60% / BC 25% / Radii 15%
# ---------------------------------------------------------------------------

def bench_serving(rg, graphs, rates=(200, 400, 800, 1600, 3200, 12800), per_rate=600, seed=5, workers=4, slo_ms=100.0):
    rng = np.random.default_rng(seed)

    def draw(nq):
        qs = []
        for _ in range(nq):
            gi = int(rng.integers(0, len(graphs)))
            u = rng.random()
            kind = "bfs" if u < 0.6 else ("bc" if u < 0.85 else "radii")
            src = int(rng.integers(0, graphs[gi].n)) if kind != "radii" else int(rng.integers(0, 1 << 20))
            qs.append((gi, kind, src))
        return qs

    # one page-locked result buffer per (graph, kind), used by both arms
    bufs = {(gi, kind): rg.pinned_empty(G.n, np.float64 if kind == "bc" else np.int32)
            for gi, G in enumerate(graphs) for kind in ("bfs", "bc", "radii")}

    # plain: one query at a time through the single-query entry points
    plain_qs = draw(60)
    plain_out = []
    plain_s = 0.0
    per_kind = {}
    for gi, kind, src in plain_qs:
        G, buf = graphs[gi], bufs[(gi, kind)]
        t0 = time.perf_counter()
        if kind == "bfs":
            G.bfs("push", src, depth_out=buf, parents=False)
        elif kind == "bc":
            G.bc_sources(np.array([src], np.uint32), "push", out=buf)
        else:
            G.radii_seeds(rg.radii_query_seeds(src, G.n), "push", out=buf)
        dt = time.perf_counter() - t0
        plain_s += dt
        k = per_kind.setdefault(f"{kind}_s{int(G.n).bit_length() - 1}", [0, 0.0])
        k[0] += 1
        k[1] += dt
        plain_out.append(np.array(buf))  # kept for the identity check, outside the timed span
    plain_qps = len(plain_qs) / plain_s
    out = {"graphs": [int(g.n) for g in graphs], "mix": "BFS 60% / BC 25% / Radii 15%",
           "plain_queries_per_s": round(plain_qps, 1),
           "plain_ms_per_query": {k: {"queries": c, "ms": round(1e3 * t / c, 3), "share_of_plain_time":
                                      round(t / plain_s, 3)} for k, (c, t) in sorted(per_kind.items())},
           "rates": []}
    with rg.Server(graphs, workers=workers, max_batch=64) as S:
        # identical results: the plain sample served in one burst
        ts = [S.submit(gi, kind, src) for gi, kind, src in plain_qs]
        identical = True
        for (gi, kind, _), t, want in zip(plain_qs, ts, plain_out):
            got = S.wait(t, gi, kind, out=bufs[(gi, kind)])[0]
            if kind == "bc":
                ok = np.array_equal(np.isnan(got), np.isnan(want)) and np.allclose(
                    got[~np.isnan(got)], want[~np.isnan(want)], rtol=1e-9, atol=0)
            else:
                ok = np.array_equal(got, want)
            identical &= bool(ok)
        out["identical_results"] = identical
        best = 0.0
        for rate in rates:
            qs = draw(max(per_rate, int(rate * 0.5)))  # at least half a second of arrivals
            S.reset_stats()
            inbox = queue.Queue()

            def waiter():
                for _ in range(len(qs)):
                    t, gi, kind = inbox.get()
                    S.wait(t, gi, kind, out=bufs[(gi, kind)])

            w = threading.Thread(target=waiter)
            w.start()
            gaps = rng.exponential(1.0 / rate, size=len(qs))
            t_next = time.perf_counter()
            for (gi, kind, src), gap in zip(qs, gaps):  # Poisson arrivals
                t_next += gap
                delay = t_next - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                inbox.put((S.submit(gi, kind, src), gi, kind))
            w.join()
            st = S.stats()
            best = max(best, st["qps"])
            out["rates"].append({"offered_qps": rate, "qps": round(st["qps"], 1), "p50_ms": round(st["p50_ms"], 3),
                                 "p99_ms": round(st["p99_ms"], 3), "launches": st["launches"],
                                 "queries": st["completed"], "coalesced": st["batched"]})
        out["best_qps"] = round(best, 1)
        out["speedup_vs_plain"] = round(best / plain_qps, 2)
        # the highest offered rate served with p99 within the latency objective
        ok = [r for r in out["rates"] if r["p99_ms"] <= slo_ms]
        out["slo"] = {"p99_ms": slo_ms, "max_offered_qps_within": max((r["offered_qps"] for r in ok), default=None),
                      "served_qps_there": max((r["qps"] for r in ok), default=None)}
    return out


# ---------------------------------------------------------------------------
# CPU baseline: the oracle port (OpenMP, all host cores)
# ---------------------------------------------------------------------------

def workload_name(scale):
    return (f"RADAR PageRank(20 it)+BFS+BC(1 src)+Radii(64) on RMAT s{scale} ef16 seed 1, symmetric, "
            "degree-sorted, autotuned schedule")


def host_cpu():
    """Host CPU the CPU legs ran on: logical cores, model and last-level cache."""
    info = {"nproc": os.cpu_count()}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            k, _, v = line.partition(":")
            k, v = k.strip(), v.strip()
            if k in ("Model name", "Vendor ID", "Architecture", "L3 cache", "L2 cache", "Socket(s)"):
                info[k.lower().replace(" ", "_").replace("(s)", "s")] = v
    except (OSError, subprocess.SubprocessError):
        pass
    return info


def port_run(off, adj, root, bc_src, pr_iters, with_delta=False, cores=None):
    """The oracle port (OpenMP, all host cores) on the degree-sorted graph, as
    the RADAR binaries run: PageRank (pr_iters iterations), BFS from `root`,
    BC from bc_src, Radii (64 hashInt samples) and optionally PageRankDelta
    (3 rounds).  Inputs are ORIGINAL ids.  Returns (seconds, edges, results):
    edges counted by the port's own edgeMap as the GPU counts them; results
    in ORIGINAL id order (PageRank ranks, BFS depths, BC dependencies, radii)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    cores = cores or os.cpu_count() or 1
    ids, so, sa = orc.degree_sort(off, adj)
    n = len(off) - 1
    seeds = orc.radii_seeds(n)
    t, e, res = {}, {}, {}
    runs = {
        "pagerank": lambda: orc.pagerank(so, sa, "radar", pr_iters, cores)[0],
        "bfs": lambda: orc.bfs(so, sa, int(ids[root]), "radar", cores)[0],
        "bc": lambda: orc.bc(so, sa, ids[bc_src], "radar", cores)[0],
        "radii": lambda: orc.radii(so, sa, ids[seeds], "radar", cores)[0],
    }
    if with_delta:
        runs["pagerank_delta_3"] = lambda: orc.pagerank_delta(so, sa, "radar", 3, cores)[0]
    for k, fn in runs.items():
        orc.take_edges()
        t0 = time.time()
        res[k] = fn()
        t[k] = time.time() - t0
        e[k] = orc.take_edges()
    out = {"pagerank": res["pagerank"][ids], "bfs": orc.depths_from_parents(res["bfs"])[ids],
           "bc": res["bc"][ids], "radii": res["radii"][ids]}
    return t, e, out


def gpu_results(gs, root, bc_src, pr_iters):
    """The same four results from the GPU (ORIGINAL id order), untimed."""
    return {"pagerank": gs.pagerank("radar", pr_iters)[0], "bfs": gs.bfs("radar", root, parents=False)[1],
            "bc": gs.bc_sources(bc_src, "radar")[0], "radii": gs.radii("radar")[0]}


def max_rel(a, b):
    """Largest |a-b| / max(|a|,|b|) over the values that are finite in both
    (0 where both are 0), and whether NaN positions agree."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    nan_ok = bool(np.array_equal(np.isnan(a), np.isnan(b)))
    fin = np.isfinite(a) & np.isfinite(b)
    den = np.maximum(np.abs(a[fin]), np.abs(b[fin]))
    err = np.abs(a[fin] - b[fin])
    rel = np.where(den > 0, err / np.where(den > 0, den, 1), 0.0)
    inf_ok = bool(np.array_equal(a[~fin & ~np.isnan(a)], b[~fin & ~np.isnan(b)]))
    return float(rel.max()) if rel.size else 0.0, nan_ok and inf_ok


def parity(gpu, port, rtol=1e-9):
    """Per app: bit-exact for depths and radii, relative 1e-9 with NaN
    positions equal for ranks and dependencies (the tolerances of the tests)."""
    out = {}
    for k in ("pagerank", "bc"):
        r, same_nan = max_rel(gpu[k], port[k])
        out[k] = {"max_rel": float(f"{r:.3e}"), "nan_positions_equal": same_nan, "ok": bool(same_nan and r <= rtol)}
    for k in ("bfs", "radii"):
        out[k] = {"identical": bool(np.array_equal(gpu[k], port[k]))}
        out[k]["ok"] = out[k]["identical"]
    out["all_ok"] = all(v["ok"] for v in out.values())
    return out


def reference_arm(args):
    """--impl reference: the reference algorithm on the host cores (the oracle
    port, OpenMP, all threads), same workload, metric and config as the GPU
    arm.  The graph is generated and cleaned by the oracle itself (the GAP
    generator and the loader's clean-up restated in oracle.cc), so this arm
    loads no product library."""
    world, rank, local, pg = dist_init()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    off, adj = orc.rmat_csr(args.scale, 16, 1)
    n, m = len(off) - 1, len(adj)
    deg = np.diff(off.astype(np.int64)).astype(np.uint32)
    root = int(orc.source_picker(deg, 1)[0])
    bc_src = orc.bc_sources(deg, 1)
    steps = []
    for i in range(args.warmup + args.steps):
        t, e, _ = port_run(off, adj, root, bc_src, args.cpu_pr_iters)  # the headline: four apps
        if i >= args.warmup:
            steps.append((t, e))
    tot_t = sum(sum(t.values()) for t, _ in steps)
    tot_e = sum(sum(e.values()) for _, e in steps)
    v = tot_e / tot_t / 1e9
    cores = os.cpu_count() or 1
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "GTEPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * tot_t / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args.scale, n, m),
        "cpu_baseline": {"value": round(v, 4), "unit": "GTEPS", "cores": cores, "kind": "port",
                         "sample": f"PageRank {args.cpu_pr_iters} iterations + BFS + BC 1 source + Radii 64 "
                                   "sources per step on the full graph, edges counted by the port's edgeMap",
                         "host": host_cpu()},
        "e2e": {"value": round(v, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def bench_config(scale, n, m):
    """The `config` both arms print (identical keys and values)."""
    return {"workload": workload_name(scale), "n": n, "m": m, "parallelism": "replicas",
            "l2": "inputs larger than L2 (no flush)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--scale", type=int, default=24)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-extra", action="store_true", help="skip the batched and served legs")
    ap.add_argument("--only", default="", help="comma list of extra legs to run (default all): " + ",".join(EXTRA_LEGS))
    ap.add_argument("--cpu-pr-iters", type=int, default=2)
    ap.add_argument("--pr-shape", type=int, default=0,
                    help="pin PageRank's pull sweep shape (RG_OPT_SWEEP_SHAPE, e.g. 81 or 161) after autotuning "
                         "(for profiler captures of one shape); 0 keeps the tuned choice")
    ap.add_argument("--step-only", action="store_true",
                    help="stop after the timed step (for profiler captures of it): no e2e, legs or CPU baseline")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return reference_arm(args)

    world, rank, local, pg = dist_init()
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    import radar_graph as rg
    rg.lib()
    t0 = time.time()
    off, adj = make_graph(rg, args.scale, 16, 1)
    gen_s = time.time() - t0
    n, m = len(off) - 1, len(adj)
    hbm, peak_kind = peaks()

    g = rg.Graph.from_csr(off, adj)
    gs = g.degree_sort()
    g.free()
    root = int(gs.pick_roots(1)[0])  # GAP SourcePicker, as the reference arm picks it
    bc_src = gs.bc_pick_sources(1)
    tuning = gs.autotune("radar")
    if args.pr_shape:
        tuning["pagerank"][1]["sweep_shape"] = args.pr_shape
        gs.set_tuning(tuning)
    rg.set_kernel_timing(True)
    for _ in range(args.warmup):
        run_step(rg, gs, root, bc_src, {})
    barrier(pg)
    rg.lib().rg_synchronize()
    clocks = Clocks(local)
    cuda_profiler(True)
    stats = {}
    tot_ms, tot_edges, launches = 0.0, 0, 0
    wall0 = time.time()
    for _ in range(args.steps):
        ms, e, L = run_step(rg, gs, root, bc_src, stats)
        tot_ms += ms
        tot_edges += e
        launches += L
    rg.lib().rg_synchronize()
    wall = time.time() - wall0
    barrier(pg)
    cuda_profiler(False)
    clk = clocks.stop()
    rg.set_kernel_timing(False)
    value, ms_step = replica_rate(pg, tot_ms / args.steps, tot_edges / args.steps)
    if args.step_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(value, 3), "unit": "GTEPS", "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
                              "config": bench_config(args.scale, n, m), "gpu_launches": int(launches),
                              "apps_ms": {k: round(v["ms"] / args.steps, 3) for k, v in stats.items()},
                              "note": "--step-only: the timed step alone, for profiler captures"}), flush=True)
        gs.free()
        return 0

    # roofline of the dominant kernel: the PageRank edge sweep (pull or push,
    # whichever the autotuner chose), timed per launch with CUDA events
    pr = stats["pagerank"]
    sweep_ms = pr["edge_ms"] / max(pr["edge_launches"], 1)
    sweep_bytes = 4 * m + 4 * (n + 1) + 8 * n + 8 * n
    achieved = sweep_bytes / (sweep_ms / 1e3) / 1e9
    pr_opts = tuning["pagerank"][1]
    if pr_opts["direction"] == 1:  # the pull sweep's template: <hub cache, edges per lane, cache mode>
        shape = pr_opts["sweep_shape"]
        sweep_kernel = f"pr_pull_sweep<{int(pr_opts['hub_smem_kb'] > 0)}, {shape // 10}, {shape % 10}>"
    else:
        sweep_kernel = "pr_push_sweep"
    # the graph's gather ceiling: stream the edge array and gather 8 bytes per
    # edge, nothing else -- what any pull over this graph must at least do
    cuda_profiler(True)  # a profiled range of its own, for captures of the probe
    gather_ms = gather_ceiling_ms(gs)
    cuda_profiler(False)
    traffic = measured_traffic(sweep_kernel, args.scale)
    apps = app_rates(stats, args.steps, hbm)
    for k in apps:
        apps[k]["tuned"] = tuning[k][1]

    # e2e through the C ABI: every step moves the CSR from pinned host memory
    # and degree-sorts it (rg_graph_create_sorted: offsets uploaded, the
    # neighbour array read over the host link by the relabel), runs the four
    # apps and copies every result back into host buffers (pinned, allocated
    # once and reused as a serving loop would)
    h2d = 4 * (n + 1) + 4 * m
    d2h = 8 * n + 4 * n + 4 * n + 8 * n + 4 * n
    off_p, adj_p = rg.pinned_empty(n + 1, np.uint32), rg.pinned_empty(m, np.uint32)
    off_p[:], adj_p[:] = off, adj
    ranks_p, par_p = rg.pinned_empty(n, np.float64), rg.pinned_empty(n, np.uint32)
    depth_p, deps_p, radii_p = rg.pinned_empty(n, np.int32), rg.pinned_empty(n, np.float64), rg.pinned_empty(n, np.int32)
    # The result copies run asynchronously (RG_OPT_ASYNC_RESULTS): each app's
    # copy overlaps the next app, and rg_synchronize -- inside the timed span
    # -- waits for the last of them.
    e2e_ms, e2e_edges = 0.0, 0
    rg.set_option("async_results", 1)
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        with rg.Graph.from_csr_sorted(off_p, adj_p) as g2:
            g2.set_tuning(tuning)
            g2.pagerank("radar", 20, out=ranks_p)
            e = rg.last_timing()["edges_traversed"]
            g2.bfs("radar", root, depth_out=depth_p, parents=par_p)
            e += rg.last_timing()["edges_traversed"]
            g2.bc_sources(bc_src, "radar", out=deps_p)
            e += rg.last_timing()["edges_traversed"]
            g2.radii("radar", out=radii_p)
            e += rg.last_timing()["edges_traversed"]
            rg.synchronize()
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_ms += dt * 1e3
            e2e_edges += e
    rg.set_option("async_results", 0)
    e2e_v, _ = replica_rate(pg, e2e_ms / args.steps, e2e_edges / args.steps)
    e2e = {"value": round(e2e_v, 4), "unit": "GTEPS",
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_ms / args.steps, 3)}

    extra = {}
    # PageRankDelta (the first row past the four apps) on the same graph
    prd = {}
    for i in range(4):
        _, prd_rounds, _ = gs.pagerank_delta("radar", 100)
        t = rg.last_timing()
        if i:
            prd.setdefault("ms", []).append(t["total_ms"])
            prd["edges"], prd["bytes"] = t["edges_traversed"], t["algorithmic_bytes"]
    prd_ms = min(prd["ms"])
    extra["pagerank_delta"] = {"gteps": round(prd["edges"] / (prd_ms / 1e3) / 1e9, 3), "ms": round(prd_ms, 3),
                               "rounds": prd_rounds,
                               "hbm_frac_of_measured": round(prd["bytes"] / (prd_ms / 1e3) / 1e9 / hbm, 4),
                               "variant": "radar", "max_iters": 100}
    legs = set(args.only.split(",")) if args.only else set(EXTRA_LEGS)
    with_cpu = world == 1 and not args.no_cpu
    if rank == 0 and not args.no_extra:
        cuda_profiler(True)
        if "er_contrast" in legs:
            extra["er_contrast"] = bench_er_contrast(rg, args.scale, with_cpu, hbm)
        if "config2" in legs:
            extra["config2_rmat22"] = bench_config2(rg, with_cpu)
        if "graph_build" in legs:
            extra["graph_build"] = bench_input(rg, args.scale)
        if "triangles" in legs:
            extra["triangles"] = bench_triangles(rg, gs, with_cpu)
        if "directed" in legs:
            extra["directed"] = bench_directed(rg, args.scale, with_cpu)
        if "batched" in legs:
            extra["batched"] = bench_batched(rg)
        if "batched_sources" in legs:
            extra["batched_sources"] = bench_batched_sources(rg, gs)
        if "serving" in legs:
            gsv = []
            for sc in (20, 22):
                o2, a2 = make_graph(rg, sc, 16, 1)
                with rg.Graph.from_csr(o2, a2) as gg:
                    gsv.append(gg.degree_sort())
            gsv.append(gs)
            extra["serving"] = bench_serving(rg, gsv)
            for G in gsv[:2]:
                G.free()
        cuda_profiler(False)

    # CPU baseline and parity on the bench graph: the oracle port (all host
    # cores) runs the four RADAR apps with the same inputs -- PageRank for the
    # full 20 iterations -- and every GPU result is compared with its output
    cpu, par = None, None
    if rank == 0 and with_cpu:
        t, e, port = port_run(off, adj, root, bc_src, 20, with_delta=True)
        t_prd, e_prd = t.pop("pagerank_delta_3"), e.pop("pagerank_delta_3")
        par = parity(gpu_results(gs, root, bc_src, 20), port)
        tot_t = sum(t.values())
        extra["pagerank_delta"]["cpu_port_gteps_3_rounds"] = round(e_prd / t_prd / 1e9, 4)
        cpu = {"value": round(sum(e.values()) / tot_t / 1e9, 4), "unit": "GTEPS", "cores": os.cpu_count(),
               "kind": "port",
               "sample": "oracle port, OpenMP, all host cores: RADAR PageRank 20 iterations + BFS + BC 1 source + "
                         f"Radii 64 sources on the full graph ({tot_t:.1f} s)",
               "seconds": {k: round(v, 3) for k, v in t.items()}, "host": host_cpu()}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args.scale, n, m),
            "parity": par,
            "apps_hbm_frac": {k: v["hbm_frac_of_measured"] for k, v in apps.items()},
            "apps": apps,
            "roofline": {"bound": "hbm", "kernel": sweep_kernel,
                         "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(achieved / hbm, 4), "traffic": traffic, "peak_kind": peak_kind,
                         "bytes_per_launch": sweep_bytes, "avg_launch_ms": round(sweep_ms, 4),
                         "gather_ceiling_ms": round(gather_ms, 4),
                         "frac_of_gather_ceiling": round(gather_ms / sweep_ms, 4)},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk,
            "wall_s": round(wall, 3),
            "graph_generation_s": round(gen_s, 1),
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    gs.free()
    return 0


if __name__ == "__main__":
    sys.exit(main())
