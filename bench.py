"""Benchmark: RADAR PageRank / BFS / BC / Radii on a symmetric R-MAT scale-24
graph (edge factor 16, a=0.57 b=0.19 c=0.19, seed 1) on one GB300.

A step is one pass of the four RADAR apps over the resident graph: PageRank
20 iterations, BFS from one root, BC from one source, Radii with 64 samples.
`value` = edges traversed / device time (GTEPS), inputs resident in HBM; the
graph (about 2 GB of edges) is far larger than L2, so no flush is needed
between steps.  `e2e` = the same through the public C ABI from host buffers:
every step uploads the CSR, degree-sorts it on the device and copies every
app's result back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--scale S] [--impl reference]

Under torchrun each rank runs an independent replica on its own GPU
(replicas only: the engine has no cross-GPU exchange); rank 0 prints the
whole-job line.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "radar-graph_gb300"))

METRIC = "GTEPS + % HBM roofline per app (RMAT s24); batched queries/s, p50/p99 vs plain"


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
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allsum(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def make_graph(rg, scale, ef, seed):
    t0 = time.time()
    src, dst = rg.generate_edges(scale, ef, seed)
    off, adj = rg.csr_from_edges(1 << scale, src, dst)
    del src, dst
    return off, adj, time.time() - t0


def pick_root(off, seed=27491095):
    """SourcePicker rule (GAP benchmark.h:47-64): uniform, nonzero degree."""
    rng = np.random.default_rng(seed)
    deg = np.diff(off.astype(np.int64))
    while True:
        r = int(rng.integers(0, len(deg)))
        if deg[r] > 0:
            return r


def run_step(rg, gs, root, bc_src, stats):
    """One pass of the four RADAR apps; returns (device ms, edges, launches)."""
    ms, edges, launches = 0.0, 0, 0
    per = {}
    gs.pagerank("radar", 20)
    t = rg.last_timing()
    per["pagerank"] = t
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


def cpu_baseline(off, adj, seconds_budget=20.0):
    """The oracle port (OpenMP, all host cores) on a bounded sample of the same
    workload: RADAR PageRank (2 iterations), BFS, BC (1 source), Radii."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    cores = os.cpu_count() or 1
    ids, so, sa = orc.degree_sort(off, adj)
    n = len(off) - 1
    m = len(adj)
    root = pick_root(off)
    deg = np.diff(off.astype(np.int64)).astype(np.uint32)
    src = orc.bc_sources(deg, 1)
    seeds = orc.radii_seeds(n)
    t0 = time.time()
    orc.pagerank(so, sa, "radar", 2, cores)
    t_pr = time.time() - t0
    edges = 2 * m
    t0 = time.time()
    par, _ = orc.bfs(so, sa, int(ids[root]), "radar", cores)
    t_bfs = time.time() - t0
    reached = par != 0xFFFFFFFF
    e_bfs = int(np.diff(so.astype(np.int64))[reached].sum())
    t0 = time.time()
    orc.bc(so, sa, ids[src], "radar", cores)
    t_bc = time.time() - t0
    t0 = time.time()
    orc.radii(so, sa, ids[seeds], "radar", cores)
    t_radii = time.time() - t0
    # Radii/BC edge counts are taken from the GPU run's own counters by the caller
    return {"t": {"pagerank": t_pr, "bfs": t_bfs, "bc": t_bc, "radii": t_radii},
            "edges": {"pagerank": edges, "bfs": e_bfs}, "cores": cores}


def reference_arm(args):
    """--impl reference: the reference algorithm on the host cores (the oracle
    port, OpenMP, all threads), same workload and metric as the GPU arm."""
    world, rank, local, pg = dist_init(args)
    if rank != 0:
        return 0
    import radar_graph as rg
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    off, adj, _ = make_graph(rg, args.scale, 16, 1)
    n, m = len(off) - 1, len(adj)
    cores = os.cpu_count() or 1
    ids, so, sa = orc.degree_sort(off, adj)
    root = pick_root(off)
    deg = np.diff(off.astype(np.int64)).astype(np.uint32)
    src = orc.bc_sources(deg, 1)
    seeds = orc.radii_seeds(n)
    sdeg = np.diff(so.astype(np.int64))

    def step():
        e = 0
        t0 = time.time()
        orc.pagerank(so, sa, "radar", args.cpu_pr_iters, cores)
        e += args.cpu_pr_iters * m
        par, _ = orc.bfs(so, sa, int(ids[root]), "radar", cores)
        e += int(sdeg[par != 0xFFFFFFFF].sum())
        d, _ = orc.bc(so, sa, ids[src], "radar", cores)
        e += 2 * int(sdeg[~np.isnan(d)].sum())
        orc.radii(so, sa, ids[seeds], "radar", cores)
        return e, time.time() - t0

    for _ in range(args.warmup):
        step()
    tot_e, tot_t = 0, 0.0
    for _ in range(args.steps):
        e, t = step()
        tot_e += e
        tot_t += t
    v = tot_e / tot_t / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "GTEPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * tot_t / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"RADAR PageRank({args.cpu_pr_iters} it)+BFS+BC(1)+Radii(64), RMAT s{args.scale} ef16 "
                               f"seed 1, symmetric, degree-sorted", "n": n, "m": m},
        "cpu_baseline": {"value": round(v, 4), "unit": "GTEPS", "cores": cores, "kind": "port",
                         "sample": f"PageRank {args.cpu_pr_iters} iterations + BFS + BC 1 source + Radii 64 "
                                   f"sources per step on the full graph"},
        "e2e": {"value": round(v, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--scale", type=int, default=24)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--cpu-pr-iters", type=int, default=2)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return reference_arm(args)

    world, rank, local, pg = dist_init(args)
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local)) if world > 1 else None
    import radar_graph as rg
    rg.lib()
    off, adj, gen_s = make_graph(rg, args.scale, 16, 1)
    n, m = len(off) - 1, len(adj)
    root = pick_root(off)
    hbm, peak_kind = peaks()

    g = rg.Graph.from_csr(off, adj)
    gs = g.degree_sort()
    g.free()
    bc_src = gs.bc_pick_sources(1)
    rg.set_kernel_timing(True)
    stats = {}
    for _ in range(args.warmup):
        run_step(rg, gs, root, bc_src, {})
    barrier(pg)
    rg.lib().rg_synchronize()
    clocks = Clocks(local)
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
    clk = clocks.stop()
    rg.set_kernel_timing(False)
    ms_step = allmax(pg, tot_ms / args.steps)
    edges_all = allsum(pg, tot_edges / args.steps)
    value = edges_all / (ms_step / 1e3) / 1e9

    # roofline of the dominant kernel: the PageRank edge sweep
    pr = stats["pagerank"]
    sweep_ms = pr["edge_ms"] / max(pr["edge_launches"], 1)
    sweep_bytes = 4 * m + 4 * (n + 1) + 8 * n + 8 * n
    achieved = sweep_bytes / (sweep_ms / 1e3) / 1e9
    apps = {}
    for k, s in stats.items():
        apps[k] = {"gteps": round(s["edges"] / (s["ms"] / 1e3) / 1e9, 3),
                   "ms": round(s["ms"] / args.steps, 3),
                   "hbm_frac": round(s["bytes"] / (s["ms"] / 1e3) / 1e9 / hbm, 4)}

    # e2e through the C ABI from host buffers
    e2e = None
    if rank == 0 or True:
        e2e_ms, e2e_edges = 0.0, 0
        h2d = 4 * (n + 1) + 4 * m
        d2h = 8 * n + (4 + 4) * n + 8 * n + 4 * n
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            with rg.Graph.from_csr(off, adj) as g1, g1.degree_sort() as g2:
                g2.pagerank("radar", 20)
                e = rg.last_timing()["edges_traversed"]
                g2.bfs("radar", root)
                e += rg.last_timing()["edges_traversed"]
                g2.bc_sources(bc_src, "radar")
                e += rg.last_timing()["edges_traversed"]
                g2.radii("radar")
                e += rg.last_timing()["edges_traversed"]
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                e2e_ms += dt * 1e3
                e2e_edges += e
        e2e = {"value": round(e2e_edges / (e2e_ms / 1e3) / 1e9 * world, 4), "unit": "GTEPS",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": round(e2e_ms / args.steps, 3)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        c = cpu_baseline(off, adj)
        # edge counts of BC/Radii from the GPU run (identical traversal)
        e_bc = stats["bc"]["edges"] / args.steps
        e_radii = stats["radii"]["edges"] / args.steps
        t = c["t"]
        tot_e = c["edges"]["pagerank"] + c["edges"]["bfs"] + e_bc + e_radii
        tot_t = sum(t.values())
        cpu = {"value": round(tot_e / tot_t / 1e9, 4), "unit": "GTEPS", "cores": c["cores"], "kind": "port",
               "sample": "oracle port, OpenMP: RADAR PageRank 2 iterations + BFS + BC 1 source + Radii 64 sources "
                         f"on the full graph ({tot_t:.1f} s)",
               "seconds": {k: round(v, 3) for k, v in t.items()}}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"RADAR PageRank(20 it)+BFS+BC(1 src)+Radii(64) on RMAT s{args.scale} ef16 seed 1, "
                                   "symmetric, degree-sorted", "n": n, "m": m, "parallelism": "replicas",
                       "l2": "inputs larger than L2 (no flush)", "graph_build_s": round(gen_s, 1)},
            "apps": apps,
            "roofline": {"bound": "hbm", "kernel": "pr_push_sweep<hub prefix>", "achieved": round(achieved, 1),
                         "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4), "traffic": None,
                         "peak_kind": peak_kind, "bytes_per_launch": sweep_bytes,
                         "avg_launch_ms": round(sweep_ms, 4)},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk,
            "wall_s": round(wall, 3),
        }
        print(json.dumps(line), flush=True)
    gs.free()
    return 0


if __name__ == "__main__":
    sys.exit(main())
