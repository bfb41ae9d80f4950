"""Times the oracle port against the reference's own RADAR binaries on the
same graph and host threads (test infrastructure: the evidence behind using
the port as the CPU baseline where the reference binaries cannot run).

The reference binaries come from `make -C oracle ref` (built from the
reference sources, output in oracle/_ref/; needs the reference tree).  The
graph is the oracle's seeded R-MAT (the GAP generator restated), written as a
Ligra AdjacencyGraph file; each binary runs with -s and -rounds R and its own
"Run Time(sec)" lines are parsed (the median of the rounds after the first).
The port runs the same app on the degree-sorted graph, as the RADAR binaries
do after their -preprocess 1 default, with OMP_NUM_THREADS threads.

    python oracle/port_vs_reference.py [--scale 20] [--threads N] [--rounds 3]
"""

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import oracle as orc  # noqa: E402

REF = os.path.join(HERE, "_ref", "RADAR")


def write_adjacency(path, off, adj):
    with open(path, "w") as f:
        f.write(f"AdjacencyGraph\n{len(off) - 1}\n{len(adj)}\n")
        np.savetxt(f, off[:-1], fmt="%d")
        np.savetxt(f, adj, fmt="%d")


def ref_times(app, args, path, threads, rounds):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="close")
    r = subprocess.run([os.path.join(REF, app), "-s", "-rounds", str(rounds), *args, path], capture_output=True,
                       text=True, env=env, timeout=3600)
    if r.returncode != 0:
        raise RuntimeError(f"{app} failed: {r.stderr[-500:]}")
    t = [float(x) for x in re.findall(r"Run Time\(sec\)\s*:\s*([0-9.eE+-]+)", r.stdout)]
    return statistics.median(t[1:] if len(t) > 1 else t)


def port_time(fn, reps):
    t = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        t.append(time.perf_counter() - t0)
    return statistics.median(t[1:] if len(t) > 1 else t)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=20)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--rounds", type=int, default=3)
    a = ap.parse_args()
    if not os.path.exists(os.path.join(REF, "PageRank")):
        sys.exit("reference binaries missing: make -C oracle ref REF=<reference root>")
    off, adj = orc.rmat_csr(a.scale, 16, 1)
    n = len(off) - 1
    deg = np.diff(off.astype(np.int64)).astype(np.uint32)
    root = int(orc.source_picker(deg, 1)[0])
    ids, so, sa = orc.degree_sort(off, adj)
    seeds = orc.radii_seeds(n)
    bc_src = orc.bc_sources(deg, 1)
    T = a.threads
    out = {"graph": f"RMAT s{a.scale} ef16 seed 1 (n={n}, m={len(adj)})", "threads": T, "rounds": a.rounds}
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "g.adj")
        write_adjacency(path, off, adj)
        cases = {
            "PageRank 20 it": (("PageRank", ["-maxiters", "20"]),
                               lambda: orc.pagerank(so, sa, "radar", 20, T)),
            "BFS": (("BFS", ["-r", str(root)]), lambda: orc.bfs(so, sa, int(ids[root]), "radar", T)),
            "BC 1 source": (("BC-manyiter-v2", ["-maxiters", "1"]), lambda: orc.bc(so, sa, ids[bc_src], "radar", T)),
            "Radii": (("Radii", []), lambda: orc.radii(so, sa, ids[seeds], "radar", T)),
        }
        for name, ((app, args), fn) in cases.items():
            tr = ref_times(app, args, path, T, a.rounds)
            tp = port_time(fn, a.rounds + 1)
            out[name] = {"reference_s": round(tr, 4), "port_s": round(tp, 4), "port_over_reference": round(tp / tr, 3)}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
