"""Generates the golden vectors in tests/golden/ by running the REFERENCE's own
OpenMP apps (built from the reference sources by `make -C oracle ref`, which
needs the reference tree; the fixtures are committed so the tests do not).

For each seeded graph the raw symmetric adjacency (both directions, with the
duplicates and self-loops the generator produced) is written as a Ligra
AdjacencyGraph text file and fed to oracle/_ref/<variant>/<App>.dump, which
runs the unmodified app and captures its result arrays (see
oracle/ref_driver.cc).  Outputs are stored in ORIGINAL id order.

    python tests/golden/make_golden.py [--ref /path/to/reference]
"""

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "radar-graph_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import radar_graph as rg  # noqa: E402  (generator only: it makes the inputs)
import oracle as orc  # noqa: E402

REFBIN = os.path.join(ROOT, "oracle", "_ref")

# name: (scale, edge_factor, seed, uniform, hub_threads)
# hub_threads: thread count for the HUBDUP/RADAR binaries, chosen so that the
# reference's numHubs = 2^25 / (threads * elem [+ extra]) stays <= n
# (numHubs > n makes those apps read/write out of bounds).
GRAPHS = {
    "rmat10": (10, 16, 1, False, None),
    "er10": (10, 8, 2, True, None),
    "rmat12": (12, 8, 1, False, None),
    "rmat13": (13, 8, 3, False, 1024),
}


def raw_adjacency(n, src, dst):
    """Both directions of every edge, grouped by source (stable), no clean-up."""
    s = np.concatenate([src, dst]).astype(np.int64)
    d = np.concatenate([dst, src]).astype(np.uint32)
    order = np.argsort(s, kind="stable")
    s, d = s[order], d[order]
    off = np.searchsorted(s, np.arange(n), side="left").astype(np.uint32)
    return off, d


def tiny_graph():
    """12 vertices: duplicates, self-loops, isolated vertices 9-11, two components."""
    edges = [(0, 1), (0, 1), (1, 2), (2, 0), (2, 2), (3, 4), (4, 5), (5, 3), (5, 6), (6, 7), (7, 8), (8, 6),
             (1, 3), (0, 0), (4, 4)]
    src = np.array([e[0] for e in edges], np.uint32)
    dst = np.array([e[1] for e in edges], np.uint32)
    return 12, src, dst


def write_text(path, off_n, adj):
    with open(path, "w") as f:
        f.write("AdjacencyGraph\n%d\n%d\n" % (len(off_n), len(adj)))
        f.write("\n".join(str(int(x)) for x in off_n) + "\n")
        if len(adj):
            f.write("\n".join(str(int(x)) for x in adj) + "\n")


def read_dump(path):
    recs = []
    with open(path, "rb") as f:
        data = f.read()
    p = 0
    while p < len(data):
        nb = int.from_bytes(data[p:p + 8], "little")
        recs.append(data[p + 8:p + 8 + nb])
        p += 8 + nb
    return recs


def run(variant, app, gpath, args, threads, workdir):
    exe = os.path.join(REFBIN, variant, app + ".dump")
    out = os.path.join(workdir, f"{variant}_{app}.bin")
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    # the sorting variants' own default is -preprocess 1 (ligra.h:566)
    pre = ["-preprocess", "1"] if variant in ("degree-sorting", "RADAR") else []
    cmd = [exe, "-s"] + pre + args + ["-dump", out, gpath]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, cwd=workdir)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd} failed:\n{r.stdout}\n{r.stderr}")
    recs = read_dump(out)
    off = np.frombuffer(recs[0], np.uint32).copy()
    adj = np.frombuffer(recs[1], np.uint32).copy()
    new_ids = np.frombuffer(recs[2], np.uint32).copy()
    return off, adj, new_ids, recs[3:], r.stdout


def to_orig(arr, new_ids, preprocessed):
    return arr[new_ids] if preprocessed else arr


def make(name, n, src, dst, hub_threads, workdir, out):
    off_n, adj = raw_adjacency(n, src, dst)
    gpath = os.path.join(workdir, name + ".adj")
    write_text(gpath, off_n, adj)
    res = {"raw_off": off_n, "raw_adj": adj}
    T = 8
    # loaded graph + PageRank (push, not preprocessed)
    off, cadj, _, cap, _ = run("push-new-orig", "PageRank", gpath, ["-maxiters", "20"], T, workdir)
    res["off"], res["adj"] = off, cadj
    deg = np.diff(off.astype(np.int64))
    nz = np.nonzero(deg)[0]
    roots = [int(nz[0]), int(nz[len(nz) // 2])] if len(nz) else [0]
    res["bfs_roots"] = np.array(roots, np.uint32)

    def pr_of(cap):
        a, b = (np.frombuffer(c, np.float64) for c in cap[:2])
        return a.copy() if not np.any(b) else b.copy()

    res["pr_push"] = pr_of(cap)
    _, _, _, cap, _ = run("push-pull", "PageRank", gpath, ["-maxiters", "20"], T, workdir)
    res["pr_push-pull"] = pr_of(cap)
    _, _, nid, cap, _ = run("degree-sorting", "PageRank", gpath, ["-maxiters", "20"], T, workdir)
    res["new_ids"] = nid
    res["pr_degree-sorting"] = to_orig(pr_of(cap), nid, True)
    # early-stop case: the L1 break (PageRank.C:172) before maxiters
    _, _, _, cap, so = run("push-new-orig", "PageRank", gpath, ["-maxiters", "200"], T, workdir)
    res["pr200_push"] = pr_of(cap)
    res["pr200_iters"] = np.array([int(so.split("Num Iters = ")[1].split()[0])], np.int64)

    # PageRankDelta: p is freed third-from-last among the n-double blocks
    # (PageRankDelta.C:148-154 frees p, then Delta and nghSum)
    def prd_of(cap):
        blocks = [c for c in cap if len(c) == 8 * n]
        return np.frombuffer(blocks[-3], np.float64).copy()

    def iters_of(stdout):
        return int(stdout.split("Num Iters = ")[1].split()[0])

    for variant, pre in (("push", False), ("push-pull", False), ("degree-sorting", True)):
        vdir = {"push": "push-new-orig"}.get(variant, variant)
        _, _, nid, cap, so = run(vdir, "PageRankDelta", gpath, ["-maxiters", "20"], T, workdir)
        res[f"prd_{variant}"] = to_orig(prd_of(cap), nid, pre)
        res[f"prd_iters_{variant}"] = np.array([iters_of(so)], np.int64)
    _, _, _, cap, so = run("push-new-orig", "PageRankDelta", gpath, ["-maxiters", "5"], T, workdir)
    res["prd5_push"] = prd_of(cap)  # stopped by -maxiters before the L1 break
    res["prd5_iters"] = np.array([iters_of(so)], np.int64)

    # BFS: depths from the reference parents (internal ids), per root
    for variant, pre in (("push", False), ("push-pull", False), ("degree-sorting", True)):
        vdir = {"push": "push-new-orig"}.get(variant, variant)
        for ri, r in enumerate(roots):
            _, _, nid, cap, _ = run(vdir, "BFS", gpath, ["-r", str(r)], T, workdir)
            par = np.frombuffer(cap[-1], np.uint32).copy()
            depth = orc.depths_from_parents(par)
            res[f"bfs{ri}_{variant}"] = to_orig(depth, nid, pre)
    # BC: 1 source and 4 chained sources
    for variant, pre in (("push", False), ("push-pull", False), ("degree-sorting", True)):
        vdir = {"push": "push-new-orig"}.get(variant, variant)
        for k in (1, 4):
            _, _, nid, cap, _ = run(vdir, "BC-manyiter-v2", gpath, ["-maxiters", str(k)], T, workdir)
            res[f"bc{k}_{variant}"] = to_orig(np.frombuffer(cap[2], np.float64).copy(), nid, pre)
    # Radii: one thread so seed collisions resolve in loop order (largest i wins)
    for variant, pre in (("push", False), ("push-pull", False), ("degree-sorting", True)):
        vdir = {"push": "push-new-orig"}.get(variant, variant)
        _, _, nid, cap, _ = run(vdir, "Radii", gpath, [], 1, workdir)
        res[f"radii_{variant}"] = to_orig(np.frombuffer(cap[2], np.int32).copy(), nid, pre)
    # HUBDUP / RADAR where their hub count fits the graph
    if hub_threads:
        for variant, pre in (("hubdup", False), ("radar", True)):
            vdir = {"radar": "RADAR"}.get(variant, variant)
            _, _, nid, cap, _ = run(vdir, "PageRank", gpath, ["-maxiters", "20"], hub_threads, workdir)
            res[f"pr_{variant}"] = to_orig(pr_of(cap), nid, pre)
            _, _, nid, cap, so = run(vdir, "PageRankDelta", gpath, ["-maxiters", "20"], hub_threads, workdir)
            res[f"prd_{variant}"] = to_orig(prd_of(cap), nid, pre)
            res[f"prd_iters_{variant}"] = np.array([iters_of(so)], np.int64)
            # hubdup BC is skipped: it builds its hub bitmap without clearing
            # it (hubdup/Ligra/apps/BC-manyiter-v2.C:267, no hubMap.reset()),
            # so its output depends on uninitialised heap memory
            if variant == "radar":
                _, _, nid, cap, _ = run(vdir, "BC-manyiter-v2", gpath, ["-maxiters", "4"], hub_threads, workdir)
                res[f"bc4_{variant}"] = to_orig(np.frombuffer(cap[2], np.float64).copy(), nid, pre)
        # RADAR BFS (hubdup BFS has a wrong-depth bug: BFS.C:161 seeds the
        # per-thread copies from Parents indexed by vertex id, not hub slot)
        for ri, r in enumerate(roots):
            _, _, nid, cap, _ = run("RADAR", "BFS", gpath, ["-r", str(r)], hub_threads, workdir)
            par = np.frombuffer(cap[-1], np.uint32).copy()
            res[f"bfs{ri}_radar"] = to_orig(orc.depths_from_parents(par), nid, True)
    # triangle count (GAP tc_local, undirected edge list, -s symmetrises)
    el = os.path.join(workdir, name + ".el")
    with open(el, "w") as f:
        for u in range(len(off) - 1):
            for v in cadj[off[u]:off[u + 1]]:
                if u < v:
                    f.write(f"{u} {int(v)}\n")
    if os.path.getsize(el) > 0:
        r = subprocess.run([os.path.join(REFBIN, "gap", "tc_local"), "-f", el, "-s", "-n", "1", "-a"],
                           capture_output=True, text=True, env=dict(os.environ, OMP_NUM_THREADS="8"))
        if r.returncode != 0:
            raise RuntimeError(f"tc_local failed:\n{r.stdout}\n{r.stderr}")
        tri = [ln for ln in r.stdout.splitlines() if ln.strip().endswith(" triangles")]
        res["tc_total"] = np.array([int(tri[-1].split()[0])], np.int64)
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **res)
    print(f"{name}: n={n} m={len(cadj)} keys={len(res)}")


# directed graphs: name -> (scale, edge_factor, seed, uniform, hub_threads)
DIRECTED = {
    "drmat10": (10, 8, 11, False, None),
    "der10": (10, 8, 12, True, None),
    "drmat13": (13, 8, 13, False, 1024),
}


def run_directed(variant, app, gpath, args, threads, workdir):
    """Like run() without -s: the dump holds out-lists, in-lists, new_ids."""
    exe = os.path.join(REFBIN, variant, app + ".dump")
    out = os.path.join(workdir, f"d_{variant}_{app}.bin")
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    pre = ["-preprocess", "1"] if variant in ("degree-sorting", "RADAR") else []
    cmd = [exe] + pre + args + ["-dump", out, gpath]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, cwd=workdir)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd} failed:\n{r.stdout}\n{r.stderr}")
    recs = read_dump(out)
    arrs = [np.frombuffer(recs[i], np.uint32).copy() for i in range(5)]
    return arrs, recs[5:], r.stdout


def make_directed(name, n, src, dst, hub_threads, workdir, out):
    """Directed golden vectors: the raw out-lists (src -> dst, with repeats
    and self loops) as a Ligra file, the reference apps run without -s."""
    order = np.argsort(src, kind="stable")
    s, d = src[order].astype(np.int64), dst[order].astype(np.uint32)
    off_n = np.searchsorted(s, np.arange(n), side="left").astype(np.uint32)
    gpath = os.path.join(workdir, name + ".adj")
    write_text(gpath, off_n, d)
    res = {"raw_off": off_n, "raw_adj": d}
    T = 8
    (off, adj, in_off, in_adj, _), cap, _ = run_directed("push-new-orig", "PageRank", gpath, ["-maxiters", "20"], T,
                                                         workdir)
    res.update(off=off, adj=adj, in_off=in_off, in_adj=in_adj)
    outdeg = np.diff(off.astype(np.int64))
    nz = np.nonzero(outdeg)[0]
    roots = [int(nz[0]), int(nz[len(nz) // 2])]
    res["bfs_roots"] = np.array(roots, np.uint32)

    def pr_of(cap):
        a, b = (np.frombuffer(c, np.float64) for c in cap[:2])
        return a.copy() if not np.any(b) else b.copy()

    def prd_of(cap):
        blocks = [c for c in cap if len(c) == 8 * n]
        return np.frombuffer(blocks[-3], np.float64).copy()

    res["pr_push"] = pr_of(cap)
    variants = (("push", "push-new-orig", False), ("push-pull", "push-pull", False),
                ("degree-sorting", "degree-sorting", True))
    for variant, vdir, pre in variants:
        if variant != "push":
            (_, _, _, _, nid), cap, _ = run_directed(vdir, "PageRank", gpath, ["-maxiters", "20"], T, workdir)
            res[f"pr_{variant}"] = to_orig(pr_of(cap), nid, pre)
            if pre:
                res["new_ids"] = nid  # in-degree order (-preprocess 1)
        (_, _, _, _, nid), cap, so = run_directed(vdir, "PageRankDelta", gpath, ["-maxiters", "20"], T, workdir)
        res[f"prd_{variant}"] = to_orig(prd_of(cap), nid, pre)
        res[f"prd_iters_{variant}"] = np.array([int(so.split("Num Iters = ")[1].split()[0])], np.int64)
        for ri, r in enumerate(roots):
            (_, _, _, _, nid), cap, _ = run_directed(vdir, "BFS", gpath, ["-r", str(r)], T, workdir)
            par = np.frombuffer(cap[-1], np.uint32).copy()
            res[f"bfs{ri}_{variant}"] = to_orig(orc.depths_from_parents(par), nid, pre)
        for k in (1, 2, 3):
            (_, _, _, _, nid), cap, _ = run_directed(vdir, "BC-manyiter-v2", gpath, ["-maxiters", str(k)], T,
                                                     workdir)
            res[f"bc{k}_{variant}"] = to_orig(np.frombuffer(cap[2], np.float64).copy(), nid, pre)
        (_, _, _, _, nid), cap, _ = run_directed(vdir, "Radii", gpath, [], 1, workdir)
        res[f"radii_{variant}"] = to_orig(np.frombuffer(cap[2], np.int32).copy(), nid, pre)
    if hub_threads:
        for variant, vdir, pre in (("hubdup", "hubdup", False), ("radar", "RADAR", True)):
            (_, _, _, _, nid), cap, _ = run_directed(vdir, "PageRank", gpath, ["-maxiters", "20"], hub_threads,
                                                     workdir)
            res[f"pr_{variant}"] = to_orig(pr_of(cap), nid, pre)
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **res)
    print(f"{name}: n={n} m={len(adj)} keys={len(res)} (directed)")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    a = ap.parse_args()
    if not os.path.exists(os.path.join(REFBIN, "RADAR", "BFS.dump")):
        sys.exit("reference binaries missing: run `make -C oracle ref` first")
    with tempfile.TemporaryDirectory() as wd:
        n, s, d = tiny_graph()
        make("tiny", n, s, d, None, wd, a.out)
        for name, (scale, ef, seed, uni, ht) in GRAPHS.items():
            s, d = rg.generate_edges(scale, ef, seed, uni)
            make(name, 1 << scale, s, d, ht, wd, a.out)
        for name, (scale, ef, seed, uni, ht) in DIRECTED.items():
            s, d = rg.generate_edges(scale, ef, seed, uni)
            make_directed(name, 1 << scale, s, d, ht, wd, a.out)


if __name__ == "__main__":
    main()
