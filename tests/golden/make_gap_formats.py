"""Golden triangle totals for GAP's text edge-list formats.

One seeded edge list (repeats and self loops kept, as generated) is written
as .el, .wel, .gr, .graph (METIS), and .mtx (general, and symmetric with each
undirected edge listed once).  The reference's GAP tc_local (built from the
reference sources by oracle/Makefile into oracle/_ref/gap) reads each file
with -s and reports the triangle total.  The totals and the edge list go to
gap_formats.npz; tests/test_host_formats.py writes the same files, reads them
with rg_read_edges, cleans them up and checks the totals with the oracle.

    python tests/golden/make_gap_formats.py
"""

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "radar-graph_gb300"))

FORMATS = ("el", "wel", "gr", "graph", "mtx", "sym.mtx")


def edge_list(scale=10, ef=8, seed=3):
    import radar_graph as rg
    src, dst = rg.generate_edges(scale, ef, seed, False)
    # a few explicit self loops and repeats on top of the generator's own
    src = np.concatenate([src, np.array([5, 5, 7], np.uint32)])
    dst = np.concatenate([dst, np.array([5, 9, 7], np.uint32)])
    return src, dst


def write_formats(src, dst, base):
    """Writes base.<fmt> for every format; returns {fmt: path}."""
    n = int(max(src.max(), dst.max())) + 1
    rng = np.random.default_rng(11)
    w = rng.integers(1, 100, size=len(src))
    paths = {}
    p = base + ".el"
    with open(p, "w") as f:
        f.writelines(f"{u} {v}\n" for u, v in zip(src, dst))
    paths["el"] = p
    p = base + ".wel"
    with open(p, "w") as f:
        f.writelines(f"{u} {v} {x}\n" for u, v, x in zip(src, dst, w))
    paths["wel"] = p
    p = base + ".gr"  # DIMACS shape; GAP keeps the ids as written
    with open(p, "w") as f:
        f.write(f"c written by make_gap_formats\np sp {n} {len(src)}\n")
        f.writelines(f"a {u} {v} {x}\n" for u, v, x in zip(src, dst, w))
    paths["gr"] = p
    # METIS: line u lists u's out-neighbours 1-based.  Each line ends with a
    # space: GAP's ReadInMetis (reader.h:126, 132) reads a line with
    # `edge_stream >> v >> std::ws`, and the number that ends the line sets
    # eofbit, so the following std::ws fails and that last neighbour is
    # dropped unless whitespace follows it.  With the trailing space GAP reads
    # every listed neighbour, which is what rg_read_edges does.
    p = base + ".graph"
    order = np.argsort(src, kind="stable")
    lists = [[] for _ in range(n)]
    for i in order:
        lists[int(src[i])].append(int(dst[i]) + 1)
    with open(p, "w") as f:
        f.write(f"% written by make_gap_formats\n{n} {len(src)}\n")
        f.writelines("".join(f"{x} " for x in ls) + "\n" for ls in lists)
    paths["graph"] = p
    p = base + ".mtx"
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern general\n% entries 1-based\n")
        f.write(f"{n} {n} {len(src)}\n")
        f.writelines(f"{u + 1} {v + 1}\n" for u, v in zip(src, dst))
    paths["mtx"] = p
    p = base + ".sym.mtx"  # symmetric: each undirected pair once, reader adds the mirror
    pairs = sorted({(max(int(u), int(v)), min(int(u), int(v))) for u, v in zip(src, dst)})
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real symmetric\n")
        f.write(f"{n} {n} {len(pairs)}\n")
        f.writelines(f"{a + 1} {b + 1} 0.5\n" for a, b in pairs)
    paths["sym.mtx"] = p
    return paths


def main():
    tc = os.path.join(ROOT, "oracle", "_ref", "gap", "tc_local")
    if not os.path.exists(tc):
        raise SystemExit("build the reference binaries first: make -C oracle ref")
    src, dst = edge_list()
    totals = {}
    with tempfile.TemporaryDirectory() as d:
        for fmt, path in write_formats(src, dst, os.path.join(d, "g")).items():
            r = subprocess.run([tc, "-f", path, "-s", "-n", "1", "-a"], capture_output=True, text=True,
                               env=dict(os.environ, OMP_NUM_THREADS="8"))
            if r.returncode != 0:
                raise RuntimeError(f"tc_local on {fmt} failed:\n{r.stdout}\n{r.stderr}")
            tri = [ln for ln in r.stdout.splitlines() if ln.strip().endswith(" triangles")]
            totals[fmt] = int(tri[-1].split()[0])
            print(fmt, totals[fmt])
    np.savez_compressed(os.path.join(HERE, "gap_formats.npz"), src=src, dst=dst,
                        formats=np.array(list(totals.keys())), totals=np.array(list(totals.values()), np.int64))


if __name__ == "__main__":
    main()
