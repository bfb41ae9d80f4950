"""The command-line apps (bin/PageRank, bin/BFS, bin/BC, bin/Radii): the
reference's flags (-s -r -maxiters -rounds -preprocess -b) on a Ligra
AdjacencyGraph file, results written with -out and compared with the golden
outputs of the reference's own binaries."""

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, assert_close

BIN = os.path.join(ROOT, "radar-graph_gb300", "bin")


def _bin(app):
    p = os.path.join(BIN, app)
    if not os.path.exists(p):
        pytest.skip("CLI apps not built")
    return p


def _run(app, *args):
    return subprocess.run([_bin(app), *map(str, args)], capture_output=True, text=True, timeout=600)


def _write_raw(golden, name, tmp_path):
    """The golden graph as the reference read it: the raw (uncleaned) file."""
    import radar_graph as rg
    g = golden[name]
    raw_off = np.append(g["raw_off"], np.uint32(len(g["raw_adj"])))
    path = tmp_path / f"{name}.adj"
    rg.write_adjacency(path, raw_off, g["raw_adj"])
    return path


def test_usage_and_flags():
    r = _run("BFS")
    assert r.returncode == 2 and "usage" in r.stderr
    r = _run("PageRank", "-maxiters", "3", "/nonexistent/graph.adj")  # no -s: read as a directed graph
    assert r.returncode == 1 and "Unable to open" in r.stderr
    r = _run("BC", "-s", "-variant", "nosuch", "graph.adj")
    assert r.returncode == 2 and "variant" in r.stderr
    r = _run("Radii", "-s", "/nonexistent/graph.adj")
    assert r.returncode == 1 and "Unable to open" in r.stderr


def test_no_device_fails_cleanly(golden, tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    path = _write_raw(golden, "tiny", tmp_path)
    r = _run("BFS", "-s", "-r", "0", path)
    assert r.returncode == 1 and "device" in r.stderr.lower()


VARIANTS = {"push": "push", "push-pull": "push-pull", "degree-sorting": "degree-sorting"}


@pytest.mark.gpu
@pytest.mark.parametrize("variant", sorted(VARIANTS))
def test_cli_matches_reference(golden, tmp_path, variant):
    name = "rmat12"
    g = golden[name]
    path = _write_raw(golden, name, tmp_path)
    out = tmp_path / "out.txt"
    common = ["-s", "-rounds", "1", "-variant", variant, "-out", out]

    r = _run("PageRank", "-maxiters", "20", *common, path)
    assert r.returncode == 0, r.stderr
    assert "Run Time(sec)" in r.stdout
    assert_close(np.loadtxt(out), g[f"pr_{variant}"], what="PageRank via CLI")

    for i, root in enumerate(g["bfs_roots"]):
        r = _run("BFS", "-r", int(root), *common, path)
        assert r.returncode == 0, r.stderr
        assert np.array_equal(np.loadtxt(out, dtype=np.int64), g[f"bfs{i}_{variant}"])

    for k in (1, 4):
        r = _run("BC", "-maxiters", k, *common, path)
        assert r.returncode == 0, r.stderr
        assert_close(np.loadtxt(out), g[f"bc{k}_{variant}"], what=f"BC {k} via CLI")

    r = _run("Radii", *common, path)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.loadtxt(out, dtype=np.int64), g[f"radii_{variant}"])


@pytest.mark.gpu
def test_cli_preprocess_flag(golden, tmp_path):
    """-preprocess -1 turns RADAR's default degree sort off; results are the same."""
    g = golden["rmat12"]
    path = _write_raw(golden, "rmat12", tmp_path)
    out = tmp_path / "out.txt"
    for pre in ("1", "-1"):
        r = _run("BFS", "-s", "-rounds", "0", "-preprocess", pre, "-r", int(g["bfs_roots"][0]), "-out", out, path)
        assert r.returncode == 0, r.stderr
        assert ("DegSort Time" in r.stdout) == (pre == "1")
        assert np.array_equal(np.loadtxt(out, dtype=np.int64), g["bfs0_push"])


@pytest.mark.gpu
@pytest.mark.parametrize("variant", sorted(VARIANTS))
def test_cli_pagerank_delta(golden, tmp_path, variant):
    g = golden["rmat12"]
    path = _write_raw(golden, "rmat12", tmp_path)
    out = tmp_path / "out.txt"
    r = _run("PageRankDelta", "-s", "-rounds", "0", "-maxiters", "20", "-variant", variant, "-out", out, path)
    assert r.returncode == 0, r.stderr
    assert_close(np.loadtxt(out), g[f"prd_{variant}"], what="PageRankDelta via CLI")


@pytest.mark.gpu
def test_cli_prints_a_json_result_line(golden, tmp_path):
    """Every run ends with one JSON result line: app, variant, graph, size,
    time, GTEPS and the fraction of the HBM roofline (here against a given
    peak), and the GPU's name."""
    import json
    path = _write_raw(golden, "rmat12", tmp_path)
    r = _run("BFS", "-s", "-rounds", "0", "-r", 1, "-hbm-gbs", "6791.4", path)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    j = lines[0]
    assert j["app"] == "BFS" and j["variant"] == "radar" and j["graph"] == str(path)
    assert j["n"] == 4096 and j["m"] == len(golden["rmat12"]["adj"]) and j["degree_sorted"] is True
    assert j["gteps"] > 0 and j["edges"] > 0 and j["peak_kind"] == "given" and j["hbm_peak_gbs"] == 6791.4
    assert j["hbm_frac"] == pytest.approx(j["achieved_gbs"] / 6791.4, rel=1e-3)
    assert j["gpu"]
