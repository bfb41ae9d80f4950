import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "radar-graph_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")
# graph goldens (every .npz but the GAP edge-list format totals)
ALL_GOLDEN = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                    if os.path.basename(p) != "gap_formats.npz")
# directed graphs carry their in-lists; the rest are symmetric
DIRECTED_NAMES = [n for n in ALL_GOLDEN if "in_off" in np.load(os.path.join(GOLDEN, n + ".npz")).files]
GOLDEN_NAMES = [n for n in ALL_GOLDEN if n not in DIRECTED_NAMES]

# Tolerance for double results (PageRank ranks, BC dependencies): relative
# 1e-9, the bar the reference comparison is held to.  Integer results (BFS
# depths, Radii, the degree-sort permutation, the cleaned CSR) are bit-exact.
RTOL = 1e-9


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return {n: dict(np.load(os.path.join(GOLDEN, n + ".npz"))) for n in GOLDEN_NAMES}


@pytest.fixture(scope="session")
def golden_directed():
    return {n: dict(np.load(os.path.join(GOLDEN, n + ".npz"))) for n in DIRECTED_NAMES}


def assert_close(a, b, rtol=RTOL, what=""):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.shape == b.shape, what
    na, nb = np.isnan(a), np.isnan(b)
    assert np.array_equal(na, nb), f"{what}: NaN positions differ ({na.sum()} vs {nb.sum()})"
    a, b = a[~na], b[~nb]
    inf = np.isinf(a) | np.isinf(b)
    assert np.array_equal(a[inf], b[inf]), f"{what}: inf values differ"
    a, b = a[~inf], b[~inf]
    err = np.abs(a - b)
    tol = rtol * np.maximum(np.abs(a), np.abs(b))
    bad = err > tol
    assert not bad.any(), (f"{what}: {bad.sum()} values beyond rel {rtol}; worst rel "
                           f"{(err / np.maximum(np.abs(b), 1e-300)).max():.3e}")
