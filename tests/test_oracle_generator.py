"""The oracle's own graph inputs (CPU): its restatement of the GAP generator
(generator.h:52-114) and of the symmetric loader's clean-up (IO.h:429-474)
give the same edge lists and CSRs as the library's host generator, so the
reference arm of the benchmark and the large parity tests can build their
graphs without the product; GAP's SourcePicker (benchmark.h:47-64) draws
nonzero-degree roots deterministically."""

import numpy as np
import pytest

import oracle as orc
import radar_graph as rg


@pytest.mark.parametrize("scale,ef,seed,uniform", [(10, 16, 1, False), (12, 8, 5, True), (14, 16, 1, False),
                                                   (13, 32, 9, True)])
def test_oracle_generator_equals_library(scale, ef, seed, uniform):
    a = orc.generate_edges(scale, ef, seed, uniform)
    b = rg.generate_edges(scale, ef, seed, uniform)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    o1, a1 = orc.csr_from_edges(1 << scale, *a)
    o2, a2 = rg.csr_from_edges(1 << scale, *b)
    assert np.array_equal(o1, o2) and np.array_equal(a1, a2)


def test_oracle_csr_matches_the_loader_cleanup():
    """Both directions, sorted lists, repeats and self loops dropped."""
    src = np.array([0, 1, 1, 2, 3, 3], np.uint32)
    dst = np.array([1, 0, 2, 2, 0, 0], np.uint32)
    off, adj = orc.csr_from_edges(4, src, dst)
    assert off.tolist() == [0, 2, 4, 5, 6]
    assert adj.tolist() == [1, 3, 0, 2, 1, 0]
    with pytest.raises(ValueError):
        orc.csr_from_edges(2, np.array([0], np.uint32), np.array([5], np.uint32))


def test_source_picker_draws_nonzero_degree_roots():
    off, _ = orc.rmat_csr(12, 4, 3)
    deg = np.diff(off.astype(np.int64)).astype(np.uint32)
    r = orc.source_picker(deg, 64)
    assert (deg[r] > 0).all()
    assert np.array_equal(r, orc.source_picker(deg, 64))
    assert np.array_equal(r[:10], orc.source_picker(deg, 10))  # one generator, continued
