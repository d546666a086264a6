"""The checker-side workload generator (oracle/gen.c) against the product's
generator, byte for byte: the reference arm of bench.py builds its R-MAT graph
and sources through the oracle only, so both arms must time the same graph."""
import numpy as np
import pytest

import dfqbfs as d
import oracle


@pytest.mark.parametrize("scale,ef,seed", [(1, 1, 0), (4, 2, 9), (10, 16, 1), (12, 8, 5), (14, 32, 3), (16, 16, 2)])
def test_rmat_matches_product_generator(scale, ef, seed):
    off, cols = oracle.gen_rmat(scale, ef, seed=seed)
    g = d.gen_rmat(scale, ef, seed=seed)
    assert np.array_equal(off, g.offsets)
    assert np.array_equal(cols, g.cols)


def test_rmat_thread_count_does_not_change_the_graph():
    a = oracle.gen_rmat(15, 16, seed=4, threads=1)
    b = oracle.gen_rmat(15, 16, seed=4, threads=7)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_rmat_other_quadrant_probabilities():
    off, cols = oracle.gen_rmat(13, 8, a=0.45, b=0.15, c=0.15, seed=11)
    g = d.gen_rmat(13, 8, a=0.45, b=0.15, c=0.15, seed=11)
    assert np.array_equal(off, g.offsets) and np.array_equal(cols, g.cols)


@pytest.mark.parametrize("k", [0, 1, 64, 3000])
def test_pick_sources_matches_product(k):
    g = d.gen_rmat(11, 4, seed=6)  # some isolated vertices at this density
    assert (np.diff(g.offsets) == 0).any()
    got = oracle.pick_sources(g.offsets, k, seed=8)
    assert np.array_equal(got, g.pick_sources(k, seed=8))
    assert (np.diff(g.offsets)[got] > 0).all()


def test_pick_sources_rejects_a_graph_without_edges():
    with pytest.raises(ValueError):
        oracle.pick_sources(np.zeros(5, np.int32), 3, seed=1)
