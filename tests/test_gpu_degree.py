"""Degree statistics on the device (tbfs_graph_degree_stats) against the
restatement of the reference's degree.c (oracle_degree_stats, pinned to the
reference's own code in test_degree_oracle.py): maximum, first vertex of
maximum degree in the caller's numbering, mean, accumulated log2
distribution and its percentages bit for bit; the standard deviation, summed
in degree order on the device side and in vertex order by the reference,
within a relative 1e-12."""
import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from golden_data import FIXTURE_NAMES, load
from turbobfs_gb300 import graphs

pytestmark = pytest.mark.gpu


def _check(g, cp, ic, symmetric):
    din, dout, und = oracle.degree_vectors(cp, ic, symmetric)
    for kind, deg in (("in", din), ("out", dout), ("undirected", und)):
        got = g.degree_stats(kind, full=True)
        want = oracle.degree_stats(deg)
        nb = len(got["dist_ac"])
        assert got["max"] == want["max"] and got["argmax"] == want["argmax"], kind
        assert got["sum"] == int(deg.astype(np.int64).sum())
        assert got["mean"] == want["mean"]
        assert got["sd"] == pytest.approx(want["sd"], rel=1e-12)
        assert np.array_equal(got["dist_ac"], want["dist_ac"][:nb]), kind
        assert np.array_equal(got["dist_rel_ac"], want["dist_rel_ac"][:nb]), kind
        assert (want["dist_ac"][nb:] == 0).all()
        assert np.array_equal(got["dist"], np.bincount(deg, minlength=want["max"] + 1))


@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_fixtures(gpu_available, name):
    fx = load(name)
    with tb.Graph(fx.col_ptr, fx.row_idx, symmetric=fx.symmetric) as g:
        _check(g, fx.col_ptr, fx.row_idx, fx.symmetric)


@pytest.mark.parametrize("keep_order", [False, True])
def test_rmat_regrouped_numbering(gpu_available, keep_order):
    """RMAT-16 is stored regrouped by degree unless keep_order: the first
    vertex of maximum degree must still be the caller's."""
    h = graphs.rmat(16, 16, seed=3)
    with tb.Graph.from_host_csc(h, keep_order=keep_order) as g:
        _check(g, h.col_ptr, h.row_idx, True)


def test_directed_and_ties(gpu_available):
    rng = np.random.default_rng(11)
    n = 50000
    src = rng.integers(0, n, 400000).astype(np.int32)
    dst = (rng.zipf(1.6, 400000) % n).astype(np.int32)
    h = graphs.from_edges(n, src, dst)
    with tb.Graph.from_host_csc(h) as g:
        _check(g, h.col_ptr, h.row_idx, False)
    # several vertices share a maximum that is a power of two; isolated vertices
    cp = np.array([0, 4, 4, 8, 9, 13, 13], np.int32)
    ic = np.array([1, 2, 3, 4, 0, 1, 3, 5, 0, 0, 1, 2, 3], np.int32)
    with tb.Graph(cp, ic) as g:
        _check(g, cp, ic, False)
