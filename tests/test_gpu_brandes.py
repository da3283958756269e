"""GPU parity of the Brandes betweenness sweep (tbfs_brandes) against the
oracle's restatement of the same summation order.

Bar: bit-exact (float64 compared with ==) on graphs whose out-lists are the
caller's CSC (symmetric graphs), in both vertex numberings, and on directed
graphs kept in the caller's numbering (the device transpose lists each
out-list by ascending column, as the oracle does); to 1e-12 relative on
directed graphs regrouped by degree, whose out-lists follow the new
numbering."""
import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from golden_data import FIXTURE_NAMES, load
from turbobfs_gb300 import graphs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_brandes_fixtures_bit_exact(gpu_available, name):
    fx = load(name)
    if not fx.symmetric:
        pytest.skip("directed fixture: covered by the tolerance test")
    rng = np.random.default_rng(1)
    roots = rng.integers(0, fx.n, min(fx.n, 24)).astype(np.int32)
    want, wovf = oracle.brandes(fx.col_ptr, fx.row_idx, roots)
    with tb.Graph(fx.col_ptr, fx.row_idx, fx.n, symmetric=True) as g:
        bc, ovf = g.betweenness(roots)
    assert ovf == wovf
    assert np.array_equal(bc, want)


@pytest.mark.parametrize("kind", ["er", "rmat12", "rmat16", "grid", "hub"])
def test_brandes_synthetic_bit_exact_both_numberings(gpu_available, kind):
    if kind == "er":
        h = graphs.erdos_renyi(20000, 80000, seed=3)
    elif kind == "hub":  # lists of 6000 and 12000 entries: segmented sums
        rng = np.random.default_rng(4)
        n = 20000
        src = np.concatenate([np.zeros(6000, np.int32), np.ones(12000, np.int32),
                              rng.integers(2, n, 40000, dtype=np.int32)])
        dst = np.concatenate([np.arange(2, 6002, dtype=np.int32),
                              np.arange(3000, 15000, dtype=np.int32),
                              rng.integers(2, n, 40000, dtype=np.int32)])
        h = graphs.from_edges(n, src, dst, symmetrize=True, dedup=True, drop_loops=True)
    elif kind == "rmat12":
        h = graphs.rmat(12, 16, seed=3)
    elif kind == "rmat16":
        h = graphs.rmat(16, 16, seed=3)  # hubs: the warp-summed path
    else:
        h = graphs.grid(60, seed=3)
    roots = graphs.pick_roots(h, 32, seed=2)
    want, _ = oracle.brandes(h.col_ptr, h.row_idx, roots)
    with tb.Graph.from_host_csc(h) as g, tb.Graph.from_host_csc(h, keep_order=True) as gk:
        bc, _ = g.betweenness(roots)
        bck, _ = gk.betweenness(roots)
    assert np.array_equal(bc, want)
    assert np.array_equal(bck, want)


def test_brandes_directed_to_rounding(gpu_available):
    rng = np.random.default_rng(9)
    n, m = 3000, 15000
    h = graphs.from_edges(n, rng.integers(0, n, m, dtype=np.int32),
                          rng.integers(0, n, m, dtype=np.int32))
    col = np.repeat(np.arange(n), np.diff(h.col_ptr)).astype(np.int32)
    order = np.lexsort((col, h.row_idx))
    orp = np.zeros(n + 1, np.int64)
    np.add.at(orp, h.row_idx.astype(np.int64) + 1, 1)
    orp = np.cumsum(orp).astype(np.int32)
    roots = rng.integers(0, n, 40).astype(np.int32)
    want, _ = oracle.brandes(orp, col[order], roots)
    with tb.Graph.from_host_csc(h) as g:
        bc, _ = g.betweenness(roots)
    np.testing.assert_allclose(bc, want, rtol=1e-12, atol=1e-9)
    # in the caller's numbering the device transpose lists each out-list by
    # ascending column, the oracle's order: the same sums, bit for bit
    with tb.Graph.from_host_csc(h, keep_order=True) as gk:
        bck, _ = gk.betweenness(roots)
    assert np.array_equal(bck, want)


def test_brandes_all_roots_small_and_invalid(gpu_available):
    h = graphs.rmat(9, 8, seed=6)
    want, _ = oracle.brandes(h.col_ptr, h.row_idx, np.arange(h.n, dtype=np.int32))
    with tb.Graph.from_host_csc(h) as g:
        bc, ovf = g.betweenness()
        assert ovf == 0 and np.array_equal(bc, want)
        with pytest.raises(tb.TbfsError):
            g.betweenness(np.array([h.n], dtype=np.int32))
        bc0, _ = g.betweenness(np.zeros(0, dtype=np.int32))
        assert not bc0.any()
