"""Single-source engine: results must not depend on the vertex numbering
(degree grouping vs the caller's order), on the path-count schedule
(pull_ratio), or on the direction thresholds (alpha, beta); the level trace
must describe the traversal that produced them."""
import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from turbobfs_gb300 import graphs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rmat16():
    h = graphs.rmat(16, 16, seed=11)
    return h, graphs.pick_roots(h, 6, seed=11)


def test_numbering_does_not_change_results(gpu_available, rmat16):
    h, roots = rmat16
    with tb.Graph.from_host_csc(h) as g, tb.Graph.from_host_csc(h, keep_order=True) as gk:
        for r in roots:
            for mode in ("auto", "td", "bu"):
                a, b = g.bfs(int(r), mode=mode), gk.bfs(int(r), mode=mode)
                assert np.array_equal(a.S, b.S) and np.array_equal(a.sigma, b.sigma)


@pytest.mark.parametrize("pull_ratio", [1e-6, 0.25, 4.0, 1e9])
def test_pull_ratio_extremes(gpu_available, rmat16, pull_ratio):
    h, roots = rmat16
    with tb.Graph.from_host_csc(h) as g:
        for r in roots[:3]:
            res = g.bfs(int(r), pull_ratio=pull_ratio)
            S, sg, ovf, _ = oracle.exact_bfs(h.col_ptr, h.row_idx, int(r))
            assert np.array_equal(res.S, S) and np.array_equal(res.sigma[ovf == 0], sg[ovf == 0])


@pytest.mark.parametrize("alpha,beta", [(0.5, 0.5), (1e6, 1e6), (2.0, 1e6), (1e6, 2.0)])
def test_direction_thresholds_do_not_change_results(gpu_available, rmat16, alpha, beta):
    h, roots = rmat16
    with tb.Graph.from_host_csc(h) as g:
        ref = g.bfs(int(roots[0]))
        res = g.bfs(int(roots[0]), alpha=alpha, beta=beta)
        assert np.array_equal(ref.S, res.S) and np.array_equal(ref.sigma, res.sigma)


def test_level_trace_matches_the_traversal(gpu_available, rmat16):
    h, roots = rmat16
    with tb.Graph.from_host_csc(h) as g:
        res = g.bfs(int(roots[0]), trace=64)
    tr = res.stats["trace"]
    assert len(tr) == res.stats["levels"]
    assert sum(r["vertices"] for r in tr) == res.stats["visited"]
    assert sum(r["edges"] for r in tr) == res.stats["edges"]
    assert [r["vertices"] for r in tr] == [int((res.S == d).sum()) for d in range(len(tr))]
    assert sum(r["direction"] == "bu" for r in tr) == res.stats["bu_levels"]
    starts = [r["start_us"] for r in tr]
    assert starts == sorted(starts) and res.stats["trace_end_us"] >= starts[-1]


def test_batch_trace_records_levels(gpu_available, rmat16):
    h, roots = rmat16
    with tb.Graph.from_host_csc(h) as g:
        S, sg, st = g.bfs_batch(roots, trace=64)
    tr = st[0]["trace"]
    assert len(tr) == max(s["levels"] for s in st)
    assert sum(r["direction"] == "td" for r in tr) == st[0]["td_levels"]
