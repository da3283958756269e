"""Degree profile on the device against the host restatement, and the
autotuner: candidates, cache round trip, results unchanged under tuned
parameters."""
import numpy as np
import pytest

import turbobfs_gb300 as tb
from turbobfs_gb300 import graphs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["rmat", "grid", "directed"])
def test_device_degree_profile_matches_host(gpu_available, kind):
    if kind == "rmat":
        h = graphs.rmat(14, 16, seed=1)
    elif kind == "grid":
        h = graphs.grid(100, seed=1)
    else:
        rng = np.random.default_rng(2)
        h = graphs.from_edges(5000, rng.integers(0, 5000, 30000, dtype=np.int32),
                              rng.integers(0, 5000, 30000, dtype=np.int32))
    want = graphs.degree_profile(h)
    with tb.Graph.from_host_csc(h) as g:
        got = g.degree_profile()
    assert np.array_equal(got["hist"], np.asarray(want["hist_log2"], dtype=np.int64))
    assert got["max"] == want["max"]
    assert abs(got["mean"] - want["mean"]) < 1e-12


def test_autotune_candidates_cache_and_results(gpu_available, tmp_path):
    h = graphs.rmat(15, 16, seed=3)
    roots = graphs.pick_roots(h, 3, seed=3)
    cache = str(tmp_path / "tune.txt")
    with tb.Graph.from_host_csc(h) as g:
        t1 = g.autotune(roots, cache=cache)
        assert not t1["from_cache"]
        assert t1["alpha"] in (4.0, 6.0, 9.0, 12.0, 15.0, 24.0, 60.0)
        assert t1["beta"] in (1.0, 2.0, 4.0, 18.0)
        assert t1["pull_ratio"] in (0.5, 1.0, 2.0, 4.0)
        assert t1["max_ept"] in (2, 4, 0) and t1["ctas_per_sm"] in (1, 2, 4, 0)
        t2 = g.autotune(roots, cache=cache)
        keys = ("alpha", "beta", "pull_ratio", "max_ept", "ctas_per_sm")
        assert t2["from_cache"] and all(t2[k] == t1[k] for k in keys)
        # the same family and scale shares the key
        with tb.Graph.from_host_csc(graphs.rmat(15, 16, seed=4)) as g2:
            assert g2.autotune(graphs.pick_roots(h, 1, seed=1), cache=cache)["from_cache"]
        base = g.bfs(int(roots[0]))
        tuned = g.bfs(int(roots[0]), **{k: t1[k] for k in keys})
        assert np.array_equal(base.S, tuned.S) and np.array_equal(base.sigma, tuned.sigma)


@pytest.mark.parametrize("max_ept", [1, 2, 4, 0])
@pytest.mark.parametrize("ctas_per_sm", [1, 2, 0])
def test_engine_shapes_exact(gpu_available, max_ept, ctas_per_sm):
    """Every engine shape the autotuner may pick gives the exact result, in
    every direction mode."""
    import oracle

    h = graphs.rmat(17, 16, seed=6)
    with tb.Graph.from_host_csc(h) as g:
        for r in graphs.pick_roots(h, 2, seed=6):
            S, sg, ovf, _ = oracle.exact_bfs(h.col_ptr, h.row_idx, int(r))
            for mode in ("auto", "td", "bu"):
                res = g.bfs(int(r), mode=mode, max_ept=max_ept, ctas_per_sm=ctas_per_sm)
                assert np.array_equal(res.S, S)
                assert np.array_equal(res.sigma[ovf == 0], sg[ovf == 0])


def test_autotune_batch(gpu_available, tmp_path):
    h = graphs.rmat(14, 16, seed=5)
    roots = graphs.pick_roots(h, 64, seed=5)
    cache = str(tmp_path / "tune.txt")
    with tb.Graph.from_host_csc(h) as g:
        t1 = g.autotune_batch(roots, cache=cache)
        assert not t1["from_cache"] and t1["alpha"] in (3.0, 5.0, 8.0, 15.0, 30.0)
        t2 = g.autotune_batch(roots, cache=cache)
        assert t2["from_cache"] and t2["alpha"] == t1["alpha"]
        S0, sg0, _ = g.bfs_batch(roots)
        S1, sg1, _ = g.bfs_batch(roots, alpha=t1["alpha"])
        assert np.array_equal(S0, S1) and np.array_equal(sg0, sg1)
