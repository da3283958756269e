"""GPU parity of the frontier-matrix batch (tbfs_bfs_batch) against the
exact oracle, root by root.

Bar: bit-exact.  Every root's S and sigma must equal the oracle's exact
restatement on every vertex (sigma where it fits int64), and each root's
overflow flag must equal the oracle's, in every mode, layout and row width
(W = 1, 2, 4, 8 words for up to 32, 64, 128, 256 roots per launch)."""
import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from golden_data import FIXTURE_NAMES, bfs_invariants, load
from turbobfs_gb300 import graphs

pytestmark = pytest.mark.gpu
MODES = ["auto", "td", "bu"]


def _check_roots(cp, ic, roots, S, sg, stats, want_sigma=True, layout="root"):
    if layout == "vertex":
        S = S.T
        sg = sg.T if sg is not None else None
    deg_out = None
    for i, r in enumerate(roots):
        eS, esg, ovf, levels = oracle.exact_bfs(cp, ic, int(r))
        assert np.array_equal(S[i], eS), f"S differs for root index {i} (vertex {r})"
        assert stats[i]["levels"] == levels
        assert stats[i]["visited"] == int((eS >= 0).sum())
        if want_sigma:
            ok = ovf == 0
            assert np.array_equal(sg[i][ok], esg[ok]), f"sigma differs for root index {i}"
            assert stats[i]["sigma_overflow"] == int(ovf.any())
    return deg_out


def _roots(h, k, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, h.n, k).astype(np.int32)


@pytest.mark.parametrize("name", FIXTURE_NAMES)
@pytest.mark.parametrize("mode", MODES)
def test_batch_fixtures(gpu_available, name, mode):
    fx = load(name)
    rng = np.random.default_rng(3)
    roots = np.concatenate([np.asarray(fx.roots, dtype=np.int32),
                            rng.integers(0, fx.n, 40).astype(np.int32)])
    with tb.Graph(fx.col_ptr, fx.row_idx, fx.n, symmetric=fx.symmetric) as g:
        S, sg, st = g.bfs_batch(roots, mode=mode)
        _check_roots(fx.col_ptr, fx.row_idx, roots, S, sg, st)


@pytest.mark.parametrize("k", [1, 5, 32, 33, 64, 100, 256])
@pytest.mark.parametrize("kind", ["er", "rmat", "grid"])
def test_batch_widths_synthetic(gpu_available, kind, k):
    if kind == "er":
        h = graphs.erdos_renyi(30000, 120000, seed=4)
    elif kind == "rmat":
        h = graphs.rmat(15, 16, seed=4)
    else:
        h = graphs.grid(120, seed=4)
    roots = _roots(h, k, seed=k)
    with tb.Graph.from_host_csc(h) as g:
        for mode in MODES:
            S, sg, st = g.bfs_batch(roots, mode=mode)
            _check_roots(h.col_ptr, h.row_idx, roots, S, sg, st)


def test_batch_matches_bfs_many_rmat16(gpu_available):
    h = graphs.rmat(16, 16, seed=2)
    roots = graphs.pick_roots(h, 256, seed=2)
    with tb.Graph.from_host_csc(h) as g:
        S, sg, st = g.bfs_batch(roots)
        S1, sg1, st1 = g.bfs_many(roots)
        assert np.array_equal(S, S1) and np.array_equal(sg, sg1)
        for a, b in zip(st, st1):
            assert (a["levels"], a["visited"], a["edges"], a["sigma_overflow"]) == \
                   (b["levels"], b["visited"], b["edges"], b["sigma_overflow"])


def test_batch_more_than_256_roots_and_duplicates(gpu_available):
    h = graphs.rmat(13, 8, seed=7)
    roots = _roots(h, 300, seed=1)
    roots[10] = roots[11] = roots[290]  # the same vertex in both launches
    with tb.Graph.from_host_csc(h) as g:
        S, sg, st = g.bfs_batch(roots)
        _check_roots(h.col_ptr, h.row_idx, roots, S, sg, st)
        Sv, sgv, stv = g.bfs_batch(roots, layout="vertex")
        assert np.array_equal(Sv.T, S) and np.array_equal(sgv.T, sg)


def test_batch_depths_only_and_keep_order(gpu_available):
    h = graphs.rmat(14, 16, seed=5)
    roots = _roots(h, 77, seed=5)
    with tb.Graph.from_host_csc(h) as g, tb.Graph.from_host_csc(h, keep_order=True) as gk:
        S, sg, st = g.bfs_batch(roots, sigma=False)
        assert sg is None
        _check_roots(h.col_ptr, h.row_idx, roots, S, None, st, want_sigma=False)
        S2, sg2, _ = gk.bfs_batch(roots)
        S3, sg3, _ = g.bfs_batch(roots)
        assert np.array_equal(S2, S) and np.array_equal(S3, S) and np.array_equal(sg2, sg3)


def test_batch_directed_general_graph(gpu_available):
    rng = np.random.default_rng(8)
    n, m = 20000, 90000
    src = rng.integers(0, n, m, dtype=np.int32)
    dst = rng.integers(0, n, m, dtype=np.int32)
    h = graphs.from_edges(n, src, dst)  # directed, with duplicates and self-loops
    roots = _roots(h, 70, seed=8)
    with tb.Graph.from_host_csc(h) as g:
        for mode in MODES:
            S, sg, st = g.bfs_batch(roots, mode=mode)
            _check_roots(h.col_ptr, h.row_idx, roots, S, sg, st)


def test_batch_hub_segments(gpu_available):
    """Two hubs far above the segment length (256 W entries): their lists are
    split across groups and combined by the last segment."""
    rng = np.random.default_rng(9)
    n = 40000
    hub_a, hub_b = 0, 1
    leaves = np.arange(2, n, dtype=np.int32)
    src = np.concatenate([np.full(leaves.size, hub_a, np.int32), leaves[: n // 2],
                          rng.integers(2, n, 60000).astype(np.int32)])
    dst = np.concatenate([leaves, np.full(n // 2, hub_b, np.int32)[: leaves[: n // 2].size],
                          rng.integers(2, n, 60000).astype(np.int32)])
    h = graphs.from_edges(n, src, dst, symmetrize=True)
    with tb.Graph.from_host_csc(h) as g:
        for k in (20, 200):
            roots = _roots(h, k, seed=k)
            for mode in MODES:
                S, sg, st = g.bfs_batch(roots, mode=mode)
                _check_roots(h.col_ptr, h.row_idx, roots, S, sg, st)


def test_batch_overflow_flags_per_root(gpu_available):
    """Root 0 of the 17-layer 16-wide layered graph sees 16^16 = 2^64 paths
    (overflow); roots one layer further in see 2^60 (no overflow)."""
    h = graphs.layered_bipartite(16, 17)
    roots = np.array([0, 1, 20, 21, 0, 40], dtype=np.int32)
    with tb.Graph.from_host_csc(h) as g:
        for mode in MODES:
            S, sg, st = g.bfs_batch(roots, mode=mode)
            _check_roots(h.col_ptr, h.row_idx, roots, S, sg, st)
            flags = [s["sigma_overflow"] for s in st]
            assert flags[0] == 1 and flags[4] == 1


@pytest.mark.parametrize("width,layers", [(16, 9), (16, 10), (16, 12), (300, 4), (300, 6)])
def test_batch_counts_past_32_bits(gpu_available, width, layers):
    """Launches first keep path counts in 32 bits and are redone with 64-bit
    counts when one needs more.  Layered graphs (counts up to
    width^(layers-1)): 16-wide with 2^32, 2^36 and 2^44 paths (redone);
    300-wide (in-lists of 300-600 entries, split into segments at 20 roots)
    with 2.7e7 paths (kept in 32 bits) and 2.4e12 (redone).  Exact counts,
    no overflow flag, in every mode."""
    h = graphs.layered_bipartite(width, layers)
    roots = np.arange(0, min(h.n, 20 * 7), 7, dtype=np.int32)[:20]
    with tb.Graph.from_host_csc(h) as g:
        for mode in MODES:
            S, sg, st = g.bfs_batch(roots, mode=mode)
            _check_roots(h.col_ptr, h.row_idx, roots, S, sg, st)
            assert not any(x["sigma_overflow"] for x in st)


def test_batch_device_outputs(gpu_available):
    torch = pytest.importorskip("torch")
    import ctypes

    from turbobfs_gb300 import _lib
    from turbobfs_gb300.api import _P_I32, make_options

    h = graphs.rmat(13, 16, seed=3)
    roots = _roots(h, 90, seed=3)
    with tb.Graph.from_host_csc(h) as g:
        Sd = torch.empty((90, h.n), dtype=torch.int32, device="cuda")
        sgd = torch.empty((90, h.n), dtype=torch.int64, device="cuda")
        o = make_options("auto", True, outputs_on_device=True)
        st = (_lib.Stats * 90)()
        _lib.check(tb.lib().tbfs_bfs_batch(g.handle, roots.ctypes.data_as(_P_I32), 90,
                                           ctypes.byref(o), 0, Sd.data_ptr(), sgd.data_ptr(),
                                           st), "tbfs_bfs_batch")
        torch.cuda.synchronize()
        S, sg, _ = g.bfs_batch(roots)
        assert np.array_equal(Sd.cpu().numpy(), S) and np.array_equal(sgd.cpu().numpy(), sg)


def test_batch_invalid_arguments(gpu_available):
    h = graphs.rmat(10, 8, seed=1)
    with tb.Graph.from_host_csc(h) as g:
        with pytest.raises(tb.TbfsError):
            g.bfs_batch(np.array([0, h.n], dtype=np.int32))
        with pytest.raises(tb.TbfsError):
            g.bfs_batch(np.array([-1], dtype=np.int32))
        S, sg, st = g.bfs_batch(np.zeros(0, dtype=np.int32))
        assert S.shape == (0, h.n) and st == []


def test_batch_rmat20_256_roots_invariants(gpu_available):
    """The C4 workload at full size: RMAT scale 20, 256 roots in one launch;
    size-independent invariants for every root, exact oracle for a sample."""
    h = graphs.rmat(20, 16, seed=1)
    roots = graphs.pick_roots(h, 256, seed=1)
    with tb.Graph.from_host_csc(h) as g:
        S, sg, st = g.bfs_batch(roots)
        for i in range(0, 256, 37):
            bfs_invariants(h.col_ptr, h.row_idx, int(roots[i]), S[i], sg[i])
        sample = roots[::64]
        _check_roots(h.col_ptr, h.row_idx, sample, S[::64], sg[::64], st[::64])
