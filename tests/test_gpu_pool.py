"""Device memory pool (devmem.cu) and the per-call caches of tbfs_bfs_many.

Bar: graphs built, traversed and destroyed over and over from reused pool
memory give the oracle's results; with TBFS_POOL_POISON set every fresh
allocation holds 0xA5 bytes, so a buffer the library forgot to initialise
shows up as a wrong depth or count; tbfs_bfs_many's control blocks and
events grow with k and are reused by later calls on the same graph."""
import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from turbobfs_gb300 import graphs

pytestmark = pytest.mark.gpu


def _check(h, S_got, sg_got, root):
    S, sg, ovf, _ = oracle.exact_bfs(h.col_ptr, h.row_idx, int(root))
    assert np.array_equal(S_got, S)
    assert np.array_equal(sg_got[ovf == 0], sg[ovf == 0])


@pytest.mark.parametrize("poison", [False, True])
def test_rebuilt_graphs_from_reused_memory(gpu_available, monkeypatch, poison):
    if poison:
        monkeypatch.setenv("TBFS_POOL_POISON", "1")
    cases = [graphs.rmat(12, 16, seed=3), graphs.grid(64, seed=2), graphs.rmat(14, 8, seed=4),
             graphs.erdos_renyi(3000, 12000, seed=5)]
    for rep in range(2):
        for i, h in enumerate(cases):
            roots = graphs.pick_roots(h, 3, seed=i + 1)
            keep = bool((i + rep) & 1)
            with tb.Graph.from_host_csc(h, keep_order=keep) as g:
                for mode in ("auto", "td", "bu"):
                    res = g.bfs(int(roots[0]), mode=mode)
                    _check(h, res.S, res.sigma, roots[0])
                S, sg, _ = g.bfs_many(roots)
                for j, r in enumerate(roots):
                    _check(h, S[j], sg[j], r)
        if rep == 0:
            tb.release_cached_memory()


def test_poisoned_directed_and_cooc_graphs(gpu_available, monkeypatch):
    monkeypatch.setenv("TBFS_POOL_POISON", "1")
    rng = np.random.default_rng(9)
    n, m = 2000, 9000
    I = rng.integers(0, n, m, dtype=np.int32)
    J = rng.integers(0, n, m, dtype=np.int32)
    h = graphs.from_edges(n, I, J)  # directed: column J[k] gets row I[k]
    with tb.Graph.from_cooc(I, J, n) as g:
        for root in (0, 7, 1999):
            res = g.bfs(root)
            S, sg, ovf, _ = oracle.exact_bfs(h.col_ptr, h.row_idx, root)
            assert np.array_equal(res.S, S) and np.array_equal(res.sigma[ovf == 0], sg[ovf == 0])


def test_bfs_many_caches_grow_and_are_reused(gpu_available):
    h = graphs.rmat(13, 16, seed=8)
    roots = graphs.pick_roots(h, 9, seed=8)
    with tb.Graph.from_host_csc(h) as g:
        for k in (2, 9, 1, 5):
            S, sg, stats = g.bfs_many(roots[:k])
            assert len(stats) == k and all(st["levels"] > 0 for st in stats)
            for j, r in enumerate(roots[:k]):
                _check(h, S[j], sg[j], r)


def test_poisoned_batch_brandes_and_server(gpu_available, monkeypatch):
    """Fresh blocks hold 0xA5 bytes: the frontier-matrix batch, the betweenness
    sweep and the server still give the results of the plain path and the
    oracle."""
    monkeypatch.setenv("TBFS_POOL_POISON", "1")
    h = graphs.rmat(12, 16, seed=21)
    roots = graphs.pick_roots(h, 40, seed=21)
    with tb.Graph.from_host_csc(h) as g:
        S, sg, _ = g.bfs_batch(roots)
        Sm, sgm, _ = g.bfs_many(roots)
        assert np.array_equal(S, Sm) and np.array_equal(sg, sgm)
        bc, _ = g.betweenness(roots[:6])
        want, _ = oracle.brandes(h.col_ptr, h.row_idx, roots[:6])
        assert np.array_equal(bc, want)
        with tb.Server(max_slots=8, mem_budget=64 << 20) as srv:
            tickets = [srv.submit(g, int(r)) for r in roots[:12]]
            for t, j in zip(tickets, range(12)):
                res, _ = srv.wait(t)
                assert np.array_equal(res.S, Sm[j]) and np.array_equal(res.sigma, sgm[j])
