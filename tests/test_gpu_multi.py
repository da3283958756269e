"""GPU parity of the multi-instance engine: packed arenas of many graphs
(tbfs_arena_*) and the serving loop (tbfs_server_*).

Bar: bit-exact.  Every traversal's S and sigma must equal the exact oracle
(arena) or the single traversal tbfs_bfs of the same (graph, root) run
alone (server: "the same alone and in the mix"), whatever else shares the
launch, the memory budget or the admission order."""
import threading

import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from turbobfs_gb300 import graphs

pytestmark = pytest.mark.gpu


def _mixed_graphs(count, seed, lo=6, hi=12):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        kind = i % 3
        scale = int(rng.integers(lo, hi + 1))
        if kind == 0:
            n = 1 << scale
            out.append(graphs.erdos_renyi(n, 4 * n, seed=seed + i))
        elif kind == 1:
            out.append(graphs.rmat(scale, 8, seed=seed + i))
        else:
            out.append(graphs.grid(max(2, int(2 ** (scale / 2))), seed=seed + i))
    return out


def _check_exact(h, r, S, sg, st):
    eS, esg, ovf, levels = oracle.exact_bfs(h.col_ptr, h.row_idx, int(r))
    assert np.array_equal(S, eS)
    ok = ovf == 0
    if sg is not None:
        assert np.array_equal(sg[ok], esg[ok])
        assert st["sigma_overflow"] == int(ovf.any())
    assert st["levels"] == levels
    assert st["visited"] == int((eS >= 0).sum())


def test_arena_mixed_graphs_vs_exact(gpu_available):
    gs = _mixed_graphs(60, seed=3)
    rng = np.random.default_rng(4)
    roots = np.array([int(rng.integers(0, g.n)) for g in gs], dtype=np.int32)
    with tb.Arena(gs) as a:
        S, sg, st = a.bfs(roots)
        for i, (Si, sgi) in enumerate(zip(a.split(S), a.split(sg))):
            _check_exact(gs[i], roots[i], Si, sgi, st[i])
        S2, sg2, _ = a.bfs(roots, sigma=False)
        assert sg2 is None and np.array_equal(S2, S)


def test_arena_directed_and_many_launches(gpu_available):
    """1100 graphs (two launches of up to 1024), directed with duplicate
    entries and self-loops, so out-lists are built for the pushes."""
    rng = np.random.default_rng(7)
    gs = []
    for i in range(1100):
        n = int(rng.integers(1, 200))
        m = int(rng.integers(0, 4 * n + 1))
        gs.append(graphs.from_edges(n, rng.integers(0, n, m, dtype=np.int32),
                                    rng.integers(0, n, m, dtype=np.int32)))
    roots = np.array([int(rng.integers(0, g.n)) for g in gs], dtype=np.int32)
    with tb.Arena(gs, symmetric=False) as a:
        S, sg, st = a.bfs(roots)
        for i, (Si, sgi) in enumerate(zip(a.split(S), a.split(sg))):
            _check_exact(gs[i], roots[i], Si, sgi, st[i])


def test_arena_short_and_long_lists_in_one_launch(gpu_available):
    """Deep low-degree instances share launches with shallow hub-heavy ones:
    a grid, a 2 x 4000 ladder (4000 levels), directed graphs with
    out-degrees up to 16 and with one of 17, and an RMAT graph; every one
    equals the exact oracle."""
    rng = np.random.default_rng(12)

    def outdeg_graph(n, max_out, hub):
        deg = rng.integers(0, max_out + 1, n)
        if hub:
            deg[1] = hub
        src = np.repeat(np.arange(n, dtype=np.int32), deg)
        return graphs.from_edges(n, src, rng.integers(0, n, src.size, dtype=np.int32))

    n2 = 4000
    a_ = np.arange(n2 - 1, dtype=np.int32)
    lad = graphs.from_edges(2 * n2, np.concatenate([a_, a_ + n2, np.arange(n2, dtype=np.int32)]),
                            np.concatenate([a_ + 1, a_ + 1 + n2, np.arange(n2, dtype=np.int32) + n2]),
                            symmetrize=True)
    gs = [graphs.grid(150, seed=5), lad, outdeg_graph(20000, 16, 0), outdeg_graph(20000, 16, 17),
          graphs.rmat(12, 16, seed=5)]
    roots = np.array([7, 0, 3, 1, 11], dtype=np.int32)
    with tb.Arena(gs, symmetric=False) as a:
        S, sg, st = a.bfs(roots)
        for i, (Si, sgi) in enumerate(zip(a.split(S), a.split(sg))):
            _check_exact(gs[i], roots[i], Si, sgi, st[i])


def test_arena_overflow_flag(gpu_available):
    gs = [graphs.layered_bipartite(16, 17), graphs.layered_bipartite(16, 16), graphs.rmat(8, 8, seed=1)]
    with tb.Arena(gs) as a:
        S, sg, st = a.bfs(np.zeros(3, dtype=np.int32))
        assert [s["sigma_overflow"] for s in st] == [1, 0, 0]
        for i, (Si, sgi) in enumerate(zip(a.split(S), a.split(sg))):
            _check_exact(gs[i], 0, Si, sgi, st[i])


def test_arena_invalid_input(gpu_available):
    bad = graphs.HostCSC(3, np.array([0, 2, 1, 3], np.int32), np.array([1, 2, 0], np.int32), True)
    with pytest.raises(tb.TbfsError):
        tb.Arena([graphs.rmat(6, 4, seed=1), bad])
    with tb.Arena([graphs.rmat(6, 4, seed=1)]) as a:
        with pytest.raises(tb.TbfsError):
            a.bfs(np.array([1 << 20], dtype=np.int32))


@pytest.fixture(scope="module")
def served_graphs():
    rng = np.random.default_rng(11)
    src = rng.integers(0, 5000, 20000, dtype=np.int32)
    dst = rng.integers(0, 5000, 20000, dtype=np.int32)
    hs = [graphs.rmat(14, 16, seed=1), graphs.rmat(12, 16, seed=2), graphs.grid(150, seed=3),
          graphs.erdos_renyi(20000, 80000, seed=4), graphs.from_edges(5000, src, dst),
          graphs.layered_bipartite(16, 17)]
    gs = [tb.Graph.from_host_csc(h) for h in hs]
    yield hs, gs
    for g in gs:
        g.close()


def _queries(hs, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        gi = int(rng.integers(0, len(hs)))
        out.append((gi, int(rng.integers(0, hs[gi].n))))
    return out


def test_server_results_equal_alone(gpu_available, served_graphs):
    """Results of queries that shared launches with others (in the mix) equal
    the same queries run alone: the launches must actually have carried more
    than one query each on average."""
    hs, gs = served_graphs
    qs = _queries(hs, 120, seed=1)
    with tb.Server(max_slots=64, mem_budget=1 << 30) as srv:
        tickets = [srv.submit(gs[gi], r) for gi, r in qs]
        results = [srv.wait(t) for t in tickets]
        c = srv.counters()
        split = srv.time_split()
        assert c["completed"] == len(qs) and c["launches"] >= 1
        assert split["slot_sum"] / c["launches"] > 1.0, (split, c)
    for (gi, r), (res, lat) in zip(qs, results):
        alone = gs[gi].bfs(r)
        assert np.array_equal(res.S, alone.S), (gi, r)
        assert np.array_equal(res.sigma, alone.sigma), (gi, r)
        assert res.stats["levels"] == alone.stats["levels"]
        assert res.stats["visited"] == alone.stats["visited"]
        assert res.stats["sigma_overflow"] == alone.stats["sigma_overflow"]
        assert lat > 0.0


def test_server_tight_memory_and_threads(gpu_available, served_graphs):
    """A budget that holds only a few queries at a time: the rest wait for
    memory; four host threads submit concurrently; depths-only queries mix
    with path-count queries."""
    hs, gs = served_graphs
    qs = _queries(hs, 80, seed=2)
    need = max(48 * h.n for h in hs)
    out = [None] * len(qs)
    with tb.Server(max_slots=8, mem_budget=3 * need) as srv:
        def worker(idx):
            for i in idx:
                gi, r = qs[i]
                t = srv.submit(gs[gi], r, sigma=(i % 3 != 0))
                out[i] = srv.wait(t)
        ths = [threading.Thread(target=worker, args=(range(k, len(qs), 4),)) for k in range(4)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
    for i, ((gi, r), (res, _)) in enumerate(zip(qs, out)):
        alone = gs[gi].bfs(r, sigma=(i % 3 != 0))
        assert np.array_equal(res.S, alone.S)
        if i % 3 != 0:
            assert np.array_equal(res.sigma, alone.sigma)
        else:
            assert res.sigma is None


def test_server_burst_waited_in_reverse(gpu_available, served_graphs):
    """A burst larger than the memory budget, waited for newest first: the
    delivery of finished queries frees their memory without any waiter, so
    the queued ones are admitted and nothing deadlocks."""
    hs, gs = served_graphs
    qs = _queries(hs, 40, seed=3)
    need = max(48 * h.n for h in hs)
    with tb.Server(max_slots=4, mem_budget=2 * need) as srv:
        tickets = [srv.submit(gs[gi], r) for gi, r in qs]
        results = {t: srv.wait(t) for t in reversed(tickets)}
        assert srv.counters()["completed"] == len(qs)
    for (gi, r), t in zip(qs, tickets):
        res, _ = results[t]
        alone = gs[gi].bfs(r)
        assert np.array_equal(res.S, alone.S) and np.array_equal(res.sigma, alone.sigma)


def test_server_rejects_and_oversized(gpu_available, served_graphs):
    hs, gs = served_graphs
    with tb.Server(max_slots=2, mem_budget=256 << 10) as srv:
        with pytest.raises(tb.TbfsError):
            srv.submit(gs[0], -1)
        t = srv.submit(gs[0], 0)  # needs 786 KB, more than the whole pool: fails, does not hang
        with pytest.raises(tb.TbfsError):
            srv.wait(t)
        t2 = srv.submit(gs[4], 0, sigma=False)  # 5000 vertices, depths only: 160 KB, fits
        res, _ = srv.wait(t2)
        assert np.array_equal(res.S, gs[4].bfs(0, sigma=False).S)


def test_server_routes_large_shallow_and_deep_graphs(gpu_available):
    """RMAT scale 18 (2^18 vertices, ~6 levels) goes to the single-source
    route; a 600x600 grid starts there (depth unknown) and moves to the
    shared launches once its depth (over 48 levels) is known; small graphs
    always share them.  Every result equals the query run alone."""
    hs = [graphs.rmat(18, 16, seed=5), graphs.grid(600, seed=6), graphs.rmat(10, 16, seed=7)]
    gs = [tb.Graph.from_host_csc(h) for h in hs]
    try:
        qs = [(i % 3, int(graphs.pick_roots(hs[i % 3], 1, seed=i)[0])) for i in range(18)]
        with tb.Server(max_slots=16, mem_budget=2 << 30) as srv:
            first = srv.wait(srv.submit(gs[1], qs[1][1]))  # learns the grid's depth
            tickets = [srv.submit(gs[gi], r) for gi, r in qs]
            results = [srv.wait(t) for t in tickets]
            split, c = srv.time_split(), srv.counters()
        assert first[0].stats["levels"] > 48
        # the first grid query and the six scale-18 ones take the single-source route
        assert split["plain_runs"] >= 7 and split["launch_ms"] > 0 and split["deliver_ms"] > 0
        assert split["slot_sum"] >= c["launches"] >= 1
        for (gi, r), (res, _) in zip(qs, results):
            alone = gs[gi].bfs(r)
            assert np.array_equal(res.S, alone.S) and np.array_equal(res.sigma, alone.sigma)
            assert res.stats["visited"] == alone.stats["visited"]
    finally:
        for g in gs:
            g.close()
