"""The Brandes restatement in oracle/ pinned against an independent
implementation (networkx, unnormalised betweenness), and its summation
order checked on its own terms.  CPU only."""
import numpy as np
import pytest

import oracle
from turbobfs_gb300 import graphs


def _nx_graph(h, directed):
    nx = pytest.importorskip("networkx")
    G = nx.DiGraph() if directed else nx.Graph()
    G.add_nodes_from(range(h.n))
    col = np.repeat(np.arange(h.n), np.diff(h.col_ptr))
    G.add_edges_from(zip(h.row_idx.tolist(), col.tolist()))  # entry u -> v
    return nx, G


@pytest.mark.parametrize("kind", ["er", "rmat", "grid"])
def test_oracle_brandes_matches_networkx_undirected(kind):
    if kind == "er":
        h = graphs.erdos_renyi(300, 900, seed=2)
    elif kind == "rmat":
        h = graphs.rmat(8, 8, seed=3)
    else:
        h = graphs.grid(14, seed=4)
    nx, G = _nx_graph(h, directed=False)
    roots = np.arange(h.n, dtype=np.int32)
    bc, ovf = oracle.brandes(h.col_ptr, h.row_idx, roots)
    ref = nx.betweenness_centrality(G, normalized=False)
    want = np.array([ref[v] for v in range(h.n)])
    assert ovf == 0
    # every unordered pair is counted from both ends here, once in networkx
    np.testing.assert_allclose(bc / 2.0, want, rtol=1e-9, atol=1e-9)


def test_oracle_brandes_matches_networkx_directed():
    rng = np.random.default_rng(5)
    n, m = 200, 700
    h = graphs.from_edges(n, rng.integers(0, n, m, dtype=np.int32),
                          rng.integers(0, n, m, dtype=np.int32), dedup=True, drop_loops=True)
    nx, G = _nx_graph(h, directed=True)
    # out-lists of the CSC (in-lists): the transpose, sorted by source
    col = np.repeat(np.arange(n), np.diff(h.col_ptr)).astype(np.int32)
    order = np.lexsort((col, h.row_idx))
    orp = np.zeros(n + 1, np.int64)
    np.add.at(orp, h.row_idx.astype(np.int64) + 1, 1)
    orp = np.cumsum(orp).astype(np.int32)
    ojr = col[order]
    bc, _ = oracle.brandes(orp, ojr, np.arange(n, dtype=np.int32))
    ref = nx.betweenness_centrality(G, normalized=False)
    np.testing.assert_allclose(bc, [ref[v] for v in range(n)], rtol=1e-9, atol=1e-9)


def test_oracle_brandes_subset_of_roots_and_star():
    # star: the centre lies on every leaf-to-leaf path
    n = 50
    src = np.concatenate([np.zeros(n - 1, np.int32), np.arange(1, n, dtype=np.int32)])
    dst = np.concatenate([np.arange(1, n, dtype=np.int32), np.zeros(n - 1, np.int32)])
    h = graphs.from_edges(n, src, dst, sort=True)
    bc, _ = oracle.brandes(h.col_ptr, h.row_idx, np.array([1, 2, 3], np.int32))
    # from each leaf root, the centre carries the 48 other leaves
    assert bc[0] == 3 * (n - 2)
    assert np.all(bc[1:] == 0)


def test_oracle_brandes_hub_segments_match_networkx():
    # a hub of out-degree 6000 (three segments of the summation order) on
    # top of a sparse random graph
    rng = np.random.default_rng(8)
    n = 6500
    src = np.concatenate([np.zeros(6000, np.int32), rng.integers(1, n, 9000, dtype=np.int32)])
    dst = np.concatenate([np.arange(1, 6001, dtype=np.int32), rng.integers(1, n, 9000, dtype=np.int32)])
    h = graphs.from_edges(n, src, dst, symmetrize=True, dedup=True, drop_loops=True)
    assert np.diff(h.col_ptr).max() > 2 * 2048
    nx, G = _nx_graph(h, directed=False)
    roots = np.arange(0, n, 97, dtype=np.int32)
    bc, _ = oracle.brandes(h.col_ptr, h.row_idx, roots)
    ref = nx.betweenness_centrality_subset(G, sources=roots.tolist(), targets=list(range(n)),
                                           normalized=False)
    # subset betweenness counts each (source, target) pair once, halved for
    # undirected graphs; the sweep counts it once per source
    np.testing.assert_allclose(bc, 2.0 * np.array([ref[v] for v in range(n)]), rtol=1e-9, atol=1e-7)
