"""Host graph tools (no GPU): determinism and structure of the generators,
the Matrix Market loader's CSC construction, components and root picks."""
import hashlib
import os
from pathlib import Path

import numpy as np
import pytest

from golden_data import REFERENCE_FIXTURES, load
from turbobfs_gb300 import graphs

# the reference tree (its graphData/ fixtures), where this machine has one
REF = Path(os.environ["TBFS_REFERENCE"]) if os.environ.get("TBFS_REFERENCE") else None


def _digest(g):
    h = hashlib.sha256()
    h.update(g.col_ptr.tobytes())
    h.update(g.row_idx.tobytes())
    return h.hexdigest()


def _is_symmetric_simple(g):
    n = g.n
    deg = g.degrees()
    col = np.repeat(np.arange(n, dtype=np.int64), deg)
    row = g.row_idx.astype(np.int64)
    fwd = np.sort(row * n + col)
    bwd = np.sort(col * n + row)
    no_loops = not (row == col).any()
    no_dups = fwd.shape[0] == np.unique(fwd).shape[0]
    return np.array_equal(fwd, bwd), no_loops, no_dups


def test_er_matches_golden_and_is_simple():
    g = graphs.erdos_renyi(4096, 16384, seed=1)
    fx = load("er4096")
    assert np.array_equal(g.col_ptr, fx.col_ptr) and np.array_equal(g.row_idx, fx.row_idx)
    assert g.nnz == 2 * 16384
    assert all(_is_symmetric_simple(g))


def test_generators_deterministic_and_thread_independent(monkeypatch):
    a = graphs.rmat(12, 16, seed=7)
    monkeypatch.setenv("TBFS_HOST_THREADS", "1")
    b = graphs.rmat(12, 16, seed=7)
    assert _digest(a) == _digest(b)
    c = graphs.rmat(12, 16, seed=8)
    assert _digest(a) != _digest(c)
    assert np.array_equal(load("rmat10").row_idx, graphs.rmat(10, 16, seed=2).row_idx)
    assert np.array_equal(load("grid32").row_idx, graphs.grid(32, seed=4).row_idx)


def test_rmat_structure():
    g = graphs.rmat(12, 16, seed=3)
    assert g.n == 4096
    sym, no_loops, no_dups = _is_symmetric_simple(g)
    assert sym and no_loops and no_dups
    assert g.nnz <= 2 * 16 * 4096
    deg = g.degrees()
    assert deg.max() > 20 * deg.mean()  # skewed degrees
    for i in range(g.n):  # columns sorted
        seg = g.row_idx[g.col_ptr[i]:g.col_ptr[i + 1]]
        assert (np.diff(seg) > 0).all()


def test_grid_structure():
    side = 64
    g = graphs.grid(side, delete_frac=0.10, chord_frac=0.01, max_dist=8, max_deg=6, seed=5)
    assert g.n == side * side
    sym, no_loops, no_dups = _is_symmetric_simple(g)
    assert sym and no_loops and no_dups
    assert g.degrees().max() <= 6
    grid_edges = 2 * side * (side - 1)
    kept = grid_edges - round(0.1 * grid_edges)
    chords = round(0.01 * kept)
    assert g.nnz == 2 * (kept + chords)
    col = np.repeat(np.arange(g.n), g.degrees())
    row = g.row_idx
    dist = np.abs(col % side - row % side) + np.abs(col // side - row // side)
    assert dist.max() <= 8 and (dist >= 1).all()
    assert ((dist >= 2).sum() // 2) == chords


def test_layered_bipartite():
    g = graphs.layered_bipartite(3, 4)
    assert g.n == 13 and g.nnz == 2 * (3 + 3 * 9)


def test_from_edges_flags():
    src = np.array([0, 1, 1, 2, 2], np.int32)
    dst = np.array([1, 2, 2, 2, 0], np.int32)
    raw = graphs.from_edges(3, src, dst)
    assert raw.col_ptr.tolist() == [0, 1, 2, 5]
    assert raw.row_idx.tolist() == [2, 0, 1, 1, 2]  # column 2 keeps input order
    dd = graphs.from_edges(3, src, dst, symmetrize=True, drop_loops=True, dedup=True)
    assert dd.col_ptr.tolist() == [0, 2, 4, 6]
    assert dd.row_idx.tolist() == [1, 2, 0, 2, 0, 1]
    with pytest.raises(Exception):
        graphs.from_edges(2, np.array([0], np.int32), np.array([5], np.int32))


def test_cooc_roundtrip():
    g = graphs.rmat(8, 8, seed=1)
    I, J = g.to_cooc()
    back = graphs.from_edges(g.n, I, J)
    assert np.array_equal(back.col_ptr, g.col_ptr) and np.array_equal(back.row_idx, g.row_idx)


def test_components_and_roots():
    g = graphs.rmat(12, 16, seed=3)
    mask = graphs.largest_component(g)
    roots = graphs.pick_roots(g, 64, seed=1)
    assert len(set(roots.tolist())) == 64
    assert mask[roots].all()
    assert np.array_equal(roots, graphs.pick_roots(g, 64, seed=1))
    prof = graphs.degree_profile(g)
    assert prof["hist_log2"].sum() == g.n and prof["max"] == g.degrees().max()


@pytest.mark.skipif(REF is None or not (REF / "graphData").is_dir(),
                    reason="TBFS_REFERENCE unset or without graphData/")
@pytest.mark.parametrize("name", REFERENCE_FIXTURES)
def test_mm_loader_matches_golden(name):
    fx = load(name)
    ug = 1 if "ug=1" in fx.meta["source"] else 0
    g = graphs.read_mm(REF / "graphData" / f"{name}.mtx", ug)
    assert np.array_equal(g.col_ptr, fx.col_ptr) and np.array_equal(g.row_idx, fx.row_idx)


def test_mm_loader_semantics(tmp_path):
    p = tmp_path / "t.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n% c\n3 3 3\n"
                 "1 1\n2 1\n3 2\n")
    g = graphs.read_mm(p, undirected=True)
    # diagonal (1,1) appears twice in column 0, as the reference's SSC->CSC does
    assert g.col_ptr.tolist() == [0, 3, 5, 6]
    assert sorted(g.row_idx[0:3].tolist()) == [0, 0, 1]
    d = graphs.read_mm(p, undirected=False)
    assert d.col_ptr.tolist() == [0, 2, 3, 3] and d.row_idx.tolist() == [0, 1, 2]
    bad = tmp_path / "bad.mtx"
    bad.write_text("not a matrix\n")
    with pytest.raises(Exception):
        graphs.read_mm(bad, True)
