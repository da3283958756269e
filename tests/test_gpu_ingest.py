"""Graphs built on the device (tbfs_graph_create_edges / _create_mm /
_load_mm) against the host builders they replace.

Bar: the device-built CSC equals the host builder's col_ptr / row_idx
element for element (graphs kept in the caller's numbering), for every
construction flag; Matrix Market text parsed on the device gives the host
reader's graph; malformed text fails with TBFS_ERR_IO; COOC ingest and the
transposed out-lists keep a fixed entry order."""
import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from turbobfs_gb300 import graphs
from turbobfs_gb300._lib import (BUILD_DEDUP, BUILD_DROP_LOOPS, BUILD_SORT, BUILD_SYMMETRIZE,
                                 TbfsError)

pytestmark = pytest.mark.gpu

FLAG_SETS = [0, BUILD_SYMMETRIZE, BUILD_SYMMETRIZE | BUILD_DROP_LOOPS,
             BUILD_SYMMETRIZE | BUILD_DROP_LOOPS | BUILD_DEDUP, BUILD_SORT, BUILD_DEDUP,
             BUILD_SYMMETRIZE | BUILD_SORT, BUILD_DROP_LOOPS]


def _edges(n, m, seed):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, m, dtype=np.int32)
    dst = rng.integers(0, n, m, dtype=np.int32)
    k = m // 10  # repeats and self loops on purpose
    src[:k] = src[k:2 * k]
    dst[:k] = dst[k:2 * k]
    dst[2 * k:2 * k + k // 2] = src[2 * k:2 * k + k // 2]
    return src, dst


def _host(n, src, dst, flags):
    return graphs.from_edges(n, src, dst, symmetrize=bool(flags & BUILD_SYMMETRIZE),
                             drop_loops=bool(flags & BUILD_DROP_LOOPS),
                             dedup=bool(flags & BUILD_DEDUP), sort=bool(flags & BUILD_SORT))


@pytest.mark.parametrize("flags", FLAG_SETS)
def test_device_edges_equal_host_builder(gpu_available, flags):
    n, m = 3000, 20000
    src, dst = _edges(n, m, seed=flags + 1)
    want = _host(n, src, dst, flags)
    with tb.Graph.from_edges(src, dst, n, flags, keep_order=True) as g:
        cp, ic = g.csc()
        assert g.nnz == want.nnz
    assert np.array_equal(cp, want.col_ptr)
    assert np.array_equal(ic, want.row_idx)


def test_device_edges_large_three_radix_passes(gpu_available):
    n, m = 1 << 20, 3_000_000  # 21-bit column keys: three 8-bit passes per sort
    src, dst = _edges(n, m, seed=7)
    for flags in (BUILD_SYMMETRIZE, BUILD_SYMMETRIZE | BUILD_DROP_LOOPS | BUILD_DEDUP):
        want = _host(n, src, dst, flags)
        with tb.Graph.from_edges(src, dst, n, flags, keep_order=True) as g:
            cp, ic = g.csc()
        assert np.array_equal(cp, want.col_ptr) and np.array_equal(ic, want.row_idx)


def test_device_edges_bfs_matches_oracle(gpu_available):
    n, m = 5000, 30000
    src, dst = _edges(n, m, seed=3)
    flags = BUILD_SYMMETRIZE | BUILD_DROP_LOOPS | BUILD_DEDUP
    host = _host(n, src, dst, flags)
    with tb.Graph.from_edges(src, dst, n, flags) as g:  # regrouped by degree
        for root in (0, 17, 4999):
            res = g.bfs(root)
            S, sg, ovf, _ = oracle.exact_bfs(host.col_ptr, host.row_idx, root)
            assert np.array_equal(res.S, S) and np.array_equal(res.sigma, sg)


def test_device_edges_reject_bad_input(gpu_available):
    src = np.array([0, 1, 5], np.int32)
    dst = np.array([1, 2, 0], np.int32)
    with pytest.raises(TbfsError):
        tb.Graph.from_edges(src, dst, 4, BUILD_SYMMETRIZE)  # 5 is outside [0, 4)


def _mm_text(n, src, dst, crlf=False, noise=True):
    nl = "\r\n" if crlf else "\n"
    lines = ["%%MatrixMarket matrix coordinate pattern general", "% a comment", "%"]
    lines.append(f"{n} {n} {len(src)}")
    for k, (u, v) in enumerate(zip(src.tolist(), dst.tolist())):
        if noise and k % 97 == 5:
            lines.append("% comment between entries")
        if noise and k % 89 == 3 and not crlf:  # the host reader takes "\n" as an empty line only
            lines.append("")
        pad = "  " if noise and k % 13 == 0 else ""
        val = " 1.5" if noise and k % 7 == 0 else ""
        lines.append(f"{pad}{u + 1}\t{v + 1}{val}" if k % 5 == 0 else f"{pad}{u + 1} {v + 1}{val}")
    return (nl.join(lines) + nl).encode()


@pytest.mark.parametrize("undirected", [True, False])
@pytest.mark.parametrize("crlf", [False, True])
def test_mm_text_equals_host_reader(gpu_available, tmp_path, undirected, crlf):
    n, m = 2500, 12000
    rng = np.random.default_rng(11)
    src = rng.integers(0, n, m, dtype=np.int32)
    dst = rng.integers(0, n, m, dtype=np.int32)
    text = _mm_text(n, src, dst, crlf=crlf)
    path = tmp_path / "g.mtx"
    path.write_bytes(text)
    want = graphs.read_mm(path, undirected)
    with tb.Graph.from_mm_text(text, undirected, keep_order=True) as g:
        cp, ic = g.csc()
    assert np.array_equal(cp, want.col_ptr) and np.array_equal(ic, want.row_idx)
    with tb.Graph.load_mm(path, undirected, keep_order=True) as g:
        cp2, ic2 = g.csc()
    assert np.array_equal(cp2, want.col_ptr) and np.array_equal(ic2, want.row_idx)


def test_mm_text_large(gpu_available):
    n, m = 1 << 18, 1_500_000
    rng = np.random.default_rng(5)
    src = rng.integers(0, n, m, dtype=np.int32)
    dst = rng.integers(0, n, m, dtype=np.int32)
    text = _mm_text(n, src, dst, noise=False)
    want = graphs.from_edges(n, src, dst, symmetrize=True)
    with tb.Graph.from_mm_text(text, True, keep_order=True) as g:
        cp, ic = g.csc()
    assert np.array_equal(cp, want.col_ptr) and np.array_equal(ic, want.row_idx)


def test_mm_text_extra_lines_ignored(gpu_available):
    base = b"%%MatrixMarket matrix coordinate pattern symmetric\n3 3 2\n2 1\n3 2\n3 1\n"
    with tb.Graph.from_mm_text(base, True, keep_order=True) as g:
        cp, ic = g.csc()
    assert cp.tolist() == [0, 1, 3, 4] and ic.tolist() == [1, 0, 2, 1]


@pytest.mark.parametrize("text", [
    b"not a banner\n3 3 1\n1 2\n",
    b"%%MatrixMarket matrix array real general\n3 3\n1.0\n",
    b"%%MatrixMarket matrix coordinate pattern general\n% no size line\n",
    b"%%MatrixMarket matrix coordinate pattern general\n3 3 4\n1 2\n2 3\n",   # short
    b"%%MatrixMarket matrix coordinate pattern general\n3 3 2\n1 2\n0 3\n",   # index 0
    b"%%MatrixMarket matrix coordinate pattern general\n3 3 2\n1 2\n2 4\n",   # j > N
    b"%%MatrixMarket matrix coordinate pattern general\n3 3 2\n1 2\n7\n",     # one index
])
def test_mm_text_errors(gpu_available, text):
    with pytest.raises(TbfsError) as ei:
        tb.Graph.from_mm_text(text, True)
    assert ei.value.status == 6  # TBFS_ERR_IO


def test_cooc_lists_keep_file_order(gpu_available):
    n, m = 2000, 15000
    rng = np.random.default_rng(2)
    I = rng.integers(0, n, m, dtype=np.int32)
    J = rng.integers(0, n, m, dtype=np.int32)
    want = graphs.from_edges(n, I, J)  # column J[k] gets row I[k], file order
    with tb.Graph.from_cooc(I, J, n, keep_order=True) as g:
        cp, ic = g.csc()
    assert np.array_equal(cp, want.col_ptr) and np.array_equal(ic, want.row_idx)


def test_mm_text_to_cooc(gpu_available):
    """Matrix Market -> symmetric sorted COOC on the device: the column-order
    pairs of the deduplicated symmetric CSC."""
    n, m = 3000, 15000
    rng = np.random.default_rng(12)
    src = rng.integers(0, n, m, dtype=np.int32)
    dst = rng.integers(0, n, m, dtype=np.int32)
    text = _mm_text(n, src, dst, noise=False)
    flags = BUILD_DROP_LOOPS | BUILD_DEDUP
    want = graphs.from_edges(n, src, dst, symmetrize=True, drop_loops=True, dedup=True)
    with tb.Graph.from_mm_text(text, True, flags, keep_order=True) as g:
        row, col = g.cooc()
    assert np.array_equal(row, want.row_idx)
    assert np.array_equal(col, np.repeat(np.arange(n, dtype=np.int32), np.diff(want.col_ptr)))
