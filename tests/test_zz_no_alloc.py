"""tbfs_bfs_noalloc, the entry point that allocates nothing.

It exists for callers that may not have the library call cudaMalloc or
cudaFree: code inside a host framework that hands out all device memory
from its own pool, and latency-critical loops that cannot afford the
device-wide synchronisation those calls can cause.  The caller passes the
graph and the outputs as device memory; the traversal's scratch is a static
device array in the library.  This file is named so pytest collects it
last; it must pass alone in a fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

import turbobfs_gb300 as tb
from turbobfs_gb300 import _lib, graphs

pytestmark = pytest.mark.gpu
MAX_N = 1 << 20


def _noalloc(torch, cp, ic, n, nnz, root, mode=0, out=None, sigma=True):
    S = torch.full((n,), 123, dtype=torch.int32, device="cuda")
    sg = torch.full((n,), 123, dtype=torch.int64, device="cuda") if sigma else None
    st = _lib.Stats()
    rc = tb.lib().tbfs_bfs_noalloc(
        cp.data_ptr(), ic.data_ptr(), out[0].data_ptr() if out else None,
        out[1].data_ptr() if out else None, n, nnz, root, mode, S.data_ptr(),
        sg.data_ptr() if sigma else None, None, ctypes.byref(st))
    torch.cuda.synchronize()
    return rc, S.cpu().numpy(), (sg.cpu().numpy() if sigma else None), st


def test_noalloc_matches_regular_entry_point(gpu_available):
    torch = pytest.importorskip("torch")
    h = graphs.rmat(16, 16, seed=5)
    roots = graphs.pick_roots(h, 2, seed=5)
    cp = torch.from_numpy(h.col_ptr).cuda()
    ic = torch.from_numpy(h.row_idx).cuda()
    with tb.Graph.from_host_csc(h) as g:
        for r in roots:  # two calls in a row: the shared scratch is reused
            r = int(r)
            ref = g.bfs(r)
            for mode in (0, 1, 2):
                rc, S, sg, st = _noalloc(torch, cp, ic, h.n, h.nnz, r, mode)
                assert rc == 0, tb.lib().tbfs_last_error()
                assert np.array_equal(S, ref.S)  # integer results: exact
                assert np.array_equal(sg, ref.sigma)
                assert st.levels == ref.stats["levels"] and st.visited == ref.stats["visited"]


def test_noalloc_directed_out_lists_and_depth_only(gpu_available):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    n = 30000
    src = rng.integers(0, n, 120000, dtype=np.int32)
    dst = rng.integers(0, n, 120000, dtype=np.int32)
    h = graphs.from_edges(n, src, dst)
    t = graphs.from_edges(n, dst, src)  # out-lists: the transpose of the in-lists
    dev = [torch.from_numpy(a).cuda() for a in (h.col_ptr, h.row_idx, t.col_ptr, t.row_idx)]
    with tb.Graph.from_host_csc(h) as g:
        for r in (0, 99):
            ref = g.bfs(r)
            rc, S, sg, _ = _noalloc(torch, dev[0], dev[1], n, h.nnz, r, out=(dev[2], dev[3]))
            assert rc == 0 and np.array_equal(S, ref.S) and np.array_equal(sg, ref.sigma)
            rc, S, _, _ = _noalloc(torch, dev[0], dev[1], n, h.nnz, r, out=(dev[2], dev[3]),
                                   sigma=False)
            assert rc == 0 and np.array_equal(S, ref.S)


def test_noalloc_allocates_nothing(gpu_available):
    """After a warm-up call, further calls leave the device's free memory
    unchanged (outputs preallocated and reused, torch's allocator idle)."""
    torch = pytest.importorskip("torch")
    h = graphs.rmat(14, 16, seed=7)
    cp = torch.from_numpy(h.col_ptr).cuda()
    ic = torch.from_numpy(h.row_idx).cuda()
    S = torch.empty(h.n, dtype=torch.int32, device="cuda")
    sg = torch.empty(h.n, dtype=torch.int64, device="cuda")
    st = _lib.Stats()

    def call(r):
        return tb.lib().tbfs_bfs_noalloc(cp.data_ptr(), ic.data_ptr(), None, None, h.n, h.nnz,
                                         int(r), 0, S.data_ptr(), sg.data_ptr(), None,
                                         ctypes.byref(st))

    assert call(0) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for r in graphs.pick_roots(h, 4, seed=7):
        assert call(r) == 0, tb.lib().tbfs_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_too_large_and_bad_input(gpu_available):
    torch = pytest.importorskip("torch")
    n = MAX_N + 1
    cp = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    ic = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc, _, _, _ = _noalloc(torch, cp, ic, n, 0, 0)
    assert rc == 7 and b"TBFS_NOALLOC_MAX_VERTICES" in tb.lib().tbfs_last_error()
    bad_cp = torch.tensor([0, 1, 2], dtype=torch.int32, device="cuda")
    bad_ic = torch.tensor([1, 5], dtype=torch.int32, device="cuda")  # row id 5 >= n
    rc, _, _, _ = _noalloc(torch, bad_cp, bad_ic, 2, 2, 0)
    assert rc == 1
