"""Parity on the headline workload at full size: RMAT scale 22 (edgefactor 16,
a/b/c/d = .57/.19/.19/.05, seed 1, vertex ids permuted) with the 64 roots the
benchmark times (pick_roots(h, 64, seed=1)).

Every one of the 64 traversals is checked, with the default direction
parameters, with fixed tuned ones and with the autotuner's pick (which
select different path-count schedules), by the device validator
(tbfs_bfs_validate: level consistency, a parent for every reached vertex,
sigma = parent sum), which pins S and sigma uniquely; the validator itself
is checked against the oracle and against planted mistakes in
test_gpu_validate.py.  Four roots are compared element for element with the
oracle's exact BFS, and the drop-in bfs_gpu_tdbu_csc_sc with the oracle's
emulation of the reference driver on two roots (S everywhere, its int32
sigma where the reference's count is exact)."""
import ctypes

import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from turbobfs_gb300 import _lib, graphs
from turbobfs_gb300.api import _P_I32, _P_I64, make_options

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def headline(gpu_available):
    h = graphs.rmat(22, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    roots = np.ascontiguousarray(graphs.pick_roots(h, 64, seed=1), dtype=np.int32)
    g = tb.Graph.from_host_csc(h)
    S = torch.empty((64, h.n), dtype=torch.int32, device="cuda")
    sg = torch.empty((64, h.n), dtype=torch.int64, device="cuda")
    yield h, roots, g, S, sg
    g.close()
    del S, sg
    torch.cuda.empty_cache()


def _run_many(g, roots, S, sg, **kw):
    o = make_options("auto", True, outputs_on_device=True, **kw)
    st = (_lib.Stats * len(roots))()
    _lib.check(tb.lib().tbfs_bfs_many(g.handle, roots.ctypes.data_as(_P_I32), len(roots),
                                      ctypes.byref(o), ctypes.cast(S.data_ptr(), _P_I32),
                                      ctypes.cast(sg.data_ptr(), _P_I64), st), "tbfs_bfs_many")
    return [st[i].as_dict() for i in range(len(roots))]


def _validate_all(g, roots, S, sg, stats):
    for i, r in enumerate(roots):
        v = g.validate(int(r), S[i], sg[i])
        assert v["ok"], f"root {r}: {v}"
        assert v["visited"] == stats[i]["visited"]
        assert stats[i]["sigma_overflow"] == 0


@pytest.mark.parametrize("params", [{}, {"alpha": 9, "beta": 2, "pull_ratio": 2},
                                    {"alpha": 9, "beta": 1, "pull_ratio": 2},
                                    {"max_ept": 2, "ctas_per_sm": 2}, "autotuned"],
                         ids=["default", "tuned_b2", "tuned_b1", "shape", "autotuned"])
def test_all_64_roots_validate(headline, params):
    h, roots, g, S, sg = headline
    if params == "autotuned":
        tu = g.autotune(roots[:8])
        params = {k: v for k, v in tu.items() if k != "from_cache"}
    stats = _run_many(g, roots, S, sg, **params)
    assert all(s["bu_levels"] >= 1 for s in stats)
    _validate_all(g, roots, S, sg, stats)


def test_four_roots_equal_exact_oracle(headline):
    h, roots, g, S, sg = headline
    _run_many(g, roots, S, sg, alpha=9, beta=2, pull_ratio=2)
    for i in (0, 21, 42, 63):
        Se, sge, ovf, levels = oracle.exact_bfs(h.col_ptr, h.row_idx, int(roots[i]))
        assert not ovf.any()
        assert np.array_equal(S[i].cpu().numpy(), Se)
        assert np.array_equal(sg[i].cpu().numpy(), sge)


def test_dropin_tdbu_equals_reference_emulation(headline):
    h, roots, _, _, _ = headline
    for r in roots[:2]:
        S = np.zeros(h.n, np.int32)
        sg = np.zeros(h.n, np.int32)
        assert tb.bfs_gpu_tdbu_csc_sc(h.row_idx, h.col_ptr, S, sg, int(r), h.nnz, h.n, 1, 1) == 0
        Se, sge, _ = oracle.gpu_tdbu_csc(h.col_ptr, h.row_idx, int(r))
        assert np.array_equal(S, Se)
        Sx, sgx, ovf, _ = oracle.exact_bfs(h.col_ptr, h.row_idx, int(r))
        exact = (ovf == 0) & (sgx < 2**31)
        assert np.array_equal(sg[exact], sge[exact])
