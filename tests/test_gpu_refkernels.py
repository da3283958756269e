"""The reference's own GPU kernels (compiled unchanged for sm_103a, driven by
the restatement of their host loops in oracle/ref_gpu.cu) as a second parity
source.  On every fixture and on a synthetic graph:
  * they equal the oracle's emulation of the reference drivers bit for bit,
    on every vertex (the emulation reproduces their int32 wrap-around too);
  * they equal this library's drop-in entry points wherever the reference's
    arithmetic is exact (no int32 path count wrapped on the way): S and sigma
    everywhere when no count reaches 2^31, otherwise sigma where the count
    fits the reference's type (float: up to 2^24, int32: below 2^31)."""
import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from golden_data import FIXTURE_NAMES, load
from turbobfs_gb300 import graphs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refgpu(gpu_available):
    if not oracle.refgpu_available():
        pytest.skip("the reference's kernel images (oracle/_ref/*.cubin) are not on this machine")
    return True


def _cases():
    for name in FIXTURE_NAMES:
        fx = load(name)
        yield name, fx.col_ptr, fx.row_idx, fx.roots
    h = graphs.rmat(16, 16, seed=4)
    yield "rmat16", h.col_ptr, h.row_idx, [int(r) for r in graphs.pick_roots(h, 2, seed=4)]


CASES = {name: (cp, ic, roots) for name, cp, ic, roots in _cases()}


@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_kernels_equal_emulation_and_dropin(refgpu, name):
    cp, ic, roots = CASES[name]
    n, nz = cp.shape[0] - 1, ic.shape[0]
    J = np.repeat(np.arange(n, dtype=np.int32), np.diff(cp))
    for r in roots:
        Sx, sgx, ovf, _ = oracle.exact_bfs(cp, ic, r)
        clean = not ovf.any() and sgx.max() < 2**31  # no int32 sum wraps
        f_ok = (ovf == 0) & (sgx <= 2**24)
        i_ok = (ovf == 0) & (sgx < 2**31)
        Sd = np.zeros(n, np.int32)
        # top-down, float sigma
        S, sg, _, _ = oracle.refgpu_td_csc_sc(cp, ic, r)
        Se, sge = oracle.gpu_td_csc(cp, ic, r)
        assert np.array_equal(S, Se) and np.array_equal(_bits(sg), _bits(sge))
        sgd = np.zeros(n, np.float32)
        assert tb.bfs_gpu_td_csc_sc(ic, cp, Sd, sgd, r, nz, n, 1) == 0
        assert np.array_equal(_bits(sg[f_ok]), _bits(sgd[f_ok]))
        if clean:
            assert np.array_equal(S, Sd) and np.array_equal(_bits(sg), _bits(sgd))
        # bottom-up, S only (no path counts, so nothing wraps)
        S, _, _ = oracle.refgpu_bu_csc_sc(cp, ic, r)
        assert np.array_equal(S, oracle.gpu_bu_csc(cp, ic, r))
        assert tb.bfs_gpu_bu_csc_sc(ic, cp, Sd, r, nz, n, 1, 1) == 0
        assert np.array_equal(S, Sd) and np.array_equal(S, Sx)
        # direction-optimizing, int32 sigma over the top-down levels
        S, sg, _, td, bu = oracle.refgpu_tdbu_csc_sc(cp, ic, r)
        Se, sge, _ = oracle.gpu_tdbu_csc(cp, ic, r)
        assert np.array_equal(S, Se) and np.array_equal(sg, sge)
        sgi = np.zeros(n, np.int32)
        assert tb.bfs_gpu_tdbu_csc_sc(ic, cp, Sd, sgi, r, nz, n, 1, 1) == 0
        assert np.array_equal(sg[i_ok], sgi[i_ok])
        if clean:
            assert np.array_equal(S, Sd) and np.array_equal(sg, sgi)
        # edge-parallel COOC, float sigma
        sg, _, _ = oracle.refgpu_td_cooc_sc(ic, J, n, r)
        sge = oracle.gpu_td_cooc(ic, J, n, r)
        assert np.array_equal(_bits(sg), _bits(sge))
        sgd = np.zeros(n, np.float32)
        assert tb.bfs_gpu_td_cooc_sc(ic, J, sgd, r, nz, n, 1) == 0
        assert np.array_equal(_bits(sg[f_ok]), _bits(sgd[f_ok]))


def _bits(a):
    return np.asarray(a).view(np.int32)
