"""Pin the oracle: the CPU restatement must reproduce, bit for bit, the
outputs of the reference's own sequential code frozen in tests/golden/, and
(where the reference tree was compiled on this machine) the reference's code
run live on fresh graphs."""
import numpy as np
import pytest

import oracle
from golden_data import FIXTURE_NAMES, load
from turbobfs_gb300 import graphs


def _bits(a):
    a = np.asarray(a)
    return a.view(np.int32) if a.dtype == np.float32 else a


@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_restatement_matches_reference_golden(name):
    fx = load(name)
    I, J = fx.cooc()
    for i, r in enumerate(fx.roots):
        S, sg, _ = oracle.seq_csc_f32(fx.col_ptr, fx.row_idx, r, init_S=False)
        assert np.array_equal(S, fx.get("td_S", i))
        assert np.array_equal(_bits(sg), _bits(fx.get("td_sigma", i)))
        S, sg, _ = oracle.seq_csc_f32(fx.col_ptr, fx.row_idx, r, init_S=True)
        assert np.array_equal(S, fx.get("bu_S", i))
        assert np.array_equal(_bits(sg), _bits(fx.get("bu_sigma", i)))
        S, sg, _ = oracle.seq_csc_i32(fx.col_ptr, fx.row_idx, r)
        assert np.array_equal(S, fx.get("tdbu_S", i))
        assert np.array_equal(sg, fx.get("tdbu_sigma", i))
        sg, _ = oracle.seq_cooc_f32(I, J, fx.n, r)
        assert np.array_equal(_bits(sg), _bits(fx.get("cooc_sigma", i)))


@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_exact_oracle_golden(name):
    fx = load(name)
    for i, r in enumerate(fx.roots):
        S, sg, ovf, _ = oracle.exact_bfs(fx.col_ptr, fx.row_idx, r)
        assert np.array_equal(S, fx.get("exact_S", i))
        assert np.array_equal(sg, fx.get("exact_sigma", i))
        assert np.array_equal(ovf, fx.get("exact_ovf", i))


@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_exact_agrees_with_reference_where_reference_is_exact(name):
    """The reference's depths equal the exact ones; its int32 sigma equals the
    exact count wherever that is below 2^31 and no ancestor wrapped, and its
    float sigma wherever the count is at most 2^24."""
    fx = load(name)
    for i, r in enumerate(fx.roots):
        S = fx.get("exact_S", i)
        sg = fx.get("exact_sigma", i)
        ovf = fx.get("exact_ovf", i).astype(bool)
        # float sums stay positive, so the float variants' depths are always right
        assert np.array_equal(fx.get("td_S", i), np.where(S < 0, 0, S))
        assert np.array_equal(fx.get("bu_S", i), S)
        if not ovf.any() and sg.max() < 2**31:
            assert np.array_equal(S, fx.get("tdbu_S", i))
            assert np.array_equal(fx.get("tdbu_sigma", i).astype(np.int64), sg)
        else:
            # int32 counts wrapped: the reference loses vertices (its sum > 0.1
            # test fails on a wrapped count); every depth it does assign is right
            St = fx.get("tdbu_S", i)
            assert (St[St >= 0] == S[St >= 0]).all() and (St != S).any()
        small = (~ovf) & (sg <= 2**24)
        assert np.array_equal(fx.get("td_sigma", i)[small].astype(np.int64), sg[small])
        assert np.array_equal(fx.get("cooc_sigma", i)[small].astype(np.int64), sg[small])


def test_overflow_fixture_really_overflows():
    fx = load("layered16x17")
    ovf = fx.get("exact_ovf", 0).astype(bool)
    S = fx.get("exact_S", 0)
    assert ovf.any() and (S[ovf] == 17).all()
    sg = fx.get("exact_sigma", 0)
    assert sg[S == 16].max() == 16**15  # 2^60, still exact


@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_gpu_emulations_consistent(name):
    """The emulated outputs of the reference's GPU drivers agree with its
    sequential code in the range where both are exact."""
    fx = load(name)
    I, J = fx.cooc()
    for i, r in enumerate(fx.roots):
        S = fx.get("exact_S", i)
        sg = fx.get("exact_sigma", i)
        ovf = fx.get("exact_ovf", i).astype(bool)
        assert np.array_equal(oracle.gpu_bu_csc(fx.col_ptr, fx.row_idx, r), S)
        small = (~ovf) & (sg <= 2**24)
        Sg, sgg = oracle.gpu_td_csc(fx.col_ptr, fx.row_idx, r)
        if not ovf.any() and sg.max() < 2**31:
            assert np.array_equal(Sg, np.where(S < 0, 0, S))
        assert np.array_equal(sgg[small].astype(np.int64), sg[small])
        sgc = oracle.gpu_td_cooc(I, J, fx.n, r)
        assert np.array_equal(sgc[small].astype(np.int64), sg[small])
        St, sgt, sw = oracle.gpu_tdbu_csc(fx.col_ptr, fx.row_idx, r)
        assert np.array_equal(St, S)
        if not ovf.any() and sg.max() < 2**31:
            last_td = sw if sw >= 0 else S.max()
            expect = np.where((S >= 0) & (S <= last_td), sg, 0)
            assert np.array_equal(sgt.astype(np.int64), expect)


def test_tdbu_emulation_switch_rule():
    """ER(4096): level 1 already holds more than 0.001*n vertices, so the
    reference's driver goes bottom-up from depth 1 on and reports sigma only
    for the root and its neighbours."""
    fx = load("er4096")
    S, sg, sw = oracle.gpu_tdbu_csc(fx.col_ptr, fx.row_idx, 0)
    assert sw == 1
    assert (sg[S >= 2] == 0).all() and (sg[S == 1] > 0).all() and sg[0] == 1


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not compiled here")
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_restatement_matches_reference_live(seed):
    """Fresh graphs, the reference's compiled code run live."""
    for g in (graphs.erdos_renyi(600, 1500, seed=seed), graphs.rmat(9, 8, seed=seed),
              graphs.grid(12, seed=seed)):
        roots = graphs.pick_roots(g, 2, seed=seed)
        I, J = g.to_cooc()
        for r in roots:
            r = int(r)
            Sr, sr = oracle.ref_seq_csc("csc_td", g.col_ptr, g.row_idx, r)
            So, so, _ = oracle.seq_csc_f32(g.col_ptr, g.row_idx, r, init_S=False)
            assert np.array_equal(Sr, So) and np.array_equal(_bits(sr), _bits(so))
            Sr, sr = oracle.ref_seq_csc("csc_tdbu", g.col_ptr, g.row_idx, r)
            So, so, _ = oracle.seq_csc_i32(g.col_ptr, g.row_idx, r)
            assert np.array_equal(Sr, So) and np.array_equal(sr, so)
            sr = oracle.ref_seq_cooc(I, J, g.n, r)
            so, _ = oracle.seq_cooc_f32(I, J, g.n, r)
            assert np.array_equal(_bits(sr), _bits(so))


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not compiled here")
def test_restatement_matches_reference_on_wrapping_counts():
    """int32 path counts that wrap, and float counts past 2^24: the
    restatement follows the reference's arithmetic there too."""
    g = graphs.layered_bipartite(16, 17)
    Sr, sr = oracle.ref_seq_csc("csc_tdbu", g.col_ptr, g.row_idx, 0)
    So, so, _ = oracle.seq_csc_i32(g.col_ptr, g.row_idx, 0)
    assert np.array_equal(Sr, So) and np.array_equal(sr, so)
    Sr, sr = oracle.ref_seq_csc("csc_td", g.col_ptr, g.row_idx, 0)
    So, so, _ = oracle.seq_csc_f32(g.col_ptr, g.row_idx, 0, init_S=False)
    assert np.array_equal(Sr, So) and np.array_equal(_bits(sr), _bits(so))
