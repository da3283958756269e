"""GPU parity: the CUDA engine against the oracle, through the C ABI.

Bar: bit-exact.  S (int32) and sigma (int64 path counts) of the native API
must equal the exact oracle on every vertex, in every traversal mode; the
drop-in entry points must equal the outputs the reference's GPU drivers
produce (emulated by the oracle, and frozen from the reference's own
sequential code in tests/golden/ where both are exact)."""
import ctypes

import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from golden_data import FIXTURE_NAMES, bfs_invariants, load
from turbobfs_gb300 import graphs

pytestmark = pytest.mark.gpu
MODES = ["auto", "td", "bu"]


def _exact_check(cp, ic, r, res, want_sigma=True):
    S, sg, ovf, levels = oracle.exact_bfs(cp, ic, r)
    assert np.array_equal(res.S, S)
    assert res.stats["levels"] == levels
    assert res.stats["visited"] == int((S >= 0).sum())
    deg = np.diff(np.asarray(cp, dtype=np.int64))
    if want_sigma:
        ok = ovf == 0
        assert np.array_equal(res.sigma[ok], sg[ok])
        assert res.stats["sigma_overflow"] == int(ovf.any())


@pytest.mark.parametrize("name", FIXTURE_NAMES)
@pytest.mark.parametrize("mode", MODES)
def test_native_fixtures_all_modes(gpu_available, name, mode):
    fx = load(name)
    with tb.Graph(fx.col_ptr, fx.row_idx, fx.n, symmetric=fx.symmetric) as g:
        for i, r in enumerate(fx.roots):
            res = g.bfs(r, mode=mode)
            assert np.array_equal(res.S, fx.get("exact_S", i))
            ok = fx.get("exact_ovf", i) == 0
            assert np.array_equal(res.sigma[ok], fx.get("exact_sigma", i)[ok])
            assert res.stats["sigma_overflow"] == int((~ok).any())
            res2 = g.bfs(r, mode=mode, sigma=False)
            assert np.array_equal(res2.S, res.S)


@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_native_general_path_on_symmetric_graphs(gpu_available, name):
    """Without the symmetric promise the engine builds the transpose on the
    device and pulls sigma separately; results must not change."""
    fx = load(name)
    with tb.Graph(fx.col_ptr, fx.row_idx, fx.n, symmetric=False) as g:
        for i, r in enumerate(fx.roots):
            for mode in MODES:
                res = g.bfs(r, mode=mode)
                assert np.array_equal(res.S, fx.get("exact_S", i))
                ok = fx.get("exact_ovf", i) == 0
                assert np.array_equal(res.sigma[ok], fx.get("exact_sigma", i)[ok])


@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_native_cooc_input(gpu_available, name):
    fx = load(name)
    I, J = fx.cooc()
    perm = np.random.default_rng(0).permutation(I.shape[0])  # column order not required
    with tb.Graph.from_cooc(I[perm], J[perm], fx.n) as g:
        for i, r in enumerate(fx.roots):
            res = g.bfs(r)
            assert np.array_equal(res.S, fx.get("exact_S", i))
            ok = fx.get("exact_ovf", i) == 0
            assert np.array_equal(res.sigma[ok], fx.get("exact_sigma", i)[ok])


# ------------------------------------------------- drop-in entry points

def _bits(a):
    return np.asarray(a).view(np.int32)


@pytest.mark.parametrize("name", FIXTURE_NAMES)
@pytest.mark.parametrize("fn", ["bfs_gpu_td_csc_sc", "bfs_gpu_td_csc_wa"])
def test_compat_td_csc(gpu_available, name, fn):
    fx = load(name)
    for i, r in enumerate(fx.roots):
        S = np.full(fx.n, 77, np.int32)
        sg = np.full(fx.n, -1.0, np.float32)
        assert tb.COMPAT_FUNCTIONS[fn](fx.row_idx, fx.col_ptr, S, sg, r, fx.nnz, fx.n, 2) == 0
        exact_S = fx.get("exact_S", i)
        exact = fx.get("exact_sigma", i)
        ovf = fx.get("exact_ovf", i).astype(bool)
        assert np.array_equal(S, np.where(exact_S < 0, 0, exact_S))
        fine = (~ovf) & (exact < 2**31)  # the reference's int32 sums are exact here
        Se, sge = oracle.gpu_td_csc(fx.col_ptr, fx.row_idx, r)
        if fine.all():
            assert np.array_equal(S, Se)
            assert np.array_equal(_bits(sg), _bits(sge))
        assert np.array_equal(_bits(sg[fine]), _bits(exact[fine].astype(np.float32)))
        small = (~ovf) & (exact <= 2**24)
        assert np.array_equal(_bits(sg[small]), _bits(fx.get("td_sigma", i)[small]))


@pytest.mark.parametrize("name", FIXTURE_NAMES)
@pytest.mark.parametrize("fn", ["bfs_gpu_bu_csc_sc", "bfs_gpu_bu_csc_wa"])
def test_compat_bu_csc(gpu_available, name, fn):
    fx = load(name)
    for i, r in enumerate(fx.roots):
        for bbreak in (0, 1):
            S = np.full(fx.n, 77, np.int32)
            assert tb.COMPAT_FUNCTIONS[fn](fx.row_idx, fx.col_ptr, S, r, fx.nnz, fx.n, 1,
                                           bbreak) == 0
            assert np.array_equal(S, oracle.gpu_bu_csc(fx.col_ptr, fx.row_idx, r))
            assert np.array_equal(S, fx.get("bu_S", i))


@pytest.mark.parametrize("name", FIXTURE_NAMES)
@pytest.mark.parametrize("fn", ["bfs_gpu_tdbu_csc_sc", "bfs_gpu_tdbu_csc_wa"])
def test_compat_tdbu_csc(gpu_available, name, fn):
    fx = load(name)
    for i, r in enumerate(fx.roots):
        S = np.full(fx.n, 77, np.int32)
        sg = np.full(fx.n, 77, np.int32)
        assert tb.COMPAT_FUNCTIONS[fn](fx.row_idx, fx.col_ptr, S, sg, r, fx.nnz, fx.n, 1, 1) == 0
        assert np.array_equal(S, fx.get("exact_S", i))
        exact = fx.get("exact_sigma", i)
        ovf = fx.get("exact_ovf", i).astype(bool)
        Se, sge, _ = oracle.gpu_tdbu_csc(fx.col_ptr, fx.row_idx, r)
        if not ovf.any() and exact.max() < 2**31:
            assert np.array_equal(S, Se)
            assert np.array_equal(sg, sge)


@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_compat_td_cooc(gpu_available, name):
    fx = load(name)
    I, J = fx.cooc()
    for i, r in enumerate(fx.roots):
        sg = np.full(fx.n, -1.0, np.float32)
        assert tb.bfs_gpu_td_cooc_sc(I, J, sg, r, fx.nnz, fx.n, 1) == 0
        exact = fx.get("exact_sigma", i)
        ovf = fx.get("exact_ovf", i).astype(bool)
        fine = (~ovf) & (exact < 2**31)
        if fine.all():
            assert np.array_equal(_bits(sg), _bits(oracle.gpu_td_cooc(I, J, fx.n, r)))
        small = (~ovf) & (exact <= 2**24)
        assert np.array_equal(_bits(sg[small]), _bits(fx.get("cooc_sigma", i)[small]))


def test_compat_cooc_native_and_sorted_paths(gpu_available):
    """bfs_gpu_td_cooc_sc runs straight over the pairs for graphs of at most
    32 levels and sorts them into CSC beyond: a directed shallow graph and a
    2 x 3000 ladder (3000 levels) in both directions, pairs in random order,
    equal to the oracle's emulation of the reference's COOC driver (float
    sigma; counts here stay below 2^24).  Out-of-range pairs are an error."""
    rng = np.random.default_rng(11)
    n = 20000
    src = rng.integers(0, n, 80000, dtype=np.int32)
    dst = rng.integers(0, n, 80000, dtype=np.int32)
    n2 = 3000
    a = np.arange(n2 - 1, dtype=np.int32)
    lsrc = np.concatenate([a, a + n2, np.arange(n2, dtype=np.int32)])
    ldst = np.concatenate([a + 1, a + 1 + n2, np.arange(n2, dtype=np.int32) + n2])
    cases = [("directed", n, src, dst, (0, 5, 1234)),
             ("ladder", 2 * n2, np.concatenate([lsrc, ldst]), np.concatenate([ldst, lsrc]), (0, 2500))]
    for name, nv, I, J, roots in cases:
        perm = rng.permutation(I.shape[0])
        I = np.ascontiguousarray(I[perm], np.int32)
        J = np.ascontiguousarray(J[perm], np.int32)
        for r in roots:
            sg = np.full(nv, -1.0, np.float32)
            assert tb.bfs_gpu_td_cooc_sc(I, J, sg, r, I.shape[0], nv, 1) == 0, name
            want = oracle.gpu_td_cooc(I, J, nv, r)
            assert np.array_equal(_bits(sg), _bits(want)), (name, r)
    bad = np.array([0, 1, 7], np.int32)
    sg = np.zeros(5, np.float32)
    assert tb.bfs_gpu_td_cooc_sc(bad, np.array([1, 2, 3], np.int32), sg, 0, 3, 5, 1) != 0


# ------------------------------------------------------- synthetic sizes

@pytest.mark.parametrize("kind,seed", [("er", 1), ("er", 2), ("rmat", 1), ("rmat", 2),
                                       ("grid", 1), ("grid", 2)])
def test_native_synthetic_vs_exact_oracle(gpu_available, kind, seed):
    if kind == "er":
        h = graphs.erdos_renyi(50000, 200000, seed=seed)
    elif kind == "rmat":
        h = graphs.rmat(16, 16, seed=seed)
    else:
        h = graphs.grid(200, seed=seed)
    roots = graphs.pick_roots(h, 3, seed=seed)
    with tb.Graph.from_host_csc(h) as g:
        for r in roots:
            for mode in MODES:
                res = g.bfs(int(r), mode=mode)
                _exact_check(h.col_ptr, h.row_idx, int(r), res)


def test_native_directed_random_vs_exact(gpu_available):
    rng = np.random.default_rng(5)
    n, m = 20000, 90000
    src = rng.integers(0, n, m, dtype=np.int32)
    dst = rng.integers(0, n, m, dtype=np.int32)
    h = graphs.from_edges(n, src, dst)  # directed, with duplicates and self-loops
    with tb.Graph.from_host_csc(h) as g:
        for r in (0, 17, 4242):
            for mode in MODES:
                res = g.bfs(r, mode=mode)
                _exact_check(h.col_ptr, h.row_idx, r, res)


def _out_degree_graph(n, max_out, seed, hub_out=0):
    """Directed graph whose vertices have out-degree uniform in [0, max_out]
    (vertex 1 gets hub_out out-edges when given)."""
    rng = np.random.default_rng(seed)
    deg = rng.integers(0, max_out + 1, n)
    if hub_out:
        deg[1] = hub_out
    src = np.repeat(np.arange(n, dtype=np.int32), deg)
    dst = rng.integers(0, n, src.size, dtype=np.int32)
    return graphs.from_edges(n, src, dst)


@pytest.mark.parametrize("max_out,hub_out", [(16, 0), (16, 17), (3, 0)])
def test_short_list_levels_vs_exact(gpu_available, max_out, hub_out):
    """Graphs whose out-lists are all at most 16 entries long expand their
    small top-down levels in entry-aligned items (no owner search); one list
    of 17 entries switches the graph to the general instance.  Both equal the
    exact oracle, with path counts, in every mode, from several roots."""
    h = _out_degree_graph(30000, max_out, seed=max_out + hub_out, hub_out=hub_out)
    with tb.Graph.from_host_csc(h) as g:
        for r in (0, 1, 777, 29999):
            for mode in MODES:
                _exact_check(h.col_ptr, h.row_idx, r, g.bfs(r, mode=mode))
                if mode == "td":
                    _exact_check(h.col_ptr, h.row_idx, r, g.bfs(r, mode=mode, sigma=False),
                                 want_sigma=False)


def test_short_list_deep_ladder_vs_exact(gpu_available):
    """A 2 x 20000 ladder (20000 levels of two vertices, out-degree <= 3)
    and the same ladder directed one way: every level is a short one."""
    n2 = 20000
    a = np.arange(n2 - 1, dtype=np.int32)
    src = np.concatenate([a, a + n2, np.arange(n2, dtype=np.int32)])
    dst = np.concatenate([a + 1, a + 1 + n2, np.arange(n2, dtype=np.int32) + n2])
    for sym in (True, False):
        h = graphs.from_edges(2 * n2, src, dst, symmetrize=sym)
        with tb.Graph.from_host_csc(h) as g:
            for r in (0, n2 + 5000):
                res = g.bfs(r)
                _exact_check(h.col_ptr, h.row_idx, r, res)


def test_bfs_many_matches_single(gpu_available):
    h = graphs.rmat(14, 16, seed=9)
    roots = graphs.pick_roots(h, 6, seed=2)
    with tb.Graph.from_host_csc(h) as g:
        S, sg, stats = g.bfs_many(roots)
        for i, r in enumerate(roots):
            one = g.bfs(int(r))
            assert np.array_equal(S[i], one.S) and np.array_equal(sg[i], one.sigma)
            assert stats[i]["levels"] == one.stats["levels"]


def test_sigma_overflow_detected(gpu_available):
    """16^16 = 2^64 shortest paths reach the last layer: reported, not rounded."""
    h = graphs.layered_bipartite(16, 17)
    with tb.Graph.from_host_csc(h) as g:
        for mode in MODES:
            res = g.bfs(0, mode=mode)
            assert res.stats["sigma_overflow"] == 1
            S, sg, ovf, _ = oracle.exact_bfs(h.col_ptr, h.row_idx, 0)
            assert np.array_equal(res.S, S)
            assert np.array_equal(res.sigma[ovf == 0], sg[ovf == 0])
    h2 = graphs.layered_bipartite(16, 16)  # 2^60: no overflow
    with tb.Graph.from_host_csc(h2) as g:
        res = g.bfs(0)
        assert res.stats["sigma_overflow"] == 0 and res.sigma.max() == 16**15


# --------------------------------------------- full sizes, invariants only

@pytest.mark.parametrize("mode", ["auto", "td", "bu"])
def test_rmat22_full_size_invariants(gpu_available, rmat22, mode):
    h, roots = rmat22
    with tb.Graph.from_host_csc(h) as g:
        res = g.bfs(int(roots[0]), mode=mode)
        bfs_invariants(h.col_ptr, h.row_idx, int(roots[0]), res.S, res.sigma)
        if mode == "auto":
            assert res.stats["bu_levels"] >= 1 and res.stats["td_levels"] >= 1
            ref = g.bfs(int(roots[0]), mode="td")
            assert np.array_equal(ref.S, res.S) and np.array_equal(ref.sigma, res.sigma)


def test_grid2048_full_size_invariants(gpu_available):
    h = graphs.grid(2048, seed=1)
    with tb.Graph.from_host_csc(h) as g:
        r = int(graphs.pick_roots(h, 1, seed=1)[0])
        res = g.bfs(r)
        assert res.stats["levels"] > 1000
        bfs_invariants(h.col_ptr, h.row_idx, r, res.S, res.sigma)
        I, J = h.to_cooc()
        with tb.Graph.from_cooc(I, J, h.n) as gc:
            resc = gc.bfs(r, mode="bu")
            assert np.array_equal(resc.S, res.S) and np.array_equal(resc.sigma, res.sigma)


@pytest.fixture(scope="module")
def rmat22():
    h = graphs.rmat(22, 16, seed=1)
    return h, graphs.pick_roots(h, 4, seed=1)


# ------------------------------------------------------------ edge cases

def test_edge_cases(gpu_available):
    # single vertex, no edges
    with tb.Graph(np.array([0, 0], np.int32), np.zeros(0, np.int32), 1) as g:
        res = g.bfs(0)
        assert res.S.tolist() == [0] and res.sigma.tolist() == [1]
        assert res.stats["levels"] == 1 and res.stats["visited"] == 1
    # isolated root in a larger graph, self-loops and duplicate entries
    cp = np.array([0, 0, 3, 5, 6], np.int32)
    ic = np.array([1, 2, 2, 1, 1, 3], np.int32)  # col1: 1,2,2  col2: 1,1  col3: 3
    with tb.Graph(cp, ic, 4) as g:
        res = g.bfs(0)
        assert res.S.tolist() == [0, -1, -1, -1] and res.sigma.tolist() == [1, 0, 0, 0]
        for mode in MODES:
            res = g.bfs(2, mode=mode)
            S, sg, _, _ = oracle.exact_bfs(cp, ic, 2)
            assert np.array_equal(res.S, S) and np.array_equal(res.sigma, sg)
            assert res.sigma[1] == 2  # duplicate entry counted twice, as the reference does
    # compat with repetition 0 behaves like one run
    S = np.zeros(4, np.int32)
    assert tb.bfs_gpu_bu_csc_sc(ic, cp, S, 2, 6, 4, 0, 1) == 0
    assert S.tolist() == oracle.gpu_bu_csc(cp, ic, 2).tolist()


def test_invalid_inputs_rejected(gpu_available):
    cp = np.array([0, 2, 1], np.int32)  # decreasing
    with pytest.raises(tb.TbfsError) as e:
        tb.Graph(cp, np.array([1, 0], np.int32), 2)
    assert e.value.status == 1
    with pytest.raises(tb.TbfsError):
        tb.Graph(np.array([0, 1, 2], np.int32), np.array([1, 9], np.int32), 2)  # row id 9
    with pytest.raises(tb.TbfsError):
        tb.Graph.from_cooc(np.array([0, 3], np.int32), np.array([1, 0], np.int32), 2)
    with tb.Graph(np.array([0, 1, 2], np.int32), np.array([1, 0], np.int32), 2) as g:
        with pytest.raises(tb.TbfsError):
            g.bfs(2)
        assert g.bfs(1).S.tolist() == [1, 0]


def test_barrier_timeout_is_reported_and_context_survives(gpu_available):
    """One CTA leaves before the barrier ending level 1; the other CTAs'
    bounded waits (50 ms) expire and the call reports TBFS_ERR_TIMEOUT
    instead of hanging.  The next traversal on the same graph is correct."""
    h = graphs.grid(64, seed=3)
    with tb.Graph.from_host_csc(h) as g:
        with pytest.raises(tb.TbfsError) as e:
            g.bfs(0, timeout_ns=50_000_000, inject_barrier_skip=2)
        assert e.value.status == 4
        res = g.bfs(0)
        _exact_check(h.col_ptr, h.row_idx, 0, res)


# ------------------------------------------------ symmetry found on upload

def test_symmetry_detected_without_the_flag(gpu_available):
    """A CSC uploaded without TBFS_GRAPH_SYMMETRIC that equals its transpose
    is found so on the device (tbfs_graph_info then reports the flag) and
    needs no transpose; one missing mirror entry, or one duplicated on one
    side only, makes it general.  Results equal the exact oracle either way."""
    h = graphs.rmat(12, 16, seed=9)
    col = np.repeat(np.arange(h.n), np.diff(h.col_ptr))
    variants = {"symmetric": (h.row_idx, col)}
    keep = np.ones(h.nnz, bool)
    keep[h.nnz // 3] = False
    variants["one mirror missing"] = (h.row_idx[keep], col[keep])
    k = h.nnz // 2
    variants["one-sided duplicate"] = (np.append(h.row_idx, h.row_idx[k]), np.append(col, col[k]))
    for name, (src, dst) in variants.items():
        g2 = graphs.from_edges(h.n, src.astype(np.int32), dst.astype(np.int32))
        with tb.Graph(g2.col_ptr, g2.row_idx, g2.n, symmetric=False) as g:
            flags = ctypes.c_uint32()
            tb.lib().tbfs_graph_info(g.handle, None, None, ctypes.byref(flags))
            assert bool(flags.value & 1) == (name == "symmetric"), name
            r = int(graphs.pick_roots(h, 1, seed=9)[0])
            for mode in MODES:
                _exact_check(g2.col_ptr, g2.row_idx, r, g.bfs(r, mode=mode))
