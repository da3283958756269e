"""The device validator (tbfs_bfs_validate) against the oracle: exact results
pass with the oracle's visited and edge counts; results with planted
mistakes (changed on the host before the check, the oracle's outputs
altered) are caught with the right kind and the smallest offending vertex,
exactly where the vectorised invariant checker of the tests rejects them."""
import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from golden_data import bfs_invariants, load
from turbobfs_gb300 import graphs

pytestmark = pytest.mark.gpu

KINDS = ("bad_root", "bad_depth", "skips_level", "no_parent", "sigma_mismatch")


def _graphs():
    yield "rmat16", graphs.rmat(16, 16, seed=5)  # regrouped numbering, hub lists > 128 entries
    fx = load("luxembourg_osm")
    yield "luxembourg", graphs.HostCSC(fx.n, fx.col_ptr, fx.row_idx, fx.symmetric)
    rng = np.random.default_rng(3)
    n = 3000
    yield "directed", graphs.from_edges(n, rng.integers(0, n, 20000).astype(np.int32),
                                        rng.integers(0, n, 20000).astype(np.int32))


def _numpy_ok(h, r, S, sg):
    try:
        bfs_invariants(h.col_ptr, h.row_idx, r, S, sg)
        return True
    except AssertionError:
        return False


@pytest.mark.parametrize("which", ["rmat16", "luxembourg", "directed"])
def test_exact_results_pass_and_mistakes_are_caught(gpu_available, which):
    torch = pytest.importorskip("torch")
    h = dict(_graphs())[which]
    r = int(graphs.pick_roots(h, 1, seed=2)[0])
    S, sg, ovf, _ = oracle.exact_bfs(h.col_ptr, h.row_idx, r)
    assert not ovf.any()
    deg = np.diff(h.col_ptr.astype(np.int64))
    with tb.Graph.from_host_csc(h) as g:
        v = g.validate(r, S, sg)
        assert v["ok"] and v["first_bad"] == -1
        assert v["visited"] == int((S >= 0).sum()) and v["edges"] == int(deg[S >= 0].sum())
        vd = g.validate(r, torch.from_numpy(S).cuda(), torch.from_numpy(sg).cuda())
        assert vd == v
        assert g.validate(r, S, None)["ok"]
        unreached = np.flatnonzero(S < 0)
        deepest = np.flatnonzero(S == S.max())  # no children: a change stays local
        x = int(deepest[len(deepest) // 2])
        cases = []
        s2 = sg.copy(); s2[x] += 1
        cases.append(("sigma_mismatch", S, s2, x))
        S2 = S.copy(); S2[r] = 1
        cases.append(("bad_root", S2, sg, None))
        S2 = S.copy(); S2[x] = S[x] + 2  # its parents' edges now skip a level
        cases.append(("skips_level", S2, sg, None))
        S2 = S.copy(); S2[x] = -1; s2 = sg.copy(); s2[x] = 0  # dropped from the tree
        cases.append(("skips_level", S2, s2, None))
        S2 = S.copy(); S2[x] = -5
        cases.append(("bad_depth", S2, sg, None))
        if len(unreached):
            y = int(unreached[0])  # every in-neighbour of y is unreached too
            s2 = sg.copy(); s2[y] = 7
            cases.append(("sigma_mismatch", S, s2, y))
            S2 = S.copy(); S2[y] = 5
            cases.append(("no_parent", S2, None, None))
        for kind, Sb, sgb, first in cases:
            v = g.validate(r, Sb, sgb)
            assert not v["ok"] and v[kind] >= 1, (kind, v)
            if first is not None:
                assert v["first_bad"] == first and sum(v[k] for k in KINDS) == 1, (kind, v)
            assert not _numpy_ok(h, r, Sb, sgb)


def test_rejects_bad_arguments(gpu_available):
    h = graphs.rmat(10, 8, seed=1)
    with tb.Graph.from_host_csc(h) as g:
        with pytest.raises(tb.TbfsError):
            g.validate(h.n, np.zeros(h.n, np.int32))
