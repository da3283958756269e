"""Pin the degree-statistics restatement (oracle_degree_stats) to the
reference's own degree.c (TurboBFS_CSC_TD/degree.c:22-141, compiled
unchanged into oracle/_ref where the reference tree is on this machine), on
the fixture graphs and on synthetic degree vectors -- including a maximum
degree that is a power of two, which degree_dist_ac leaves out of every
bucket."""
import numpy as np
import pytest

import oracle
from golden_data import FIXTURE_NAMES, load

needs_ref = pytest.mark.skipif(not oracle.ref_degree_available(),
                               reason="reference degree.c not compiled on this machine")


def _same(a, b):
    nb = len(b["dist_ac"])
    assert a["max"] == b["max"] and a["argmax"] == b["argmax"]
    assert a["mean"] == b["mean"]
    assert a["sd"] == b["sd"]
    assert np.array_equal(a["dist_ac"][:nb], b["dist_ac"])
    assert np.array_equal(a["dist_rel_ac"][:nb], b["dist_rel_ac"])
    assert (a["dist_ac"][nb:] == 0).all()


@needs_ref
@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_fixture_degrees_match_reference(name):
    fx = load(name)
    for deg in oracle.degree_vectors(fx.col_ptr, fx.row_idx, fx.symmetric):
        if deg.max() >= 2:
            _same(oracle.degree_stats(deg), oracle.ref_degree_stats(deg))


@needs_ref
@pytest.mark.parametrize("seed", range(8))
def test_synthetic_degrees_match_reference(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(3, 20000))
    deg = (rng.zipf(1.7, n).clip(1, 5000) - 1).astype(np.int32)
    if seed % 2 == 0:  # a maximum that is a power of two
        deg = np.minimum(deg, 1024)
        deg[int(rng.integers(0, n))] = 1024
    _same(oracle.degree_stats(deg), oracle.ref_degree_stats(deg))


def test_power_of_two_maximum_in_no_bucket():
    st = oracle.degree_stats(np.array([0, 8, 3, 8, 1, 2, 5], np.int32))
    assert st["max"] == 8 and st["argmax"] == 1
    assert st["dist_ac"][:5].tolist() == [1, 1, 2, 1, 0]  # deg 0, 1, [2,4), [4,8), never [8,16)
    assert st["mean"] == 27 / 7


def test_degree_vectors_directed_and_symmetric():
    cp = np.array([0, 1, 3, 3], np.int32)   # edges 1->0, 0->1, 2->1
    ic = np.array([1, 0, 2], np.int32)
    din, dout, und = oracle.degree_vectors(cp, ic, symmetric=False)
    assert din.tolist() == [1, 2, 0] and dout.tolist() == [1, 1, 1] and und.tolist() == [2, 3, 1]
    din, dout, und = oracle.degree_vectors(cp, ic, symmetric=True)
    assert und.tolist() == din.tolist()
