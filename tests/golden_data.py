"""Access to the golden vectors in tests/golden/ and a vectorised checker of
the BFS invariants used at sizes the oracle cannot reach quickly."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLDEN / "golden_meta.json").read_text())
FIXTURE_NAMES = sorted(META)
REFERENCE_FIXTURES = ["mycielskian4", "Tina_AskCal", "Ragusa18", "cage4", "luxembourg_osm"]


class Fixture:
    def __init__(self, name: str):
        self.name = name
        self.meta = META[name]
        self.d = np.load(GOLDEN / f"{name}.npz")
        self.col_ptr = self.d["col_ptr"]
        self.row_idx = self.d["row_idx"]
        self.roots = [int(r) for r in self.d["roots"]]
        self.n = int(self.col_ptr.shape[0] - 1)
        self.nnz = int(self.row_idx.shape[0])
        self.symmetric = bool(self.meta["symmetric"])

    def get(self, key: str, i: int) -> np.ndarray:
        return self.d[f"{key}_{i}"]

    def cooc(self):
        J = np.repeat(np.arange(self.n, dtype=np.int32), np.diff(self.col_ptr))
        return self.row_idx.astype(np.int32), J


def load(name: str) -> Fixture:
    return Fixture(name)


def bfs_invariants(col_ptr, row_idx, root, S, sigma=None) -> None:
    """Size-independent checks of a BFS result on a CSC graph (entry k of
    column v is the edge row_idx[k] -> v):
      * S[root] = 0; every edge u->v out of a reached u reaches v with
        S[v] <= S[u] + 1; every reached v != root has an in-neighbour at
        depth S[v] - 1; unreached vertices have S = -1;
      * sigma[root] = 1, sigma = 0 off the reached set, and sigma[v] equals
        the sum of sigma[u] over in-list entries u at depth S[v]-1 (mod 2^64,
        which also holds where the engine reported overflow, since its sums
        wrap in uint64)."""
    cp = np.asarray(col_ptr, dtype=np.int64)
    ic = np.asarray(row_idx, dtype=np.int64)
    n = cp.shape[0] - 1
    S = np.asarray(S)
    assert S.shape == (n,)
    assert S[root] == 0
    assert ((S >= 0) | (S == -1)).all()
    deg = np.diff(cp)
    col = np.repeat(np.arange(n, dtype=np.int64), deg)
    su, sv = S[ic], S[col]
    out_of_reached = su >= 0
    assert (sv[out_of_reached] >= 0).all(), "edge from a reached vertex to an unreached one"
    assert (sv[out_of_reached] <= su[out_of_reached] + 1).all(), "edge skips a level"
    parent = out_of_reached & (su == sv - 1)
    has_parent = np.zeros(n, dtype=bool)
    has_parent[col[parent]] = True
    need = S > 0
    assert has_parent[need].all(), "reached vertex without a parent one level up"
    if sigma is None:
        return
    sg = np.asarray(sigma).astype(np.uint64)
    assert sg[root] == 1
    assert (sg[S < 0] == 0).all()
    contrib = np.where(parent, sg[ic], np.uint64(0))
    sums = np.zeros(n, dtype=np.uint64)
    nonempty = deg > 0
    if contrib.shape[0]:
        red = np.add.reduceat(contrib, cp[:-1][nonempty])
        sums[nonempty] = red
    sums[root] = 1
    bad = np.nonzero(sums[S >= 0] != sg[S >= 0])[0]
    assert bad.size == 0, f"sigma differs from the parent sum at {bad.size} vertices"
