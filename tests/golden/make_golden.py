"""Regenerate the golden vectors in tests/golden/*.npz.

Run on a machine that has the reference tree, after
`make -C oracle ref REF=<tree>`:

    TBFS_REFERENCE=<tree> python tests/golden/make_golden.py

For every reference fixture (graphData/*.mtx, loaded with the reference's
own CSC construction and the `ug` flag its run scripts use) and for a few
seeded synthetic graphs, this stores the CSC arrays and the outputs of the
REFERENCE's OWN sequential code (oracle/_ref, compiled unchanged from the
reference sources) for each root:
    td_S, td_sigma       TurboBFS_CSC_TD  bfs_seq_td_csc  (float sigma, S 0-init)
    bu_S, bu_sigma       TurboBFS_CSC_BU  bfs_seq_td_csc  (float sigma, S -1 init)
    tdbu_S, tdbu_sigma   TurboBFS_CSC_TDBU bfs_seq_td_csc (int32 sigma)
    cooc_sigma           TurboBFS_COOC_TD bfs_seq_td_cooc (float sigma)
plus the exact path counts of the saturating 128-bit oracle (exact_S,
exact_sigma, exact_ovf), which the native int64 engine must reproduce.
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from turbobfs_gb300 import graphs  # noqa: E402

OUT = Path(__file__).resolve().parent
if not os.environ.get("TBFS_REFERENCE"):
    sys.exit("make_golden.py: set TBFS_REFERENCE to the reference tree")
REF = Path(os.environ["TBFS_REFERENCE"])

# (name, ug, roots); roots follow the run scripts (TurboBFS_CSC_TD/run_bfstdcsc.sh:10-37)
FIXTURES = [
    ("mycielskian4", 1, [0, 5, 10]),
    ("Tina_AskCal", 0, [0, 10, 3]),
    ("Ragusa18", 0, [0, 7, 22]),
    ("cage4", 0, [0, 4, 8]),
    ("luxembourg_osm", 1, [0, 57000]),
]


def record(name: str, g, roots, meta: dict) -> None:
    data = {"col_ptr": g.col_ptr, "row_idx": g.row_idx, "roots": np.array(roots, np.int32)}
    I, J = g.to_cooc()
    for i, r in enumerate(roots):
        S, sg = oracle.ref_seq_csc("csc_td", g.col_ptr, g.row_idx, r)
        data[f"td_S_{i}"], data[f"td_sigma_{i}"] = S, sg
        S, sg = oracle.ref_seq_csc("csc_bu", g.col_ptr, g.row_idx, r)
        data[f"bu_S_{i}"], data[f"bu_sigma_{i}"] = S, sg
        S, sg = oracle.ref_seq_csc("csc_tdbu", g.col_ptr, g.row_idx, r)
        data[f"tdbu_S_{i}"], data[f"tdbu_sigma_{i}"] = S, sg
        data[f"cooc_sigma_{i}"] = oracle.ref_seq_cooc(I, J, g.n, r)
        S, sg, ovf, lv = oracle.exact_bfs(g.col_ptr, g.row_idx, r)
        data[f"exact_S_{i}"], data[f"exact_sigma_{i}"], data[f"exact_ovf_{i}"] = S, sg, ovf
    np.savez_compressed(OUT / f"{name}.npz", **data)
    meta[name] = {"n": g.n, "nnz": g.nnz, "roots": list(map(int, roots)),
                  "symmetric": bool(g.symmetric)}


def main() -> None:
    if not oracle.ref_available():
        sys.exit("oracle/_ref is not built: run `make -C oracle ref REF=<reference tree>`")
    meta = {}
    for name, ug, roots in FIXTURES:
        g = graphs.read_mm(REF / "graphData" / f"{name}.mtx", ug)
        record(name, g, roots, meta)
        meta[name]["source"] = f"graphData/{name}.mtx ug={ug}"
    # C1: Erdos-Renyi n=4096, 16384 undirected edges (average degree 8), seed 1, root 0
    er = graphs.erdos_renyi(4096, 16384, seed=1)
    record("er4096", er, [0, 1, 4095], meta)
    meta["er4096"]["source"] = "erdos_renyi(4096, 16384, seed=1)"
    rm = graphs.rmat(10, 16, seed=2)
    roots = graphs.pick_roots(rm, 3, seed=3).tolist()
    record("rmat10", rm, roots, meta)
    meta["rmat10"]["source"] = "rmat(10, 16, 0.57, 0.19, 0.19, seed=2, permute)"
    gr = graphs.grid(32, seed=4)
    record("grid32", gr, [0, 527], meta)
    meta["grid32"]["source"] = "grid(32, 0.10, 0.01, 8, 6, seed=4)"
    # path counts 16^16 = 2^64 at the last layer: past int64, int32 and float's exact range
    lb = graphs.layered_bipartite(16, 17)
    record("layered16x17", lb, [0], meta)
    meta["layered16x17"]["source"] = "layered_bipartite(16, 17)"
    (OUT / "golden_meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    total = sum(p.stat().st_size for p in OUT.glob("*.npz"))
    print(f"wrote {len(meta)} fixtures, {total / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
