"""The drop-in from C.

* CPU: the reference's own TDBU driver program (bfstdbucsc_main.c and its C
  helpers, unchanged) linked against libtbfs.so instead of its .cu objects
  (oracle/Makefile target ref-dropin, built where the reference tree is):
  the executable resolves bfs_gpu_tdbu_csc_sc from libtbfs.so and runs to its
  S_check line.  Without a GPU the call returns TBFS_ERR_NO_DEVICE instead of
  crashing, so S_check reports the untouched vector.
* GPU: tests/c_dropin/dropin_main.c, a C caller of all seven entry points
  with calloc'd host arrays as the reference's drivers use them, is compiled
  with gcc against include/tbfs_compat.h and libtbfs.so and run on fixture
  graphs; its outputs equal the oracle's emulation of the reference drivers
  (where the reference's int32 arithmetic is exact) and the exact depths."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
import turbobfs_gb300 as tb
from golden_data import load
from turbobfs_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]
EXEC = ROOT / "oracle" / "_ref" / "tdbu_dropin_exec"


def _write_mm_lower(path, cp, ic):
    """Matrix Market text of a symmetric CSC: its lower triangle (row >= col),
    a diagonal entry (present twice in the symmetric CSC) once."""
    n = cp.shape[0] - 1
    col = np.repeat(np.arange(n), np.diff(cp))
    keep = ic >= col
    rows, cols = ic[keep], col[keep]
    diag = rows == cols
    if diag.any():
        d = np.flatnonzero(diag)
        rows = np.concatenate([rows[~diag], rows[d[::2]]])
        cols = np.concatenate([cols[~diag], cols[d[::2]]])
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern symmetric\n")
        f.write(f"{n} {n} {rows.shape[0]}\n")
        for i, j in zip(rows, cols):
            f.write(f"{i + 1} {j + 1}\n")


@pytest.mark.skipif(not EXEC.exists(), reason="reference driver not linked on this machine")
def test_reference_driver_links_against_libtbfs(tmp_path):
    out = subprocess.run(["ldd", str(EXEC)], capture_output=True, text=True).stdout
    assert str(_lib.LIB_PATH) in out
    fx = load("mycielskian4")
    mtx = tmp_path / "g.mtx"
    _write_mm_lower(mtx, fx.col_ptr, fx.row_idx)
    # exec file w ug format p r repet seq bbreak
    res = subprocess.run([str(EXEC), str(mtx), "0", "1", "0", "0", "0", "1", "1", "1"],
                         capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "check values of S_hgpu (sc)" in res.stdout
    if tb.device_count() > 0:
        assert "values of the GPU computed S vector are correct" in res.stdout


def _build_caller(tmp_path):
    exe = tmp_path / "dropin_main"
    subprocess.run(["gcc", "-O2", "-std=gnu11", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "c_dropin" / "dropin_main.c"), "-o", str(exe),
                    f"-L{_lib.LIB_PATH.parent}", f"-Wl,-rpath,{_lib.LIB_PATH.parent}", "-ltbfs"],
                   check=True, capture_output=True)
    return exe


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["mycielskian4", "Tina_AskCal", "Ragusa18", "luxembourg_osm",
                                  "rmat10"])
def test_c_caller_all_entry_points(gpu_available, tmp_path, name):
    exe = _build_caller(tmp_path)
    fx = load(name)
    n, nz = fx.n, fx.nnz
    I, J = fx.cooc()
    for i, r in enumerate(fx.roots[:2]):
        inp = tmp_path / "in.bin"
        np.concatenate([np.array([n, nz, r, 1], np.int32), fx.col_ptr.astype(np.int32),
                        fx.row_idx.astype(np.int32)]).tofile(inp)
        outp = tmp_path / "out.bin"
        subprocess.run([str(exe), str(inp), str(outp)], check=True, timeout=120)
        buf = np.fromfile(outp, dtype=np.int32)
        pos = 0

        def take(count):
            nonlocal pos
            a = buf[pos:pos + count]
            pos += count
            return a

        exact_S = fx.get("exact_S", i)
        exact = fx.get("exact_sigma", i)
        ovf = fx.get("exact_ovf", i).astype(bool)
        clean = not ovf.any() and exact.max() < 2**31
        Se, sge = oracle.gpu_td_csc(fx.col_ptr, fx.row_idx, r)
        for _ in range(2):  # td_csc _sc, _wa
            assert take(1)[0] == 0
            S, sg = take(n), take(n)
            assert np.array_equal(S, np.where(exact_S < 0, 0, exact_S))
            if clean:
                assert np.array_equal(sg, sge.view(np.int32))
        for _ in range(2):  # bu_csc _sc, _wa
            assert take(1)[0] == 0
            assert np.array_equal(take(n), oracle.gpu_bu_csc(fx.col_ptr, fx.row_idx, r))
        Se, sge, _ = oracle.gpu_tdbu_csc(fx.col_ptr, fx.row_idx, r)
        for _ in range(2):  # tdbu_csc _sc, _wa
            assert take(1)[0] == 0
            S, sg = take(n), take(n)
            assert np.array_equal(S, exact_S)
            if clean:
                assert np.array_equal(S, Se) and np.array_equal(sg, sge)
        assert take(1)[0] == 0  # td_cooc
        sg = take(n)
        if clean:
            assert np.array_equal(sg, oracle.gpu_td_cooc(I, J, n, r).view(np.int32))
        assert pos == buf.shape[0]
