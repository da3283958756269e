"""TEST INFRASTRUCTURE ONLY -- the parity checker.

ctypes front end of oracle/liboracle.so (tbfs_oracle.c: CPU restatement of
the reference's sequential BFS variants, emulations of what its GPU drivers
return, and an exact saturating-128-bit BFS) and, where they were built on
this machine, of the reference's own sequential sources compiled unchanged
into oracle/_ref/.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline import this package; the product never does.
"""
from __future__ import annotations

import contextlib
import ctypes
import os
import subprocess
import sys
from ctypes import POINTER, c_double, c_float, c_int, c_int64, c_uint8
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
_P_I32, _P_I64, _P_F32, _P_U8 = POINTER(c_int), POINTER(c_int64), POINTER(c_float), POINTER(c_uint8)

_lib = None
_ref = {}


def build() -> None:
    subprocess.run(["make", "-C", str(HERE), "liboracle.so"], check=True, capture_output=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = HERE / "liboracle.so"
        if not path.exists():
            build()
        L = ctypes.CDLL(str(path))
        L.oracle_seq_csc_f32.argtypes = [_P_I32, _P_I32, _P_I32, _P_F32, c_int, c_int, c_int, c_int]
        L.oracle_seq_csc_i32.argtypes = [_P_I32, _P_I32, _P_I32, _P_I32, c_int, c_int, c_int]
        L.oracle_seq_cooc_f32.argtypes = [_P_I32, _P_I32, _P_F32, c_int, c_int, c_int]
        L.oracle_exact_bfs.argtypes = [_P_I32, _P_I32, c_int, c_int, _P_I32, _P_I64, _P_U8]
        L.oracle_brandes.argtypes = [_P_I32, _P_I32, c_int, _P_I32, c_int,
                                     ctypes.POINTER(ctypes.c_double)]
        L.oracle_gpu_td_csc.argtypes = [_P_I32, _P_I32, _P_I32, _P_F32, c_int, c_int, c_int]
        L.oracle_gpu_bu_csc.argtypes = [_P_I32, _P_I32, _P_I32, c_int, c_int, c_int]
        L.oracle_gpu_tdbu_csc.argtypes = [_P_I32, _P_I32, _P_I32, _P_I32, c_int, c_int, c_int,
                                          _P_I32]
        L.oracle_gpu_td_cooc.argtypes = [_P_I32, _P_I32, _P_F32, c_int, c_int, c_int]
        L.oracle_seq_many.argtypes = [_P_I32, _P_I32, c_int, c_int, _P_I32, c_int, c_int,
                                      POINTER(c_double), _P_I64]
        L.oracle_seq_many.restype = c_double
        _lib = L
    return _lib


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _p(a, t):
    return a.ctypes.data_as(t)


# ------------------------------------------------------------ restatement

def seq_csc_f32(cp, ic, r, init_S):
    cp, ic = _i32(cp), _i32(ic)
    n = cp.shape[0] - 1
    S = np.zeros(n, np.int32)
    sg = np.zeros(n, np.float32)
    d = lib().oracle_seq_csc_f32(_p(ic, _P_I32), _p(cp, _P_I32), _p(S, _P_I32), _p(sg, _P_F32),
                                 r, ic.shape[0], n, 1 if init_S else 0)
    return S, sg, d


def seq_csc_i32(cp, ic, r):
    cp, ic = _i32(cp), _i32(ic)
    n = cp.shape[0] - 1
    S = np.zeros(n, np.int32)
    sg = np.zeros(n, np.int32)
    d = lib().oracle_seq_csc_i32(_p(ic, _P_I32), _p(cp, _P_I32), _p(S, _P_I32), _p(sg, _P_I32),
                                 r, ic.shape[0], n)
    return S, sg, d


def seq_cooc_f32(I, J, n, r):
    I, J = _i32(I), _i32(J)
    sg = np.zeros(n, np.float32)
    d = lib().oracle_seq_cooc_f32(_p(I, _P_I32), _p(J, _P_I32), _p(sg, _P_F32), r, I.shape[0], n)
    return sg, d


def exact_bfs(cp, ic, r):
    """(S, sigma int64, ovf uint8, levels): sigma exact below 2^63, ovf marks the rest."""
    cp, ic = _i32(cp), _i32(ic)
    n = cp.shape[0] - 1
    S = np.zeros(n, np.int32)
    sg = np.zeros(n, np.int64)
    ovf = np.zeros(n, np.uint8)
    lv = lib().oracle_exact_bfs(_p(cp, _P_I32), _p(ic, _P_I32), n, r, _p(S, _P_I32),
                                _p(sg, _P_I64), _p(ovf, _P_U8))
    return S, sg, ovf, lv


def brandes(orp, ojr, roots):
    """(bc float64[n], roots_with_wrapped_counts): betweenness over roots with
    the GPU sweep's summation order; (orp, ojr) are the out-lists."""
    orp, ojr = _i32(orp), _i32(ojr)
    roots = _i32(roots)
    n = orp.shape[0] - 1
    bc = np.zeros(n, np.float64)
    ovf = lib().oracle_brandes(_p(orp, _P_I32), _p(ojr, _P_I32), n, _p(roots, _P_I32),
                               int(roots.shape[0]), bc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return bc, int(ovf)


def gpu_td_csc(cp, ic, r):
    cp, ic = _i32(cp), _i32(ic)
    n = cp.shape[0] - 1
    S = np.zeros(n, np.int32)
    sg = np.zeros(n, np.float32)
    lib().oracle_gpu_td_csc(_p(ic, _P_I32), _p(cp, _P_I32), _p(S, _P_I32), _p(sg, _P_F32), r,
                            ic.shape[0], n)
    return S, sg


def gpu_bu_csc(cp, ic, r):
    cp, ic = _i32(cp), _i32(ic)
    n = cp.shape[0] - 1
    S = np.zeros(n, np.int32)
    lib().oracle_gpu_bu_csc(_p(ic, _P_I32), _p(cp, _P_I32), _p(S, _P_I32), r, ic.shape[0], n)
    return S


def gpu_tdbu_csc(cp, ic, r):
    cp, ic = _i32(cp), _i32(ic)
    n = cp.shape[0] - 1
    S = np.zeros(n, np.int32)
    sg = np.zeros(n, np.int32)
    sw = np.zeros(1, np.int32)
    lib().oracle_gpu_tdbu_csc(_p(ic, _P_I32), _p(cp, _P_I32), _p(S, _P_I32), _p(sg, _P_I32), r,
                              ic.shape[0], n, _p(sw, _P_I32))
    return S, sg, int(sw[0])


def gpu_td_cooc(I, J, n, r):
    I, J = _i32(I), _i32(J)
    sg = np.zeros(n, np.float32)
    lib().oracle_gpu_td_cooc(_p(I, _P_I32), _p(J, _P_I32), _p(sg, _P_F32), r, I.shape[0], n)
    return sg


def seq_many(cp, ic, roots, threads):
    """CPU baseline: reference-algorithm BFS from each root, `threads` at a time.
    Returns (wall seconds, per-root seconds, per-root edge counts)."""
    cp, ic, roots = _i32(cp), _i32(ic), _i32(roots)
    k = roots.shape[0]
    secs = np.zeros(k, np.float64)
    edges = np.zeros(k, np.int64)
    wall = lib().oracle_seq_many(_p(ic, _P_I32), _p(cp, _P_I32), ic.shape[0], cp.shape[0] - 1,
                                 _p(roots, _P_I32), k, threads,
                                 secs.ctypes.data_as(POINTER(c_double)), _p(edges, _P_I64))
    return wall, secs, edges


# ------------------------------------------- the reference's own sources

_REF_LIBS = {
    "csc_td": "libref_csc_td.so",
    "csc_bu": "libref_csc_bu.so",
    "csc_tdbu": "libref_csc_tdbu.so",
    "cooc_td": "libref_cooc_td.so",
}


def ref_available() -> bool:
    return all((REF_DIR / f).exists() for f in _REF_LIBS.values())


def _reflib(key):
    if key not in _ref:
        _ref[key] = ctypes.CDLL(str(REF_DIR / _REF_LIBS[key]), mode=os.RTLD_LOCAL)
    return _ref[key]


@contextlib.contextmanager
def _quiet_stdout():
    """The reference's BFS functions print timings; send fd 1 to /dev/null."""
    sys.stdout.flush()
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    try:
        os.dup2(devnull, 1)
        yield
    finally:
        libc = ctypes.CDLL(None)
        libc.fflush(None)
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)


def ref_seq_csc(variant, cp, ic, r):
    """Run the reference's bfs_seq_td_csc of `variant` (csc_td / csc_bu /
    csc_tdbu).  S starts zeroed and sigma zeroed, as the drivers' calloc does
    (TurboBFS_CSC_TD/bfstdcsc_main.c:134-137)."""
    cp, ic = _i32(cp), _i32(ic)
    n = cp.shape[0] - 1
    S = np.zeros(n, np.int32)
    sg = np.zeros(n, np.int32 if variant == "csc_tdbu" else np.float32)
    L = _reflib(variant)
    L.bfs_seq_td_csc.argtypes = [_P_I32, _P_I32, _P_I32, ctypes.c_void_p, c_int, c_int, c_int]
    with _quiet_stdout():
        L.bfs_seq_td_csc(_p(ic, _P_I32), _p(cp, _P_I32), _p(S, _P_I32),
                         sg.ctypes.data_as(ctypes.c_void_p), r, ic.shape[0], n)
    return S, sg


def ref_seq_cooc(I, J, n, r):
    I, J = _i32(I), _i32(J)
    sg = np.zeros(n, np.float32)
    L = _reflib("cooc_td")
    L.bfs_seq_td_cooc.argtypes = [_P_I32, _P_I32, _P_F32, c_int, c_int, c_int]
    with _quiet_stdout():
        L.bfs_seq_td_cooc(_p(I, _P_I32), _p(J, _P_I32), _p(sg, _P_F32), r, I.shape[0], n)
    return sg
