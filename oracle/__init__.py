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
        L.oracle_degree_stats.argtypes = [_P_I32, c_int, _P_I64, _P_I64, POINTER(c_double),
                                          POINTER(c_double), _P_I64, POINTER(c_double), c_int]
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


def degree_vectors(cp, ic, symmetric: bool):
    """(in, out, undirected) degree vectors of a CSC graph whose column v lists
    the sources u of edges u -> v: in = column lengths, out = row counts; the
    undirected degree is the reference's out_degree + in_degree of the file
    entries (TurboBFS_CSC_TD/degree.c:22-31, readMMfilef.c:56-70), which for a
    symmetric CSC (every entry mirrored) is the column length and otherwise
    in + out."""
    cp = np.asarray(cp, dtype=np.int64)
    n = cp.shape[0] - 1
    din = np.diff(cp).astype(np.int32)
    dout = np.bincount(np.asarray(ic, dtype=np.int64), minlength=n).astype(np.int32)
    und = din.copy() if symmetric else (din + dout).astype(np.int32)
    return din, dout, und


def degree_stats(deg, cap: int = 40):
    """Restatement of the reference's degree statistics of one degree vector:
    {max, argmax, mean, sd, dist_ac[cap], dist_rel_ac[cap]} (tbfs_oracle.h)."""
    deg = _i32(deg)
    mx, ix = np.zeros(1, np.int64), np.zeros(1, np.int64)
    mean, sd = c_double(), c_double()
    ac = np.zeros(cap, np.int64)
    rel = np.zeros(cap, np.float64)
    rc = lib().oracle_degree_stats(_p(deg, _P_I32), deg.shape[0], _p(mx, _P_I64), _p(ix, _P_I64),
                                   ctypes.byref(mean), ctypes.byref(sd), _p(ac, _P_I64),
                                   rel.ctypes.data_as(POINTER(c_double)), cap)
    if rc != 0:
        raise ValueError("degree_stats: cap too small for the maximum degree")
    return {"max": int(mx[0]), "argmax": int(ix[0]), "mean": mean.value, "sd": sd.value,
            "dist_ac": ac, "dist_rel_ac": rel}


# ------------------------------------------- the reference's own sources

_REF_LIBS = {
    "csc_td": "libref_csc_td.so",
    "csc_bu": "libref_csc_bu.so",
    "csc_tdbu": "libref_csc_tdbu.so",
    "cooc_td": "libref_cooc_td.so",
}
_REF_DEGREE = "libref_degree.so"


def ref_degree_available() -> bool:
    return (REF_DIR / _REF_DEGREE).exists()


def ref_degree_stats(deg):
    """The reference's own degree.c (compiled unchanged into oracle/_ref) run
    as its driver runs it (TurboBFS_CSC_TD/bfstdcsc_main.c:177-195):
    degree_max, degree_sta, degree_dist, degree_dist_rel, degree_dist_ac.
    Returns the restatement's layout: dist_ac[b] = degreeDistAc[0 / 1 /
    2^(b-1)].  Needs max >= 2 (the reference indexes degreeDistAc[1] of a
    maxDegree-long array)."""
    deg = _i32(deg)
    n = deg.shape[0]
    if "degree" not in _ref:
        _ref["degree"] = ctypes.CDLL(str(REF_DIR / _REF_DEGREE), mode=os.RTLD_LOCAL)
    L = _ref["degree"]
    mx, ix = c_int(0), c_int(-1)
    L.degree_max(_p(deg, _P_I32), ctypes.byref(mx), ctypes.byref(ix), n)
    mean, sd = c_double(), c_double()
    L.degree_sta(_p(deg, _P_I32), ctypes.byref(mean), ctypes.byref(sd), n)
    m = mx.value
    if m < 2:
        raise ValueError("ref_degree_stats needs a maximum degree of at least 2")
    dist = np.zeros(m + 1, np.int32)
    rel = np.zeros(m + 1, np.float64)
    ac = np.zeros(m, np.int32)
    relac = np.zeros(m, np.float64)
    L.degree_dist(_p(deg, _P_I32), _p(dist, _P_I32), n)
    L.degree_dist_rel(_p(dist, _P_I32), rel.ctypes.data_as(POINTER(c_double)), m, n)
    L.degree_dist_ac(_p(dist, _P_I32), rel.ctypes.data_as(POINTER(c_double)), _p(ac, _P_I32),
                     relac.ctypes.data_as(POINTER(c_double)), m)
    idx = [0, 1] + [1 << j for j in range(1, 40) if (1 << j) < m]
    return {"max": m, "argmax": ix.value, "mean": mean.value, "sd": sd.value,
            "dist_ac": ac[idx].astype(np.int64), "dist_rel_ac": relac[idx]}


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


# ------------------------------------- the reference's own GPU kernels

_refgpu = None


def refgpu_available() -> bool:
    """True when librefgpu.so and at least one of the reference's kernel
    images (oracle/_ref/*.cubin, built where the reference tree is) exist and
    a GPU is visible."""
    return _refgpu_lib() is not None and _refgpu_mask() != 0


def _refgpu_lib():
    global _refgpu
    if _refgpu is None:
        path = HERE / "librefgpu.so"
        if not path.exists():
            return None
        L = ctypes.CDLL(str(path))
        L.refgpu_load.argtypes = [ctypes.c_char_p]
        L.refgpu_last_error.restype = ctypes.c_char_p
        P = ctypes.POINTER(c_double)
        L.refgpu_td_csc_sc.argtypes = [_P_I32, _P_I32, _P_I32, _P_F32, c_int, c_int, c_int, P, _P_I32]
        L.refgpu_bu_csc_sc.argtypes = [_P_I32, _P_I32, _P_I32, c_int, c_int, c_int, c_int, P, _P_I32]
        L.refgpu_tdbu_csc_sc.argtypes = [_P_I32, _P_I32, _P_I32, _P_I32, c_int, c_int, c_int, c_int,
                                         P, _P_I32, _P_I32]
        L.refgpu_td_cooc_sc.argtypes = [_P_I32, _P_I32, _P_F32, c_int, c_int, c_int, P, _P_I32]
        _refgpu = L
    return _refgpu


def _refgpu_mask() -> int:
    L = _refgpu_lib()
    return 0 if L is None else int(L.refgpu_load(str(REF_DIR).encode()))


def _refgpu_call(name, *args):
    L = _refgpu_lib()
    if L is None or _refgpu_mask() == 0:
        raise RuntimeError("reference GPU kernel images not available")
    rc = getattr(L, name)(*args)
    if rc != 0:
        raise RuntimeError(f"{name}: {L.refgpu_last_error().decode()}")


def refgpu_tdbu_csc_sc(cp, ic, r, bbreak=1):
    """The reference's bfs_gpu_tdbu_csc_sc kernels on this GPU: (S, int32
    sigma, kernel ms, top-down levels, bottom-up levels)."""
    cp, ic = _i32(cp), _i32(ic)
    n = cp.shape[0] - 1
    S = np.zeros(n, np.int32)
    sg = np.zeros(n, np.int32)
    ms, td, bu = c_double(), np.zeros(1, np.int32), np.zeros(1, np.int32)
    _refgpu_call("refgpu_tdbu_csc_sc", _p(ic, _P_I32), _p(cp, _P_I32), _p(S, _P_I32),
                 _p(sg, _P_I32), int(r), ic.shape[0], n, int(bbreak), ctypes.byref(ms),
                 _p(td, _P_I32), _p(bu, _P_I32))
    return S, sg, ms.value, int(td[0]), int(bu[0])


def refgpu_td_csc_sc(cp, ic, r):
    """The reference's bfs_gpu_td_csc_sc kernels: (S, float sigma, ms, levels)."""
    cp, ic = _i32(cp), _i32(ic)
    n = cp.shape[0] - 1
    S = np.zeros(n, np.int32)
    sg = np.zeros(n, np.float32)
    ms, lv = c_double(), np.zeros(1, np.int32)
    _refgpu_call("refgpu_td_csc_sc", _p(ic, _P_I32), _p(cp, _P_I32), _p(S, _P_I32),
                 _p(sg, _P_F32), int(r), ic.shape[0], n, ctypes.byref(ms), _p(lv, _P_I32))
    return S, sg, ms.value, int(lv[0])


def refgpu_bu_csc_sc(cp, ic, r, bbreak=1):
    """The reference's bfs_gpu_bu_csc_sc kernel: (S, ms, levels)."""
    cp, ic = _i32(cp), _i32(ic)
    n = cp.shape[0] - 1
    S = np.zeros(n, np.int32)
    ms, lv = c_double(), np.zeros(1, np.int32)
    _refgpu_call("refgpu_bu_csc_sc", _p(ic, _P_I32), _p(cp, _P_I32), _p(S, _P_I32), int(r),
                 ic.shape[0], n, int(bbreak), ctypes.byref(ms), _p(lv, _P_I32))
    return S, ms.value, int(lv[0])


def refgpu_td_cooc_sc(I, J, n, r):
    """The reference's bfs_gpu_td_cooc_sc kernels: (float sigma, ms, levels)."""
    I, J = _i32(I), _i32(J)
    sg = np.zeros(n, np.float32)
    ms, lv = c_double(), np.zeros(1, np.int32)
    _refgpu_call("refgpu_td_cooc_sc", _p(I, _P_I32), _p(J, _P_I32), _p(sg, _P_F32), int(r),
                 I.shape[0], n, ctypes.byref(ms), _p(lv, _P_I32))
    return sg, ms.value, int(lv[0])
