"""Host graphs as numpy CSC arrays, built by the library's C graph tools
(include/tbfs_graphgen.h): Matrix Market loading with the reference's CSC
construction, seeded generators, largest component and root selection."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from ._lib import BUILD_DEDUP, BUILD_DROP_LOOPS, BUILD_SORT, BUILD_SYMMETRIZE, HostCSCStruct
from ._lib import check, lib


@dataclass
class HostCSC:
    """CSC adjacency: column v of (col_ptr, row_idx) lists the sources u of the
    edges u->v -- the reference's struct Csc (TurboBFS_CSC_TD/bfstdcsc.h:30-34)."""

    n: int
    col_ptr: np.ndarray  # int32[n+1]
    row_idx: np.ndarray  # int32[nnz]
    symmetric: bool = False

    @property
    def nnz(self) -> int:
        return int(self.row_idx.shape[0])

    def degrees(self) -> np.ndarray:
        return np.diff(self.col_ptr.astype(np.int64))

    def to_cooc(self) -> tuple[np.ndarray, np.ndarray]:
        """(I, J) with entry k the edge I[k] -> J[k], sorted by column: the
        reference's COOC (TurboBFS_COOC_TD/sparseformatransf.c:62-95)."""
        J = np.repeat(np.arange(self.n, dtype=np.int32), self.degrees())
        return self.row_idx.copy(), J

    def _struct(self) -> HostCSCStruct:
        cp = np.ascontiguousarray(self.col_ptr, dtype=np.int32)
        ic = np.ascontiguousarray(self.row_idx, dtype=np.int32)
        s = HostCSCStruct()
        s.n = self.n
        s.nnz = ic.shape[0]
        s.col_ptr = cp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        s.row_idx = ic.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        s._keep = (cp, ic)  # keep buffers alive while the struct is used
        return s


def _take(ptr, symmetric: bool) -> HostCSC:
    g = ptr.contents
    n, nnz = int(g.n), int(g.nnz)
    cp = np.ctypeslib.as_array(g.col_ptr, shape=(n + 1,)).copy()
    ic = np.ctypeslib.as_array(g.row_idx, shape=(max(nnz, 1),))[:nnz].copy()
    lib().tbfs_host_csc_free(ptr)
    return HostCSC(n, cp, ic, symmetric)


def _out():
    return ctypes.POINTER(HostCSCStruct)()


def from_edges(n: int, src, dst, symmetrize=False, drop_loops=False, dedup=False,
               sort=False) -> HostCSC:
    src = np.ascontiguousarray(src, dtype=np.int32)
    dst = np.ascontiguousarray(dst, dtype=np.int32)
    flags = ((BUILD_SYMMETRIZE if symmetrize else 0) | (BUILD_DROP_LOOPS if drop_loops else 0)
             | (BUILD_DEDUP if dedup else 0) | (BUILD_SORT if sort else 0))
    out = _out()
    P = ctypes.POINTER(ctypes.c_int32)
    check(lib().tbfs_csc_from_edges(n, src.ctypes.data_as(P), dst.ctypes.data_as(P),
                                    src.shape[0], flags, ctypes.byref(out)), "tbfs_csc_from_edges")
    return _take(out, symmetrize)


def read_mm(path: str | Path, undirected: bool) -> HostCSC:
    """Matrix Market file -> CSC exactly as the reference's drivers build it
    (undirected: stored entries mirrored, diagonal entries counted twice)."""
    out = _out()
    check(lib().tbfs_mm_read(str(path).encode(), 1 if undirected else 0, ctypes.byref(out)),
          f"tbfs_mm_read({path})")
    return _take(out, bool(undirected))


def erdos_renyi(n: int, m: int, seed: int = 1) -> HostCSC:
    out = _out()
    check(lib().tbfs_gen_er(n, m, seed, ctypes.byref(out)), "tbfs_gen_er")
    return _take(out, True)


def rmat(scale: int, edgefactor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 1, permute: bool = True) -> HostCSC:
    out = _out()
    check(lib().tbfs_gen_rmat(scale, edgefactor, a, b, c, seed, 1 if permute else 0,
                              ctypes.byref(out)), "tbfs_gen_rmat")
    return _take(out, True)


def grid(side: int, delete_frac: float = 0.10, chord_frac: float = 0.01, max_dist: int = 8,
         max_deg: int = 6, seed: int = 1) -> HostCSC:
    out = _out()
    check(lib().tbfs_gen_grid(side, delete_frac, chord_frac, max_dist, max_deg, seed,
                              ctypes.byref(out)), "tbfs_gen_grid")
    return _take(out, True)


def largest_component(g: HostCSC) -> np.ndarray:
    mask = np.zeros(g.n, dtype=np.uint8)
    size = ctypes.c_int64()
    s = g._struct()
    check(lib().tbfs_largest_component(ctypes.byref(s),
                                       mask.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                       ctypes.byref(size)), "tbfs_largest_component")
    return mask.astype(bool)


def pick_roots(g: HostCSC, k: int, seed: int = 1) -> np.ndarray:
    roots = np.zeros(k, dtype=np.int32)
    s = g._struct()
    check(lib().tbfs_pick_roots(ctypes.byref(s), k, seed,
                                roots.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))),
          "tbfs_pick_roots")
    return roots


def degree_profile(g: HostCSC) -> dict:
    hist = np.zeros(40, dtype=np.int64)
    mx = ctypes.c_int64()
    mean = ctypes.c_double()
    s = g._struct()
    check(lib().tbfs_degree_profile(ctypes.byref(s),
                                    hist.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                    ctypes.byref(mx), ctypes.byref(mean)), "tbfs_degree_profile")
    return {"hist_log2": hist, "max": int(mx.value), "mean": float(mean.value)}


def layered_bipartite(width: int, layers: int) -> HostCSC:
    """Root 0, then `layers` layers of `width` vertices, consecutive layers
    completely connected (undirected): the path count to the last layer is
    width**(layers-1).  Used to drive path counts past 2^63."""
    n = 1 + width * layers
    src, dst = [], []
    first = np.arange(1, 1 + width)
    src += [0] * width
    dst += first.tolist()
    for l in range(layers - 1):
        a = np.arange(1 + l * width, 1 + (l + 1) * width)
        b = a + width
        aa, bb = np.meshgrid(a, b, indexing="ij")
        src += aa.ravel().tolist()
        dst += bb.ravel().tolist()
    return from_edges(n, np.array(src), np.array(dst), symmetrize=True, dedup=True)
