"""Python face of the engine.

Two layers, both thin wrappers over the C ABI:

* ``Graph`` -- a device-resident graph (``tbfs_graph_create_*``) with
  ``bfs`` / ``bfs_many`` returning numpy depth (int32, -1 unreached) and
  path-count (int64) vectors plus traversal statistics.
* ``bfs_gpu_td_csc_sc`` ... ``bfs_gpu_td_cooc_sc`` -- the reference's entry
  points under their own names and argument order
  (TurboBFS_CSC_TD/bfstdcsc.h:54-66, TurboBFS_CSC_BU/bfsbucsc.h:55-67,
  TurboBFS_CSC_TDBU/bfstdbucsc.h:56-68, TurboBFS_COOC_TD/bfstdcooc.h:48-49):
  host arrays in, results written into the caller's arrays, int status out.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from ._lib import (GRAPH_KEEP_ORDER, GRAPH_SYMMETRIC, LAYOUT_ROOT_MAJOR, LAYOUT_VERTEX_MAJOR,
                   DegreeStats, Options, Stats, Validation, check, lib)

MODES = {"auto": 0, "do": 0, "td": 1, "top_down": 1, "bu": 2, "bottom_up": 2}
_P_I32 = ctypes.POINTER(ctypes.c_int32)
_P_I64 = ctypes.POINTER(ctypes.c_int64)
_P_F32 = ctypes.POINTER(ctypes.c_float)


def _i32(a) -> np.ndarray:
    a = np.asarray(a)
    if a.dtype != np.int32 or not a.flags.c_contiguous:
        a = np.ascontiguousarray(a, dtype=np.int32)
    return a


def _ptr(a: np.ndarray, typ):
    return a.ctypes.data_as(typ)


def _flags(symmetric: bool, keep_order: bool) -> int:
    return (GRAPH_SYMMETRIC if symmetric else 0) | (GRAPH_KEEP_ORDER if keep_order else 0)


def make_options(mode="auto", sigma=True, alpha=None, beta=None, timeout_ns=0,
                 outputs_on_device=False, stream=None, inject_barrier_skip=0,
                 pull_ratio=None, max_ept=None, ctas_per_sm=None) -> Options:
    o = Options()
    lib().tbfs_options_init(ctypes.byref(o))
    o.mode = MODES[mode] if isinstance(mode, str) else int(mode)
    o.want_sigma = 1 if sigma else 0
    o.outputs_on_device = 1 if outputs_on_device else 0
    if alpha is not None:
        o.alpha = float(alpha)
    if beta is not None:
        o.beta = float(beta)
    o.timeout_ns = int(timeout_ns)
    o.stream = stream
    o.inject_barrier_skip = int(inject_barrier_skip)
    if pull_ratio is not None:
        o.pull_ratio = float(pull_ratio)
    if max_ept is not None:
        o.max_ept = int(max_ept)
    if ctas_per_sm is not None:
        o.ctas_per_sm = int(ctas_per_sm)
    return o


@dataclass
class BfsResult:
    S: np.ndarray                 # int32[n], -1 = unreached
    sigma: np.ndarray | None      # int64[n] path counts (None if not requested)
    stats: dict = field(default_factory=dict)


def _trace_buffer(o: Options, trace: int):
    if not trace:
        return None
    tr = np.zeros((max(int(trace), 2), 4), dtype=np.int64)
    o.level_trace = tr.ctypes.data_as(_P_I64)
    o.level_trace_cap = tr.shape[0]
    return tr


def _parse_trace(tr: np.ndarray):
    """Per-level records {level, start_us, vertices, edges, direction} with
    start_us relative to the first level, and the end time."""
    t0 = tr[0, 0]
    recs, end = [], None
    for d, (t, qn, qe, dr) in enumerate(tr.tolist()):
        if dr == -1:
            end = (t - t0) / 1e3
            break
        if t == 0:
            break
        recs.append({"level": d, "start_us": (t - t0) / 1e3, "vertices": qn,
                     "edges": qe, "direction": "bu" if dr == 1 else "td"})
    return recs, end


class Graph:
    """A graph resident in GPU memory until ``close()``."""

    def __init__(self, col_ptr, row_idx, n: int | None = None, symmetric: bool = False,
                 keep_order: bool = False):
        cp, ic = _i32(col_ptr), _i32(row_idx)
        self.n = int(n if n is not None else cp.shape[0] - 1)
        self.nnz = int(ic.shape[0])
        self.symmetric = bool(symmetric)
        h = ctypes.c_void_p()
        check(lib().tbfs_graph_create_csc(_ptr(cp, _P_I32), _ptr(ic, _P_I32), self.n, self.nnz,
                                          _flags(symmetric, keep_order), ctypes.byref(h)),
              "tbfs_graph_create_csc")
        self._h = h

    @classmethod
    def from_host_csc(cls, g, keep_order: bool = False) -> "Graph":
        return cls(g.col_ptr, g.row_idx, g.n, symmetric=g.symmetric, keep_order=keep_order)

    @classmethod
    def from_cooc(cls, I, J, n: int, symmetric: bool = False, keep_order: bool = False) -> "Graph":
        I, J = _i32(I), _i32(J)
        self = cls.__new__(cls)
        self.n, self.nnz, self.symmetric = int(n), int(I.shape[0]), bool(symmetric)
        h = ctypes.c_void_p()
        check(lib().tbfs_graph_create_cooc(_ptr(I, _P_I32), _ptr(J, _P_I32), self.n, self.nnz,
                                           _flags(symmetric, keep_order), ctypes.byref(h)),
              "tbfs_graph_create_cooc")
        self._h = h
        return self

    @classmethod
    def _adopt(cls, h: ctypes.c_void_p, symmetric: bool) -> "Graph":
        self = cls.__new__(cls)
        self._h = h
        n, nnz = ctypes.c_int32(), ctypes.c_int64()
        check(lib().tbfs_graph_info(h, ctypes.byref(n), ctypes.byref(nnz), None), "tbfs_graph_info")
        self.n, self.nnz, self.symmetric = int(n.value), int(nnz.value), bool(symmetric)
        return self

    @classmethod
    def from_edges(cls, src, dst, n: int, build_flags: int = 0,
                   keep_order: bool = False) -> "Graph":
        """Graph built on the device from the edge list src[k] -> dst[k] with
        the host builder's construction (``graphs.BUILD_*`` flags; the same
        CSC as ``graphs.from_edges`` with those flags)."""
        src, dst = _i32(src), _i32(dst)
        h = ctypes.c_void_p()
        check(lib().tbfs_graph_create_edges(_ptr(src, _P_I32), _ptr(dst, _P_I32), int(n),
                                            int(src.shape[0]), int(build_flags),
                                            _flags(False, keep_order), ctypes.byref(h)),
              "tbfs_graph_create_edges")
        return cls._adopt(h, bool(build_flags & 1))

    @classmethod
    def from_mm_text(cls, text: bytes, undirected: bool = True, build_flags: int = 0,
                     keep_order: bool = False) -> "Graph":
        """Graph from Matrix Market coordinate text, parsed on the device."""
        h = ctypes.c_void_p()
        check(lib().tbfs_graph_create_mm(text, len(text), 1 if undirected else 0,
                                         int(build_flags), _flags(False, keep_order),
                                         ctypes.byref(h)), "tbfs_graph_create_mm")
        return cls._adopt(h, undirected)

    @classmethod
    def load_mm(cls, path, undirected: bool = True, build_flags: int = 0,
                keep_order: bool = False) -> "Graph":
        """Graph from a Matrix Market file, parsed on the device."""
        h = ctypes.c_void_p()
        check(lib().tbfs_graph_load_mm(str(path).encode(), 1 if undirected else 0,
                                       int(build_flags), _flags(False, keep_order),
                                       ctypes.byref(h)), f"tbfs_graph_load_mm({path})")
        return cls._adopt(h, undirected)

    def csc(self):
        """The resident in-lists (col_ptr, row_idx) in the caller's numbering
        (graphs created with keep_order=True)."""
        cp = np.empty(self.n + 1, np.int32)
        ic = np.empty(max(self.nnz, 1), np.int32)
        check(lib().tbfs_graph_get_csc(self.handle, _ptr(cp, _P_I32), _ptr(ic, _P_I32)),
              "tbfs_graph_get_csc")
        return cp, ic[: self.nnz]

    def cooc(self):
        """The resident in-lists as COOC pairs (row, col), column order
        (graphs created with keep_order=True)."""
        row = np.empty(max(self.nnz, 1), np.int32)
        col = np.empty(max(self.nnz, 1), np.int32)
        check(lib().tbfs_graph_get_cooc(self.handle, _ptr(row, _P_I32), _ptr(col, _P_I32)),
              "tbfs_graph_get_cooc")
        return row[: self.nnz], col[: self.nnz]

    @property
    def handle(self) -> ctypes.c_void_p:
        if self._h is None:
            raise RuntimeError("graph is closed")
        return self._h

    def bfs(self, root: int, mode="auto", sigma: bool = True, trace: int = 0,
            **kw) -> BfsResult:
        """One traversal.  trace=k records up to k-1 levels: stats["trace"]
        lists {level, start_us, vertices, edges, direction ("td"/"bu")} with
        start_us relative to the first level, and stats["trace_end_us"]."""
        o = make_options(mode, sigma, **kw)
        S = np.empty(self.n, dtype=np.int32)
        sg = np.empty(self.n, dtype=np.int64) if sigma else None
        tr = _trace_buffer(o, trace)
        st = Stats()
        check(lib().tbfs_bfs(self.handle, int(root), ctypes.byref(o), _ptr(S, _P_I32),
                             _ptr(sg, _P_I64) if sg is not None else None, ctypes.byref(st)),
              "tbfs_bfs")
        stats = st.as_dict()
        if tr is not None:
            stats["trace"], stats["trace_end_us"] = _parse_trace(tr)
        return BfsResult(S, sg, stats)

    def bfs_many(self, roots, mode="auto", sigma: bool = True, **kw):
        roots = _i32(roots)
        k = int(roots.shape[0])
        o = make_options(mode, sigma, **kw)
        S = np.empty((k, self.n), dtype=np.int32)
        sg = np.empty((k, self.n), dtype=np.int64) if sigma else None
        stats = (Stats * max(k, 1))()
        check(lib().tbfs_bfs_many(self.handle, _ptr(roots, _P_I32), k, ctypes.byref(o),
                                  _ptr(S, _P_I32), _ptr(sg, _P_I64) if sg is not None else None,
                                  stats), "tbfs_bfs_many")
        return S, sg, [stats[i].as_dict() for i in range(k)]

    def bfs_batch(self, roots, mode="auto", sigma: bool = True, layout: str = "root",
                  trace: int = 0, **kw):
        """Frontier-matrix traversal from every root at once (256 per launch).
        Returns (S, sigma, stats) like bfs_many; layout "root" gives k x n
        arrays, "vertex" gives n x k.  trace=k records the levels of the first
        launch in stats[0]["trace"] (push levels show as "td", pull as "bu")."""
        roots = _i32(roots)
        k = int(roots.shape[0])
        o = make_options(mode, sigma, **kw)
        tr = _trace_buffer(o, trace)
        lay = LAYOUT_ROOT_MAJOR if layout == "root" else LAYOUT_VERTEX_MAJOR
        shape = (k, self.n) if lay == LAYOUT_ROOT_MAJOR else (self.n, k)
        S = np.empty(shape, dtype=np.int32)
        sg = np.empty(shape, dtype=np.int64) if sigma else None
        stats = (Stats * max(k, 1))()
        check(lib().tbfs_bfs_batch(self.handle, _ptr(roots, _P_I32), k, ctypes.byref(o), lay,
                                   S.ctypes.data, sg.ctypes.data if sg is not None else None,
                                   stats), "tbfs_bfs_batch")
        out = [stats[i].as_dict() for i in range(k)]
        if tr is not None and out:
            out[0]["trace"], out[0]["trace_end_us"] = _parse_trace(tr)
        return S, sg, out

    def degree_profile(self) -> dict:
        """{'hist': int64[40] (vertices per floor(log2(deg+1))), 'max', 'mean'},
        computed on the device."""
        h = np.zeros(40, dtype=np.int64)
        mx = ctypes.c_int64()
        mean = ctypes.c_double()
        check(lib().tbfs_graph_degree_profile(self.handle, _ptr(h, _P_I64), ctypes.byref(mx),
                                              ctypes.byref(mean)), "tbfs_graph_degree_profile")
        return {"hist": h, "max": int(mx.value), "mean": float(mean.value)}

    def validate(self, root: int, S, sigma=None) -> dict:
        """Check a BFS result (S int32[n], sigma int64[n] or None; numpy
        arrays, or torch CUDA tensors) against this graph on the device
        (tbfs_bfs_validate): violation counts by kind, 'first_bad', the
        reached vertices and their in-list entries, and 'ok'."""
        v = Validation()
        on_dev = hasattr(S, "data_ptr")
        if on_dev:
            s_ptr = S.data_ptr()
            g_ptr = sigma.data_ptr() if sigma is not None else None
        else:
            S = _i32(S)
            s_ptr = S.ctypes.data
            if sigma is not None:
                sigma = np.ascontiguousarray(sigma, dtype=np.int64)
            g_ptr = sigma.ctypes.data if sigma is not None else None
        check(lib().tbfs_bfs_validate(self.handle, int(root), s_ptr, g_ptr, 1 if on_dev else 0,
                                      None, ctypes.byref(v)), "tbfs_bfs_validate")
        out = v.as_dict()
        out["ok"] = v.ok()
        return out

    def degree_stats(self, kind: str = "undirected", full: bool = False) -> dict:
        """The reference driver's degree statistics (TurboBFS_CSC_TD/degree.c:22-141),
        computed on the device: {'max', 'argmax', 'sum', 'mean', 'sd',
        'dist_ac' int64[b], 'dist_rel_ac' float64[b]} with b the buckets in
        use (degree 0, 1, then [2^(j-1), 2^j) for 2^(j-1) < max), and with
        full=True 'dist' int64[max+1] (vertices per degree).  kind: 'in',
        'out' or 'undirected' (degree_ug: out + in of the entries)."""
        kinds = {"in": 0, "out": 1, "undirected": 2}
        st = DegreeStats()
        check(lib().tbfs_graph_degree_stats(self.handle, kinds[kind], ctypes.byref(st), None, 0),
              "tbfs_graph_degree_stats")
        nb = 2
        while nb < 40 and (1 << (nb - 1)) < st.max_degree:
            nb += 1
        out = {"max": int(st.max_degree), "argmax": int(st.argmax), "sum": int(st.sum),
               "mean": float(st.mean), "sd": float(st.sd),
               "dist_ac": np.array(st.dist_ac[:nb], dtype=np.int64),
               "dist_rel_ac": np.array(st.dist_rel_ac[:nb], dtype=np.float64)}
        if full:
            dist = np.zeros(st.max_degree + 1, dtype=np.int64)
            check(lib().tbfs_graph_degree_stats(self.handle, kinds[kind], ctypes.byref(st),
                                                _ptr(dist, _P_I64), dist.shape[0]),
                  "tbfs_graph_degree_stats")
            out["dist"] = dist
        return out

    def autotune(self, roots, cache: str | None = None, **kw) -> dict:
        """Tuned {'alpha', 'beta', 'pull_ratio', 'from_cache'} for this graph
        (timed on ``roots``; cached per degree profile in ``cache``)."""
        roots = _i32(roots)
        o = make_options("auto", True, **kw)
        fc = ctypes.c_int32()
        check(lib().tbfs_autotune(self.handle, _ptr(roots, _P_I32), int(roots.shape[0]),
                                  cache.encode() if cache else None, ctypes.byref(o),
                                  ctypes.byref(fc)), "tbfs_autotune")
        return {"alpha": o.alpha, "beta": o.beta, "pull_ratio": o.pull_ratio,
                "max_ept": o.max_ept, "ctas_per_sm": o.ctas_per_sm,
                "from_cache": bool(fc.value)}

    def autotune_batch(self, roots, cache: str | None = None, sigma: bool = True, **kw) -> dict:
        """Tuned {'alpha', 'from_cache'} of the frontier-matrix batch for
        these (<= 256) roots (timed batch launches; cached per degree profile
        and root count in ``cache``)."""
        roots = _i32(roots)
        o = make_options("auto", sigma, **kw)
        fc = ctypes.c_int32()
        check(lib().tbfs_autotune_batch(self.handle, _ptr(roots, _P_I32), int(roots.shape[0]),
                                        cache.encode() if cache else None, ctypes.byref(o),
                                        ctypes.byref(fc)), "tbfs_autotune_batch")
        return {"alpha": o.alpha, "from_cache": bool(fc.value)}

    def betweenness(self, roots=None, **kw):
        """Brandes betweenness over ``roots`` (default: every vertex):
        (bc float64[n], number of roots whose path counts overflowed).
        Unnormalised; an undirected graph counts every pair from both ends."""
        roots = _i32(np.arange(self.n) if roots is None else roots)
        o = make_options("auto", True, **kw)
        bc = np.zeros(self.n, dtype=np.float64)
        ovf = ctypes.c_int32()
        check(lib().tbfs_brandes(self.handle, _ptr(roots, _P_I32), int(roots.shape[0]),
                                 ctypes.byref(o), bc.ctypes.data, ctypes.byref(ovf)),
              "tbfs_brandes")
        return bc, int(ovf.value)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().tbfs_graph_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Arena:
    """Many graphs packed in one device arena, one BFS per graph per call
    (``tbfs_arena_*``).  ``graphs`` is a list of HostCSC (or objects with
    col_ptr, row_idx, n); S and sigma come back packed in arena order, with
    ``offsets[i]`` the first vertex of graph i."""

    def __init__(self, graphs, symmetric: bool | None = None):
        gs = list(graphs)
        if not gs:
            raise ValueError("Arena needs at least one graph")
        if symmetric is None:
            symmetric = all(getattr(g, "symmetric", False) for g in gs)
        n = np.array([int(g.n) for g in gs], dtype=np.int32)
        nnz = np.array([int(np.asarray(g.row_idx).shape[0]) for g in gs], dtype=np.int64)
        cp = np.concatenate([_i32(g.col_ptr) for g in gs])
        ic = np.concatenate([_i32(g.row_idx) for g in gs]) if nnz.sum() else np.zeros(1, np.int32)
        self.n, self.nnz = n, nnz
        self.offsets = np.concatenate([[0], np.cumsum(n.astype(np.int64))])
        h = ctypes.c_void_p()
        check(lib().tbfs_arena_create(len(gs), _ptr(n, _P_I32), _ptr(nnz, _P_I64), _ptr(cp, _P_I32),
                                      _ptr(ic, _P_I32), GRAPH_SYMMETRIC if symmetric else 0,
                                      ctypes.byref(h)), "tbfs_arena_create")
        self._h = h

    def bfs(self, roots, sigma: bool = True, **kw):
        roots = _i32(roots)
        if roots.shape[0] != self.n.shape[0]:
            raise ValueError("one root per graph")
        o = make_options("td", sigma, **kw)
        tot = int(self.offsets[-1])
        S = np.empty(tot, dtype=np.int32)
        sg = np.empty(tot, dtype=np.int64) if sigma else None
        stats = (Stats * len(roots))()
        check(lib().tbfs_arena_bfs(self._h, _ptr(roots, _P_I32), ctypes.byref(o), S.ctypes.data,
                                   sg.ctypes.data if sg is not None else None, stats),
              "tbfs_arena_bfs")
        return S, sg, [stats[i].as_dict() for i in range(len(roots))]

    def split(self, packed):
        return [packed[self.offsets[i]:self.offsets[i + 1]] for i in range(len(self.n))]

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().tbfs_arena_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The serving loop (``tbfs_server_*``): submit (graph, root) queries,
    wait for them; queries admitted while device memory allows run together
    (continuous batching).  Results land in pinned host buffers."""

    def __init__(self, max_slots: int = 256, mem_budget: int = 8 << 30, **kw):
        o = make_options("td", True, **kw)
        h = ctypes.c_void_p()
        check(lib().tbfs_server_create(int(max_slots), int(mem_budget), ctypes.byref(o),
                                       ctypes.byref(h)), "tbfs_server_create")
        self._h = h
        self._bufs = {}

    def submit(self, graph: "Graph", root: int, sigma: bool = True) -> int:
        S = np.empty(graph.n, dtype=np.int32)
        sg = np.empty(graph.n, dtype=np.int64) if sigma else None
        t = ctypes.c_uint64()
        check(lib().tbfs_server_submit(self._h, graph.handle, int(root), S.ctypes.data,
                                       sg.ctypes.data if sg is not None else None,
                                       ctypes.byref(t)), "tbfs_server_submit")
        self._bufs[t.value] = (S, sg)
        return t.value

    def wait(self, ticket: int):
        """(BfsResult, latency_ms) of a submitted query."""
        st = Stats()
        lat = ctypes.c_double()
        rc = lib().tbfs_server_wait(self._h, ctypes.c_uint64(ticket), ctypes.byref(st),
                                    ctypes.byref(lat))
        S, sg = self._bufs.pop(ticket)
        check(rc, "tbfs_server_wait")
        return BfsResult(S, sg, st.as_dict()), lat.value

    def counters(self) -> dict:
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().tbfs_server_counters(self._h, ctypes.byref(a), ctypes.byref(b),
                                         ctypes.byref(c)), "tbfs_server_counters")
        return {"launches": a.value, "levels": b.value, "completed": c.value}

    def time_split(self) -> dict:
        """Host wall time of the server thread by activity (ms, cumulative)."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        d, e = ctypes.c_int64(), ctypes.c_int64()
        check(lib().tbfs_server_time_split(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                           ctypes.byref(d), ctypes.byref(e)), "tbfs_server_time_split")
        return {"launch_ms": a.value, "plain_ms": b.value, "deliver_ms": c.value,
                "plain_runs": d.value, "slot_sum": e.value}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().tbfs_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- compat ---
# Same names, argument order and in-place outputs as the reference's C
# functions; the int return is 0 on success, a tbfs_status code otherwise.

def _outbuf(a, dtype, n: int, name: str) -> np.ndarray:
    if not (isinstance(a, np.ndarray) and a.dtype == dtype and a.flags.c_contiguous
            and a.shape[0] >= n):
        raise TypeError(f"{name} must be a contiguous {np.dtype(dtype).name} array of length >= n")
    return a


def bfs_gpu_td_csc_sc(IC_h, CP_h, S_h, sigma_h, r, nz, n, repetition=1) -> int:
    IC, CP = _i32(IC_h), _i32(CP_h)
    S, sg = _outbuf(S_h, np.int32, n, "S_h"), _outbuf(sigma_h, np.float32, n, "sigma_h")
    return lib().bfs_gpu_td_csc_sc(_ptr(IC, _P_I32), _ptr(CP, _P_I32), _ptr(S, _P_I32),
                                   _ptr(sg, _P_F32), r, nz, n, repetition)


def bfs_gpu_td_csc_wa(IC_h, CP_h, S_h, sigma_h, r, nz, n, repetition=1) -> int:
    IC, CP = _i32(IC_h), _i32(CP_h)
    S, sg = _outbuf(S_h, np.int32, n, "S_h"), _outbuf(sigma_h, np.float32, n, "sigma_h")
    return lib().bfs_gpu_td_csc_wa(_ptr(IC, _P_I32), _ptr(CP, _P_I32), _ptr(S, _P_I32),
                                   _ptr(sg, _P_F32), r, nz, n, repetition)


def bfs_gpu_bu_csc_sc(I_h, CP_h, S_h, r, nz, n, repetition=1, bbreak=1) -> int:
    I, CP = _i32(I_h), _i32(CP_h)
    S = _outbuf(S_h, np.int32, n, "S_h")
    return lib().bfs_gpu_bu_csc_sc(_ptr(I, _P_I32), _ptr(CP, _P_I32), _ptr(S, _P_I32), r, nz, n,
                                   repetition, bbreak)


def bfs_gpu_bu_csc_wa(I_h, CP_h, S_h, r, nz, n, repetition=1, bbreak=1) -> int:
    I, CP = _i32(I_h), _i32(CP_h)
    S = _outbuf(S_h, np.int32, n, "S_h")
    return lib().bfs_gpu_bu_csc_wa(_ptr(I, _P_I32), _ptr(CP, _P_I32), _ptr(S, _P_I32), r, nz, n,
                                   repetition, bbreak)


def bfs_gpu_tdbu_csc_sc(I_h, CP_h, S_h, sigma_h, r, nz, n, repetition=1, bbreak=1) -> int:
    I, CP = _i32(I_h), _i32(CP_h)
    S, sg = _outbuf(S_h, np.int32, n, "S_h"), _outbuf(sigma_h, np.int32, n, "sigma_h")
    return lib().bfs_gpu_tdbu_csc_sc(_ptr(I, _P_I32), _ptr(CP, _P_I32), _ptr(S, _P_I32),
                                     _ptr(sg, _P_I32), r, nz, n, repetition, bbreak)


def bfs_gpu_tdbu_csc_wa(IC_h, CP_h, S_h, sigma_h, r, nz, n, repetition=1, bbreak=1) -> int:
    IC, CP = _i32(IC_h), _i32(CP_h)
    S, sg = _outbuf(S_h, np.int32, n, "S_h"), _outbuf(sigma_h, np.int32, n, "sigma_h")
    return lib().bfs_gpu_tdbu_csc_wa(_ptr(IC, _P_I32), _ptr(CP, _P_I32), _ptr(S, _P_I32),
                                     _ptr(sg, _P_I32), r, nz, n, repetition, bbreak)


def bfs_gpu_td_cooc_sc(I_h, J_h, sigma_h, r, nz, n, repetition=1) -> int:
    I, J = _i32(I_h), _i32(J_h)
    sg = _outbuf(sigma_h, np.float32, n, "sigma_h")
    return lib().bfs_gpu_td_cooc_sc(_ptr(I, _P_I32), _ptr(J, _P_I32), _ptr(sg, _P_F32), r, nz,
                                    n, repetition)


COMPAT_FUNCTIONS = {
    "bfs_gpu_td_csc_sc": bfs_gpu_td_csc_sc,
    "bfs_gpu_td_csc_wa": bfs_gpu_td_csc_wa,
    "bfs_gpu_bu_csc_sc": bfs_gpu_bu_csc_sc,
    "bfs_gpu_bu_csc_wa": bfs_gpu_bu_csc_wa,
    "bfs_gpu_tdbu_csc_sc": bfs_gpu_tdbu_csc_sc,
    "bfs_gpu_tdbu_csc_wa": bfs_gpu_tdbu_csc_wa,
    "bfs_gpu_td_cooc_sc": bfs_gpu_td_cooc_sc,
}


def device_count() -> int:
    return int(lib().tbfs_device_count())


def release_cached_memory() -> None:
    """Hand the device memory the library's pool keeps after frees back to
    the CUDA driver (tbfs_release_cached_memory)."""
    check(lib().tbfs_release_cached_memory(), "tbfs_release_cached_memory")
