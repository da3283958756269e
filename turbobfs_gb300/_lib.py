"""ctypes binding of libtbfs.so (the C ABI declared in include/*.h).

The library is built in-tree by ``turbobfs_gb300.build.build()``; importing a
GPU entry point without it raises immediately -- there is no fallback path.
"""
from __future__ import annotations

import ctypes
import threading
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_size_t
from ctypes import c_uint8, c_uint32, c_uint64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libtbfs.so"

TBFS_OK = 0
STATUS_NAMES = {
    0: "TBFS_OK",
    1: "TBFS_ERR_INVALID_ARG",
    2: "TBFS_ERR_CUDA",
    3: "TBFS_ERR_OUT_OF_MEMORY",
    4: "TBFS_ERR_TIMEOUT",
    5: "TBFS_ERR_NO_DEVICE",
    6: "TBFS_ERR_IO",
    7: "TBFS_ERR_UNSUPPORTED",
}
GRAPH_SYMMETRIC = 0x1
GRAPH_DEVICE_PTRS = 0x2
GRAPH_KEEP_ORDER = 0x4
LAYOUT_ROOT_MAJOR = 0
LAYOUT_VERTEX_MAJOR = 1
BATCH_MAX_ROOTS = 256
BUILD_SYMMETRIZE, BUILD_DROP_LOOPS, BUILD_DEDUP, BUILD_SORT = 0x1, 0x2, 0x4, 0x8


class Options(ctypes.Structure):
    _fields_ = [
        ("mode", c_int32),
        ("want_sigma", c_int32),
        ("outputs_on_device", c_int32),
        ("inject_barrier_skip", c_int32),
        ("alpha", c_float),
        ("beta", c_float),
        ("stream", c_void_p),
        ("timeout_ns", c_int64),
        ("level_trace", POINTER(c_int64)),
        ("level_trace_cap", c_int32),
        ("pull_ratio", c_float),
        ("max_ept", c_int32),
        ("ctas_per_sm", c_int32),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("levels", c_int32),
        ("td_levels", c_int32),
        ("bu_levels", c_int32),
        ("sigma_overflow", c_int32),
        ("visited", c_int64),
        ("edges", c_int64),
        ("device_ms", c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


DEGREE_IN, DEGREE_OUT, DEGREE_UNDIRECTED = 0, 1, 2
DEGREE_BUCKETS = 40


class DegreeStats(ctypes.Structure):
    _fields_ = [
        ("max_degree", c_int64),
        ("argmax", c_int64),
        ("sum", c_int64),
        ("mean", c_double),
        ("sd", c_double),
        ("dist_ac", c_int64 * DEGREE_BUCKETS),
        ("dist_rel_ac", c_double * DEGREE_BUCKETS),
    ]


class Validation(ctypes.Structure):
    _fields_ = [
        ("bad_root", c_int64),
        ("bad_depth", c_int64),
        ("skips_level", c_int64),
        ("no_parent", c_int64),
        ("sigma_mismatch", c_int64),
        ("first_bad", c_int64),
        ("visited", c_int64),
        ("edges", c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}

    def ok(self) -> bool:
        return (self.bad_root == 0 and self.bad_depth == 0 and self.skips_level == 0
                and self.no_parent == 0 and self.sigma_mismatch == 0)


class HostCSCStruct(ctypes.Structure):
    _fields_ = [
        ("n", c_int32),
        ("reserved", c_int32),
        ("nnz", c_int64),
        ("col_ptr", POINTER(c_int32)),
        ("row_idx", POINTER(c_int32)),
    ]


_P_I32 = POINTER(c_int32)
_P_I64 = POINTER(c_int64)
_P_F32 = POINTER(c_float)

_SIGNATURES = {
    # native engine (tbfs.h)
    "tbfs_options_init": (None, [POINTER(Options)]),
    "tbfs_graph_create_csc": (c_int, [_P_I32, _P_I32, c_int32, c_int64, c_uint32, POINTER(c_void_p)]),
    "tbfs_graph_create_cooc": (c_int, [_P_I32, _P_I32, c_int32, c_int64, c_uint32, POINTER(c_void_p)]),
    "tbfs_graph_destroy": (None, [c_void_p]),
    "tbfs_graph_info": (c_int, [c_void_p, _P_I32, _P_I64, POINTER(c_uint32)]),
    "tbfs_bfs": (c_int, [c_void_p, c_int32, POINTER(Options), _P_I32, _P_I64, POINTER(Stats)]),
    "tbfs_bfs_validate": (c_int, [c_void_p, c_int32, c_void_p, c_void_p, c_int32, c_void_p,
                                  POINTER(Validation)]),
    "tbfs_graph_last_stats": (c_int, [c_void_p, POINTER(Stats)]),
    "tbfs_bfs_many": (c_int, [c_void_p, _P_I32, c_int32, POINTER(Options), _P_I32, _P_I64,
                              POINTER(Stats)]),
    "tbfs_bfs_batch": (c_int, [c_void_p, _P_I32, c_int32, POINTER(Options), c_int32, c_void_p,
                               c_void_p, POINTER(Stats)]),
    "tbfs_graph_degree_profile": (c_int, [c_void_p, _P_I64, _P_I64, POINTER(c_double)]),
    "tbfs_graph_degree_stats": (c_int, [c_void_p, c_int32, POINTER(DegreeStats), _P_I64, c_int64]),
    "tbfs_graph_create_edges": (c_int, [_P_I32, _P_I32, c_int32, c_int64, c_uint32, c_uint32,
                                        POINTER(c_void_p)]),
    "tbfs_graph_create_mm": (c_int, [c_char_p, c_int64, c_int32, c_uint32, c_uint32,
                                     POINTER(c_void_p)]),
    "tbfs_graph_load_mm": (c_int, [c_char_p, c_int32, c_uint32, c_uint32, POINTER(c_void_p)]),
    "tbfs_graph_get_csc": (c_int, [c_void_p, _P_I32, _P_I32]),
    "tbfs_graph_get_cooc": (c_int, [c_void_p, _P_I32, _P_I32]),
    "tbfs_autotune": (c_int, [c_void_p, _P_I32, c_int32, c_char_p, POINTER(Options),
                              POINTER(c_int32)]),
    "tbfs_autotune_batch": (c_int, [c_void_p, _P_I32, c_int32, c_char_p, POINTER(Options),
                                    POINTER(c_int32)]),
    "tbfs_brandes": (c_int, [c_void_p, _P_I32, c_int32, POINTER(Options), c_void_p,
                             POINTER(c_int32)]),
    "tbfs_arena_create": (c_int, [c_int32, _P_I32, _P_I64, _P_I32, _P_I32, c_uint32,
                                  POINTER(c_void_p)]),
    "tbfs_arena_info": (c_int, [c_void_p, _P_I32, _P_I64, _P_I64]),
    "tbfs_arena_bfs": (c_int, [c_void_p, _P_I32, POINTER(Options), c_void_p, c_void_p,
                               POINTER(Stats)]),
    "tbfs_arena_destroy": (None, [c_void_p]),
    "tbfs_server_create": (c_int, [c_int32, c_int64, POINTER(Options), POINTER(c_void_p)]),
    "tbfs_server_submit": (c_int, [c_void_p, c_void_p, c_int32, c_void_p, c_void_p,
                                   POINTER(c_uint64)]),
    "tbfs_server_wait": (c_int, [c_void_p, c_uint64, POINTER(Stats), POINTER(c_double)]),
    "tbfs_server_counters": (c_int, [c_void_p, _P_I64, _P_I64, _P_I64]),
    "tbfs_server_time_split": (c_int, [c_void_p, POINTER(c_double), POINTER(c_double), POINTER(c_double),
                                        POINTER(c_int64), POINTER(c_int64)]),
    "tbfs_server_destroy": (None, [c_void_p]),
    "tbfs_bfs_noalloc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_int64,
                                 c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                                 POINTER(Stats)]),
    "tbfs_release_cached_memory": (c_int, []),
    "tbfs_host_alloc_pinned": (c_int, [c_size_t, POINTER(c_void_p)]),
    "tbfs_host_free_pinned": (None, [c_void_p]),
    "tbfs_status_string": (c_char_p, [c_int]),
    "tbfs_last_error": (c_char_p, []),
    "tbfs_version": (c_int32, []),
    "tbfs_device_count": (c_int32, []),
    # drop-in replacements (tbfs_compat.h)
    "bfs_gpu_td_csc_sc": (c_int, [_P_I32, _P_I32, _P_I32, _P_F32, c_int, c_int, c_int, c_int]),
    "bfs_gpu_td_csc_wa": (c_int, [_P_I32, _P_I32, _P_I32, _P_F32, c_int, c_int, c_int, c_int]),
    "bfs_gpu_bu_csc_sc": (c_int, [_P_I32, _P_I32, _P_I32, c_int, c_int, c_int, c_int, c_int]),
    "bfs_gpu_bu_csc_wa": (c_int, [_P_I32, _P_I32, _P_I32, c_int, c_int, c_int, c_int, c_int]),
    "bfs_gpu_tdbu_csc_sc": (c_int, [_P_I32, _P_I32, _P_I32, _P_I32, c_int, c_int, c_int, c_int, c_int]),
    "bfs_gpu_tdbu_csc_wa": (c_int, [_P_I32, _P_I32, _P_I32, _P_I32, c_int, c_int, c_int, c_int, c_int]),
    "bfs_gpu_td_cooc_sc": (c_int, [_P_I32, _P_I32, _P_F32, c_int, c_int, c_int, c_int]),
    # host graph tools (tbfs_graphgen.h)
    "tbfs_host_csc_free": (None, [POINTER(HostCSCStruct)]),
    "tbfs_csc_from_edges": (c_int, [c_int32, _P_I32, _P_I32, c_int64, c_uint32,
                                    POINTER(POINTER(HostCSCStruct))]),
    "tbfs_mm_read": (c_int, [c_char_p, c_int32, POINTER(POINTER(HostCSCStruct))]),
    "tbfs_gen_er": (c_int, [c_int32, c_int64, c_uint64, POINTER(POINTER(HostCSCStruct))]),
    "tbfs_gen_rmat": (c_int, [c_int32, c_int32, c_double, c_double, c_double, c_uint64, c_int32,
                              POINTER(POINTER(HostCSCStruct))]),
    "tbfs_gen_grid": (c_int, [c_int32, c_double, c_double, c_int32, c_int32, c_uint64,
                              POINTER(POINTER(HostCSCStruct))]),
    "tbfs_largest_component": (c_int, [POINTER(HostCSCStruct), POINTER(c_uint8), _P_I64]),
    "tbfs_pick_roots": (c_int, [POINTER(HostCSCStruct), c_int32, c_uint64, _P_I32]),
    "tbfs_degree_profile": (c_int, [POINTER(HostCSCStruct), _P_I64, _P_I64, POINTER(c_double)]),
}

_lock = threading.Lock()
_lib = None


def lib() -> ctypes.CDLL:
    """Load libtbfs.so once; raise if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is not built; run turbobfs_gb300.build.build() first "
                    "(there is no CPU fallback for the BFS engine)")
            handle = ctypes.CDLL(str(LIB_PATH))
            for name, (restype, argtypes) in _SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = restype
                fn.argtypes = argtypes
            _lib = handle
    return _lib


def exported_names() -> list[str]:
    return sorted(_SIGNATURES)


class TbfsError(RuntimeError):
    def __init__(self, status: int, where: str = ""):
        self.status = status
        detail = lib().tbfs_last_error().decode(errors="replace")
        name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"{where}: {name}: {detail}" if where else f"{name}: {detail}")


def check(status: int, where: str = "") -> None:
    if status != TBFS_OK:
        raise TbfsError(status, where)
