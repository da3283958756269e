"""turbobfs_gb300 -- GB300-native (sm_103a) linear-algebra BFS.

Depth vector S and shortest-path-count vector sigma of a CSC / COOC graph,
computed by one persistent CUDA kernel per traversal, behind the C ABI in
include/tbfs.h (native) and include/tbfs_compat.h (the reference's entry
points).  See ``turbobfs_gb300.api`` for the Python face.
"""
from .api import (COMPAT_FUNCTIONS, Arena, BfsResult, Graph, Server, bfs_gpu_bu_csc_sc, bfs_gpu_bu_csc_wa,
                  bfs_gpu_td_cooc_sc, bfs_gpu_td_csc_sc, bfs_gpu_td_csc_wa, bfs_gpu_tdbu_csc_sc,
                  bfs_gpu_tdbu_csc_wa, device_count, make_options,
                  release_cached_memory)
from ._lib import TbfsError, lib

__all__ = [
    "Graph", "Arena", "Server", "BfsResult", "TbfsError", "lib", "make_options", "device_count",
    "release_cached_memory",
    "COMPAT_FUNCTIONS", "bfs_gpu_td_csc_sc", "bfs_gpu_td_csc_wa", "bfs_gpu_bu_csc_sc",
    "bfs_gpu_bu_csc_wa", "bfs_gpu_tdbu_csc_sc", "bfs_gpu_tdbu_csc_wa", "bfs_gpu_td_cooc_sc",
]
