"""Build recipe for the in-tree shared library ``turbobfs_gb300/libtbfs.so``.

The CUDA translation units are compiled for sm_103a only (GB300), the C host
tools with gcc, all in parallel, then linked with nvcc (static cudart).  No
PyTorch extension machinery is involved: the product is a plain C ABI.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libtbfs.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CU_SOURCES = ["bfs_engine.cu", "batch_engine.cu", "multi_engine.cu", "graph_ingest.cu", "api.cu",
              "batch_api.cu", "multi_api.cu", "brandes.cu", "tune.cu",
              "noalloc.cu", "mm_ingest.cu", "devmem.cu", "validate.cu", "cooc_engine.cu"]
C_SOURCES = ["host_graph.c"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtbfs.so")
    return cand


def _headers() -> list[Path]:
    return sorted(INCLUDE.glob("*.h")) + sorted(CSRC.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str], verbose: bool) -> str:
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n"
                           f"{res.stdout}\n{res.stderr}")
    return res.stdout + res.stderr


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False,
          defines: dict | None = None, lib_path: Path | None = None,
          build_dir: Path | None = None) -> Path:
    """Compile and link libtbfs.so if any source changed; return its path.

    `defines` sets the engine's compile-time tuning knobs (TBFS_EPT edges per
    lane per round, TBFS_BLOCK threads per CTA, TBFS_MIN_BLOCKS); a tuned
    variant is normally linked to its own `lib_path` / `build_dir`."""
    nvcc = nvcc_path()
    lib = Path(lib_path) if lib_path else LIB
    bdir = Path(build_dir) if build_dir else BUILD
    bdir.mkdir(parents=True, exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    inc = [f"-I{INCLUDE}", f"-I{CSRC}"]
    dflags = [f"-D{k}={v}" for k, v in sorted((defines or {}).items())]
    for src in CU_SOURCES:
        s = CSRC / src
        o = bdir / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "--expt-relaxed-constexpr", *dflags, *inc, "-c", str(s), "-o", str(o)]
            if ptxas_verbose:
                cmd.insert(3, "-Xptxas=-v")
            jobs.append(cmd)
    for src in C_SOURCES:
        s = CSRC / src
        o = bdir / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["gcc", "-O3", "-std=gnu11", "-fPIC", "-Wall", "-Wextra",
                         "-Wno-unused-parameter", *inc, "-c", str(s), "-o", str(o)])
    outputs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outputs = list(ex.map(lambda c: _run(c, verbose), jobs))
    if force or jobs or _stale(lib, objs):
        tmp = lib.with_suffix(".so.tmp")
        _run([nvcc, ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"], verbose)
        os.replace(tmp, lib)
    if ptxas_verbose:
        for out in outputs:
            sys.stdout.write(out)
    return lib


def build_oracle(verbose: bool = False) -> Path:
    """Build the checker: the CPU restatement (oracle/liboracle.so), the host
    driver of the reference's GPU kernel images (oracle/librefgpu.so) and, when
    the reference tree is present on this machine, the reference's own
    sequential sources and GPU kernel images (oracle/_ref/)."""
    odir = ROOT / "oracle"
    _run(["make", "-C", str(odir), "liboracle.so", "librefgpu.so", f"NVCC={nvcc_path()}"], verbose)
    # the reference tree: $TBFS_REFERENCE, else where the build container
    # mounts it; absent on other machines, which then use prebuilt files only
    ref = Path(os.environ.get("TBFS_REFERENCE") or "/root/reference")
    if (ref / "TurboBFS_CSC_TD").is_dir():
        _run(["make", "-C", str(odir), "ref", f"REF={ref}", f"NVCC={nvcc_path()}"], verbose)
        if LIB.exists():
            _run(["make", "-C", str(odir), "ref-dropin", f"REF={ref}"], verbose)
    return odir / "liboracle.so"


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv))
    print(build_oracle(verbose=True))
