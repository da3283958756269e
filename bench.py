#!/usr/bin/env python3
"""Benchmark: direction-optimizing BFS with path counts on RMAT scale 22.

Workload: RMAT scale 22, edgefactor 16 (a/b/c/d = .57/.19/.19/.05, vertex ids
permuted, symmetrised, self-loops and duplicates removed: n = 4,194,304,
128.3M CSC entries), 64 seeded roots drawn from the giant component.  One
step = one BFS (depth S int32 + path counts sigma int64) from each of the 64
roots.  Metric: GTEPS = sum over roots of the undirected edges in the root's
component / time.

  value     device-timed (CUDA events on the launching stream, graph
            resident in HBM, outputs written to HBM)
  e2e       the same through the C ABI with host buffers: every step uploads
            the CSC from pinned host memory, runs the 64 traversals and
            copies every S and sigma back to pinned host memory
  roofline  the persistent BFS kernel: algorithmic bytes per traversal
            (4*nnz_c + 8*n_c + 12*n) / its mean CUDA-event duration, against
            the measured HBM copy bandwidth
  cpu_baseline  the reference's sequential BFS algorithm (oracle restatement)
            on the host cores, one BFS per core, on a sample of the roots

--impl reference times that CPU algorithm alone on this workload.
Under torchrun (N > 1) every rank runs the same workload on its own GPU
(replicas; BFS from a single source does not shard without a per-level
exchange) and value is the sum over ranks of the work / the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GTEPS (undirected edges in the root's component / BFS time), direction-optimizing BFS with path counts"
UNIT = "GTEPS"
WORKLOAD = "rmat22_do_bfs_sigma_64roots"


def parse_args(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["tbfs", "reference"], default="tbfs")
    p.add_argument("--scale", type=int, default=22)
    p.add_argument("--roots", type=int, default=64)
    p.add_argument("--mode", default="auto")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--cpu-threads", type=int, default=0)
    p.add_argument("--no-autotune", action="store_true",
                   help="default alpha/beta/pull_ratio instead of the autotuned ones")
    p.add_argument("--part", choices=["all", "batched", "serving", "ingest", "brandes",
                                      "directed", "grid"],
                   default="all", help="run only that report and print it")
    p.add_argument("--no-batched", action="store_true", help="skip the batched report")
    p.add_argument("--no-serving", action="store_true", help="skip the serving report")
    p.add_argument("--no-ingest", action="store_true", help="skip the ingest report")
    p.add_argument("--ingest-scale", type=int, default=21)
    p.add_argument("--no-directed", action="store_true", help="skip the directed-graph report")
    p.add_argument("--directed-scale", type=int, default=22)
    p.add_argument("--no-grid", action="store_true", help="skip the high-diameter grid report")
    p.add_argument("--grid-side", type=int, default=2048)
    p.add_argument("--no-brandes", action="store_true", help="skip the betweenness report")
    p.add_argument("--brandes-scale", type=int, default=20)
    p.add_argument("--brandes-roots", type=int, default=16)
    p.add_argument("--batch-scale", type=int, default=20)
    p.add_argument("--batch-roots", type=int, default=256)
    p.add_argument("--arena-graphs", type=int, default=512)
    p.add_argument("--serving-graphs", type=int, default=64)
    p.add_argument("--serving-max-scale", type=int, default=24)
    p.add_argument("--serving-max-side", type=int, default=4096)
    p.add_argument("--serving-rates", default="100,400,1600")
    p.add_argument("--serving-queries", type=int, default=2000)
    return p.parse_args(argv)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def make_workload(scale: int, nroots: int):
    from turbobfs_gb300 import graphs

    h = graphs.rmat(scale, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    roots = graphs.pick_roots(h, nroots, seed=1)
    return h, roots


def config(h, nroots, world, extra=None):
    c = {
        "workload": WORKLOAD if h.n == 1 << 22 else f"rmat{int(np.log2(h.n))}_do_bfs_sigma_{nroots}roots",
        "graph": "RMAT scale %d, edgefactor 16, a/b/c/d=.57/.19/.19/.05, permuted, symmetrised, "
                 "no self-loops, deduplicated" % int(np.log2(h.n)),
        "n": h.n,
        "nnz": h.nnz,
        "roots": nroots,
        "root_seed": 1,
        "graph_seed": 1,
        "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
        "l2": "inputs larger than L2 (CSC row_idx %d MB vs 126 MB L2); no flush" % (h.nnz * 4 // 2**20),
    }
    if extra:
        c.update(extra)
    return c


def cpu_threads(requested: int) -> int:
    n = requested if requested > 0 else (os.cpu_count() or 1)
    return max(1, min(n, 64))


def lscpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def cpu_baseline(h, roots, threads: int) -> dict:
    import oracle

    sample = roots[:threads]
    wall, secs, edges = oracle.seq_many(h.col_ptr, h.row_idx, sample, threads)
    gteps = float(edges.sum() / 2 / wall / 1e9)
    return {"value": gteps, "unit": UNIT, "cores": int(threads), "kind": "port",
            "sample": f"{len(sample)} of the {len(roots)} roots, one single-threaded BFS per "
                      f"core at a time ({lscpu_model()}); wall {wall:.2f} s, "
                      f"mean {float(np.mean(secs)):.2f} s per BFS",
            "algorithm": "restatement of TurboBFS_CSC_TDBU/bfstdcsc_seq.c (int sigma)"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        for line in (getattr(self, "out", "") or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        busy = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


KERNEL_SOURCES = ["turbobfs_gb300/csrc/bfs_engine.cu", "turbobfs_gb300/csrc/device_common.cuh",
                  "turbobfs_gb300/csrc/tbfs_internal.h"]


def kernel_source_hash() -> str:
    """sha256 over the single-source kernel's sources, in a fixed order."""
    import hashlib

    h = hashlib.sha256()
    for rel in KERNEL_SOURCES:
        h.update((ROOT / rel).read_bytes())
    return h.hexdigest()


def traffic_per_launch(scale: int):
    """dram bytes (read + write) per traversal from the committed ncu summary,
    with a note; None when the summary is absent or was measured on other
    kernel sources (its kernel_source_sha256 line differs from the sources
    built here)."""
    f = ROOT / "profiles" / f"bfs_persistent_kernel_rmat{scale}.md"
    if not f.exists():
        return None, f"no profiles/{f.name}"
    traffic, sha = None, None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                traffic = int(line.split(":", 1)[1].strip())
            except ValueError:
                traffic = None
        if line.startswith("kernel_source_sha256:"):
            sha = line.split(":", 1)[1].strip()
    if traffic is None:
        return None, f"profiles/{f.name} holds no traffic line"
    if sha != kernel_source_hash():
        return None, f"profiles/{f.name} was measured on other kernel sources"
    return traffic, f"ncu dram bytes of one launch, profiles/{f.name} (same kernel sources)"


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    h, roots = make_workload(args.scale, args.roots)
    threads = cpu_threads(args.cpu_threads)
    import oracle

    sample = roots[:threads]
    for _ in range(args.warmup):
        oracle.seq_many(h.col_ptr, h.row_idx, sample, threads)
    walls, edges_total = [], 0
    for _ in range(args.steps):
        wall, secs, edges = oracle.seq_many(h.col_ptr, h.row_idx, sample, threads)
        walls.append(wall)
        edges_total += int(edges.sum())
    t = sum(walls)
    value = edges_total / 2 / t / 1e9
    cb = {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
          "sample": f"each step: {len(sample)} of the {len(roots)} roots, one single-threaded "
                    f"BFS per core at a time ({lscpu_model()})",
          "algorithm": "restatement of TurboBFS_CSC_TDBU/bfstdcsc_seq.c (int sigma)"}
    # n_gpus: the N this arm was launched for, so the two arms' lines pair up;
    # the reference path itself runs on host cores only (cpu_baseline.cores)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": max(world, args.gpus),
            "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic (seeded RMAT generator)", "impl": "reference",
            "config": config(h, args.roots, 1, {"sample_roots_per_step": len(sample)}),
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    try:
        rg = reference_gpu(h, roots)
        if rg:
            line["reference_gpu"] = rg
    except Exception as exc:  # noqa: BLE001 -- reported in the line
        line["reference_gpu"] = {"error": repr(exc)}
    print(json.dumps(line), flush=True)
    return 0


def reference_gpu(h, roots, k=4):
    """The reference's own GPU kernels on this GPU (compiled unchanged for
    sm_103a, driven by the restatement of their host loops): the
    direction-optimizing bfs_gpu_tdbu_csc_sc kernels and the top-down
    bfs_gpu_td_csc_sc kernels, from k of the roots; GTEPS over the sum of
    their kernel times (the reference's own event timing of each launch).
    None when the kernel images were not built for this machine."""
    import oracle

    try:
        import torch

        if not torch.cuda.is_available():
            return None
    except Exception:  # noqa: BLE001
        return None
    if not oracle.refgpu_available():
        return None
    deg = np.diff(h.col_ptr.astype(np.int64))
    out = {"kernels": "TurboBFS_CSC_TDBU/bfsgputdbucsc_sc.cu, TurboBFS_CSC_TD/bfsgputdcsc_sc.cu "
                      "(thread per column) and TurboBFS_COOC_TD/bfsgputdcooc_sc.cu (thread per "
                      "entry), compiled unchanged for sm_103a; the warp-per-column variants are "
                      "not run (unsynchronised shared-memory staging)",
           "roots": k}
    J = np.repeat(np.arange(h.n, dtype=np.int32), deg)

    def cooc(cp, ic, r):  # edge-parallel COOC kernels; no S, reached = sigma > 0
        sg, ms, lv = oracle.refgpu_td_cooc_sc(ic, J, h.n, r)
        return (np.where(sg > 0, 1, -1), None, ms, lv)

    for name, fn in (("tdbu_csc_sc", oracle.refgpu_tdbu_csc_sc),
                     ("td_csc_sc", oracle.refgpu_td_csc_sc), ("td_cooc_sc", cooc)):
        fn(h.col_ptr, h.row_idx, int(roots[0]))  # warm-up (module load, first allocations)
        ms, edges, wall = 0.0, 0, 0.0
        for r in roots[:k]:
            t0 = time.perf_counter()
            res = fn(h.col_ptr, h.row_idx, int(r))
            wall += time.perf_counter() - t0
            S, t = res[0], res[2]
            ms += t
            reached = S >= 0 if name != "td_csc_sc" else (S > 0) | (np.arange(h.n) == r)
            edges += int(deg[reached].sum()) // 2
        out[name] = {"gteps_kernels": edges / (ms * 1e-3) / 1e9, "ms_per_bfs_kernels": ms / k,
                     "ms_per_call_wall": 1e3 * wall / k}
    return out


def aggregate(t_ms: float, units: float, world: int, device="cpu"):
    """Replicas: the slowest rank's time and the whole job's units (each rank
    ran its own copy of the workload; nothing is exchanged on the data
    path).  Returns (t_ms, units) unchanged for a single process."""
    if world <= 1:
        return float(t_ms), float(units)
    import torch
    import torch.distributed as dist

    tt = torch.tensor([float(t_ms)], dtype=torch.float64, device=device)
    uu = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    dist.all_reduce(uu, op=dist.ReduceOp.SUM)
    return float(tt.item()), float(uu.item())


def run_tbfs(args, world, rank, local):
    import torch

    import turbobfs_gb300 as tb
    from turbobfs_gb300 import _lib
    from turbobfs_gb300.api import _P_I32, _P_I64, make_options

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    h, roots = make_workload(args.scale, args.roots)
    k = int(roots.shape[0])
    n = h.n
    g = tb.Graph.from_host_csc(h)
    S_dev = torch.empty((k, n), dtype=torch.int32, device="cuda")
    sg_dev = torch.empty((k, n), dtype=torch.int64, device="cuda")
    tuning = {"autotuned": False}
    kw = {}
    if not args.no_autotune and args.mode == "auto":
        # the library's autotuner, timed on 8 of the roots (not cached)
        tu = g.autotune(roots[:8])
        kw = {k: v for k, v in tu.items() if k != "from_cache"}
        tuning = {"autotuned": True, "sample_roots": 8, **kw}
    o = make_options(args.mode, True, outputs_on_device=True, **kw)
    stats = (_lib.Stats * k)()
    roots_c = np.ascontiguousarray(roots, dtype=np.int32)
    import ctypes

    def step():
        _lib.check(tb.lib().tbfs_bfs_many(
            g.handle, roots_c.ctypes.data_as(_P_I32), k, ctypes.byref(o),
            ctypes.cast(S_dev.data_ptr(), _P_I32), ctypes.cast(sg_dev.data_ptr(), _P_I64),
            stats), "tbfs_bfs_many")

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 0)):
        step()
    edges_per_step = sum(stats[i].edges for i in range(k))
    per_root = [stats[i].as_dict() for i in range(k)]
    barrier()
    launch_ms = []
    with ClockSampler(local) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record()
        for _ in range(args.steps):
            step()
            launch_ms += [stats[i].device_ms for i in range(k)]
        e1.record()
        barrier()
    t_ms, units = aggregate(e0.elapsed_time(e1), args.steps * edges_per_step / 2, world, "cuda")
    value = units / (t_ms / 1e3) / 1e9
    parity = check_results(g, roots, S_dev, sg_dev, stats, kw)

    # roofline of the persistent BFS kernel
    alg_bytes = []
    for i in range(k):
        visited = int(per_root[i]["visited"])
        alg_bytes.append(4 * per_root[i]["edges"] + 8 * visited + 12 * n)
    mean_bytes = float(np.mean(alg_bytes))
    mean_launch_ms = float(np.mean(launch_ms))
    achieved = mean_bytes / (mean_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    traffic, traffic_note = traffic_per_launch(args.scale)

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(h, roots_c, args.steps, o, edges_per_step, world)

    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(h, roots, cpu_threads(args.cpu_threads))
    levels = [r["levels"] for r in per_root]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64",
        "data": "synthetic (seeded RMAT generator; no public dataset named)",
        "impl": "tbfs",
        "config": config(h, k, world, {"mode": args.mode, "tuning": tuning,
                                       "outputs": "S int32 + sigma int64 in HBM",
                                       "levels_min_max": [min(levels), max(levels)],
                                       "td_bu_levels_root0": [per_root[0]["td_levels"],
                                                              per_root[0]["bu_levels"]]}),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_note": traffic_note,
                     "kernel": "bfs_persistent_kernel",
                     "algorithmic_bytes_per_launch": mean_bytes,
                     "mean_launch_ms": mean_launch_ms,
                     "peak_source": f"{peak_kind} hbm_gbs"},
        "gpu_launches": args.steps * k,
        "clocks": clk.summary(),
    }
    line["parity"] = parity
    if e2e:
        line["e2e"] = e2e
    if cb:
        line["cpu_baseline"] = cb
    # secondary reports: a failure is recorded in its own key, so that the
    # headline line is still printed
    reports = [("batched", batched_report, args.no_batched),
               ("serving", serving_report, args.no_serving),
               ("ingest", ingest_report, args.no_ingest),
               ("brandes", brandes_report, args.no_brandes),
               ("directed", directed_report, args.no_directed),
               ("grid", grid_report, args.no_grid)]
    if rank == 0 and world == 1:
        for key, fn, skip in reports:
            if skip:
                continue
            try:
                line[key] = fn(args)
            except Exception as exc:  # noqa: BLE001 -- reported, not swallowed
                print(f"bench: {key} report failed: {exc!r}", file=sys.stderr, flush=True)
                line[key] = {"error": repr(exc)}
    line["summary"] = summary(line)
    if rank == 0:
        print(json.dumps(line), flush=True)
    g.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def check_results(g, roots, S_dev, sg_dev, stats, params):
    """Every timed traversal's S and sigma checked against the graph on the
    device (tbfs_bfs_validate: level-consistent edges, a parent for every
    reached vertex, sigma = sum of the parents' sigma), which pins both
    vectors uniquely; runs after the timed region."""
    bad, first = 0, None
    for i, r in enumerate(roots):
        v = g.validate(int(r), S_dev[i], sg_dev[i])
        if not v["ok"] or v["visited"] != stats[i].visited or stats[i].sigma_overflow:
            bad += 1
            first = first if first is not None else {"root": int(r), **v}
    out = {"roots_checked": len(roots), "mismatches": bad,
           "checker": "tbfs_bfs_validate on the device (Graph500-style invariants, sigma = parent "
                      "sum), on the results of the last timed step",
           "params": params or "defaults"}
    if first is not None:
        out["first_failure"] = first
    return out


def summary(line):
    """The headline numbers of every report in one short key, printed last."""
    out = {"value_gteps": round(line["value"], 2), "frac": round(line["roofline"]["frac"], 4),
           "parity_mismatches": line["parity"]["mismatches"]}
    if "e2e" in line:
        out["e2e_gteps"] = round(line["e2e"]["value"], 2)
        if "dropin_pageable" in line["e2e"]:
            out["dropin_pageable_gteps"] = round(line["e2e"]["dropin_pageable"]["value"], 2)
    b = line.get("batched", {}).get("frontier_matrix")
    if b:
        out["batched_speedup_vs_plain"] = round(b["speedup_vs_plain"], 3)
        out["batched_depths_only_speedup"] = round(b["depths_only"]["speedup_vs_plain"], 3)
        out["batched_frac_batch_bytes"] = round(b["roofline"]["frac"], 4)
    a = line.get("batched", {}).get("arena")
    if a:
        out["arena_speedup_vs_plain"] = round(a["speedup_vs_plain"], 2)
    sv = line.get("serving", {}).get("sweep")
    if sv:
        out["serving_p50_p99_ms"] = {str(int(x["rate_qps"])): [round(x["server"]["p50_ms"], 2),
                                                               round(x["server"]["p99_ms"], 2)]
                                     for x in sv}
    gr = line.get("grid", {}).get("auto")
    if gr:
        out["grid_us_per_level"] = round(gr["us_per_level"], 2)
    gt = line.get("grid", {}).get("autotuned")
    if gt:
        out["grid_us_per_level_autotuned"] = round(gt["us_per_level"], 2)
    return out


def run_e2e(h, roots_c, steps, o_dev, edges_per_step, world):
    """Public C ABI with host buffers: upload the CSC from pinned memory,
    traverse from every root, copy all S and sigma rows back to pinned memory."""
    import ctypes

    import turbobfs_gb300 as tb
    from turbobfs_gb300 import _lib
    from turbobfs_gb300.api import _P_I32, _P_I64, make_options

    L = tb.lib()
    k, n, nnz = int(roots_c.shape[0]), h.n, h.nnz

    def pinned(nbytes):
        p = ctypes.c_void_p()
        _lib.check(L.tbfs_host_alloc_pinned(nbytes, ctypes.byref(p)), "pinned")
        return p

    bufs = []
    try:
        p_cp, p_ic = pinned(4 * (n + 1)), pinned(4 * nnz)
        p_S, p_sg = pinned(4 * k * n), pinned(8 * k * n)
        bufs = [p_cp, p_ic, p_S, p_sg]
        cp = np.ctypeslib.as_array(ctypes.cast(p_cp, _P_I32), shape=(n + 1,))
        ic = np.ctypeslib.as_array(ctypes.cast(p_ic, _P_I32), shape=(nnz,))
        cp[:] = h.col_ptr
        ic[:] = h.row_idx
        o = make_options("auto", True)
        o.alpha, o.beta, o.mode = o_dev.alpha, o_dev.beta, o_dev.mode
        o.pull_ratio = o_dev.pull_ratio
        o.max_ept, o.ctas_per_sm = o_dev.max_ept, o_dev.ctas_per_sm
        stats = (_lib.Stats * k)()

        split = {"create_ms": 0.0, "traverse_and_copy_ms": 0.0, "destroy_ms": 0.0}

        def one(acc=None):
            hdl = ctypes.c_void_p()
            t0 = time.perf_counter()
            _lib.check(L.tbfs_graph_create_csc(ctypes.cast(p_cp, _P_I32), ctypes.cast(p_ic, _P_I32),
                                               n, nnz, _lib.GRAPH_SYMMETRIC, ctypes.byref(hdl)),
                       "tbfs_graph_create_csc")
            t1 = time.perf_counter()
            try:
                _lib.check(L.tbfs_bfs_many(hdl, roots_c.ctypes.data_as(_P_I32), k, ctypes.byref(o),
                                           ctypes.cast(p_S, _P_I32), ctypes.cast(p_sg, _P_I64),
                                           stats), "tbfs_bfs_many")
            finally:
                t2 = time.perf_counter()
                L.tbfs_graph_destroy(hdl)
                t3 = time.perf_counter()
            if acc is not None:
                acc["create_ms"] += 1e3 * (t1 - t0)
                acc["traverse_and_copy_ms"] += 1e3 * (t2 - t1)
                acc["destroy_ms"] += 1e3 * (t3 - t2)

        one()  # warm
        t0 = time.perf_counter()
        for _ in range(steps):
            one(split)
        t = time.perf_counter() - t0
        dev_ms = sum(stats[i].device_ms for i in range(k))
        split = {key: round(v / steps, 3) for key, v in split.items()}
        split["traversals_device_ms"] = round(dev_ms, 3)
        out = {"value": world * steps * edges_per_step / 2 / t / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": 4 * (n + 1) + 4 * nnz + 4 * k,
               "d2h_bytes_per_step": 12 * k * n,
               "ms_per_step": 1e3 * t / steps,
               "split_per_step": split,
               "path": "tbfs_graph_create_csc (pinned host CSC) + tbfs_bfs_many (pinned host "
                       "S/sigma) + tbfs_graph_destroy per step, host wall clock"}
        out["dropin_pageable"] = dropin_e2e(h, roots_c[:8])
        out["dropin_cooc_pageable"] = dropin_cooc_e2e(h, roots_c[:4])
        return out
    finally:
        for b in bufs:
            L.tbfs_host_free_pinned(b)


def dropin_e2e(h, roots):
    """The reference's own calling pattern: one bfs_gpu_tdbu_csc_sc call per
    root on calloc'd (pageable) host arrays (TurboBFS_CSC_TDBU/bfstdbucsc_main.c:
    127-137,294); every call uploads the CSC, traverses, copies S and sigma back
    and frees.  Host wall clock over the roots."""
    import turbobfs_gb300 as tb

    n, nnz = h.n, h.nnz
    S = np.zeros(n, np.int32)
    sg = np.zeros(n, np.int32)
    assert tb.bfs_gpu_tdbu_csc_sc(h.row_idx, h.col_ptr, S, sg, int(roots[0]), nnz, n, 1, 1) == 0
    edges = 0
    deg = np.diff(h.col_ptr.astype(np.int64))
    ts = []
    for r in roots:
        t0 = time.perf_counter()
        assert tb.bfs_gpu_tdbu_csc_sc(h.row_idx, h.col_ptr, S, sg, int(r), nnz, n, 1, 1) == 0
        ts.append(time.perf_counter() - t0)
        edges += int(deg[S >= 0].sum()) // 2  # the root's component edges, outside the timing
    t_med = float(np.median(ts))
    return {"value": edges / len(roots) / t_med / 1e9, "unit": UNIT, "roots": len(roots),
            "ms_per_call": 1e3 * t_med, "ms_per_call_mean": 1e3 * float(np.mean(ts)),
            "h2d_bytes_per_call": 4 * (n + 1) + 4 * nnz, "d2h_bytes_per_call": 8 * n,
            "path": "bfs_gpu_tdbu_csc_sc with pageable numpy arrays, one call per root; "
                    "median call (host memory speed varies from box to box)"}


def dropin_cooc_e2e(h, roots):
    """bfs_gpu_td_cooc_sc (TurboBFS_COOC_TD/bfstdcooc.h:48-49) on the same
    graph as COOC pairs with pageable host arrays, one call per root: the
    upload, the sort of the pairs into CSC on the device, the traversal and the
    float sigma's copy back, host wall clock."""
    import turbobfs_gb300 as tb

    n, nnz = h.n, h.nnz
    J = np.repeat(np.arange(n, dtype=np.int32), np.diff(h.col_ptr))
    sg = np.zeros(n, np.float32)
    assert tb.bfs_gpu_td_cooc_sc(h.row_idx, J, sg, int(roots[0]), nnz, n, 1) == 0
    deg = np.diff(h.col_ptr.astype(np.int64))
    ts, edges = [], 0
    for r in roots:
        t0 = time.perf_counter()
        assert tb.bfs_gpu_td_cooc_sc(h.row_idx, J, sg, int(r), nnz, n, 1) == 0
        ts.append(time.perf_counter() - t0)
        reached = (sg > 0) | (np.arange(n) == r)
        edges += int(deg[reached].sum()) // 2
    t_med = float(np.median(ts))
    return {"value": edges / len(roots) / t_med / 1e9, "unit": UNIT, "roots": len(roots),
            "ms_per_call": 1e3 * t_med, "ms_per_call_mean": 1e3 * float(np.mean(ts)),
            "path": "bfs_gpu_td_cooc_sc with pageable numpy arrays (row, column pairs), one call "
                    "per root, median call; a graph of at most 32 levels is traversed straight "
                    "over the pairs, a deeper one sorted into CSC first"}


# ------------------------------------------------------------ batched ----

def _event_ms(fn, reps=3, warm=3):
    import torch

    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def batched_report(args):
    """C4: (a) k roots on one RMAT graph as one frontier-matrix launch
    (tbfs_bfs_batch) against k back-to-back single-source traversals
    (tbfs_bfs_many) of the same roots; (b) many mixed graphs in one packed
    arena, one root each, in one launch (tbfs_arena_bfs) against one
    single-source traversal per resident graph.  Device outputs, CUDA-event
    timing on the legacy default stream both sides."""
    import ctypes

    import torch

    import turbobfs_gb300 as tb
    from turbobfs_gb300 import _lib, graphs
    from turbobfs_gb300.api import _P_I32, _P_I64, make_options

    L = tb.lib()
    out = {}
    # (a) frontier matrix
    h = graphs.rmat(args.batch_scale, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    k = args.batch_roots
    roots = np.ascontiguousarray(graphs.pick_roots(h, k, seed=1), dtype=np.int32)
    n = h.n
    with tb.Graph.from_host_csc(h) as g:
        S = torch.empty((k, n), dtype=torch.int32, device="cuda")
        sg = torch.empty((k, n), dtype=torch.int64, device="cuda")
        st = (_lib.Stats * k)()
        o = make_options("auto", True, outputs_on_device=True)

        def batch():
            _lib.check(L.tbfs_bfs_batch(g.handle, roots.ctypes.data_as(_P_I32), k, ctypes.byref(o),
                                        _lib.LAYOUT_ROOT_MAJOR, S.data_ptr(), sg.data_ptr(), st),
                       "tbfs_bfs_batch")

        def plain():
            _lib.check(L.tbfs_bfs_many(g.handle, roots.ctypes.data_as(_P_I32), k, ctypes.byref(o),
                                       ctypes.cast(S.data_ptr(), _P_I32),
                                       ctypes.cast(sg.data_ptr(), _P_I64), st), "tbfs_bfs_many")

        t_plain = _event_ms(plain)
        S_ref, sg_ref = S[::37].clone(), sg[::37].clone()
        t_batch = _event_ms(batch)
        same = bool(torch.equal(S[::37], S_ref) and torch.equal(sg[::37], sg_ref))
        edges = sum(st[i].edges for i in range(k)) / 2
        per_root = sum(4 * st[i].edges + 8 * st[i].visited + 12 * n for i in range(k))
        # the batch's own mandatory bytes: every root's S and sigma written once
        # (12 k n) and one pass over the lists and their pointers
        batch_bytes = 12 * k * n + 4 * h.nnz + 8 * n
        peak, peak_kind = measured_peak()
        out["frontier_matrix"] = {
            "workload": f"RMAT scale {args.batch_scale}, edgefactor 16, {k} roots in one launch, "
                        "S int32 + sigma int64 (root-major, in HBM)",
            "n": n, "nnz": h.nnz,
            "batched_gteps": edges / t_batch / 1e6, "batched_ms": t_batch,
            "plain_gteps": edges / t_plain / 1e6, "plain_ms": t_plain,
            "speedup_vs_plain": t_plain / t_batch,
            "launches": {"batched": (k + 255) // 256, "plain": k},
            "results_identical_to_plain": same,
            "roofline": {"bound": "hbm", "algorithmic_bytes": batch_bytes,
                         "achieved_gbs": batch_bytes / (t_batch / 1e3) / 1e9,
                         "frac": batch_bytes / (t_batch / 1e3) / 1e9 / peak,
                         "peak": peak, "peak_source": f"{peak_kind} hbm_gbs",
                         "note": "the batch's own bytes: 12 k n of S and sigma written once plus "
                                 "one pass over col_ptr / row_idx; the kernels' measured DRAM "
                                 "traffic is in profiles/fm_kernels_rmat19_256roots_traffic.md"},
            "per_root_bytes": {"bytes": per_root,
                               "gbs": per_root / (t_batch / 1e3) / 1e9,
                               "note": "sum over roots of 4 nnz_c + 8 n_c + 12 n, what k "
                                       "single-source traversals would read and write"},
        }
        o2 = make_options("auto", False, outputs_on_device=True)

        def batch_s():
            _lib.check(L.tbfs_bfs_batch(g.handle, roots.ctypes.data_as(_P_I32), k, ctypes.byref(o2),
                                        _lib.LAYOUT_ROOT_MAJOR, S.data_ptr(), None, st),
                       "tbfs_bfs_batch")

        def plain_s():
            _lib.check(L.tbfs_bfs_many(g.handle, roots.ctypes.data_as(_P_I32), k, ctypes.byref(o2),
                                       ctypes.cast(S.data_ptr(), _P_I32), None, st), "tbfs_bfs_many")

        tb_s, tp_s = _event_ms(batch_s), _event_ms(plain_s)
        out["frontier_matrix"]["depths_only"] = {
            "batched_gteps": edges / tb_s / 1e6, "plain_gteps": edges / tp_s / 1e6,
            "speedup_vs_plain": tp_s / tb_s}
        del S, sg
    # (b) packed arena of mixed graphs
    if args.arena_graphs > 0:
        rng = np.random.default_rng(5)
        gs, kinds = [], []
        for i in range(args.arena_graphs):
            lg = float(rng.uniform(10, 20))
            nv = int(2 ** lg)
            kind = ("er", "rmat", "grid")[i % 3]
            if kind == "er":
                hh = graphs.erdos_renyi(nv, 4 * nv, seed=100 + i)
            elif kind == "rmat":
                hh = graphs.rmat(max(1, int(round(lg))), 16, seed=100 + i)
            else:
                hh = graphs.grid(max(2, int(round(nv ** 0.5))), seed=100 + i)
            gs.append(hh)
            kinds.append(kind)
        aroots = np.array([int(graphs.pick_roots(hh, 1, seed=7)[0]) for hh in gs], dtype=np.int32)
        arena = tb.Arena(gs)
        tot = int(arena.offsets[-1])
        S = torch.empty(tot, dtype=torch.int32, device="cuda")
        sg = torch.empty(tot, dtype=torch.int64, device="cuda")
        ast = (_lib.Stats * len(gs))()
        oa = make_options("td", True, outputs_on_device=True)

        def arena_run():
            _lib.check(L.tbfs_arena_bfs(arena._h, aroots.ctypes.data_as(_P_I32), ctypes.byref(oa),
                                        S.data_ptr(), sg.data_ptr(), ast), "tbfs_arena_bfs")

        t_arena = _event_ms(arena_run)
        a_edges = sum(ast[i].edges for i in range(len(gs))) / 2
        a_levels = max(ast[i].levels for i in range(len(gs)))
        resident = [tb.Graph.from_host_csc(hh) for hh in gs]
        Sp = [torch.empty(hh.n, dtype=torch.int32, device="cuda") for hh in gs]
        sgp = [torch.empty(hh.n, dtype=torch.int64, device="cuda") for hh in gs]
        op = make_options("auto", True, outputs_on_device=True)
        pst = _lib.Stats()

        def plain_all():
            for gi, gg in enumerate(resident):
                _lib.check(L.tbfs_bfs(gg.handle, int(aroots[gi]), ctypes.byref(op),
                                      ctypes.cast(Sp[gi].data_ptr(), _P_I32),
                                      ctypes.cast(sgp[gi].data_ptr(), _P_I64), ctypes.byref(pst)),
                           "tbfs_bfs")

        t_plain_a = _event_ms(plain_all, reps=1, warm=1)
        same = True
        for gi in range(0, len(gs), 51):
            lo = int(arena.offsets[gi])
            same &= bool(torch.equal(S[lo:lo + gs[gi].n], Sp[gi]) and
                         torch.equal(sg[lo:lo + gs[gi].n], sgp[gi]))
        out["arena"] = {
            "workload": f"{len(gs)} graphs (ER avg degree 8 / RMAT edgefactor 16 / 2D grid, "
                        "n log-uniform in 2^10..2^20), one int32 offset arena, one root each "
                        "(giant component), one launch",
            "vertices": tot, "entries": int(arena.nnz.sum()), "max_levels": int(a_levels),
            "arena_gteps": a_edges / t_arena / 1e6, "arena_ms": t_arena,
            "plain_gteps": a_edges / t_plain_a / 1e6, "plain_ms": t_plain_a,
            "plain_path": "one direction-optimizing tbfs_bfs per resident graph, back to back",
            "speedup_vs_plain": t_plain_a / t_arena,
            "results_identical_to_plain": same}
        for gg in resident:
            gg.close()
        arena.close()
        del S, sg, Sp, sgp
    torch.cuda.empty_cache()
    return out


# ------------------------------------------------------------ serving ----

def serving_graph_set(count, max_scale, max_side):
    """count resident graphs: 5/8 RMAT (scales 12..max_scale, spread evenly,
    the largest once each), 3/8 grids (sides log-spaced 64..max_side)."""
    from turbobfs_gb300 import graphs

    n_rmat = (count * 5) // 8
    n_grid = count - n_rmat
    scales = np.linspace(12, max_scale, n_rmat).round().astype(int)
    sides = np.exp(np.linspace(np.log(64), np.log(max_side), n_grid)).round().astype(int)
    hs = []
    for i, sc in enumerate(scales):
        hs.append(("rmat%d" % sc, graphs.rmat(int(sc), 16, seed=200 + i)))
    for i, sd in enumerate(sides):
        hs.append(("grid%d" % sd, graphs.grid(int(sd), seed=300 + i)))
    return hs


def plain_fifo(gs, qg, qr, arrivals):
    """One-at-a-time serving on the same arrivals: a worker thread takes the
    queries in arrival order and runs each with tbfs_bfs (results to host
    memory) once it has arrived and the previous one finished.  Returns the
    latencies (ms, arrival to results in host memory), the span (s) and the
    service time of every query (s)."""
    import queue
    import threading

    q = queue.Queue()
    fin = np.zeros(len(qg))
    service = np.zeros(len(qg))
    t0 = time.perf_counter()

    def worker():
        while True:
            i = q.get()
            if i is None:
                return
            ts = time.perf_counter()
            gs[int(qg[i])].bfs(qr[i])
            fin[i] = time.perf_counter() - t0
            service[i] = fin[i] - (ts - t0)

    th = threading.Thread(target=worker, daemon=True)
    th.start()
    for i, a in enumerate(arrivals):
        now = time.perf_counter() - t0
        if a > now:
            time.sleep(a - now)
        q.put(i)
    q.put(None)
    th.join()
    return (fin - arrivals) * 1e3, float(fin.max() - arrivals[0]), list(service)


def serving_report(args):
    """C5: Poisson arrivals of (graph, root) queries over resident graphs,
    swept rate; the server (continuous batching) against the plain path
    (one tbfs_bfs at a time, FIFO)."""
    import turbobfs_gb300 as tb
    from turbobfs_gb300 import graphs

    t_gen = time.perf_counter()
    hs = serving_graph_set(args.serving_graphs, args.serving_max_scale, args.serving_max_side)
    t_gen = time.perf_counter() - t_gen
    gs = [tb.Graph.from_host_csc(h) for _, h in hs]
    hbm = sum(4 * (h.n + 1) + 4 * h.nnz for _, h in hs)
    rng = np.random.default_rng(9)
    nq = args.serving_queries
    qg = rng.integers(0, len(gs), nq)
    qr = []
    for gi in qg:
        h = hs[int(gi)][1]
        # roots uniform over non-isolated vertices
        deg = np.diff(h.col_ptr)
        nz = np.flatnonzero(deg)
        qr.append(int(nz[int(rng.integers(0, nz.size))]) if nz.size else 0)
    # every graph's workspace warmed once; per-query edges from one
    # traversal each (not timed)
    for g in gs:
        g.bfs(0)
    edges_total = 0.0
    for gi, r in zip(qg, qr):
        edges_total += gs[int(gi)].bfs(r).stats["edges"] / 2
    svc = []
    rates = [float(x) for x in args.serving_rates.split(",") if x]
    sweep = []
    with tb.Server(max_slots=512, mem_budget=48 << 30) as srv:
        for rate in rates:
            gaps = rng.exponential(1.0 / rate, nq)
            arrivals = np.cumsum(gaps)
            # plain path, run for real: one host thread serves the queries
            # one at a time (tbfs_bfs, results to host memory) in arrival
            # order, fed at the same arrival times
            lat_p, plain_span, service = plain_fifo(gs, qg, qr, arrivals)
            svc.extend(service)
            # server: submit at the arrival times, wait for all
            c0, ts0 = srv.counters(), srv.time_split()
            tickets = []
            t0 = time.perf_counter()
            for a, gi, r in zip(arrivals, qg, qr):
                now = time.perf_counter() - t0
                if a > now:
                    time.sleep(a - now)
                tickets.append(srv.submit(gs[int(gi)], r))
            lat_s = []
            for tk in tickets:
                _, lat = srv.wait(tk)
                lat_s.append(lat)
            span = time.perf_counter() - t0
            c1, ts1 = srv.counters(), srv.time_split()
            nl = max(1, c1["launches"] - c0["launches"])
            split = {k: round(ts1[k] - ts0[k], 3) for k in ("launch_ms", "plain_ms", "deliver_ms")}
            split["routed_queries"] = ts1["plain_runs"] - ts0["plain_runs"]
            split["mean_slots_per_launch"] = round((ts1["slot_sum"] - ts0["slot_sum"]) / nl, 2)
            lat_s = np.array(lat_s)
            sweep.append({
                "rate_qps": rate, "queries": nq,
                "server": {"p50_ms": float(np.percentile(lat_s, 50)),
                           "p99_ms": float(np.percentile(lat_s, 99)),
                           "gteps": edges_total / span / 1e9, "span_s": span,
                           "launches": c1["launches"] - c0["launches"],
                           "levels": c1["levels"] - c0["levels"],
                           "server_thread": split},
                "plain_fifo": {"p50_ms": float(np.percentile(lat_p, 50)),
                               "p99_ms": float(np.percentile(lat_p, 99)),
                               "gteps": edges_total / plain_span / 1e9, "span_s": plain_span},
            })
    # results of the mix equal the plain results (spot check)
    same = True
    with tb.Server(max_slots=64, mem_budget=16 << 30) as srv:
        sel = list(range(0, nq, max(1, nq // 24)))
        tks = [srv.submit(gs[int(qg[i])], qr[i]) for i in sel]
        for i, tk in zip(sel, tks):
            res, _ = srv.wait(tk)
            alone = gs[int(qg[i])].bfs(qr[i])
            same &= bool(np.array_equal(res.S, alone.S) and np.array_equal(res.sigma, alone.sigma))
    for g in gs:
        g.close()
    return {"workload": f"{len(hs)} resident graphs: {sum(1 for nm, _ in hs if nm.startswith('rmat'))} "
                        f"RMAT (scales 12..{args.serving_max_scale}), "
                        f"{sum(1 for nm, _ in hs if nm.startswith('grid'))} grids (sides 64..{args.serving_max_side}); "
                        "(graph, root) uniform; Poisson arrivals; S + sigma copied to host per query",
            "graph_bytes": hbm, "generation_s": t_gen,
            "plain_mean_service_ms": float(np.mean(svc) * 1e3),
            "sweep": sweep, "results_identical_to_plain": same,
            "latency": "submit to results in host memory, host wall clock; server: continuous "
                       "batching; plain: one host thread running tbfs_bfs one query at a time in "
                       "arrival order on the same arrivals"}


def mm_text(h) -> bytes:
    """Matrix Market text of a symmetric CSC: its lower triangle (row > column,
    1-based), one entry per line, indices right-aligned in fixed-width fields."""
    col = np.repeat(np.arange(h.n, dtype=np.int64), np.diff(h.col_ptr))
    row = h.row_idx.astype(np.int64)
    keep = row > col
    i, j = row[keep] + 1, col[keep] + 1
    w = len(str(h.n))
    lines = np.full((i.shape[0], 2 * w + 2), ord(" "), dtype=np.uint8)
    for field, x in ((0, i), (1, j)):
        v = x.copy()
        for d in range(w - 1, -1, -1):
            digit = (v % 10).astype(np.uint8) + ord("0")
            pos = field * (w + 1) + d
            lines[:, pos] = np.where((v > 0) | (d == w - 1), digit, ord(" "))
            v //= 10
    lines[:, -1] = ord("\n")
    head = ("%%%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n"
            % (h.n, h.n, i.shape[0])).encode()
    return head + lines.tobytes()


def ingest_report(args):
    """Matrix Market text -> resident graph: the host reader (the reference's
    sequential construction) plus an upload, against the text parsed and the
    CSC built on the device (tbfs_graph_load_mm), on the same file."""
    import tempfile

    import turbobfs_gb300 as tb
    from turbobfs_gb300 import graphs

    scale = args.ingest_scale
    h = graphs.rmat(scale, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    text = mm_text(h)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "rmat.mtx")
        with open(path, "wb") as f:
            f.write(text)
        # warm-up of both paths (page cache, CUDA context, first allocations)
        with tb.Graph.load_mm(path, True) as g:
            pass
        t0 = time.perf_counter()
        hh = graphs.read_mm(path, True)
        t1 = time.perf_counter()
        with tb.Graph.from_host_csc(hh) as g:
            t2 = time.perf_counter()
        host_ms, upload_ms = (t1 - t0) * 1e3, (t2 - t1) * 1e3
        dev = []
        for _ in range(3):
            t3 = time.perf_counter()
            with tb.Graph.load_mm(path, True) as g:
                t4 = time.perf_counter()
            dev.append((t4 - t3) * 1e3)
        mem = []
        for _ in range(3):
            t5 = time.perf_counter()
            with tb.Graph.from_mm_text(text, True) as g:
                t6 = time.perf_counter()
            mem.append((t6 - t5) * 1e3)
        with tb.Graph.load_mm(path, True, keep_order=True) as g:
            cp, ic = g.csc()
        same = bool(np.array_equal(cp, hh.col_ptr) and np.array_equal(ic, hh.row_idx))
    return {"workload": f"RMAT scale {scale} lower triangle as Matrix Market text "
                        f"({len(text) / 2**20:.0f} MiB, {hh.nnz // 2} entries), undirected",
            "n": int(hh.n), "nnz": int(hh.nnz), "text_bytes": len(text),
            "host_reader_ms": host_ms, "host_upload_ms": upload_ms,
            "host_path_ms": host_ms + upload_ms,
            "device_load_mm_ms": min(dev), "device_from_text_ms": min(mem),
            "speedup_vs_host_path": (host_ms + upload_ms) / min(dev),
            "csc_identical_to_host_reader": same,
            "timing": "host wall clock around each call, after one warm-up; device path = file "
                      "read into pinned memory + parse + build + degree grouping + resident "
                      "graph; host path = tbfs_mm_read + tbfs_graph_create_csc"}


def brandes_report(args):
    """Betweenness (forward traversal + dependency sweep per root) on RMAT:
    device time per root through tbfs_brandes, against the oracle's
    single-threaded restatement of the same computation (the CPU baseline,
    also the bit-exact checker) on two of the roots."""
    import oracle
    import turbobfs_gb300 as tb
    from turbobfs_gb300 import graphs

    scale, k = args.brandes_scale, args.brandes_roots
    h = graphs.rmat(scale, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    roots = graphs.pick_roots(h, k, seed=3)
    with tb.Graph.from_host_csc(h) as g:
        g.betweenness(roots[:2])  # warm-up
        t0 = time.perf_counter()
        bc, ovf = g.betweenness(roots)
        gpu_s = time.perf_counter() - t0
        bc2, _ = g.betweenness(roots[:2])
    t1 = time.perf_counter()
    want, _ = oracle.brandes(h.col_ptr, h.row_idx, roots[:2])
    cpu_s = time.perf_counter() - t1
    deg = np.diff(h.col_ptr).astype(np.int64)
    S, _, _, _ = oracle.exact_bfs(h.col_ptr, h.row_idx, int(roots[0]))
    m_c = int(deg[S >= 0].sum()) // 2
    return {"workload": f"RMAT scale {scale}, edgefactor 16, {k} roots from the giant component, "
                        "unnormalised betweenness (S, sigma forward + Brandes sweep per root)",
            "n": int(h.n), "nnz": int(h.nnz), "roots": k, "component_edges": m_c,
            "gpu_ms_per_root": gpu_s * 1e3 / k,
            "gpu_gteps": 2 * m_c * k / gpu_s / 1e9,
            "cpu_baseline": {"ms_per_root": cpu_s * 1e3 / 2, "cores": 1, "kind": "port",
                             "sample": "2 of the roots, one thread (oracle_brandes)"},
            "speedup_vs_cpu": (cpu_s / 2) / (gpu_s / k),
            "bit_identical_to_oracle": bool(np.array_equal(bc2, want)),
            "sigma_overflow_roots": int(ovf),
            "metric_note": "gteps counts each component edge twice per root (forward and sweep); "
                           "host wall clock around tbfs_brandes"}


def directed_report(args):
    """Directed graph: every undirected RMAT edge kept in one direction (a
    hash of the pair picks which), uploaded without TBFS_GRAPH_SYMMETRIC so
    the out-lists are built on the device.  Direction-optimizing BFS (pushes
    over out-lists, pulls over in-lists) against pulls only (mode bu, the
    structure of the reference's column-per-thread kernels), S + sigma, with
    two roots checked against the oracle."""
    import oracle
    import turbobfs_gb300 as tb
    from turbobfs_gb300 import graphs

    scale = args.directed_scale
    hs = graphs.rmat(scale, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    col = np.repeat(np.arange(hs.n, dtype=np.int64), np.diff(hs.col_ptr))
    row = hs.row_idx.astype(np.int64)
    pick = (((row ^ col) * 0x9E3779B1) >> 16) & 1
    keep = pick == (row < col)
    h = graphs.from_edges(hs.n, row[keep].astype(np.int32), col[keep].astype(np.int32))
    del hs, col, row
    deg_in = np.diff(h.col_ptr)
    rng = np.random.default_rng(4)
    cand = np.nonzero(deg_in > 0)[0]
    roots = cand[rng.integers(0, cand.shape[0], 16)].astype(np.int32)
    out = {"workload": f"RMAT scale {scale}, edgefactor 16, each undirected edge kept in one "
                       "direction; 16 roots with in-edges; S + sigma",
           "n": int(h.n), "nnz": int(h.nnz)}
    t0 = time.perf_counter()
    with tb.Graph.from_host_csc(h) as g:  # not symmetric: device transpose
        out["upload_with_transpose_ms"] = (time.perf_counter() - t0) * 1e3
        for mode in ("auto", "bu"):
            for r in roots[:2]:
                g.bfs(int(r), mode=mode)
            ms, edges = [], []
            for r in roots:
                res = g.bfs(int(r), mode=mode)
                ms.append(res.stats["device_ms"])
                edges.append(res.stats["edges"])
            out[f"{mode}_ms_per_bfs"] = float(np.mean(ms))
            out[f"{mode}_gteps"] = float(np.sum(edges) / (np.sum(ms) * 1e-3) / 1e9)
        same = True
        for r in roots[:2]:
            res = g.bfs(int(r))
            S, sg, ovf, _ = oracle.exact_bfs(h.col_ptr, h.row_idx, int(r))
            same &= bool(np.array_equal(res.S, S) and np.array_equal(res.sigma[ovf == 0], sg[ovf == 0]))
    out["push_pull_speedup_vs_pull_only"] = out["bu_ms_per_bfs"] / out["auto_ms_per_bfs"]
    out["identical_to_oracle"] = same
    out["gteps_edges"] = "out-list entries of the root's reached vertices (stats.edges)"
    return out


def grid_report(args):
    """High-diameter graph: the 2D grid with deletions and chords, thousands of
    levels, so the per-level cost of the persistent kernel shows.  Native
    traversals in every mode (device-timed, graph resident), and the two
    reference entry points this graph runs through, COOC top-down and CSC
    bottom-up (host arrays, upload inside each call, host wall clock).  Every
    result is checked against the oracle's exact BFS: S everywhere, sigma where
    the count is below 2^63 (on a grid most counts are not)."""
    import oracle
    import turbobfs_gb300 as tb
    from turbobfs_gb300 import graphs

    side = args.grid_side
    h = graphs.grid(side, seed=1)
    roots = graphs.pick_roots(h, 2, seed=1)
    want = [oracle.exact_bfs(h.col_ptr, h.row_idx, int(r)) for r in roots]
    out = {"workload": f"{side}x{side} 2D grid, 10% of edges deleted, 1% chords within Manhattan "
                       f"distance 8, degree <= 6; n={h.n}, {h.nnz} CSC entries; 2 roots; S + sigma",
           "n": h.n, "nnz": int(h.nnz)}
    same = True
    with tb.Graph.from_host_csc(h) as g:
        for mode in ("auto", "td", "bu"):
            g.bfs(int(roots[0]), mode=mode)  # warm
            ms, lv, ed = [], [], []
            for r, (S, sg, ovf, _) in zip(roots, want):
                res = g.bfs(int(r), mode=mode)
                ms.append(res.stats["device_ms"])
                lv.append(res.stats["levels"])
                ed.append(res.stats["edges"] / 2)
                ok = ovf == 0
                same &= bool(np.array_equal(res.S, S) and np.array_equal(res.sigma[ok], sg[ok]))
            out[mode] = {"ms_per_bfs": float(np.mean(ms)), "levels": int(np.mean(lv)),
                         "us_per_level": float(1e3 * np.sum(ms) / np.sum(lv)),
                         "gteps": float(np.sum(ed) / np.sum(ms) / 1e6)}
        # the engine shape and direction parameters tuned for this graph's
        # degree profile (CTAs per SM above all: small levels are latency-bound)
        kw = {k: v for k, v in g.autotune(roots[:1]).items() if k != "from_cache"}
        g.bfs(int(roots[0]), **kw)  # warm
        ms, lv = [], []
        for r, (S, sg, ovf, _) in zip(roots, want):
            res = g.bfs(int(r), **kw)
            ms.append(res.stats["device_ms"])
            lv.append(res.stats["levels"])
            ok = ovf == 0
            same &= bool(np.array_equal(res.S, S) and np.array_equal(res.sigma[ok], sg[ok]))
        out["autotuned"] = {"ms_per_bfs": float(np.mean(ms)), "levels": int(np.mean(lv)),
                            "us_per_level": float(1e3 * np.sum(ms) / np.sum(lv)),
                            "params": {k: (round(v, 3) if isinstance(v, float) else v)
                                       for k, v in kw.items()}}
    # the reference's entry points: graph built from the host arrays in every call
    n, nz = h.n, int(h.nnz)
    J = np.repeat(np.arange(n, dtype=np.int32), np.diff(h.col_ptr))
    I = h.row_idx
    r = int(roots[0])
    S0, sg0, ovf0, _ = want[0]
    sig = np.zeros(n, np.float32)
    tb.bfs_gpu_td_cooc_sc(I, J, sig, r, nz, n, 1)  # warm
    t0 = time.perf_counter()
    rc = tb.bfs_gpu_td_cooc_sc(I, J, sig, r, nz, n, 1)
    t_cooc = time.perf_counter() - t0
    ok = ovf0 == 0
    same &= rc == 0 and bool(np.array_equal(sig[ok], sg0[ok].astype(np.float32)))
    Sb = np.zeros(n, np.int32)
    t0 = time.perf_counter()
    rc = tb.bfs_gpu_bu_csc_sc(h.row_idx, h.col_ptr, Sb, r, nz, n, 1)
    t_bu = time.perf_counter() - t0
    same &= rc == 0 and bool(np.array_equal(Sb, S0))
    out["bfs_gpu_td_cooc_sc_ms"] = 1e3 * t_cooc
    out["bfs_gpu_bu_csc_sc_ms"] = 1e3 * t_bu
    out["entry_points_note"] = ("host wall clock per call: device allocation, upload (COOC: "
                                "sort into CSC on the device), one traversal, result copy, free")
    out["identical_to_oracle"] = same
    out["cpu_baseline_note"] = (f"not timed: the reference's sequential BFS scans all {nz} entries "
                                f"at each of the {out['auto']['levels']} levels")
    return out


def main():
    args = parse_args()
    world, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if args.part != "all":
        import torch

        torch.cuda.set_device(local)
        rep = {"batched": batched_report, "serving": serving_report,
               "ingest": ingest_report, "brandes": brandes_report,
               "directed": directed_report, "grid": grid_report}[args.part](args)
        print(json.dumps({"part": args.part, args.part: rep}), flush=True)
        return 0
    return run_tbfs(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
