"""bench.py's wiring, checked without a GPU: every report the default run
makes exists and has its skip flag, every --part maps to a report, and the
reference arm prints the contract's JSON line on the host cores."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402

REPORTS = ["batched", "serving", "ingest", "brandes", "directed", "grid"]


def test_every_report_has_a_function_a_flag_and_a_part():
    args = bench.parse_args([])
    for name in REPORTS:
        assert callable(getattr(bench, f"{name}_report")), name
        assert getattr(args, f"no_{name}") is False, name
        assert bench.parse_args(["--part", name]).part == name


def test_skip_flags_parse():
    args = bench.parse_args([f"--no-{name}" for name in REPORTS])
    assert all(getattr(args, f"no_{name}") for name in REPORTS)


@pytest.mark.timeout(600)
def test_reference_arm_prints_the_contract_line():
    """The reference arm runs the CPU restatement of the reference's
    sequential BFS on a bounded sample of the RMAT-22 workload."""
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], cwd=ROOT, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["config"]["workload"] == "rmat22_do_bfs_sigma_64roots"
