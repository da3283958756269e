"""The C ABI surface, checked without running any GPU work: every function
declared in include/*.h is exported by libtbfs.so, bound by the Python layer,
and calls that need a device fail cleanly when none is visible."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import turbobfs_gb300 as tb
from turbobfs_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, re.M):
            if m.group(1) not in {"if", "while", "for", "return", "sizeof"}:
                names.add(m.group(1))
    return names


def exported_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_every_declared_function_is_exported_and_bound():
    declared = declared_functions()
    assert len(declared) >= 30
    exported = exported_symbols()
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    assert declared <= set(_lib.exported_names()) | {"tbfs_set_error"}
    lib = tb.lib()
    for name in declared:
        assert getattr(lib, name) is not None


def test_compat_symbols_present():
    for name in tb.COMPAT_FUNCTIONS:
        assert name in exported_symbols()


def test_version_and_status_strings():
    lib = tb.lib()
    assert lib.tbfs_version() == 100
    for code, name in _lib.STATUS_NAMES.items():
        s = lib.tbfs_status_string(code).decode()
        assert s and s != "unknown status"
    assert lib.tbfs_status_string(99).decode() == "unknown status"


def test_options_layout_and_defaults():
    o = tb.make_options()
    assert ctypes.sizeof(_lib.Options) == 64 and ctypes.sizeof(_lib.Stats) == 40
    assert o.mode == 0 and o.want_sigma == 1 and o.alpha == 15.0 and o.beta == 2.0 and o.pull_ratio == 1.0


@pytest.mark.skipif(tb.device_count() > 0, reason="checks behaviour without a GPU")
def test_no_device_is_a_clean_error():
    cp = np.array([0, 1, 2], np.int32)
    ic = np.array([1, 0], np.int32)
    with pytest.raises(tb.TbfsError) as e:
        tb.Graph(cp, ic)
    assert e.value.status == 5
    S = np.zeros(2, np.int32)
    sg = np.zeros(2, np.float32)
    assert tb.bfs_gpu_td_csc_sc(ic, cp, S, sg, 0, 2, 2, 1) == 5
    assert tb.bfs_gpu_td_cooc_sc(ic, np.array([0, 1], np.int32), sg, 0, 2, 2, 1) == 5


def test_invalid_arguments_rejected_before_device_use():
    S = np.zeros(2, np.int32)
    sg = np.zeros(2, np.float32)
    cp = np.array([0, 1, 2], np.int32)
    ic = np.array([1, 0], np.int32)
    assert tb.bfs_gpu_td_csc_sc(ic, cp, S, sg, 5, 2, 2, 1) == 1  # root out of range
    assert tb.bfs_gpu_bu_csc_sc(ic, cp, S, -1, 2, 2, 1, 1) == 1
    assert tb.bfs_gpu_tdbu_csc_sc(ic, cp, S, np.zeros(2, np.int32), 0, -3, 2, 1, 1) == 1
    with pytest.raises(TypeError):
        tb.bfs_gpu_td_csc_sc(ic, cp, S, np.zeros(2, np.float64), 0, 2, 2, 1)
