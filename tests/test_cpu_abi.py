"""CPU-side checks of the C ABI library: it loads and exports every entry
point include/adg.h declares (no GPU work is issued here)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "adg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(adg_\w+)\s*\(", src, re.M)))


def test_header_declares_entry_points():
    names = header_functions()
    assert "adg_ctx_create" in names and "adg_ader" in names and len(names) >= 20


def test_library_exports_every_declared_symbol():
    import adg_gb300

    L = adg_gb300.lib()
    missing = [n for n in header_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_flop_counts_are_consistent():
    import adg_gb300

    alg, issued = adg_gb300.flops_per_element(2, 3)
    assert alg == 139280.0  # dense matvec count of the method at D=2, P=3
    alg1, _ = adg_gb300.flops_per_element(2, 1)
    assert alg1 == 2552.0
    alg3d, _ = adg_gb300.flops_per_element(3, 2)
    assert alg3d == 180250.0
    assert 0 < issued < alg


def test_bad_config_is_rejected_without_gpu_work():
    import ctypes

    import adg_gb300

    cfg = adg_gb300.AdgConfig()
    cfg.D, cfg.P = 2, 7  # unsupported degree
    h = ctypes.c_void_p()
    assert adg_gb300.lib().adg_ctx_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
