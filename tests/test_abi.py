"""The C-ABI library loads and exports every entry point include/les_gb300.h
declares (no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    txt = open(os.path.join(ROOT, "include", "les_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(les_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(gpu_lib):
    L = ctypes.CDLL(gpu_lib.LIB_PATH)
    names = declared()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_estimate_bytes_without_gpu(gpu_lib):
    cfg = gpu_lib.make_config(256, s_flag=1)
    b = gpu_lib.estimate_device_bytes(cfg)
    assert 5e9 < b < 60e9
    small = gpu_lib.estimate_device_bytes(gpu_lib.make_config(32))
    assert small < b / 100


def test_config_struct_layout():
    from les_gb300.config import LesConfig
    assert ctypes.sizeof(LesConfig) == 12 * 4 + 11 * 8
