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
    """les_config in include/les_gb300.h: 12 ints, then 13 doubles; the
    ctypes mirror and the field enumeration follow the header."""
    from les_gb300.config import LesConfig, FIELDS
    assert ctypes.sizeof(LesConfig) == 12 * 4 + 13 * 8
    assert LesConfig.q_flag.offset == 11 * 4 and LesConfig.dqdz_top.offset == 12 * 4 + 12 * 8
    txt = open(os.path.join(ROOT, "include", "les_gb300.h")).read()
    enum = re.search(r"typedef enum les_field \{(.*?)\} les_field;", txt, flags=re.S).group(1)
    enum = re.sub(r"/\*.*?\*/", "", enum, flags=re.S)
    names = [n.strip().split("=")[0].strip() for n in enum.split(",") if n.strip()]
    assert names[-1] == "LES_NUM_FIELDS" and len(names) - 1 == len(FIELDS)
    assert names.index("LES_Q") == FIELDS.index("q")
    assert names.index("LES_ZO") == FIELDS.index("zo")
    assert names.index("LES_SGS_Q3_SFC") == FIELDS.index("sgs_q3")
