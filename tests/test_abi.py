"""The C-ABI library loads and exports every symbol include/gmr.h declares."""
import ctypes
import re
from pathlib import Path

import numpy as np

import gmr
from gmr import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "gmr.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    names = set(re.findall(r"\b(gmr_[a-z0-9_]+|run_gpu_right_multiply_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_legacy_pair():
    names = declared_functions()
    assert "run_gpu_right_multiply_layered" in names
    assert "run_gpu_right_multiply_batched" in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    assert set(declared_functions()) <= set(_lib.EXPORTED)


def test_struct_layouts_match_reference():
    # gpu-engine/layered_types.h:45-75: LayeredRule {int,int,float}, GPUSchedule
    assert ctypes.sizeof(gmr.LayeredRule) == 12
    assert gmr.GPUSchedule.emit_total.offset == 48
    assert ctypes.sizeof(gmr.GPUSchedule) == 80


def test_version_and_error_strings():
    lib = gmr.lib()
    assert lib.gmr_version().startswith(b"gmr")
    h = ctypes.c_void_p()
    rc = lib.gmr_grammar_load(b"/nonexistent/base", ctypes.byref(h))
    assert rc == 3 and b"cannot open" in lib.gmr_last_error()


def _bad_device_plan(**over):
    """A gmr_device_plan that fails the entry point's host-side checks (each
    case below breaks one), so nothing reaches the GPU."""
    lvl = np.array([0, 2, 3], dtype=np.int64)
    seg = np.array([0, 1, 2, 3], dtype=np.int64)
    dp = _lib.DevicePlan()
    dp.rows, dp.cols, dp.depth, dp.n_ops, dp.n_terms = 4, 3, 2, 3, 2
    dp.lvl_off, dp.seg_off = lvl.ctypes.data, seg.ctypes.data
    dp.ops, dp.em_src, dp.seg_row, dp.seg_start, dp.term_val, dp.term_col, dp.V = [256] * 7
    dp.op_c = None
    keep = [lvl, seg]
    for k, v in over.items():
        if isinstance(v, np.ndarray):
            keep.append(v)
            v = v.ctypes.data
        setattr(dp, k, v)
    return dp, keep


def test_noalloc_rejects_bad_plans_before_any_launch():
    lib = gmr.lib()
    cases = [
        (dict(em_src=None), 1, b"null emission array"),
        (dict(seg_row=None), 1, b"null emission array"),
        (dict(seg_off=np.array([1, 1, 2, 3], dtype=np.int64)), 2, b"do not start at 0"),
        (dict(seg_off=np.array([0, 2, 1, 3], dtype=np.int64)), 2, b"segment offsets decrease"),
        (dict(lvl_off=np.array([0, 4, 3], dtype=np.int64)), 2, b"level offsets decrease"),
        (dict(lvl_off=np.array([0, 2, 5], dtype=np.int64)), 2, b"do not cover"),
        (dict(op_c=258), 1, b"misaligned"),
    ]
    for over, code, msg in cases:
        dp, keep = _bad_device_plan(**over)
        rc = lib.gmr_multiply_noalloc(ctypes.byref(dp), 0, ctypes.c_void_p(256), ctypes.c_void_p(256), 4, None)
        assert rc == code and msg in lib.gmr_last_error(), (over, rc, lib.gmr_last_error())
