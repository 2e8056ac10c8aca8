"""The C-ABI library loads and exports every symbol include/gmr.h declares."""
import ctypes
import re
from pathlib import Path

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
