"""ctypes wrapper of the oracle (oracle.c) -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, by the smoke check in __graft_entry__.py, by the CPU
baseline leg of bench.py and by `bench.py --impl reference`, as the checker
and as the timed baselines (the reference's CPU sweep, and its GPU engine run
through RefGpu).  The product path (g-mm-repair_gb300/gmr) never imports it.  Each function names the
reference code it restates (see oracle.c).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
PLUS, BOOL, TROP = 0, 1, 2
NAMES = {0: "plustimes", 1: "boolean", 2: "tropical"}
_lib = None


REFGPU_LIB = HERE / "librefgpu.so"
REFGPU_PTX = HERE / "_ref" / "gpu_engine.ptx"


def build(force: bool = False) -> Path:
    src = HERE / "oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "-B", "liboracle.so"], check=True)
    lsrc = HERE / "ref" / "ref_gpu.cpp"
    if force or not REFGPU_LIB.exists() or REFGPU_LIB.stat().st_mtime < lsrc.stat().st_mtime:
        # the launcher needs the CUDA driver headers; without them the
        # reference-GPU baseline is simply unavailable
        subprocess.run(["make", "-s", "-C", str(HERE), "-B", "librefgpu.so"], check=False,
                       capture_output=True)
    return LIB


def reference_root() -> Path:
    """Root of the reference tree: $GMR_REFERENCE, default /root/reference."""
    return Path(os.environ.get("GMR_REFERENCE", "/root/reference"))


def build_ref() -> bool:
    """Builds the reference's own sources into oracle/_ref (only where the
    reference tree exists)."""
    root = reference_root()
    if not (root / "gpu-engine").is_dir():
        return False
    r = subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"GMR_REFERENCE={root}"], capture_output=True,
                       text=True)
    return r.returncode == 0


def lib():
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(str(LIB))
        P, I = C.c_void_p, C.POINTER(C.c_int)
        l.orc_build_schedule.argtypes = [C.c_int, C.c_long, I, I, I, C.c_long, I, C.POINTER(P)]
        l.orc_sched_free.argtypes = [P]
        l.orc_sched_int.argtypes = [P, C.c_int, C.POINTER(C.c_long)]
        l.orc_sched_arr.argtypes = [P, C.c_int]
        l.orc_sched_arr.restype = I
        l.orc_sched_coeff.argtypes = [P]
        l.orc_sched_coeff.restype = C.POINTER(C.c_float)
        l.orc_sweep_f64.argtypes = [P, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_float), C.c_int, C.c_int,
                                    C.POINTER(C.c_double)]
        l.orc_cpu_reference.argtypes = [P, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int,
                                        P, C.c_int]
        l.orc_expand.argtypes = [C.c_int, C.c_long, I, I, I, C.c_long, I, I]
        l.orc_expand.restype = C.c_long
        l.orc_brute_force.argtypes = [C.c_long, I, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_float), C.c_int,
                                      C.c_int, C.POINTER(C.c_double)]
        _lib = l
    return _lib


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


class RefSchedule:
    """The reference's BuiltSchedule (build_schedule.cpp:42-227), restated."""

    INTS = ["alpha", "depth", "max_width", "num_raw", "num_layered", "num_pt", "emit_total", "num_term"]

    def __init__(self, alpha, rules, C_seq, kinds=None, reps=None):
        rules = np.ascontiguousarray(np.asarray(rules, dtype=np.int32).reshape(-1))
        C_seq = np.ascontiguousarray(C_seq, dtype=np.int32)
        kinds = None if kinds is None else np.ascontiguousarray(kinds, dtype=np.int32)
        reps = None if reps is None else np.ascontiguousarray(reps, dtype=np.int32)
        h = C.c_void_p()
        lib().orc_build_schedule(int(alpha), len(rules) // 2, _ip(rules), _ip(kinds), _ip(reps), len(C_seq),
                                 _ip(C_seq), C.byref(h))
        self._h = h
        v = C.c_long()
        for i, n in enumerate(self.INTS):
            lib().orc_sched_int(h, i, C.byref(v))
            setattr(self, n, int(v.value))
        L, D = self.num_layered, self.depth

        def arr(which, n):
            if n == 0:
                return np.zeros(0, np.int32)
            return np.ctypeslib.as_array(lib().orc_sched_arr(h, which), shape=(n,)).copy()

        self.left, self.right = arr(0, L), arr(1, L)
        self.coeff = (np.ctypeslib.as_array(lib().orc_sched_coeff(h), shape=(L,)).copy() if L
                      else np.zeros(0, np.float32))
        self.level_offsets, self.level_widths = arr(2, D + 1), arr(3, D + 1)
        self.emit_offsets = arr(4, D + 1)
        self.emit_pos, self.emit_row = arr(5, self.emit_total), arr(6, self.emit_total)
        self.term_emit_sym, self.term_emit_row = arr(7, self.num_term), arr(8, self.num_term)
        self.term_orig = arr(9, self.alpha)

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().orc_sched_free(self._h)
            self._h = C.c_void_p()

    def rules_lrc(self):
        out = np.zeros(self.num_layered, dtype=[("l", "<i4"), ("r", "<i4"), ("c", "<f4")])
        out["l"], out["r"], out["c"] = self.left, self.right, self.coeff
        return out

    def gpu_schedule(self) -> dict:
        return dict(max_depth=self.depth, max_width=self.max_width, level_offsets=self.level_offsets,
                    level_widths=self.level_widths, emit_offsets=self.emit_offsets, emit_pos=self.emit_pos,
                    emit_row=self.emit_row, term_emit_sym=self.term_emit_sym, term_emit_row=self.term_emit_row)

    def terminal_tables(self, cols):
        """val/col index tables as gpu_engine_test.cu:373-380 builds them."""
        t = self.term_orig[1:].astype(np.int64)
        return ((t - 1) // cols).astype(np.int32), ((t - 1) % cols).astype(np.int32)

    def sweep_f64(self, semiring, V, x, rows, cols) -> np.ndarray:
        V = np.ascontiguousarray(V, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros(rows, dtype=np.float64)
        lib().orc_sweep_f64(self._h, semiring, V.ctypes.data_as(C.POINTER(C.c_double)),
                            x.ctypes.data_as(C.POINTER(C.c_float)), rows, cols,
                            y.ctypes.data_as(C.POINTER(C.c_double)))
        return y

    def cpu_reference(self, semiring, V, x, rows, cols, threads=1) -> np.ndarray:
        Vf = np.ascontiguousarray(V, dtype=np.float32)
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros(rows, dtype=np.float32 if semiring == PLUS else np.int32)
        lib().orc_cpu_reference(self._h, semiring, Vf.ctypes.data_as(C.POINTER(C.c_float)),
                                x.ctypes.data_as(C.POINTER(C.c_float)), rows, cols,
                                y.ctypes.data_as(C.c_void_p), threads)
        return y


def expand(alpha, rules, C_seq, kinds=None, reps=None) -> np.ndarray:
    """CSRV string re-expanded from a grammar (cpu_selftest.cpp:119-156)."""
    rules = np.ascontiguousarray(np.asarray(rules, dtype=np.int32).reshape(-1))
    C_seq = np.ascontiguousarray(C_seq, dtype=np.int32)
    kinds = None if kinds is None else np.ascontiguousarray(kinds, dtype=np.int32)
    reps = None if reps is None else np.ascontiguousarray(reps, dtype=np.int32)
    n = lib().orc_expand(int(alpha), len(rules) // 2, _ip(rules), _ip(kinds), _ip(reps), len(C_seq), _ip(C_seq),
                         None)
    out = np.zeros(max(n, 1), dtype=np.int32)
    lib().orc_expand(int(alpha), len(rules) // 2, _ip(rules), _ip(kinds), _ip(reps), len(C_seq), _ip(C_seq),
                     _ip(out))
    return out[:n]


def brute_force(vc, semiring, V, x, rows, cols) -> np.ndarray:
    """y = M x straight from the CSRV string (cpu_selftest.cpp:104-117)."""
    vc = np.ascontiguousarray(vc, dtype=np.int32)
    V = np.ascontiguousarray(V, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.zeros(rows, dtype=np.float64)
    lib().orc_brute_force(len(vc), _ip(vc), semiring, V.ctypes.data_as(C.POINTER(C.c_double)),
                          x.ctypes.data_as(C.POINTER(C.c_float)), rows, cols,
                          y.ctypes.data_as(C.POINTER(C.c_double)))
    return y


class RefGpu:
    """The reference's own GPU kernels (gpu-engine/gpu_engine.cu, compiled to
    PTX in _ref/) run with the reference's host sequence restated in
    ref/ref_gpu.cpp: the plain per-level sweep of the reference on this GPU.
    Baseline and test infrastructure only."""

    _lib = None

    @classmethod
    def available(cls) -> str | None:
        """None when usable, else why not."""
        if not REFGPU_PTX.exists():
            return "the reference engine's device code (oracle/_ref/gpu_engine.ptx) was not built here"
        if not REFGPU_LIB.exists():
            return "oracle/librefgpu.so was not built (CUDA driver headers missing)"
        return None

    def __init__(self, device: int = 0):
        why = self.available()
        if why:
            raise RuntimeError(why)
        if RefGpu._lib is None:
            l = C.CDLL(str(REFGPU_LIB))
            l.refgpu_error.restype = C.c_char_p
            l.refgpu_open.argtypes = [C.c_char_p, C.c_int]
            I, F = C.POINTER(C.c_int), C.POINTER(C.c_float)
            l.refgpu_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, I, I, F, C.c_int,
                                     C.c_int, C.c_int, I, I, I, I, C.c_int, I, I, C.c_int, F, C.c_void_p, C.c_int,
                                     C.c_int, F]
            RefGpu._lib = l
        if RefGpu._lib.refgpu_open(str(REFGPU_PTX).encode(), device) != 0:
            raise RuntimeError(RefGpu._lib.refgpu_error().decode())

    def run(self, sched: "RefSchedule", semiring: int, V, X, rows: int, cols: int, iters: int = 1):
        """X: [cols][B] float32 (the reference's batched layout; B = 1 runs the
        single-vector kernels).  Returns (Y [rows][B], ms per iteration)."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        if X.ndim == 1:
            X = X.reshape(-1, 1)
        B = X.shape[1]
        vi, ci = sched.terminal_tables(cols)
        rules = sched.rules_lrc()
        Vf = np.ascontiguousarray(V, dtype=np.float32)
        Y = np.zeros((rows, B), dtype=np.float32 if semiring == PLUS else np.int32)
        ms = C.c_float()
        keep = [np.ascontiguousarray(a, dtype=np.int32) for a in
                (vi, ci, sched.level_offsets, sched.emit_offsets, sched.emit_pos, sched.emit_row,
                 sched.term_emit_sym, sched.term_emit_row)]
        rc = RefGpu._lib.refgpu_run(semiring, rows, cols, sched.alpha, sched.num_layered,
                                    rules.ctypes.data_as(C.c_void_p), _ip(keep[0]), _ip(keep[1]),
                                    Vf.ctypes.data_as(C.POINTER(C.c_float)), len(Vf), sched.depth,
                                    sched.max_width, _ip(keep[2]), _ip(keep[3]), _ip(keep[4]), _ip(keep[5]),
                                    sched.emit_total, _ip(keep[6]), _ip(keep[7]), sched.num_term,
                                    X.ctypes.data_as(C.POINTER(C.c_float)), Y.ctypes.data_as(C.c_void_p), B,
                                    int(iters), C.byref(ms))
        if rc != 0:
            raise RuntimeError(RefGpu._lib.refgpu_error().decode())
        return Y, ms.value / iters
