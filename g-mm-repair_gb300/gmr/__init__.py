"""gmr -- GB300-native right multiplication over RePair grammar-compressed matrices.

Python host layer over the C-ABI library ``libgmr.so`` (declared in
include/gmr.h).  It mirrors the reference's interface for this path:

* the file format and loaders of gpu-engine/gpu_engine_test.cu:291-345
  (:class:`Grammar`, ``Grammar.load``);
* the schedule builder, build_schedule.cpp:42-227 (:class:`Plan`);
* the engine entry points gpu_engine.h:99-136 (:func:`run_gpu_right_multiply_layered`,
  :func:`run_gpu_right_multiply_batched`) and the load-once handle API
  (:class:`Engine`).

There is no CPU fallback: every multiply runs the CUDA kernels of libgmr.so,
and importing a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L
from ._lib import Config, GPUSchedule, LayeredRule

PLUS_TIMES, BOOLEAN, TROPICAL = 0, 1, 2
SEMIRINGS = {"plustimes": PLUS_TIMES, "boolean": BOOLEAN, "bool": BOOLEAN, "tropical": TROPICAL,
             "minplus": TROPICAL}
TROPICAL_INF = 1_000_000_000

VARIANT_AUTO, VARIANT_PLAIN, VARIANT_FUSED, VARIANT_GRAPH, VARIANT_PERSISTENT = 0, 1, 2, 3, 4
EMIT_AUTO, EMIT_ATOMIC, EMIT_SEGMENTED, EMIT_ROWS = 0, 1, 2, 3
PUSH_AUTO, PUSH_NEVER, PUSH_ALWAYS, PUSH_INTERLEAVE = 0, 1, 2, 3
LEVEL_PUSH, LEVEL_INTERLEAVE, LEVEL_STAGE = 32, 64, 128

__all__ = [
    "GmrError", "Csrv", "Grammar", "Plan", "Engine", "gen_mosaic", "gen_copy_graph", "repair", "semiring_id",
    "pack_bits", "unpack_bits", "run_gpu_right_multiply_layered", "run_gpu_right_multiply_batched",
    "PLUS_TIMES", "BOOLEAN", "TROPICAL", "TROPICAL_INF", "Config",
]


class GmrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{L.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def lib():
    return L.load()


def _check(rc: int):
    if rc != L.GMR_OK:
        raise GmrError(rc, lib().gmr_last_error().decode())


def semiring_id(s) -> int:
    if isinstance(s, str):
        return SEMIRINGS[s.lower()]
    return int(s)


def _i32(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(L.I32P)


def _f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(L.F64P)


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(L.F32P)


def _view(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    ctype = np.ctypeslib.as_ctypes_type(dtype)
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(n,)).copy()


def pack_bits(X: np.ndarray) -> np.ndarray:
    """[n][B] of 0/1 -> [n][ceil(B/32)] uint32, bit b%32 of word b//32 = column b."""
    X = np.asarray(X) != 0
    n, B = X.shape
    W = (B + 31) // 32
    pad = np.zeros((n, W * 32), dtype=np.uint64)
    pad[:, :B] = X
    bits = pad.reshape(n, W, 32) << np.arange(32, dtype=np.uint64)
    return bits.sum(axis=2).astype(np.uint32)


def unpack_bits(Yw: np.ndarray, B: int) -> np.ndarray:
    """Inverse of :func:`pack_bits` -> int32 0/1 array [n][B]."""
    Yw = np.asarray(Yw, dtype=np.uint32)
    n, W = Yw.shape
    bits = (Yw[:, :, None] >> np.arange(32, dtype=np.uint32)) & 1
    return bits.reshape(n, W * 32)[:, :B].astype(np.int32)


# ---------------------------------------------------------------- CSRV
class Csrv:
    """Uncompressed matrix as a CSRV string (codes val*cols+col+1, 0 = row end)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().gmr_csrv_free(self._h)
            self._h = C.c_void_p()

    @property
    def info(self) -> L.CsrvInfo:
        i = L.CsrvInfo()
        _check(lib().gmr_csrv_get_info(self._h, C.byref(i)))
        return i

    @property
    def rows(self) -> int:
        return self.info.rows

    @property
    def cols(self) -> int:
        return self.info.cols

    @property
    def nnz(self) -> int:
        return self.info.nnz

    def codes(self) -> np.ndarray:
        return _view(lib().gmr_csrv_codes(self._h), self.info.len, np.int32)

    def values(self) -> np.ndarray:
        return _view(lib().gmr_csrv_V(self._h), self.info.n_vals, np.float64)

    @classmethod
    def from_dense(cls, M) -> "Csrv":
        M, p = _f64(M)
        h = C.c_void_p()
        _check(lib().gmr_csrv_from_dense(M.shape[0], M.shape[1], p, C.byref(h)))
        return cls(h)

    @classmethod
    def from_codes(cls, rows, cols, codes, V) -> "Csrv":
        codes, pc = _i32(codes)
        V, pv = _f64(V)
        h = C.c_void_p()
        _check(lib().gmr_csrv_create(rows, cols, len(codes), pc, len(V), pv, C.byref(h)))
        return cls(h)

    def dense(self) -> np.ndarray:
        """Dense float64 matrix (small inputs only)."""
        i = self.info
        M = np.zeros((i.rows, i.cols))
        V = self.values()
        r = 0
        for c in self.codes():
            if c == 0:
                r += 1
                continue
            M[r, (c - 1) % i.cols] = V[(c - 1) // i.cols]
        return M


def gen_mosaic(rows, cols, founders, switch_rate, mutation, seed, threads=0) -> Csrv:
    h = C.c_void_p()
    _check(lib().gmr_gen_mosaic(rows, cols, founders, switch_rate, mutation, seed, threads, C.byref(h)))
    return Csrv(h)


def gen_copy_graph(nodes, degree, copy_prob, weighted, seed, threads=0) -> Csrv:
    h = C.c_void_p()
    _check(lib().gmr_gen_copy_graph(nodes, degree, copy_prob, int(weighted), seed, threads, C.byref(h)))
    return Csrv(h)


# ---------------------------------------------------------------- grammar
class Grammar:
    """RePair grammar (alpha, rules, C, V) -- gpu-engine/grammar.h:41-63."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().gmr_grammar_free(self._h)
            self._h = C.c_void_p()

    @property
    def info(self) -> L.GrammarInfo:
        i = L.GrammarInfo()
        _check(lib().gmr_grammar_get_info(self._h, C.byref(i)))
        return i

    @property
    def alpha(self) -> int:
        return self.info.alpha

    @property
    def n_rules(self) -> int:
        return self.info.n_rules

    def rules(self) -> np.ndarray:
        n = self.info.n_rules
        return _view(lib().gmr_grammar_rules(self._h), 2 * n, np.int32).reshape(n, 2)

    def kinds(self) -> np.ndarray:
        return _view(lib().gmr_grammar_kinds(self._h), self.info.n_rules, np.int32)

    def reps(self) -> np.ndarray:
        return _view(lib().gmr_grammar_reps(self._h), self.info.n_rules, np.int32)

    def C(self) -> np.ndarray:
        return _view(lib().gmr_grammar_C(self._h), self.info.c_len, np.int32)

    def values(self) -> np.ndarray:
        return _view(lib().gmr_grammar_V(self._h), self.info.n_vals, np.float64)

    @classmethod
    def load(cls, base) -> "Grammar":
        h = C.c_void_p()
        _check(lib().gmr_grammar_load(os.fsencode(str(base)), C.byref(h)))
        return cls(h)

    def save(self, base):
        _check(lib().gmr_grammar_save(self._h, os.fsencode(str(base))))

    @classmethod
    def from_arrays(cls, alpha, rules, C_seq, V, kinds=None, reps=None) -> "Grammar":
        rules = np.asarray(rules, dtype=np.int32).reshape(-1, 2)
        r, pr = _i32(rules.reshape(-1))
        c, pc = _i32(C_seq)
        v, pv = _f64(V)
        if kinds is not None:
            k, pk = _i32(kinds)
        else:
            k, pk = None, None
        if reps is not None:
            rp, prp = _i32(reps)
        else:
            rp, prp = None, None
        h = C.c_void_p()
        _check(lib().gmr_grammar_create(int(alpha), len(rules), pr, pk, prp, len(c), pc, len(v), pv, C.byref(h)))
        return cls(h)


def repair(m: Csrv, threads=0, device: int | None = None) -> Grammar:
    """RePair grammar of a CSRV string on the host (threads), or the identical
    grammar computed on GPU `device`."""
    h = C.c_void_p()
    if device is None:
        _check(lib().gmr_repair_compress(m._h, threads, C.byref(h)))
    else:
        _check(lib().gmr_repair_compress_device(m._h, int(device), C.byref(h)))
    return Grammar(h)


# ---------------------------------------------------------------- plan
class Plan:
    """Level-major, child-sorted schedule (replaces build_schedule.cpp:42-227)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().gmr_plan_free(self._h)
            self._h = C.c_void_p()

    @classmethod
    def build(cls, g: Grammar, rows: int, cols: int, device: int | None = None, validate: bool = False) -> "Plan":
        """Level-major plan of a grammar.  device=None builds on the host;
        device=d builds the identical plan on GPU d."""
        h = C.c_void_p()
        if device is None:
            _check(lib().gmr_plan_build(g._h, rows, cols, C.byref(h)))
        else:
            _check(lib().gmr_plan_build_device(g._h, rows, cols, int(device), int(bool(validate)), C.byref(h)))
        return cls(h)

    @classmethod
    def from_layered(cls, rows, cols, alpha, rules_lrc, val_indices, col_indices, V, sched) -> "Plan":
        """From the reference's proper-layered schedule (host arrays).

        rules_lrc: structured (left, right, coeff) rows; sched: dict with the
        GPUSchedule arrays (level_offsets, level_widths, emit_offsets, emit_pos,
        emit_row, term_emit_sym, term_emit_row, max_depth, max_width)."""
        keep = []
        rules = _layered_rules(rules_lrc)
        keep.append(rules)
        vi, pvi = _i32(val_indices)
        ci, pci = _i32(col_indices)
        v, pv = _f32(V)
        gs = _gpu_schedule(sched, keep)
        h = C.c_void_p()
        _check(lib().gmr_plan_from_layered(rows, cols, alpha, len(rules), rules, pvi, pci, pv, len(v),
                                           C.byref(gs), C.byref(h)))
        return cls(h)

    @property
    def stats(self) -> dict:
        s = L.PlanStats()
        _check(lib().gmr_plan_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in L.PlanStats._fields_}

    def level_ops(self) -> np.ndarray:
        d = self.stats["depth"]
        out = np.zeros(d + 1, dtype=np.int64)
        _check(lib().gmr_plan_level_ops(self._h, out.ctypes.data_as(C.POINTER(C.c_int64)), d + 1))
        return out

    def level_emits(self) -> np.ndarray:
        d = self.stats["depth"]
        out = np.zeros(d + 1, dtype=np.int64)
        _check(lib().gmr_plan_level_emits(self._h, out.ctypes.data_as(C.POINTER(C.c_int64)), d + 1))
        return out

    _ARRAYS = {"op_l": (0, np.int32), "op_r": (1, np.int32), "op_c": (2, np.float32), "lvl_off": (3, np.int64),
               "em_off": (4, np.int64), "em_src": (5, np.int32), "em_row": (6, np.int32),
               "term_val": (7, np.int32), "term_col": (8, np.int32), "V": (9, np.float32),
               "seg_off": (10, np.int64), "seg_row": (11, np.int32), "seg_start": (12, np.int64),
               "par_off": (13, np.int64), "par_src": (14, np.int32), "erow_off": (15, np.int64),
               "erow_row": (16, np.int32), "tcol_off": (17, np.int64), "tcol_q": (18, np.int32),
               "le_off": (19, np.int64), "le_src": (20, np.int32), "le_tgt": (21, np.int32),
               "le_split": (22, np.int32)}

    def array(self, name: str) -> np.ndarray:
        which, dt = self._ARRAYS[name]
        ptr, n = C.c_void_p(), C.c_int64()
        _check(lib().gmr_plan_array(self._h, which, C.byref(ptr), C.byref(n)))
        return _view(ptr, n.value, dt)

    def alg_bytes(self, semiring, B: int) -> float:
        return float(lib().gmr_plan_alg_bytes(self._h, semiring_id(semiring), B))

    def prepare_left(self):
        """Builds the reverse adjacency for the left product (y = x^T M)."""
        _check(lib().gmr_plan_prepare_left(self._h))

    def window_stats(self, rules_per_cta: int = 128, words: int = 32) -> np.ndarray:
        """[depth][5] per level: share of runs of rules_per_cta rules whose
        left-child window fits 64 / 128 / 200 KB of `words`-word values, mean
        window density, share of left children that are slots."""
        d = max(self.stats["depth"], 1)
        out = np.zeros(d * 5, dtype=np.float64)
        n = C.c_int()
        _check(lib().gmr_plan_window_stats(self._h, int(rules_per_cta), int(words),
                                           out.ctypes.data_as(L.F64P), len(out), C.byref(n)))
        return out[: n.value * 5].reshape(n.value, 5)

    def describe(self) -> str:
        cap = 1 << 16
        while True:
            buf = C.create_string_buffer(cap)
            rc = lib().gmr_plan_describe(self._h, buf, cap)
            if rc == L.GMR_OK:
                return buf.value.decode()
            if rc != 6:
                _check(rc)
            cap *= 4


def _layered_rules(rules_lrc):
    """numpy (n,3) [left, right, coeff] or structured -> ctypes LayeredRule array."""
    if isinstance(rules_lrc, C.Array):
        return rules_lrc
    a = np.asarray(rules_lrc)
    n = len(a)
    arr = (LayeredRule * max(n, 1))()
    if n:
        buf = np.frombuffer(arr, dtype=np.dtype([("l", "<i4"), ("r", "<i4"), ("c", "<f4")]), count=n)
        if a.dtype.names:
            buf["l"], buf["r"], buf["c"] = a[a.dtype.names[0]], a[a.dtype.names[1]], a[a.dtype.names[2]]
        else:
            buf["l"], buf["r"], buf["c"] = a[:, 0], a[:, 1], a[:, 2]
    return arr


def _gpu_schedule(d: dict, keep: list) -> GPUSchedule:
    def ip(name):
        a = np.ascontiguousarray(d[name], dtype=np.int32)
        if a.size == 0:
            a = np.zeros(1, dtype=np.int32)
        keep.append(a)
        return a.ctypes.data_as(C.POINTER(C.c_int))

    gs = GPUSchedule()
    gs.max_depth = int(d["max_depth"])
    gs.max_width = int(d["max_width"])
    gs.level_offsets = ip("level_offsets")
    gs.level_widths = ip("level_widths")
    gs.emit_offsets = ip("emit_offsets")
    gs.emit_pos = ip("emit_pos")
    gs.emit_row = ip("emit_row")
    gs.emit_total = int(len(d["emit_pos"]))
    gs.term_emit_sym = ip("term_emit_sym")
    gs.term_emit_row = ip("term_emit_row")
    gs.num_term_emit = int(len(d["term_emit_sym"]))
    keep.append(gs)
    return gs


# ---------------------------------------------------------------- engine
def _elem_dtype(semiring: int):
    return {PLUS_TIMES: np.float32, BOOLEAN: np.uint32, TROPICAL: np.int32}[semiring]


class Engine:
    """A plan resident on one GPU; multiplies X (cols x B) into Y (rows x B).

    Element types: float32 for (+,x); uint32 bit-packed words (32 right-hand
    sides per word) for (OR,AND); int32 for (min,+) with >= 1e9 = +inf."""

    def __init__(self, plan: Plan, device: int = 0):
        h = C.c_void_p()
        _check(lib().gmr_engine_create(plan._h, device, C.byref(h)))
        self._h = h
        s = plan.stats
        self.rows, self.cols, self.depth = s["rows"], s["cols"], s["depth"]

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().gmr_engine_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        self.close()

    @staticmethod
    def _cfg(variant=0, emit_mode=0, ops_per_cta=0, vec_tile=0, tile_levels=0, spin_limit=0, push=0, lane_bytes=0):
        return Config(variant, vec_tile, ops_per_cta, emit_mode, tile_levels, spin_limit, push, lane_bytes)

    def status(self):
        """(failed, phase) of the last persistent multiply (after a stream synchronize)."""
        f, p = C.c_int(), C.c_int()
        _check(lib().gmr_engine_status(self._h, C.byref(f), C.byref(p)))
        return f.value, p.value

    def multiply_device(self, semiring, x_ptr: int, y_ptr: int, B: int, stream: int = 0, **cfg):
        c = self._cfg(**cfg)
        _check(lib().gmr_engine_multiply(self._h, semiring_id(semiring), C.c_void_p(x_ptr), C.c_void_p(y_ptr), B,
                                         C.byref(c), C.c_void_p(stream)))

    def multiply(self, X: np.ndarray, semiring="plustimes", B: int | None = None, **cfg) -> np.ndarray:
        """Host arrays in and out (copies inside).  X: [cols] or [cols][words]."""
        sr = semiring_id(semiring)
        dt = _elem_dtype(sr)
        X = np.ascontiguousarray(X, dtype=dt)
        if X.ndim == 1:
            X = X.reshape(-1, 1)
        words = X.shape[1]
        if B is None:
            B = words * 32 if sr == BOOLEAN else words
        Y = np.empty((self.rows, words), dtype=dt)
        c = self._cfg(**cfg)
        _check(lib().gmr_engine_multiply_host(self._h, sr, X.ctypes.data_as(C.c_void_p),
                                              Y.ctypes.data_as(C.c_void_p), B, C.byref(c)))
        return Y

    def time_launches(self, semiring, x_ptr: int, y_ptr: int, B: int, stream: int = 0, **cfg) -> np.ndarray:
        """Device time (ms) of every launch of one multiply (prologue, levels, final fold)."""
        c = self._cfg(**cfg)
        cap = 4096
        ms = np.zeros(cap, dtype=np.float32)
        n = C.c_int()
        _check(lib().gmr_engine_time_launches(self._h, semiring_id(semiring), C.c_void_p(x_ptr), C.c_void_p(y_ptr),
                                              B, C.byref(c), C.c_void_p(stream), ms.ctypes.data_as(L.F32P), cap,
                                              C.byref(n)))
        return ms[: n.value].copy()

    N_LEVEL_VARIANTS = 20

    def mode_costs(self, semiring, B: int):
        """[slots][3 prev mode][3 mode] ms of the last autotune's emission-mode
        chain search for (semiring, B) (-1 = not measured), or None."""
        cap = (self.depth + 2) * 9
        out = np.zeros(cap, dtype=np.float32)
        n = C.c_int()
        _check(lib().gmr_engine_mode_costs(self._h, semiring_id(semiring), int(B), out.ctypes.data_as(L.F32P), cap,
                                           C.byref(n)))
        return out[: n.value * 9].reshape(n.value, 3, 3) if n.value else None

    def lane_bytes(self, semiring, B: int) -> int:
        """Bytes each lane moves per value access in a default multiply of (semiring, B)."""
        return int(lib().gmr_engine_lane_bytes(self._h, semiring_id(semiring), int(B)))

    def enable_left(self, plan: "Plan"):
        """Upload the reverse adjacency needed by the left product y = x^T M."""
        _check(lib().gmr_engine_enable_left(self._h, plan._h))

    def multiply_host_many(self, semiring, x_ptrs, y_ptrs, B: int, **cfg):
        """n multiplies from host X buffers into host Y buffers (raw addresses,
        page-locked for the copies to overlap), pipelined through two device
        staging pairs."""
        n = len(x_ptrs)
        if len(y_ptrs) != n:
            raise ValueError("as many Y buffers as X buffers")
        xs = (C.c_void_p * n)(*[C.c_void_p(int(p)) for p in x_ptrs])
        ys = (C.c_void_p * n)(*[C.c_void_p(int(p)) for p in y_ptrs])
        c = self._cfg(**cfg)
        _check(lib().gmr_engine_multiply_host_many(self._h, semiring_id(semiring), xs, ys, n, B, C.byref(c)))

    def multiply_left_device(self, semiring, x_ptr: int, y_ptr: int, B: int, stream: int = 0):
        """y[cols][words] = x^T M for x[rows][words] (device pointers)."""
        _check(lib().gmr_engine_multiply_left(self._h, semiring_id(semiring), C.c_void_p(x_ptr),
                                              C.c_void_p(y_ptr), B, C.c_void_p(stream)))

    def fixpoint_device(self, semiring, x_ptr: int, y_ptr: int, B: int, max_iters: int = 1000,
                        stream: int = 0) -> int:
        """x <- x (+) M x until it stops changing (boolean / tropical, square M); returns the iterations."""
        it = C.c_int()
        _check(lib().gmr_engine_fixpoint(self._h, semiring_id(semiring), C.c_void_p(x_ptr), C.c_void_p(y_ptr), B,
                                         max_iters, C.c_void_p(stream), C.byref(it)))
        return it.value

    def set_level_variants(self, semiring, B: int, table):
        """Install a per-launch variant table (len depth + 2) used by AUTO multiplies; None clears."""
        if table is None:
            _check(lib().gmr_engine_set_level_variants(self._h, semiring_id(semiring), B, None, 0))
            return
        t = np.ascontiguousarray(table, dtype=np.uint8)
        _check(lib().gmr_engine_set_level_variants(self._h, semiring_id(semiring), B,
                                                   t.ctypes.data_as(C.POINTER(C.c_uint8)), len(t)))

    def level_variants(self, semiring, B: int):
        n = C.c_int()
        buf = np.zeros(4096, dtype=np.uint8)
        _check(lib().gmr_engine_get_level_variants(self._h, semiring_id(semiring), B,
                                                   buf.ctypes.data_as(C.POINTER(C.c_uint8)), len(buf), C.byref(n)))
        return buf[: n.value].copy() if n.value else None

    def autotune(self, semiring, x_ptr: int, y_ptr: int, B: int, stream: int = 0, reps: int = 3,
                 energy_tolerance: float = 0.0) -> np.ndarray:
        """Exhaustive per-launch autotuner; installs the best table and returns times[slot][variant] (ms).
        energy_tolerance > 0 prefers each launch's source-chunked twin (fewer DRAM bytes) when it is at
        most that fraction slower."""
        depth = self.depth
        ms = np.zeros((depth + 2) * self.N_LEVEL_VARIANTS, dtype=np.float32)
        _check(lib().gmr_engine_autotune_energy(self._h, semiring_id(semiring), C.c_void_p(x_ptr),
                                                C.c_void_p(y_ptr), B, C.c_void_p(stream), reps,
                                                float(energy_tolerance), ms.ctypes.data_as(L.F32P), len(ms)))
        return ms.reshape(depth + 2, self.N_LEVEL_VARIANTS)

    @property
    def last_launches(self) -> int:
        return int(lib().gmr_engine_last_launches(self._h))

    @property
    def device_bytes(self) -> int:
        return int(lib().gmr_engine_device_bytes(self._h))


class Pack:
    """Several engines multiplied by one CUDA-graph launch (one branch per engine)."""

    def __init__(self, engines):
        self.engines = list(engines)
        arr = (C.c_void_p * len(self.engines))(*[e._h.value for e in self.engines])
        h = C.c_void_p()
        _check(lib().gmr_pack_create(arr, len(self.engines), C.byref(h)))
        self._h = h

    def multiply_device(self, semirings, x_ptrs, y_ptrs, Bs, stream: int = 0):
        n = len(self.engines)
        sr = (C.c_int * n)(*[semiring_id(s) for s in semirings])
        xs = (C.c_void_p * n)(*x_ptrs)
        ys = (C.c_void_p * n)(*y_ptrs)
        bs = (C.c_int * n)(*Bs)
        _check(lib().gmr_pack_multiply(self._h, sr, xs, ys, bs, C.c_void_p(stream)))

    GRAPH, PERSISTENT, LEVELS = 0, 1, 2

    def set_mode(self, mode: int, spin_limit: int = 0):
        """Pack.GRAPH (default): one CUDA-graph launch of per-engine branches;
        Pack.LEVELS: one launch per level over every grammar;
        Pack.PERSISTENT: one cooperative kernel for the whole pack."""
        _check(lib().gmr_pack_set_mode(self._h, int(mode), int(spin_limit)))

    def status(self):
        """(ran_persistent, failed, phase) of the last multiply (after a stream synchronize)."""
        a, f, p = C.c_int(), C.c_int(), C.c_int()
        _check(lib().gmr_pack_status(self._h, C.byref(a), C.byref(f), C.byref(p)))
        return bool(a.value), f.value, p.value

    @property
    def last_launches(self) -> int:
        return int(lib().gmr_pack_last_launches(self._h))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().gmr_pack_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        self.close()


def measure_gather_bandwidth(buffer_bytes: int, device: int = 0, sequential: bool = False) -> float:
    """Random (or, sequential=True, in-order) 128-byte line read bandwidth
    (GB/s) over a buffer of that size."""
    g = C.c_float()
    _check(lib().gmr_measure_gather_bandwidth(device, int(buffer_bytes), int(bool(sequential)), C.byref(g)))
    return float(g.value)


GATHER_MODES = {"load16": 0, "seq16": 1, "load32": 2, "bulk": 3}


def measure_gather(buffer_bytes: int, mode: str = "load16", depth: int = 4, unit_bytes: int = 128,
                   device: int = 0) -> float:
    """Gather bandwidth (GB/s) of random units of unit_bytes over a buffer of
    that size along one load path: "load16" / "load32" lane loads with `depth`
    loads in flight per thread, "seq16" the same in order, "bulk" one bulk copy
    per unit into shared memory with `depth` copies in flight per warp."""
    g = C.c_float()
    _check(lib().gmr_measure_gather(device, int(buffer_bytes), GATHER_MODES[mode], int(depth), int(unit_bytes),
                                    C.byref(g)))
    return float(g.value)


# ---------------------------------------------------------------- legacy ABI
def _legacy_args(rows, cols, alpha, rules_lrc, val_indices, col_indices, V, sched):
    keep = []
    rules = _layered_rules(rules_lrc)
    keep.append(rules)
    vi, pvi = _i32(val_indices if len(val_indices) else np.zeros(1, np.int32))
    ci, pci = _i32(col_indices if len(col_indices) else np.zeros(1, np.int32))
    v, pv = _f32(V)
    keep += [vi, ci, v]
    gs = _gpu_schedule(sched, keep)
    n_rules = len(np.asarray(rules_lrc)) if not isinstance(rules_lrc, C.Array) else len(rules_lrc)
    return keep, rules, pvi, pci, pv, len(v), gs, n_rules


def run_gpu_right_multiply_layered(rows, cols, alpha, rules_lrc, val_indices, col_indices, V, x, sched,
                                   iters=1) -> np.ndarray:
    """Calls the drop-in entry point; returns y (float32, or int32 for the
    Boolean/tropical semirings chosen by the SEMIRING environment variable)."""
    keep, rules, pvi, pci, pv, nv, gs, n = _legacy_args(rows, cols, alpha, rules_lrc, val_indices, col_indices, V,
                                                        sched)
    x, px = _f32(x)
    y = np.zeros(max(rows, 1), dtype=np.float32)
    lib().run_gpu_right_multiply_layered(rows, cols, alpha, n, rules, pvi, pci, pv, nv, px, C.byref(gs),
                                         y.ctypes.data_as(L.F32P), iters)
    sr = semiring_id(os.environ.get("SEMIRING", "plustimes"))
    return y[:rows].view(np.int32) if sr != PLUS_TIMES else y[:rows]


def run_gpu_right_multiply_batched(rows, cols, alpha, rules_lrc, val_indices, col_indices, V, X, sched, B,
                                   iters=1) -> np.ndarray:
    keep, rules, pvi, pci, pv, nv, gs, n = _legacy_args(rows, cols, alpha, rules_lrc, val_indices, col_indices, V,
                                                        sched)
    X, px = _f32(np.asarray(X).reshape(-1))
    Y = np.zeros(max(rows * B, 1), dtype=np.float32)
    lib().run_gpu_right_multiply_batched(rows, cols, alpha, n, rules, pvi, pci, pv, nv, px, C.byref(gs),
                                         Y.ctypes.data_as(L.F32P), B, iters)
    sr = semiring_id(os.environ.get("SEMIRING", "plustimes"))
    Y = Y[: rows * B].reshape(rows, B)
    return Y.view(np.int32) if sr != PLUS_TIMES else Y
