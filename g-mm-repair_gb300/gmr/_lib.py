"""ctypes bindings of libgmr.so (declarations mirror include/gmr.h)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libgmr.so"

GMR_OK = 0
STATUS_NAMES = {
    1: "GMR_ERR_ARG", 2: "GMR_ERR_FORMAT", 3: "GMR_ERR_IO", 4: "GMR_ERR_CUDA", 5: "GMR_ERR_OOM",
    6: "GMR_ERR_RANGE", 7: "GMR_ERR_TIMEOUT", 8: "GMR_ERR_STATE",
}


class LayeredRule(C.Structure):
    """gpu-engine/layered_types.h:45-49"""
    _fields_ = [("left", C.c_int), ("right", C.c_int), ("coeff", C.c_float)]


class GPUSchedule(C.Structure):
    """gpu-engine/layered_types.h:61-75"""
    _fields_ = [
        ("max_depth", C.c_int), ("max_width", C.c_int),
        ("level_offsets", C.POINTER(C.c_int)), ("level_widths", C.POINTER(C.c_int)),
        ("emit_offsets", C.POINTER(C.c_int)), ("emit_pos", C.POINTER(C.c_int)),
        ("emit_row", C.POINTER(C.c_int)), ("emit_total", C.c_int),
        ("term_emit_sym", C.POINTER(C.c_int)), ("term_emit_row", C.POINTER(C.c_int)),
        ("num_term_emit", C.c_int),
    ]


class GrammarInfo(C.Structure):
    _fields_ = [("alpha", C.c_int), ("n_rules", C.c_int64), ("c_len", C.c_int64), ("n_vals", C.c_int),
                ("has_runlen", C.c_int)]


class CsrvInfo(C.Structure):
    _fields_ = [("rows", C.c_int), ("cols", C.c_int), ("len", C.c_int64), ("nnz", C.c_int64),
                ("n_vals", C.c_int)]


class PlanStats(C.Structure):
    _fields_ = [
        ("rows", C.c_int), ("cols", C.c_int), ("depth", C.c_int), ("n_vals", C.c_int), ("has_coeff", C.c_int),
        ("n_ops", C.c_int64), ("n_emit", C.c_int64), ("n_term_emit", C.c_int64), ("n_terms", C.c_int64),
        ("max_level_ops", C.c_int64),
        ("ref_layered", C.c_int64), ("ref_raw", C.c_int64), ("ref_passthrough", C.c_int64),
        ("ref_max_width", C.c_int64), ("ref_emit", C.c_int64), ("ref_term_emit", C.c_int64),
        ("ref_alpha", C.c_int64),
    ]


class DevicePlan(C.Structure):
    """gmr_device_plan of include/gmr.h"""
    _fields_ = [
        ("rows", C.c_int), ("cols", C.c_int), ("depth", C.c_int), ("n_ops", C.c_int64), ("n_terms", C.c_int64),
        ("lvl_off", C.c_void_p), ("seg_off", C.c_void_p), ("ops", C.c_void_p), ("op_c", C.c_void_p),
        ("em_src", C.c_void_p), ("seg_row", C.c_void_p), ("seg_start", C.c_void_p), ("term_val", C.c_void_p),
        ("term_col", C.c_void_p), ("V", C.c_void_p),
    ]


class Config(C.Structure):
    _fields_ = [("variant", C.c_int), ("vec_tile", C.c_int), ("ops_per_cta", C.c_int), ("emit_mode", C.c_int),
                ("tile_levels", C.c_int), ("spin_limit", C.c_int), ("push", C.c_int), ("lane_bytes", C.c_int)]


P = C.c_void_p
I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)
F32P = C.POINTER(C.c_float)

_SIGS = {
    "gmr_last_error": (C.c_char_p, []),
    "gmr_version": (C.c_char_p, []),
    "gmr_grammar_load": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "gmr_grammar_save": (C.c_int, [P, C.c_char_p]),
    "gmr_grammar_create": (C.c_int, [C.c_int, C.c_int64, I32P, I32P, I32P, C.c_int64, I32P, C.c_int, F64P,
                                     C.POINTER(P)]),
    "gmr_grammar_get_info": (C.c_int, [P, C.POINTER(GrammarInfo)]),
    "gmr_grammar_rules": (I32P, [P]),
    "gmr_grammar_kinds": (I32P, [P]),
    "gmr_grammar_reps": (I32P, [P]),
    "gmr_grammar_C": (I32P, [P]),
    "gmr_grammar_V": (F64P, [P]),
    "gmr_grammar_free": (None, [P]),
    "gmr_csrv_create": (C.c_int, [C.c_int, C.c_int, C.c_int64, I32P, C.c_int, F64P, C.POINTER(P)]),
    "gmr_csrv_from_dense": (C.c_int, [C.c_int, C.c_int, F64P, C.POINTER(P)]),
    "gmr_csrv_get_info": (C.c_int, [P, C.POINTER(CsrvInfo)]),
    "gmr_csrv_codes": (I32P, [P]),
    "gmr_csrv_V": (F64P, [P]),
    "gmr_csrv_free": (None, [P]),
    "gmr_gen_mosaic": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint64, C.c_int,
                                 C.POINTER(P)]),
    "gmr_gen_copy_graph": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_int, C.c_uint64, C.c_int, C.POINTER(P)]),
    "gmr_repair_compress": (C.c_int, [P, C.c_int, C.POINTER(P)]),
    "gmr_repair_compress_device": (C.c_int, [P, C.c_int, C.POINTER(P)]),
    "gmr_plan_build": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(P)]),
    "gmr_plan_build_device": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(P)]),
    "gmr_plan_from_layered": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(LayeredRule), I32P, I32P,
                                        F32P, C.c_int, C.POINTER(GPUSchedule), C.POINTER(P)]),
    "gmr_plan_get_stats": (C.c_int, [P, C.POINTER(PlanStats)]),
    "gmr_plan_level_ops": (C.c_int, [P, C.POINTER(C.c_int64), C.c_int]),
    "gmr_plan_level_emits": (C.c_int, [P, C.POINTER(C.c_int64), C.c_int]),
    "gmr_plan_alg_bytes": (C.c_double, [P, C.c_int, C.c_int]),
    "gmr_plan_array": (C.c_int, [P, C.c_int, C.POINTER(P), C.POINTER(C.c_int64)]),
    "gmr_plan_describe": (C.c_int, [P, C.c_char_p, C.c_size_t]),
    "gmr_plan_window_stats": (C.c_int, [P, C.c_int, C.c_int, F64P, C.c_int, C.POINTER(C.c_int)]),
    "gmr_plan_free": (None, [P]),
    "gmr_engine_create": (C.c_int, [P, C.c_int, C.POINTER(P)]),
    "gmr_engine_multiply": (C.c_int, [P, C.c_int, P, P, C.c_int, C.POINTER(Config), P]),
    "gmr_engine_multiply_host": (C.c_int, [P, C.c_int, P, P, C.c_int, C.POINTER(Config)]),
    "gmr_engine_multiply_host_many": (C.c_int, [P, C.c_int, C.POINTER(P), C.POINTER(P), C.c_int, C.c_int,
                                                C.POINTER(Config)]),
    "gmr_engine_time_launches": (C.c_int, [P, C.c_int, P, P, C.c_int, C.POINTER(Config), P, F32P, C.c_int,
                                           C.POINTER(C.c_int)]),
    "gmr_engine_set_level_variants": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(C.c_uint8), C.c_int]),
    "gmr_engine_get_level_variants": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(C.c_uint8), C.c_int,
                                                C.POINTER(C.c_int)]),
    "gmr_engine_autotune": (C.c_int, [P, C.c_int, P, P, C.c_int, P, C.c_int, F32P, C.c_int]),
    "gmr_engine_autotune_energy": (C.c_int, [P, C.c_int, P, P, C.c_int, P, C.c_int, C.c_float, F32P, C.c_int]),
    "gmr_measure_gather_bandwidth": (C.c_int, [C.c_int, C.c_int64, C.c_int, F32P]),
    "gmr_measure_gather": (C.c_int, [C.c_int, C.c_int64, C.c_int, C.c_int, C.c_int, F32P]),
    "gmr_engine_status": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "gmr_engine_last_launches": (C.c_int64, [P]),
    "gmr_plan_prepare_left": (C.c_int, [P]),
    "gmr_engine_enable_left": (C.c_int, [P, P]),
    "gmr_engine_multiply_left": (C.c_int, [P, C.c_int, P, P, C.c_int, P]),
    "gmr_engine_fixpoint": (C.c_int, [P, C.c_int, P, P, C.c_int, C.c_int, P, C.POINTER(C.c_int)]),
    "gmr_engine_lane_bytes": (C.c_int, [P, C.c_int, C.c_int]),
    "gmr_engine_mode_costs": (C.c_int, [P, C.c_int, C.c_int, F32P, C.c_int, C.POINTER(C.c_int)]),
    "gmr_pack_create": (C.c_int, [C.POINTER(P), C.c_int, C.POINTER(P)]),
    "gmr_pack_multiply": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(P), C.POINTER(P), C.POINTER(C.c_int), P]),
    "gmr_pack_last_launches": (C.c_int64, [P]),
    "gmr_pack_set_mode": (C.c_int, [P, C.c_int, C.c_int]),
    "gmr_pack_status": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "gmr_pack_free": (None, [P]),
    "gmr_engine_device_bytes": (C.c_int64, [P]),
    "gmr_engine_free": (None, [P]),
    "gmr_plan_launch_features": (C.c_int, [P, C.c_int, C.c_int, F32P, C.c_int, C.POINTER(C.c_int)]),
    "gmr_mlp_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(P)]),
    "gmr_mlp_info": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int64)]),
    "gmr_mlp_params": (C.c_int, [P, F32P, F32P, C.c_int64]),
    "gmr_mlp_set_norm": (C.c_int, [P, F32P, F32P]),
    "gmr_mlp_predict": (C.c_int, [P, F32P, C.c_int, F32P]),
    "gmr_mlp_gradients": (C.c_int, [P, F32P, F32P, C.c_int, F32P, C.c_int64, F32P]),
    "gmr_mlp_train": (C.c_int, [P, F32P, F32P, C.c_int, C.c_int, C.c_int, C.c_float, C.c_uint64, F32P]),
    "gmr_mlp_save": (C.c_int, [P, C.c_char_p]),
    "gmr_mlp_load": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "gmr_mlp_free": (None, [P]),
    "gmr_engine_choose_learned": (C.c_int, [P, P, P, C.c_int, C.c_int, F32P, C.c_int]),
    "gmr_multiply_noalloc": (C.c_int, [C.POINTER(DevicePlan), C.c_int, P, P, C.c_int, P]),
    "run_gpu_right_multiply_layered": (None, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(LayeredRule), I32P,
                                              I32P, F32P, C.c_int, F32P, C.POINTER(GPUSchedule), F32P, C.c_int]),
    "run_gpu_right_multiply_batched": (None, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(LayeredRule), I32P,
                                              I32P, F32P, C.c_int, F32P, C.POINTER(GPUSchedule), F32P, C.c_int,
                                              C.c_int]),
}

EXPORTED = tuple(_SIGS)

_lib = None


def load() -> C.CDLL:
    """Loads libgmr.so; raises if the library has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (no fallback path exists)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
