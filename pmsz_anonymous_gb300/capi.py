"""ctypes declarations of the C ABI (include/pmsz.h, include/pmsz_host.h).

The shared library is built in-tree by ``pmsz_anonymous_gb300._build`` and
loaded from ``pmsz_anonymous_gb300/lib/``.  There is no fallback: if the
library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

c_i32, c_u32, c_i64, c_u64 = ctypes.c_int32, ctypes.c_uint32, ctypes.c_int64, ctypes.c_uint64
c_size, c_double, c_int, c_void_p = ctypes.c_size_t, ctypes.c_double, ctypes.c_int, ctypes.c_void_p

PMSZ_OK, PMSZ_ERR_ARG, PMSZ_ERR_OOM, PMSZ_ERR_NOT_CONVERGED, PMSZ_ERR_CUDA, PMSZ_ERR_IO = range(6)
PMSZ_FLAG_FULL_SWEEPS = 1
PMSZ_FLAG_TIMING = 2
PMSZ_FLAG_EDITS_ONLY = 4
PMSZ_FLAG_NAIVE = 8
PMSZ_FLAG_AUTOTUNE = 16
PMSZ_FLAG_PACKED_DELTAS = 32
PMSZ_FLAG_HOST_LOOP = 64


class Opts(ctypes.Structure):
    _fields_ = [("q", c_i32), ("flags", c_u32), ("max_sweeps", c_i64)]


class SweepRecord(ctypes.Structure):
    _fields_ = [("fmax", c_u64), ("fmin", c_u64), ("fdir", c_u64), ("requested", c_u64),
                ("changed", c_u64), ("progressed", c_u64), ("active", c_u64), ("bad", c_u64)]


class Result(ctypes.Structure):
    _fields_ = [("sweeps", c_i64), ("iteration", c_i64), ("edits", c_u64),
                ("sweep_log", ctypes.POINTER(SweepRecord)), ("sweep_log_cap", c_i64),
                ("ms_first_pass", c_double), ("ms_detect", c_double), ("ms_apply", c_double),
                ("launches", c_i64), ("ms_total", c_double)]


class VerifyResult(ctypes.Structure):
    _fields_ = [("dir_mismatch", c_u64), ("ext_mismatch", c_u64), ("as_mismatch", c_u64),
                ("ds_mismatch", c_u64), ("bound_strict", c_u64), ("bound_beyond_clamp", c_u64)]


class Field(ctypes.Structure):
    _fields_ = [("f", c_void_p), ("fhat", c_void_p), ("nx", c_size), ("ny", c_size), ("nz", c_size),
                ("eb", c_double), ("elem_size", c_u32), ("reserved", c_u32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", c_size), ("max_jobs", c_i32), ("q", c_i32), ("max_sweeps", c_i64)]


class JobInfo(ctypes.Structure):
    _fields_ = [("done", c_i32), ("status", c_i32), ("sweeps", c_i64), ("edits", c_u64), ("queue_ms", c_double),
                ("run_ms", c_double), ("latency_ms", c_double)]


class Tune(ctypes.Structure):
    _fields_ = [("zchunk", c_i32), ("jump_rounds", c_i32), ("ms_zchunk", ctypes.c_float * 4),
                ("ms_rounds", ctypes.c_float * 4)]


class HostOutputs(ctypes.Structure):
    _fields_ = [("deltas", c_void_p), ("clamp", c_void_p), ("n_clamp", c_u64), ("edit_count", c_u64),
                ("verify", ctypes.POINTER(VerifyResult))]


# name -> (restype, argtypes), one line per declaration in include/*.h
_P = c_void_p
SIGNATURES = {
    "pmsz_correct_f32": (c_int, [_P, _P, c_size, c_size, c_size, c_double, _P, _P, _P]),
    "pmsz_correct_f64": (c_int, [_P, _P, c_size, c_size, c_size, c_double, _P, _P, _P]),
    "pmsz_correct_naive_f32": (c_int, [_P, _P, c_size, c_size, c_size, c_double, _P, _P, _P]),
    "pmsz_correct_naive_f64": (c_int, [_P, _P, c_size, c_size, c_size, c_double, _P, _P, _P]),
    "pmsz_codes_f32": (c_int, [_P, c_size, c_size, c_size, _P, _P]),
    "pmsz_codes_f64": (c_int, [_P, c_size, c_size, c_size, _P, _P]),
    "pmsz_rank_offset": (c_int, [c_int, _P, _P, _P]),
    "pmsz_labels": (c_int, [_P, c_size, c_size, c_size, _P, _P, _P]),
    "pmsz_verify_f32": (c_int, [_P, _P, c_size, c_size, c_size, c_double, _P, _P]),
    "pmsz_verify_f64": (c_int, [_P, _P, c_size, c_size, c_size, c_double, _P, _P]),
    "pmsz_extract_edits_f32": (c_int, [_P, _P, _P, c_size, c_double, c_int, _P, _P, _P, _P, _P]),
    "pmsz_extract_edits_f64": (c_int, [_P, _P, _P, c_size, c_double, c_int, _P, _P, _P, _P, _P]),
    "pmsz_reconstruct_f32": (c_int, [_P, _P, _P, c_u64, c_size, c_double, c_int, _P, _P]),
    "pmsz_reconstruct_f64": (c_int, [_P, _P, _P, c_u64, c_size, c_double, c_int, _P, _P]),
    "pmsz_gen_perlin_f32": (c_int, [_P, c_size, c_size, c_size, _P, _P, _P, c_int, _P]),
    "pmsz_gen_perlin_f64": (c_int, [_P, c_size, c_size, c_size, _P, _P, _P, c_int, _P]),
    "pmsz_standin_f32": (c_int, [_P, _P, c_size, c_double, c_int, c_u64, _P]),
    "pmsz_standin_f64": (c_int, [_P, _P, c_size, c_double, c_int, c_u64, _P]),
    "pmsz_strerror": (ctypes.c_char_p, [c_int]),
    "pmsz_last_error": (ctypes.c_char_p, []),
    "pmsz_version": (c_int, []),
    "pmsz_encode_deltas": (c_int, [_P, c_size, c_int, _P, _P]),
    "pmsz_encode_packed_deltas": (c_int, [_P, c_size, _P, _P]),
    "pmsz_encode_clamps": (c_int, [_P, c_size, c_size, _P, _P]),
    "pmsz_decode_deltas": (c_int, [_P, c_size, c_size, c_int, _P]),
    "pmsz_decode_clamps": (c_int, [_P, c_size, c_size, _P, _P]),
    "pmsz_free": (None, [_P]),
    "pmsz_zstd_version": (c_u32, []),
    "pmsz_server_create": (c_int, [_P, _P]),
    "pmsz_server_submit": (c_int, [_P, _P, _P]),
    "pmsz_server_wait": (c_int, [_P, c_u64, c_double, _P]),
    "pmsz_server_release": (c_int, [_P, c_u64]),
    "pmsz_server_destroy": (c_int, [_P]),
    "pmsz_correct_batch": (c_int, [_P, c_int, _P, _P, _P, _P]),
    "pmsz_correct_noalloc": (c_int, [_P, _P, c_size, c_size, c_size, c_size, c_double, _P, _P, _P]),
    "pmsz_correct_host_f32": (c_int, [_P, _P, c_size, c_size, c_size, c_double, _P, _P, _P, _P]),
    "pmsz_correct_host_f64": (c_int, [_P, _P, c_size, c_size, c_size, c_double, _P, _P, _P, _P]),
    "pmsz_autotune_f32": (c_int, [_P, _P, c_size, c_size, c_size, _P, _P]),
    "pmsz_autotune_f64": (c_int, [_P, _P, c_size, c_size, c_size, _P, _P]),
    "pmsz_tune_get": (c_int, [c_size, c_size, c_size, c_size, _P]),
    "pmsz_tune_batch_get": (c_int, [c_size, c_int, c_size, _P]),
    "pmsz_tune_set": (c_int, [c_size, c_size, c_size, c_size, _P]),
    "pmsz_tune_save": (c_int, [ctypes.c_char_p]),
    "pmsz_tune_load": (c_int, [ctypes.c_char_p]),
    "pmsz_tune_clear": (None, []),
}

_lock = threading.Lock()
_lib = None


class PmszError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"pmsz status {status}: {message}")
        self.status = status
        self.message = message


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libpmsz_gb300.so (building it first if it is absent)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not os.path.exists(path):
                if not build_if_missing:
                    raise RuntimeError(f"{path} is missing: run pmsz_anonymous_gb300._build.build()")
                _build.build()
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(status: int, allow=(PMSZ_OK,)) -> int:
    if status not in allow:
        msg = load().pmsz_last_error()
        raise PmszError(status, msg.decode() if msg else "")
    return status
