"""ctypes wrapper of the CPU oracle (``oracle/pmsz_oracle.c``).

TEST INFRASTRUCTURE ONLY: tests/, the smoke() entry point and the CPU-baseline
leg of bench.py use it as the parity checker; the product path never imports
it.  Every function here mirrors one C function, which cites the reference
file:line it restates.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libpmsz_oracle.so")
_lock = threading.Lock()
_lib = None

OK, ERR_ARG, ERR_OOM, ERR_NOT_CONVERGED = 0, 1, 2, 3

_I64 = ctypes.c_int64
_P = ctypes.c_void_p


class SweepRecord(ctypes.Structure):
    _fields_ = [("fmax", ctypes.c_uint64), ("fmin", ctypes.c_uint64),
                ("fdir", ctypes.c_uint64), ("requested", ctypes.c_uint64),
                ("changed", ctypes.c_uint64)]


class Result(ctypes.Structure):
    _fields_ = [("sweeps", ctypes.c_int64), ("edits_applied", ctypes.c_int64),
                ("status", ctypes.c_int)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    src = os.path.join(_HERE, "pmsz_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "libpmsz_oracle.so"],
                       check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            for suf in ("f32", "f64"):
                getattr(L, f"pmszo_label_{suf}").argtypes = [_P, _I64, _I64, _I64, _P, _P]
                getattr(L, f"pmszo_correct_{suf}").argtypes = [
                    _P, _P, _I64, _I64, _I64, ctypes.c_double, ctypes.c_int,
                    _I64, _P, _P, _P]
                getattr(L, f"pmszo_verify_{suf}").argtypes = [
                    _P, _P, _I64, _I64, _I64, ctypes.c_double, _P]
                getattr(L, f"pmszo_extract_edits_{suf}").argtypes = [
                    _P, _P, _P, _I64, ctypes.c_double, ctypes.c_int, _P, _P,
                    _P, _P]
                getattr(L, f"pmszo_correct_naive_{suf}").argtypes = [
                    _P, _P, _I64, _I64, _I64, ctypes.c_double, ctypes.c_int, _I64, _P, _P, _P]
                getattr(L, f"pmszo_reconstruct_{suf}").argtypes = [
                    _P, _P, _P, _I64, _I64, ctypes.c_double, ctypes.c_int, _P]
                getattr(L, f"pmszo_perlin_{suf}").argtypes = [_P, _I64, _I64, _I64, _P, _P, _P, ctypes.c_int]
                getattr(L, f"pmszo_standin_{suf}").argtypes = [_P, _P, _I64, ctypes.c_double, ctypes.c_int,
                                                               ctypes.c_uint64]
            L.pmszo_path_compress.argtypes = [_P, _P, _I64]
            L.pmszo_pack_nbits.argtypes = [_P, _I64, ctypes.c_uint, _P]
            L.pmszo_pack_nbits.restype = ctypes.c_int64
            L.pmszo_unpack_nbits.argtypes = [_P, _I64, _I64, ctypes.c_uint, _P]
            L.pmszo_bits_for_max.argtypes = [ctypes.c_uint]
            L.pmszo_bits_for_max.restype = ctypes.c_uint
            L.pmszo_set_threads.argtypes = [ctypes.c_int]
            L.pmszo_num_threads.restype = ctypes.c_int
            _lib = L
    return _lib


def _suf(a: np.ndarray) -> str:
    if a.dtype == np.float32:
        return "f32"
    if a.dtype == np.float64:
        return "f64"
    raise TypeError(f"unsupported dtype {a.dtype}")


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def _dims(a: np.ndarray):
    """Fields are numpy arrays of shape (nz, ny, nx), x fastest."""
    nz, ny, nx = a.shape
    return nx, ny, nz


def set_threads(n: int) -> None:
    lib().pmszo_set_threads(int(n))


def num_threads() -> int:
    return int(lib().pmszo_num_threads())


def label(v: np.ndarray):
    """Steepest ascent/descent flat indices of every voxel (pMSz.cu:686-783)."""
    v = np.ascontiguousarray(v)
    nx, ny, nz = _dims(v)
    asc = np.empty(v.size, np.int64)
    desc = np.empty(v.size, np.int64)
    rc = getattr(lib(), f"pmszo_label_{_suf(v)}")(_ptr(v), nx, ny, nz, _ptr(asc), _ptr(desc))
    if rc != OK:
        raise ValueError(f"label failed: {rc}")
    return asc, desc


def correct(f: np.ndarray, fhat: np.ndarray, eb: float, q: int = 5,
            max_sweeps: int = 100000):
    """Snapshot-semantics correction loop (pMSz.cu:1872-2074).

    Returns (corrected field, counters, status, sweeps, per-sweep records as an
    (sweeps, 5) uint64 array [fmax, fmin, fdir, requested, changed]).
    """
    f = np.ascontiguousarray(f)
    out = np.array(fhat, dtype=f.dtype, copy=True, order="C")
    nx, ny, nz = _dims(f)
    cnt = np.zeros(f.size, np.uint8)
    log = (SweepRecord * int(max_sweeps))()
    res = Result()
    rc = getattr(lib(), f"pmszo_correct_{_suf(f)}")(
        _ptr(f), _ptr(out), nx, ny, nz, float(eb), int(q), int(max_sweeps),
        _ptr(cnt), ctypes.cast(log, _P), ctypes.byref(res))
    if rc not in (OK, ERR_NOT_CONVERGED):
        raise ValueError(f"correct failed: {rc}")
    n = int(res.sweeps)
    recs = np.array([[log[i].fmax, log[i].fmin, log[i].fdir, log[i].requested,
                      log[i].changed] for i in range(n)], dtype=np.uint64).reshape(n, 5)
    return out, cnt.reshape(f.shape), int(res.status), n, recs


def correct_naive(f: np.ndarray, fhat: np.ndarray, eb: float, q: int = 5, max_sweeps: int = 100000):
    """naive-MSz loop (naive_MSz.cu:1887-2220), snapshot semantics; same
    return convention as correct()."""
    f = np.ascontiguousarray(f)
    out = np.array(fhat, dtype=f.dtype, copy=True, order="C")
    nx, ny, nz = _dims(f)
    cnt = np.zeros(f.size, np.uint8)
    log = (SweepRecord * int(max_sweeps))()
    res = Result()
    rc = getattr(lib(), f"pmszo_correct_naive_{_suf(f)}")(
        _ptr(f), _ptr(out), nx, ny, nz, float(eb), int(q), int(max_sweeps), _ptr(cnt),
        ctypes.cast(log, _P), ctypes.byref(res))
    if rc not in (OK, ERR_NOT_CONVERGED):
        raise ValueError(f"correct_naive failed: {rc}")
    n = int(res.sweeps)
    recs = np.array([[log[i].fmax, log[i].fmin, log[i].fdir, log[i].requested, log[i].changed]
                     for i in range(n)], dtype=np.uint64).reshape(n, 5)
    return out, cnt.reshape(f.shape), int(res.status), n, recs


def path_compress(direction: np.ndarray) -> np.ndarray:
    """Root of every vertex's direction chain (PathCompression, pMSz.cu:255-271)."""
    d = np.ascontiguousarray(direction, dtype=np.int64)
    out = np.empty_like(d)
    lib().pmszo_path_compress(_ptr(d), _ptr(out), d.size)
    return out


def verify(f: np.ndarray, fp: np.ndarray, eb: float) -> dict:
    """[dir, extremum, AS label, DS label, bound] mismatch counts."""
    f = np.ascontiguousarray(f)
    fp = np.ascontiguousarray(fp, dtype=f.dtype)
    nx, ny, nz = _dims(f)
    out = np.zeros(5, np.uint64)
    rc = getattr(lib(), f"pmszo_verify_{_suf(f)}")(_ptr(f), _ptr(fp), nx, ny, nz, float(eb), _ptr(out))
    if rc != OK:
        raise ValueError(f"verify failed: {rc}")
    keys = ("dir_mismatch", "ext_mismatch", "as_mismatch", "ds_mismatch", "bound_violations")
    return {k: int(v) for k, v in zip(keys, out)}


def extract_edits(prev: np.ndarray, cur: np.ndarray, f: np.ndarray, eb: float, q: int = 5):
    """(deltas uint8[n], clamp list, edit_count) as extract_edits_kernel (pMSz.cu:2090-2138)."""
    prev = np.ascontiguousarray(prev).ravel()
    cur = np.ascontiguousarray(cur, dtype=prev.dtype).ravel()
    f = np.ascontiguousarray(f, dtype=prev.dtype).ravel()
    deltas = np.empty(prev.size, np.uint8)
    clamp = np.empty(prev.size, prev.dtype)
    nc = ctypes.c_int64()
    ec = ctypes.c_int64()
    rc = getattr(lib(), f"pmszo_extract_edits_{_suf(prev)}")(
        _ptr(prev), _ptr(cur), _ptr(f), prev.size, float(eb), int(q), _ptr(deltas),
        _ptr(clamp), ctypes.byref(nc), ctypes.byref(ec))
    if rc != OK:
        raise ValueError(f"extract failed: {rc}")
    return deltas, clamp[: nc.value].copy(), int(ec.value)


def reconstruct(prev: np.ndarray, deltas: np.ndarray, clamp: np.ndarray, eb: float, q: int = 5):
    prev = np.ascontiguousarray(prev).ravel()
    deltas = np.ascontiguousarray(deltas, dtype=np.uint8)
    clamp = np.ascontiguousarray(clamp, dtype=prev.dtype)
    out = np.empty_like(prev)
    rc = getattr(lib(), f"pmszo_reconstruct_{_suf(prev)}")(
        _ptr(prev), _ptr(deltas), _ptr(clamp), clamp.size, prev.size, float(eb), int(q), _ptr(out))
    if rc != OK:
        raise ValueError(f"reconstruct failed: {rc}")
    return out


def pack_nbits(sym: np.ndarray, nbits: int) -> bytes:
    sym = np.ascontiguousarray(sym, dtype=np.uint8)
    out = np.empty((sym.size * nbits + 7) // 8 + 1, np.uint8)
    n = lib().pmszo_pack_nbits(_ptr(sym), sym.size, nbits, _ptr(out))
    if n < 0:
        raise ValueError("symbol exceeds the n-bit range")
    return out[:n].tobytes()


def unpack_nbits(packed: bytes, n: int, nbits: int) -> np.ndarray:
    buf = np.frombuffer(packed, np.uint8).copy()
    out = np.empty(n, np.uint8)
    rc = lib().pmszo_unpack_nbits(_ptr(buf), buf.size, n, nbits, _ptr(out))
    if rc != OK:
        raise ValueError("packed too small")
    return out


def bits_for_max(m: int) -> int:
    return int(lib().pmszo_bits_for_max(int(m)))


def perlin_field(shape, seed: int, octaves: int, base_freq: float, persistence: float = 0.5,
                 lacunarity: float = 2.0, dtype=np.float32) -> np.ndarray:
    """Normalised Perlin fBm field of shape (nz, ny, nx) on the host cores,
    bit-identical to pmsz_anonymous_gb300.fields.perlin_field (the noise of
    generate_perlin.py:17-59, its permutation recipe :105-108)."""
    from pmsz_anonymous_gb300 import fields  # numpy only: permutation and octave table
    nz, ny, nx = (int(v) for v in shape)
    out = np.empty((nz, ny, nx), dtype=dtype)
    perm = np.ascontiguousarray(fields.permutation(seed), dtype=np.int32)
    amps, freqs = fields.octave_table(octaves, base_freq, persistence, lacunarity)
    amps, freqs = np.ascontiguousarray(amps), np.ascontiguousarray(freqs)
    rc = getattr(lib(), f"pmszo_perlin_{_suf(out)}")(_ptr(out), nx, ny, nz, _ptr(perm), _ptr(amps), _ptr(freqs),
                                                      int(octaves))
    if rc != OK:
        raise ValueError(f"perlin failed: {rc}")
    return out


def standin(f: np.ndarray, eb: float, compressor: str, seed: int = 0) -> np.ndarray:
    """The labelled compressor stand-in of fields.standin on the host cores
    ("sz3": plateaus, "zfp": bounded noise), bit-identical to it."""
    kinds = {"sz3": 0, "zfp": 1}
    if compressor not in kinds:
        raise ValueError(f"unknown compressor {compressor!r} (expected 'sz3' or 'zfp')")
    f = np.ascontiguousarray(f)
    out = np.empty_like(f)
    rc = getattr(lib(), f"pmszo_standin_{_suf(f)}")(_ptr(f), _ptr(out), f.size, float(eb), kinds[compressor],
                                                     int(seed) & 0xFFFFFFFFFFFFFFFF)
    if rc != OK:
        raise ValueError(f"standin failed: {rc}")
    return out
