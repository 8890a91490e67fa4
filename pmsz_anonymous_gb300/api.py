"""Python entry points over the C ABI, on torch CUDA tensors.

Fields are contiguous tensors of shape (nz, ny, nx) (x fastest), float32 or
float64, on a CUDA device.  Every call goes through libpmsz_gb300.so on the
current torch stream; there is no CPU path.
"""
from __future__ import annotations

import ctypes
import threading
from dataclasses import dataclass, field

import numpy as np
import torch

from . import capi
from . import fields as _fields

SWEEP_KEYS = ("fmax", "fmin", "fdir", "requested", "changed", "progressed", "active", "bad")


def _suffix(t: torch.Tensor) -> str:
    if t.dtype == torch.float32:
        return "f32"
    if t.dtype == torch.float64:
        return "f64"
    raise TypeError(f"fields must be float32 or float64, got {t.dtype}")


def _check_field(t: torch.Tensor, name: str):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dim() != 3 or not t.is_contiguous():
        raise ValueError(f"{name} must be a contiguous (nz, ny, nx) tensor")


def _dims(t: torch.Tensor):
    nz, ny, nx = t.shape
    return int(nx), int(ny), int(nz)


def _stream(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


@dataclass
class CorrectResult:
    status: int
    sweeps: int
    iteration: int
    edits: int
    log: np.ndarray = field(repr=False)  # (sweeps, 8) uint64, columns SWEEP_KEYS
    ms_first_pass: float = 0.0
    ms_detect: float = 0.0
    ms_apply: float = 0.0
    launches: int = 0
    ms_total: float = 0.0

    @property
    def converged(self) -> bool:
        return self.status == capi.PMSZ_OK


_tls = threading.local()


def _sweep_log(cap: int):
    """A per-thread sweep-log buffer of at least `cap` records, reused across
    calls (the library writes the records of the sweeps it runs)."""
    buf = getattr(_tls, "log", None)
    if buf is None or len(buf) < cap:
        buf = (capi.SweepRecord * int(cap))()
        _tls.log = buf
    return buf


def _log_rows(log, k: int, first: int = 0) -> np.ndarray:
    """Records first .. first+k-1 as a (k, 8) uint64 array, columns SWEEP_KEYS."""
    if k <= 0:
        return np.zeros((0, len(SWEEP_KEYS)), dtype=np.uint64)
    w = len(SWEEP_KEYS)
    return np.frombuffer(log, dtype=np.uint64, count=k * w, offset=first * ctypes.sizeof(capi.SweepRecord)).reshape(k, w).copy()


def correct(f: torch.Tensor, fhat: torch.Tensor, eb: float, q: int = 5, max_sweeps: int = 10000,
            full_sweeps: bool = False, timing: bool = False, stream=None, strategy: str = "pmsz",
            autotune: bool = False, host_loop: bool = False) -> CorrectResult:
    """Correct fhat in place so that its extrema and both segmentations match f
    (c_loops, pMSz.cu:1872-2074).  strategy="naive" runs the naive-MSz loop
    instead (naive_MSz.cu:1887-2220; full_sweeps and timing do not apply).
    autotune=True tunes the field's shape class on these inputs first when the
    tuning table has no entry for it (PMSZ_FLAG_AUTOTUNE).  host_loop=True
    enqueues the list sweeps from the host instead of a CUDA graph
    (PMSZ_FLAG_HOST_LOOP; same results).
    Raises PmszError except for PMSZ_ERR_NOT_CONVERGED, which is reported in
    the result."""
    _check_field(f, "f")
    _check_field(fhat, "fhat")
    if f.shape != fhat.shape or f.dtype != fhat.dtype or f.device != fhat.device:
        raise ValueError("f and fhat must share shape, dtype and device")
    L = capi.load()
    flags = ((capi.PMSZ_FLAG_FULL_SWEEPS if full_sweeps else 0) | (capi.PMSZ_FLAG_TIMING if timing else 0) |
             (capi.PMSZ_FLAG_AUTOTUNE if autotune else 0) | (capi.PMSZ_FLAG_HOST_LOOP if host_loop else 0))
    opts = capi.Opts(int(q), flags, int(max_sweeps))
    log = _sweep_log(int(max_sweeps))
    res = capi.Result(0, 0, 0, ctypes.cast(log, ctypes.POINTER(capi.SweepRecord)), int(max_sweeps))
    nx, ny, nz = _dims(f)
    with torch.cuda.device(f.device):
        if strategy not in ("pmsz", "naive"):
            raise ValueError(f"unknown strategy {strategy!r}")
        entry = "pmsz_correct_naive_" if strategy == "naive" else "pmsz_correct_"
        st = getattr(L, entry + _suffix(f))(
            f.data_ptr(), fhat.data_ptr(), nx, ny, nz, float(eb), ctypes.byref(opts), ctypes.byref(res),
            _stream(stream))
    capi.check(st, allow=(capi.PMSZ_OK, capi.PMSZ_ERR_NOT_CONVERGED))
    n = int(res.sweeps)
    rows = _log_rows(log, n)
    return CorrectResult(st, n, int(res.iteration), int(res.edits), rows, float(res.ms_first_pass),
                         float(res.ms_detect), float(res.ms_apply), int(res.launches), float(res.ms_total))


def correct_host(f: torch.Tensor, fhat: torch.Tensor, eb: float, q: int = 5, max_sweeps: int = 10000,
                 deltas: torch.Tensor | None = None, clamp: torch.Tensor | None = None,
                 edits_only: bool = False, verify: bool = False, device=None, stream=None,
                 packed_deltas: bool = False):
    """pmsz_correct_host_*: the single-rank main pipeline on HOST tensors (pin
    them for full copy bandwidth).  fhat is replaced by the corrected field
    unless edits_only.  deltas (uint8, n) and clamp (field dtype, n) receive
    the edit output when given; with packed_deltas, deltas receives the
    symbols packed as the reference's pack_nbits does (packed_len(n, q)
    bytes, PMSZ_FLAG_PACKED_DELTAS).  Returns (CorrectResult, dict with
    n_clamp, edit_count and, with verify, the verification counts)."""
    for t, name in ((f, "f"), (fhat, "fhat")):
        if t.device.type != "cpu" or not t.is_contiguous() or t.dtype not in (torch.float32, torch.float64):
            raise ValueError(f"{name} must be a contiguous float32/float64 host tensor")
    if f.shape != fhat.shape or f.dtype != fhat.dtype or f.dim() != 3:
        raise ValueError("f and fhat must be 3-D host tensors of one shape and dtype")
    n = f.numel()
    dn = packed_len(n, q) if packed_deltas else n
    if deltas is not None and (deltas.dtype != torch.uint8 or deltas.numel() < dn or deltas.device.type != "cpu"):
        raise ValueError(f"deltas must be a host uint8 tensor of {dn} entries")
    if clamp is not None and (clamp.dtype != f.dtype or clamp.numel() < n or clamp.device.type != "cpu"):
        raise ValueError("clamp must be a host tensor of the field dtype with n entries")
    L = capi.load()
    flags = ((capi.PMSZ_FLAG_EDITS_ONLY if edits_only else 0) |
             (capi.PMSZ_FLAG_PACKED_DELTAS if packed_deltas else 0))
    opts = capi.Opts(int(q), flags, int(max_sweeps))
    log = _sweep_log(int(max_sweeps))
    res = capi.Result(0, 0, 0, ctypes.cast(log, ctypes.POINTER(capi.SweepRecord)), int(max_sweeps))
    vres = capi.VerifyResult()
    outs = capi.HostOutputs(deltas.data_ptr() if deltas is not None else None,
                            clamp.data_ptr() if clamp is not None else None, 0, 0,
                            ctypes.pointer(vres) if verify else None)
    nz, ny, nx = f.shape
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    with torch.cuda.device(dev):
        st = getattr(L, f"pmsz_correct_host_{_suffix(f)}")(
            f.data_ptr(), fhat.data_ptr(), nx, ny, nz, float(eb), ctypes.byref(opts), ctypes.byref(res),
            ctypes.byref(outs), _stream(stream))
    capi.check(st, allow=(capi.PMSZ_OK, capi.PMSZ_ERR_NOT_CONVERGED))
    k = int(res.sweeps)
    rows = _log_rows(log, k)
    extra = {"n_clamp": int(outs.n_clamp), "edit_count": int(outs.edit_count)}
    if verify:
        extra["verify"] = {name: int(getattr(vres, name)) for name, _ in capi.VerifyResult._fields_}
    return (CorrectResult(st, k, int(res.iteration), int(res.edits), rows, float(res.ms_first_pass),
                          float(res.ms_detect), float(res.ms_apply), int(res.launches), float(res.ms_total)),
            extra)


def codes(v: torch.Tensor, stream=None) -> torch.Tensor:
    """Steepest-direction code byte of every voxel (iscriticle data_type=1)."""
    _check_field(v, "v")
    out = torch.empty(v.shape, dtype=torch.uint8, device=v.device)
    nx, ny, nz = _dims(v)
    with torch.cuda.device(v.device):
        capi.check(getattr(capi.load(), f"pmsz_codes_{_suffix(v)}")(v.data_ptr(), nx, ny, nz, out.data_ptr(),
                                                                    _stream(stream)))
    return out


def rank_offsets() -> np.ndarray:
    """(15, 3) int array of the (dx, dy, dz) of each stencil rank."""
    L = capi.load()
    out = np.zeros((15, 3), np.int64)
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    for r in range(15):
        capi.check(L.pmsz_rank_offset(r, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        out[r] = (a.value, b.value, c.value)
    return out


def labels(code: torch.Tensor, stream=None):
    """(AS labels, DS labels) as int64 flat indices, by pointer jumping."""
    if code.dtype != torch.uint8 or code.dim() != 3 or not code.is_cuda:
        raise TypeError("codes must be a (nz, ny, nx) uint8 CUDA tensor")
    nz, ny, nx = code.shape
    a = torch.empty(code.shape, dtype=torch.int32, device=code.device)
    d = torch.empty(code.shape, dtype=torch.int32, device=code.device)
    with torch.cuda.device(code.device):
        capi.check(capi.load().pmsz_labels(code.data_ptr(), nx, ny, nz, a.data_ptr(), d.data_ptr(), _stream(stream)))
    mask = (1 << 32) - 1
    return a.to(torch.int64) & mask, d.to(torch.int64) & mask


def verify(f: torch.Tensor, fp: torch.Tensor, eb: float, stream=None) -> dict:
    _check_field(f, "f")
    _check_field(fp, "fp")
    out = capi.VerifyResult()
    nx, ny, nz = _dims(f)
    with torch.cuda.device(f.device):
        capi.check(getattr(capi.load(), f"pmsz_verify_{_suffix(f)}")(
            f.data_ptr(), fp.data_ptr(), nx, ny, nz, float(eb), ctypes.byref(out), _stream(stream)))
    return {k: int(getattr(out, k)) for k, _ in capi.VerifyResult._fields_}


def extract_edits(prev: torch.Tensor, cur: torch.Tensor, f: torch.Tensor, eb: float, q: int = 5, stream=None):
    """(deltas uint8 tensor, clamp-value tensor, edit_count)."""
    n = prev.numel()
    deltas = torch.empty(n, dtype=torch.uint8, device=prev.device)
    clamp = torch.empty(n, dtype=prev.dtype, device=prev.device)
    nc, ec = ctypes.c_uint64(), ctypes.c_uint64()
    with torch.cuda.device(prev.device):
        capi.check(getattr(capi.load(), f"pmsz_extract_edits_{_suffix(prev)}")(
            prev.data_ptr(), cur.data_ptr(), f.data_ptr(), n, float(eb), int(q), deltas.data_ptr(),
            clamp.data_ptr(), ctypes.byref(nc), ctypes.byref(ec), _stream(stream)))
    return deltas, clamp[: nc.value], int(ec.value)


def reconstruct(prev: torch.Tensor, deltas: torch.Tensor, clamp: torch.Tensor, eb: float, q: int = 5,
                out: torch.Tensor = None, stream=None) -> torch.Tensor:
    """The corrected field rebuilt from the decompressed field `prev`, the
    delta symbols and the clamp list (the inverse of extract_edits; device
    tensors).  `out` defaults to a new tensor; it may be `prev` itself."""
    if not isinstance(prev, torch.Tensor) or not prev.is_cuda or not prev.is_contiguous():
        raise TypeError("prev must be a contiguous CUDA tensor")
    n = prev.numel()
    if deltas.dtype != torch.uint8 or deltas.numel() != n or deltas.device != prev.device:
        raise ValueError("deltas must be a uint8 tensor of prev's size on prev's device")
    if clamp.dtype != prev.dtype or clamp.device != prev.device:
        raise ValueError("clamp must have prev's dtype and device")
    deltas, clamp = deltas.contiguous(), clamp.contiguous()
    if out is None:
        out = torch.empty_like(prev)
    elif out.shape != prev.shape or out.dtype != prev.dtype or out.device != prev.device or not out.is_contiguous():
        raise ValueError("out must be a contiguous tensor like prev")
    with torch.cuda.device(prev.device):
        capi.check(getattr(capi.load(), f"pmsz_reconstruct_{_suffix(prev)}")(
            prev.data_ptr(), deltas.data_ptr(), clamp.data_ptr() if clamp.numel() else None, clamp.numel(), n,
            float(eb), int(q), out.data_ptr(), _stream(stream)))
    return out


def gen_perlin(shape, seed: int, octaves: int, base_freq: float, persistence: float = 0.5,
               lacunarity: float = 2.0, dtype=torch.float32, device="cuda", stream=None) -> torch.Tensor:
    """Normalised Perlin fBm on the device (same bits as fields.perlin_field)."""
    nz, ny, nx = shape
    out = torch.empty(shape, dtype=dtype, device=device)
    perm = np.ascontiguousarray(_fields.permutation(seed), dtype=np.int32)
    amps, freqs = _fields.octave_table(octaves, base_freq, persistence, lacunarity)
    with torch.cuda.device(out.device):
        capi.check(getattr(capi.load(), f"pmsz_gen_perlin_{_suffix(out)}")(
            out.data_ptr(), nx, ny, nz, perm.ctypes.data, amps.ctypes.data, freqs.ctypes.data, int(octaves),
            _stream(stream)))
    return out


def standin(f: torch.Tensor, eb: float, compressor: str, seed: int = 0, stream=None) -> torch.Tensor:
    """Decompressed stand-in of f ("sz3" plateaus or "zfp" noise), same bits as fields.standin."""
    kind = {"sz3": 0, "zfp": 1}.get(compressor)
    if kind is None:
        raise ValueError(f"unknown compressor {compressor!r} (expected 'sz3' or 'zfp')")
    out = torch.empty_like(f)
    with torch.cuda.device(f.device):
        capi.check(getattr(capi.load(), f"pmsz_standin_{_suffix(f)}")(
            f.data_ptr(), out.data_ptr(), f.numel(), float(eb), kind, int(seed), _stream(stream)))
    return out


# ---- host encoders (no GPU needed) -------------------------------------------------------------

def _take(L, ptr: ctypes.c_void_p, n: int) -> bytes:
    if not ptr.value or n == 0:
        return b""
    data = ctypes.string_at(ptr.value, n)
    L.pmsz_free(ptr)
    return data


def encode_deltas(deltas: np.ndarray, q: int = 5) -> bytes:
    """_deltas.bin payload: bit-packed delta symbols, zstd level 5."""
    L = capi.load()
    d = np.ascontiguousarray(deltas, dtype=np.uint8).ravel()
    out, n = ctypes.c_void_p(), ctypes.c_size_t()
    capi.check(L.pmsz_encode_deltas(d.ctypes.data, d.size, int(q), ctypes.byref(out), ctypes.byref(n)))
    return _take(L, out, n.value)


def symbol_bits(q: int = 5) -> int:
    """bits_for_max(q) (pMSz.cu:2352-2356): ceil(log2(q + 1)) bits per delta symbol."""
    return max(1, int(q).bit_length())


def packed_len(n: int, q: int = 5) -> int:
    """Bytes of n delta symbols packed at symbol_bits(q) bits each."""
    return (int(n) * symbol_bits(q) + 7) // 8


def encode_packed_deltas(packed) -> bytes:
    """_deltas.bin payload from already packed symbols (pmsz_encode_packed_deltas)."""
    a = np.ascontiguousarray(np.asarray(packed, dtype=np.uint8))
    L = capi.load()
    out, ln = ctypes.c_void_p(), ctypes.c_size_t()
    capi.check(L.pmsz_encode_packed_deltas(a.ctypes.data, a.size, ctypes.byref(out), ctypes.byref(ln)))
    return _take(L, out, ln.value)


def encode_clamps(values: np.ndarray) -> bytes:
    """_edits.bin payload: raw clamp values, zstd level 3 (empty for none)."""
    L = capi.load()
    v = np.ascontiguousarray(values)
    if v.dtype not in (np.float32, np.float64):
        raise TypeError("clamp values must be float32 or float64")
    out, n = ctypes.c_void_p(), ctypes.c_size_t()
    capi.check(L.pmsz_encode_clamps(v.ctypes.data if v.size else None, v.size, v.itemsize,
                                    ctypes.byref(out), ctypes.byref(n)))
    return _take(L, out, n.value)


def decode_deltas(blob: bytes, n: int, q: int = 5) -> np.ndarray:
    L = capi.load()
    out = np.empty(n, np.uint8)
    buf = np.frombuffer(blob, np.uint8)
    capi.check(L.pmsz_decode_deltas(buf.ctypes.data if buf.size else None, buf.size, n, int(q), out.ctypes.data))
    return out


def decode_clamps(blob: bytes, dtype) -> np.ndarray:
    L = capi.load()
    dt = np.dtype(dtype)
    buf = np.frombuffer(blob, np.uint8)
    out, cnt = ctypes.c_void_p(), ctypes.c_size_t()
    capi.check(L.pmsz_decode_clamps(buf.ctypes.data if buf.size else None, buf.size, dt.itemsize,
                                    ctypes.byref(out), ctypes.byref(cnt)))
    raw = _take(L, out, cnt.value * dt.itemsize)
    return np.frombuffer(raw, dt).copy()


def zstd_version() -> int:
    return int(capi.load().pmsz_zstd_version())


def correct_batch(items, q: int = 5, max_sweeps: int = 10000, stream=None, autotune: bool = False):
    """Correct many fields together (pmsz_correct_batch).  items: sequence of
    (f, fhat, eb) CUDA tensors / floats; each fhat is corrected in place.
    autotune=True tunes every shape class of the batch that the tuning table
    lacks on its first field first (PMSZ_FLAG_AUTOTUNE).
    Returns a list of CorrectResult, one per item."""
    items = list(items)
    n = len(items)
    fields = (capi.Field * n)()
    logs = _sweep_log(n * int(max_sweeps))  # field k's records start at k * max_sweeps
    rec = ctypes.sizeof(capi.SweepRecord)
    results = (capi.Result * n)()
    statuses = (ctypes.c_int * n)()
    device = None
    for k, (f, fh, eb) in enumerate(items):
        _check_field(f, "f")
        _check_field(fh, "fhat")
        if f.shape != fh.shape or f.dtype != fh.dtype:
            raise ValueError("f and fhat must share shape and dtype")
        device = device or f.device
        nx, ny, nz = _dims(f)
        fields[k] = capi.Field(f.data_ptr(), fh.data_ptr(), nx, ny, nz, float(eb), f.element_size(), 0)
        results[k].sweep_log = ctypes.cast(ctypes.addressof(logs) + k * int(max_sweeps) * rec,
                                           ctypes.POINTER(capi.SweepRecord))
        results[k].sweep_log_cap = int(max_sweeps)
    opts = capi.Opts(int(q), capi.PMSZ_FLAG_AUTOTUNE if autotune else 0, int(max_sweeps))
    with torch.cuda.device(device):
        st = capi.load().pmsz_correct_batch(fields, n, ctypes.byref(opts), results, statuses, _stream(stream))
    if st not in (capi.PMSZ_OK, capi.PMSZ_ERR_NOT_CONVERGED, capi.PMSZ_ERR_ARG):
        capi.check(st)
    out = []
    for k in range(n):
        m = int(results[k].sweeps)
        rows = _log_rows(logs, m, k * int(max_sweeps))
        out.append(CorrectResult(int(statuses[k]), m, int(results[k].iteration), int(results[k].edits), rows))
    return out


class Server:
    """Continuous-batching correction server (pmsz_server_*).  submit() takes
    (f, fhat, eb) CUDA tensors (fhat corrected in place; keep both alive until
    the job finishes) and returns a job id; wait() returns a dict with the
    job's status, sweeps, edits and queue / run / latency in ms."""

    def __init__(self, hbm_budget_bytes: int = 0, max_jobs: int = 256, q: int = 5, max_sweeps: int = 10000):
        self._lib = capi.load()
        cfg = capi.ServerConfig(int(hbm_budget_bytes), int(max_jobs), int(q), int(max_sweeps))
        h = ctypes.c_void_p()
        capi.check(self._lib.pmsz_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._keep = {}

    def submit(self, f: torch.Tensor, fhat: torch.Tensor, eb: float) -> int:
        _check_field(f, "f")
        _check_field(fhat, "fhat")
        nz, ny, nx = f.shape
        fld = capi.Field(f.data_ptr(), fhat.data_ptr(), nx, ny, nz, float(eb), f.element_size(), 0)
        jid = ctypes.c_uint64()
        capi.check(self._lib.pmsz_server_submit(self._h, ctypes.byref(fld), ctypes.byref(jid)))
        self._keep[jid.value] = (f, fhat)
        return jid.value

    def wait(self, job_id: int, timeout_s: float = -1.0) -> dict:
        info = capi.JobInfo()
        capi.check(self._lib.pmsz_server_wait(self._h, int(job_id), float(timeout_s), ctypes.byref(info)))
        d = {k: getattr(info, k) for k, _ in capi.JobInfo._fields_}
        if info.done:
            self._keep.pop(job_id, None)
            self._lib.pmsz_server_release(self._h, int(job_id))
        return d

    def close(self):
        if self._h is not None:
            capi.check(self._lib.pmsz_server_destroy(self._h))
            self._h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _tune_dict(t) -> dict:
    return {"zchunk": int(t.zchunk), "jump_rounds": int(t.jump_rounds),
            "ms_zchunk": {z: float(m) for z, m in zip((8, 16, 32, 64), t.ms_zchunk) if m > 0},
            "ms_rounds": {r: float(m) for r, m in zip((1, 2, 4, 8), t.ms_rounds) if m > 0}}


def autotune(f: torch.Tensor, fhat: torch.Tensor, stream=None) -> dict:
    """Time the tile depths and pointer-jumping rounds per launch on this field
    pair (pmsz_autotune_*), record the fastest for its shape class and return
    the choice with the measured times (ms per candidate)."""
    _check_field(f, "f")
    _check_field(fhat, "fhat")
    if f.shape != fhat.shape or f.dtype != fhat.dtype or f.device != fhat.device:
        raise ValueError("f and fhat must share shape, dtype and device")
    t = capi.Tune()
    nx, ny, nz = _dims(f)
    with torch.cuda.device(f.device):
        st = getattr(capi.load(), "pmsz_autotune_" + _suffix(f))(f.data_ptr(), fhat.data_ptr(), nx, ny, nz,
                                                                 ctypes.byref(t), _stream(stream))
    capi.check(st)
    return _tune_dict(t)


def tune_get(shape, dtype) -> tuple:
    """(recorded, {"zchunk", "jump_rounds"}) for a shape (nz, ny, nx) and dtype."""
    nz, ny, nx = (int(v) for v in shape)
    t = capi.Tune()
    st = capi.load().pmsz_tune_get(nx, ny, nz, torch.empty(0, dtype=dtype).element_size(), ctypes.byref(t))
    if st < 0:
        capi.check(-st)
    d = _tune_dict(t)
    return bool(st), {"zchunk": d["zchunk"], "jump_rounds": d["jump_rounds"]}


def tune_batch_get(total_voxels: int, count: int, dtype) -> tuple:
    """(recorded, zchunk): the first-pass tile depth of a batch's size class
    (its total voxels and field count), tuned over whole batches."""
    t = capi.Tune()
    st = capi.load().pmsz_tune_batch_get(int(total_voxels), int(count), torch.empty(0, dtype=dtype).element_size(),
                                         ctypes.byref(t))
    if st < 0:
        capi.check(-st)
    return bool(st), int(t.zchunk)


def tune_set(shape, dtype, zchunk: int, jump_rounds: int) -> None:
    """Record a tile depth and rounds per launch for the shape class of shape (nz, ny, nx)."""
    nz, ny, nx = (int(v) for v in shape)
    t = capi.Tune(int(zchunk), int(jump_rounds))
    capi.check(capi.load().pmsz_tune_set(nx, ny, nz, torch.empty(0, dtype=dtype).element_size(), ctypes.byref(t)))


def tune_save(path: str) -> None:
    capi.check(capi.load().pmsz_tune_save(str(path).encode()))


def tune_load(path: str) -> None:
    capi.check(capi.load().pmsz_tune_load(str(path).encode()))


def tune_clear() -> None:
    capi.load().pmsz_tune_clear()
