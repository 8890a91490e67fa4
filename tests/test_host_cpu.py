"""CPU tests of the native library that need no GPU: it loads, exports every
symbol the headers declare, and its host encoder matches the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from pmsz_anonymous_gb300 import _build, capi, fields as F

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return capi.load()


def _declared():
    names = set()
    for h in ("pmsz.h", "pmsz_host.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(pmsz_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"
    assert set(capi.SIGNATURES) == names


def test_status_strings(lib):
    assert lib.pmsz_strerror(0) == b"ok"
    assert lib.pmsz_strerror(3) == b"not converged"
    assert lib.pmsz_version() >= 100


def test_argument_errors_without_gpu(lib):
    # null pointers and bad sizes are rejected before any CUDA call
    assert lib.pmsz_correct_f32(None, None, 4, 4, 4, 1e-3, None, None, None) == capi.PMSZ_ERR_ARG
    assert b"null" in lib.pmsz_last_error()


def test_delta_encoder_matches_oracle_pack(lib):
    from pmsz_anonymous_gb300 import api
    rng = np.random.default_rng(0)
    d = rng.integers(0, 6, 10007).astype(np.uint8)
    blob = api.encode_deltas(d, 5)
    np.testing.assert_array_equal(api.decode_deltas(blob, d.size, 5), d)
    # the payload inside the zstd frame is the oracle's 3-bit pack
    import ctypes
    L = ctypes.CDLL("libzstd.so.1")
    L.ZSTD_decompress.restype = ctypes.c_size_t
    L.ZSTD_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]
    packed = O.pack_nbits(d, 3)
    buf = ctypes.create_string_buffer(len(packed))
    n = L.ZSTD_decompress(buf, len(packed), blob, len(blob))
    assert n == len(packed) and buf.raw == packed


def test_clamp_encoder_round_trip(lib):
    from pmsz_anonymous_gb300 import api
    assert api.encode_clamps(np.zeros(0, np.float64)) == b""
    v = np.linspace(-1, 1, 999).astype(np.float32)
    np.testing.assert_array_equal(api.decode_clamps(api.encode_clamps(v), np.float32), v)
    assert api.zstd_version() >= 10500


def test_rank_table(lib):
    from pmsz_anonymous_gb300 import api
    off = api.rank_offsets()
    # lexicographic (dz, dy, dx) order, centre at rank 7, opposite ranks r / 14-r
    keys = [tuple(o[::-1]) for o in off]
    assert keys == sorted(keys)
    assert tuple(off[7]) == (0, 0, 0)
    for r in range(15):
        assert tuple(off[r]) == tuple(-off[14 - r])
    # the 14 non-centre offsets are the reference's stencil (pMSz.cu:186-193)
    from tests import refpy
    assert {tuple(o) for i, o in enumerate(off) if i != 7} == set(refpy.DIRS)


def test_fields_are_normalised_and_bounded():
    f = F.perlin_field((8, 9, 10), 0, 4, 1 / 32, dtype=np.float32)
    assert f.dtype == np.float32 and f.min() == 0.0 and f.max() == 1.0
    for comp in ("sz3", "zfp"):
        fh = F.standin(f, 1e-3, comp)
        assert np.all(np.abs(f - fh) <= np.float32(1e-3))
    assert np.array_equal(F.perlin_field((4, 5, 6), 3, 2, 0.1), F.perlin_field((4, 5, 6), 3, 2, 0.1))


def _tune(lib, shape, elem):
    t = capi.Tune()
    nz, ny, nx = shape
    return lib.pmsz_tune_get(nx, ny, nz, elem, ctypes.byref(t)), t


def test_tuning_table_round_trip_without_gpu(lib, tmp_path):
    lib.pmsz_tune_clear()
    try:
        found, t = _tune(lib, (64, 64, 64), 8)
        assert found == 0 and (t.zchunk, t.jump_rounds) == (32, 1)  # defaults
        assert lib.pmsz_tune_set(64, 64, 64, 8, ctypes.byref(capi.Tune(16, 4))) == capi.PMSZ_OK
        found, t = _tune(lib, (33, 50, 61), 8)  # same ceil-log2 class as 64^3
        assert found == 1 and (t.zchunk, t.jump_rounds) == (16, 4)
        found, t = _tune(lib, (64, 64, 64), 4)  # the tile depth is per element size; rounds are not
        assert found == 0 and (t.zchunk, t.jump_rounds) == (32, 4)
        assert lib.pmsz_tune_set(300, 20, 7, 4, ctypes.byref(capi.Tune(64, 2))) == capi.PMSZ_OK
        path = str(tmp_path / "tune.txt")
        assert lib.pmsz_tune_save(path.encode()) == capi.PMSZ_OK
        text = open(path).read().splitlines()
        assert text[0] == "pmsz-tune 1" and len(text) == 3
        lib.pmsz_tune_clear()
        assert _tune(lib, (64, 64, 64), 8)[0] == 0
        assert lib.pmsz_tune_load(path.encode()) == capi.PMSZ_OK
        found, t = _tune(lib, (64, 64, 64), 8)
        assert found == 1 and (t.zchunk, t.jump_rounds) == (16, 4)
        found, t = _tune(lib, (7, 20, 300), 4)
        assert found == 1 and (t.zchunk, t.jump_rounds) == (64, 2)
    finally:
        lib.pmsz_tune_clear()


def test_batch_tuning_entries_load_and_save(lib, tmp_path):
    lib.pmsz_tune_clear()
    try:
        t = capi.Tune()
        assert lib.pmsz_tune_batch_get(200_000_000, 64, 4, ctypes.byref(t)) == 0 and t.zchunk == 32
        p = tmp_path / "b.txt"
        p.write_text("pmsz-tune 1\nb 4 28 6 16\n4 5 5 5 8 2\n")
        assert lib.pmsz_tune_load(str(p).encode()) == capi.PMSZ_OK
        assert lib.pmsz_tune_batch_get(200_000_000, 64, 4, ctypes.byref(t)) == 1 and t.zchunk == 16
        assert lib.pmsz_tune_batch_get(200_000_000, 64, 8, ctypes.byref(t)) == 0  # per element size
        q = tmp_path / "c.txt"
        assert lib.pmsz_tune_save(str(q).encode()) == capi.PMSZ_OK
        assert sorted(q.read_text().splitlines()[1:]) == ["4 5 5 5 8 2", "b 4 28 6 16"]
        assert lib.pmsz_tune_batch_get(0, 64, 4, ctypes.byref(t)) < 0
    finally:
        lib.pmsz_tune_clear()


def test_tuning_table_rejects_bad_entries(lib, tmp_path):
    bad = [capi.Tune(0, 1), capi.Tune(300, 1), capi.Tune(32, 0), capi.Tune(32, 17)]
    for t in bad:
        assert lib.pmsz_tune_set(8, 8, 8, 4, ctypes.byref(t)) == capi.PMSZ_ERR_ARG
    assert lib.pmsz_tune_set(8, 8, 8, 2, ctypes.byref(capi.Tune(32, 1))) == capi.PMSZ_ERR_ARG
    assert lib.pmsz_tune_get(8, 8, 8, 3, ctypes.byref(capi.Tune())) < 0
    p = tmp_path / "bad.txt"
    p.write_text("pmsz-tune 1\n4 3 3 3 0 1\n")
    assert lib.pmsz_tune_load(str(p).encode()) == capi.PMSZ_ERR_IO
    p.write_text("pmsz-tune 1\nb 4 3 3 300\n")
    assert lib.pmsz_tune_load(str(p).encode()) == capi.PMSZ_ERR_IO
    p.write_text("something else\n")
    assert lib.pmsz_tune_load(str(p).encode()) == capi.PMSZ_ERR_IO
    assert lib.pmsz_tune_load(str(tmp_path / "missing.txt").encode()) == capi.PMSZ_ERR_IO
    assert lib.pmsz_tune_get(8, 8, 8, 4, ctypes.byref(capi.Tune())) == 0  # nothing was recorded


def test_packed_delta_encoder_matches_symbol_encoder(lib):
    from pmsz_anonymous_gb300 import api as A
    rng = np.random.default_rng(7)
    for q in (1, 3, 5, 8, 255):
        sym = rng.integers(0, q + 1, 10_001).astype(np.uint8)
        nb = A.symbol_bits(q)
        packed = O.pack_nbits(sym, nb)
        assert len(packed) == A.packed_len(sym.size, q)
        assert A.encode_packed_deltas(np.frombuffer(packed, np.uint8)) == A.encode_deltas(sym, q)


def test_reconstruct_argument_errors_without_gpu(lib):
    # checked before any CUDA call: null pointers, n, q and the error bound
    buf = (ctypes.c_double * 8)()
    sym = (ctypes.c_uint8 * 8)()
    p, d = ctypes.addressof(buf), ctypes.addressof(sym)
    assert lib.pmsz_reconstruct_f64(None, d, None, 0, 8, 1e-3, 5, p, None) == capi.PMSZ_ERR_ARG
    assert lib.pmsz_reconstruct_f64(p, d, None, 3, 8, 1e-3, 5, p, None) == capi.PMSZ_ERR_ARG  # clamps without a list
    assert lib.pmsz_reconstruct_f64(p, d, None, 0, 0, 1e-3, 5, p, None) == capi.PMSZ_ERR_ARG
    assert lib.pmsz_reconstruct_f64(p, d, None, 0, 8, 1e-3, 0, p, None) == capi.PMSZ_ERR_ARG
    assert lib.pmsz_reconstruct_f32(p, d, None, 0, 8, -1.0, 5, p, None) == capi.PMSZ_ERR_ARG
    assert b"error bound" in lib.pmsz_last_error()


def _cli_run(args, cwd):
    import subprocess
    _build.build()
    exe = os.path.join(os.path.dirname(_build.__file__), "lib", "pmsz")
    return subprocess.run([exe] + args, cwd=cwd, capture_output=True, text=True, timeout=60)


def test_cli_argument_errors_without_gpu(tmp_path):
    # every one of these fails in argument parsing or file reading, before
    # any CUDA call
    p = _cli_run(["x.bin,4,4,4", "1e-3", "sz3", "2", "1", "1"], tmp_path)
    assert p.returncode == 2 and "PX PY PZ" in p.stderr
    p = _cli_run(["x.bin,4,4,4", "-1", "sz3", "1", "1", "1"], tmp_path)
    assert p.returncode == 2 and "error bound" in p.stderr
    p = _cli_run(["x.bin,4,4,4", "1e-3", "lz4", "1", "1", "1"], tmp_path)
    assert p.returncode == 2 and "compressor" in p.stderr
    p = _cli_run(["--reconstruct", "x.bin,4,4,4", "1e-3"], tmp_path)
    assert p.returncode == 2 and "--out" in p.stderr
    p = _cli_run(["--reconstruct", "x.bin,4,4", "1e-3", "--out", "r.bin"], tmp_path)
    assert p.returncode == 2 and "dimensions" in p.stderr
    p = _cli_run(["--reconstruct", str(tmp_path / "missing.bin") + ",4,4,4", "1e-3", "--out", "r.bin"], tmp_path)
    assert p.returncode == 1 and "cannot open" in p.stderr
    np.zeros(64).tofile(tmp_path / "decp.bin")
    p = _cli_run(["--reconstruct", str(tmp_path / "decp.bin"), "4", "4", "4", "1e-3", "--out", "r.bin",
                  "--deltas", str(tmp_path / "none.bin")], tmp_path)
    assert p.returncode == 1 and "none.bin" in p.stderr
    assert not (tmp_path / "r.bin").exists()


def test_python_api_rejects_host_tensors_without_gpu():
    # the Python layer checks its tensors before any CUDA call
    torch = pytest.importorskip("torch")
    from pmsz_anonymous_gb300 import api
    f = torch.zeros((4, 4, 4), dtype=torch.float64)
    d = torch.zeros(64, dtype=torch.uint8)
    with pytest.raises(TypeError):
        api.reconstruct(f, d, torch.zeros(0, dtype=torch.float64), 1e-3)
    with pytest.raises(TypeError):
        api.correct(f, f.clone(), 1e-3)
