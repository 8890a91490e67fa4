"""The edit-file encoder against the reference's own encoder (CPU).

tests/golden/encoder_cases.npz holds the bytes that the reference's
compress_symbols_0_N (pMSz.cu:2359-2369; the _deltas.bin payload) and
compress_zstd<T> (pMSz.cu:2261-2277; the _edits.bin payload) produced, built
from the unmodified pMSz.cu by tests/golden/make_encoder_fixtures.py, for the
reference kernels' own extract output, an oracle-corrected field and
synthetic streams.  zstd output is byte-stable only for one libzstd version,
so the compressed bytes are compared when the loaded libzstd is the one that
made them; the uncompressed payloads (the packed symbols, the raw values) are
compared always, and so is the oracle's pack_nbits restatement."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = np.load(os.path.join(HERE, "golden", "encoder_cases.npz"))


@pytest.fixture(scope="module")
def api():
    from pmsz_anonymous_gb300 import _build
    _build.build()
    from pmsz_anonymous_gb300 import api as A
    return A


def _zstd_decompress(blob: bytes, size: int) -> bytes:
    L = ctypes.CDLL("libzstd.so.1")
    L.ZSTD_decompress.restype = ctypes.c_size_t
    L.ZSTD_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]
    buf = ctypes.create_string_buffer(max(size, 1))
    n = L.ZSTD_decompress(buf, size, blob, len(blob))
    assert n == size
    return buf.raw[:size]


def _same_zstd(api) -> bool:
    return api.zstd_version() == int(CASES["zstd_version"])


@pytest.mark.parametrize("i", range(int(CASES["n_delta"])))
def test_delta_payload_matches_reference_encoder(api, i):
    sym, q = CASES[f"d{i}_in"], int(CASES[f"d{i}_q"])
    ref = CASES[f"d{i}_out"].tobytes()
    bits = api.symbol_bits(q)
    packed = _zstd_decompress(ref, api.packed_len(sym.size, q))
    assert packed == O.pack_nbits(sym, bits)                     # the oracle's restatement of pack_nbits
    np.testing.assert_array_equal(api.decode_deltas(ref, sym.size, q), sym)
    ours = api.encode_deltas(sym, q)
    assert _zstd_decompress(ours, len(packed)) == packed
    if _same_zstd(api):
        assert ours == ref                                      # byte for byte, _deltas.bin
        assert api.encode_packed_deltas(np.frombuffer(packed, np.uint8)) == ref


@pytest.mark.parametrize("i", range(int(CASES["n_clamp"])))
def test_clamp_payload_matches_reference_encoder(api, i):
    vals = CASES[f"c{i}_in"]
    ref = CASES[f"c{i}_out"].tobytes()
    ours = api.encode_clamps(vals)
    if vals.size == 0:
        assert ref == b"" and ours == b""                       # compress_zstd of nothing is nothing
        return
    assert _zstd_decompress(ref, vals.nbytes) == vals.tobytes()
    np.testing.assert_array_equal(api.decode_clamps(ref, vals.dtype).view(np.uint8), vals.view(np.uint8))
    if _same_zstd(api):
        assert ours == ref                                      # byte for byte, _edits.bin


def test_fixture_was_made_with_this_zstd(api):
    """The byte comparisons above ran (this container's libzstd made them)."""
    if not _same_zstd(api):
        pytest.skip(f"libzstd {api.zstd_version()} here, {int(CASES['zstd_version'])} made the fixtures: "
                    "payloads compared, compressed bytes not")
