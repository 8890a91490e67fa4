"""Host-buffer entry points (pmsz_correct_host_*) and the drop-in CLI.

The host call copies f and fhat in slab by slab while the first pass runs on
the slabs already present; its result must equal the device-buffer call bit
for bit, and its edit output must equal pmsz_extract_edits on the same pair.
The CLI's _deltas.bin / _edits.bin must decode to the same edit output."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from pmsz_anonymous_gb300 import _build, capi, fields as F

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def api():
    from pmsz_anonymous_gb300 import api as A
    return A


HOST_CASES = [
    ((256, 256, 256), torch.float32, "zfp", 1e-3, 31),   # several copy slabs, a short last one
    ((70, 33, 45), torch.float64, "sz3", 2e-3, 32),      # nz not a multiple of the 32-plane chunk
    ((5, 17, 33), torch.float32, "zfp", 5e-3, 33),
    ((130, 96, 160), torch.float64, "zfp", 1e-4, 34),    # 5 chunks, 2 slabs of 64 MiB
]


@pytest.mark.parametrize("case", HOST_CASES, ids=lambda c: f"{c[0]}-{str(c[1])[6:]}-{c[2]}")
def test_host_call_matches_device_call(cuda, case):
    shape, dt, comp, eb, seed = case
    A = api()
    f = A.gen_perlin(shape, seed, 4, 1 / 16, dtype=dt, device=cuda)
    fh = A.standin(f, eb, comp, seed)
    ref = fh.clone()
    r = A.correct(f, ref, eb)
    d_ref, c_ref, ec_ref = A.extract_edits(fh, ref, f, eb)
    n = f.numel()
    hf, hfh = f.cpu().pin_memory(), fh.cpu().pin_memory()
    deltas = torch.empty(n, dtype=torch.uint8).pin_memory()
    clamp = torch.empty(n, dtype=dt).pin_memory()
    for edits_only in (False, True):
        work = hfh.clone().pin_memory()
        rh, extra = A.correct_host(hf, work, eb, deltas=deltas, clamp=clamp, edits_only=edits_only, verify=True)
        assert (rh.status, rh.sweeps, rh.edits) == (r.status, r.sweeps, r.edits)
        np.testing.assert_array_equal(rh.log, r.log)
        if edits_only:
            assert torch.equal(work.view(torch.uint8), hfh.view(torch.uint8))
        else:
            assert torch.equal(work.view(torch.uint8), ref.cpu().view(torch.uint8))
        assert torch.equal(deltas, d_ref.cpu().view(-1))
        assert extra["n_clamp"] == c_ref.numel()
        assert torch.equal(clamp[: extra["n_clamp"]].view(torch.uint8), c_ref.cpu().view(torch.uint8))
        assert extra["edit_count"] == ec_ref
        v = extra["verify"]
        assert v["dir_mismatch"] == 0 and v["ext_mismatch"] == 0 and v["bound_beyond_clamp"] == 0
    # packed on the GPU: the oracle's pack_nbits of the same symbols, and the
    # same _deltas.bin payload as packing on the host
    packed = torch.empty(A.packed_len(n), dtype=torch.uint8).pin_memory()
    A.correct_host(hf, hfh.clone().pin_memory(), eb, deltas=packed, edits_only=True, packed_deltas=True)
    sym = d_ref.cpu().numpy()
    assert packed.numpy().tobytes() == O.pack_nbits(sym, A.symbol_bits(5))
    assert A.encode_packed_deltas(packed.numpy()) == A.encode_deltas(sym)


def test_host_call_with_pageable_buffers_and_naive_flag(cuda):
    """Pageable (not pinned) host arrays, both strategies, through the raw C
    entry point with a NULL outputs pointer."""
    shape, eb = (40, 36, 30), 1e-3
    f = F.perlin_field(shape, 35, 4, 1 / 16, dtype=np.float32)
    fh = F.standin(f, eb, "sz3", 35)
    L = capi.load()
    nz, ny, nx = shape
    for flags, ref_fn in ((0, O.correct), (capi.PMSZ_FLAG_NAIVE, O.correct_naive)):
        ref = ref_fn(f, fh, eb)[0]
        work = fh.copy()
        opts, res = capi.Opts(5, flags, 10000), capi.Result()
        st = L.pmsz_correct_host_f32(f.ctypes.data, work.ctypes.data, nx, ny, nz, eb, ctypes.byref(opts),
                                     ctypes.byref(res), None, None)
        assert st == capi.PMSZ_OK
        np.testing.assert_array_equal(work.view(np.uint8), ref.view(np.uint8))


def _cli():
    _build.build()
    exe = os.path.join(os.path.dirname(_build.__file__), "lib", "pmsz")
    assert os.path.exists(exe), "the pmsz CLI was not built"
    return exe


@pytest.mark.parametrize("naive", [False, True])
def test_cli_outputs_decode_to_the_edit_output(cuda, tmp_path, naive):
    exe = _cli()
    shape, eb = (24, 20, 28), 1e-3
    f = F.perlin_field(shape, 36, 4, 1 / 16, dtype=np.float64)
    fh = F.standin(f, eb, "zfp", 36)
    (tmp_path / "stat_result").mkdir()
    path, decp, out = tmp_path / "field.bin", tmp_path / "decp.bin", tmp_path / "corrected.bin"
    f.tofile(path)
    fh.tofile(decp)
    nz, ny, nx = shape
    cmd = [exe, f"{path},{nx},{ny},{nz}", repr(eb), "zfp", "1", "1", "1", "--decp", str(decp), "--out", str(out),
           "--verify"] + (["--naive"] if naive else [])
    p = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    for key in ("iteration is:", "Edit count:", "comfputational overhead is:", "overall edit ratio is:"):
        assert key in p.stdout
    ref, cnt, st, sw, recs = (O.correct_naive if naive else O.correct)(f, fh, eb)
    got = np.fromfile(out, np.float64).reshape(shape)
    np.testing.assert_array_equal(got.view(np.uint8), ref.view(np.uint8))
    deltas, clamp, ec = O.extract_edits(fh, ref, f, eb)
    A = api()
    blob_d = (tmp_path / "_deltas.bin").read_bytes()
    blob_e = (tmp_path / "_edits.bin").read_bytes()
    np.testing.assert_array_equal(A.decode_deltas(blob_d, f.size), deltas)
    np.testing.assert_array_equal(A.decode_clamps(blob_e, np.float64).view(np.uint8), clamp.view(np.uint8))
    assert blob_d == A.encode_deltas(deltas) and blob_e == A.encode_clamps(clamp)
    assert f"Edit count: {ec}" in p.stdout
    assert (tmp_path / "stat_result").iterdir()


def test_cli_rejects_multi_rank_grids_and_bad_arguments(tmp_path):
    exe = _cli()
    p = subprocess.run([exe, "x.bin,4,4,4", "1e-3", "sz3", "2", "1", "1"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=60)
    assert p.returncode != 0 and "PX PY PZ" in p.stderr
    p = subprocess.run([exe, "x.bin,4,4", "1e-3", "sz3", "1", "1", "1"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=60)
    assert p.returncode != 0
    p = subprocess.run([exe, str(tmp_path / "missing.bin") + ",4,4,4", "1e-3", "sz3", "1", "1", "1"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert p.returncode != 0


def test_cli_reconstruct_rebuilds_the_corrected_field(cuda, tmp_path):
    # correction with the CLI, then its decoder mode on the decompressed field
    # and the two edit files: the corrected field, byte for byte
    exe = _cli()
    shape, eb = (24, 20, 28), 1e-3
    f = F.perlin_field(shape, 37, 4, 1 / 16, dtype=np.float64)
    fh = F.standin(f, eb, "zfp", 37)
    path, decp, out, rec = (tmp_path / n for n in ("field.bin", "decp.bin", "corrected.bin", "rebuilt.bin"))
    f.tofile(path)
    fh.tofile(decp)
    nz, ny, nx = shape
    p = subprocess.run([exe, f"{path},{nx},{ny},{nz}", repr(eb), "zfp", "1", "1", "1", "--decp", str(decp),
                        "--out", str(out)], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    p = subprocess.run([exe, "--reconstruct", f"{decp},{nx},{ny},{nz}", repr(eb), "--out", str(rec)], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert "reconstructed" in p.stdout
    assert rec.read_bytes() == out.read_bytes()
    assert rec.read_bytes() != decp.read_bytes()
    p = subprocess.run([exe, "--reconstruct", f"{decp},{nx},{ny},{nz}", repr(eb), "--out", str(rec), "--deltas",
                        str(tmp_path / "missing.bin")], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert p.returncode != 0


@pytest.mark.parametrize("name", ["sz3", "zfp"])
def test_cli_edit_files_match_the_reference_encoder(cuda, tmp_path, name):
    """The CLI on the fields whose edit output the reference's own kernels
    produced (tests/golden/extract_perlin_*.npz): its _deltas.bin and
    _edits.bin carry the payloads that the reference's own encoder made of
    that output (tests/golden/encoder_cases.npz), byte for byte when this
    machine's libzstd is the one that made them."""
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    g = np.load(os.path.join(here, "golden", f"extract_perlin_{name}.npz"))
    cases = np.load(os.path.join(here, "golden", "encoder_cases.npz"))
    k = next(i for i in range(int(cases["n_delta"])) if str(cases[f"d{i}_name"]) == f"reference_extract_{name}")
    c = next(i for i in range(int(cases["n_clamp"])) if str(cases[f"c{i}_name"]) == f"reference_extract_{name}")
    exe = _cli()
    f, fh, eb = g["f"], g["fh"], float(g["eb"])
    path, decp = tmp_path / "field.bin", tmp_path / "decp.bin"
    f.tofile(path)
    fh.tofile(decp)
    nz, ny, nx = f.shape
    p = subprocess.run([exe, f"{path},{nx},{ny},{nz}", repr(eb), name, "1", "1", "1", "--decp", str(decp)],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    A = api()
    blob_d = (tmp_path / "_deltas.bin").read_bytes()
    blob_e = (tmp_path / "_edits.bin").read_bytes()
    ref_d, ref_e = cases[f"d{k}_out"].tobytes(), cases[f"c{c}_out"].tobytes()
    np.testing.assert_array_equal(A.decode_deltas(blob_d, f.size), A.decode_deltas(ref_d, f.size))
    np.testing.assert_array_equal(A.decode_clamps(blob_e, np.float64).view(np.uint8),
                                  A.decode_clamps(ref_e, np.float64).view(np.uint8))
    if A.zstd_version() == int(cases["zstd_version"]):
        assert blob_d == ref_d and blob_e == ref_e


# Fields of several 64 MiB copy slabs run sweeps 1..6 behind the host copy
# (each sweep two planes behind the one before); max_sweeps 2, 3 and 5 cut the
# pipelined sweeps short (K = 0 / 2 / 4), sz3 plateaus defer many voxels.
WAVE_CASES = [
    ((384, 256, 256), torch.float64, "zfp", 1e-4, 10000, 61),   # 6 slabs of 64 planes
    ((384, 256, 256), torch.float32, "sz3", 1e-3, 10000, 62),   # 3 slabs of 128 planes
    ((400, 256, 256), torch.float32, "zfp", 1e-2, 10000, 63),   # a short last slab, many clamps
    ((96, 256, 256), torch.float64, "zfp", 1e-4, 10000, 68),    # two slabs: waves after both
    ((384, 256, 256), torch.float64, "zfp", 1e-4, 2, 64),
    ((384, 256, 256), torch.float64, "zfp", 1e-4, 3, 65),
    ((384, 256, 256), torch.float64, "sz3", 1e-3, 5, 66),
]


@pytest.mark.parametrize("case", WAVE_CASES, ids=lambda c: f"{c[0][0]}-{str(c[1])[6:]}-{c[2]}-max{c[4]}")
def test_host_wavefront_matches_device_call(cuda, case):
    shape, dt, comp, eb, max_sweeps, seed = case
    A = api()
    f = A.gen_perlin(shape, seed, 5, 1 / 32, dtype=dt, device=cuda)
    fh = A.standin(f, eb, comp, seed)
    ref = fh.clone()
    r = A.correct(f, ref, eb, max_sweeps=max_sweeps)
    hf, hfh = f.cpu().pin_memory(), fh.cpu().pin_memory()
    work = hfh.clone().pin_memory()
    rh, _ = A.correct_host(hf, work, eb, max_sweeps=max_sweeps)
    assert (rh.status, rh.sweeps, rh.iteration, rh.edits) == (r.status, r.sweeps, r.iteration, r.edits)
    np.testing.assert_array_equal(rh.log, r.log)
    assert torch.equal(work.view(torch.uint8), ref.cpu().view(torch.uint8))
    if max_sweeps == 10000:
        assert r.status == capi.PMSZ_OK and r.sweeps > 7  # the pipeline ran to its depth and beyond


def test_host_wavefront_nan_input_fails_like_the_device_call(cuda):
    A = api()
    shape, eb = (384, 256, 256), 1e-3
    f = A.gen_perlin(shape, 67, 4, 1 / 32, dtype=torch.float32, device=cuda)
    fh = A.standin(f, eb, "zfp", 67)
    fh[300, 7, 9] = float("nan")  # in the third slab: the first ones ran their sweeps already
    with pytest.raises(capi.PmszError) as dev:
        A.correct(f, fh.clone(), eb)
    hfh = fh.cpu().pin_memory()
    work = hfh.clone().pin_memory()
    with pytest.raises(capi.PmszError) as host:
        A.correct_host(f.cpu().pin_memory(), work, eb)
    assert host.value.status == dev.value.status == capi.PMSZ_ERR_ARG
    assert torch.equal(work.view(torch.uint8), hfh.view(torch.uint8))  # the caller's buffer is left as it was
