"""GPU parity: every CUDA entry point, called through the C ABI, against the
CPU oracle on the same seeded inputs.  Integer / index / field outputs must be
bit-identical; counts per sweep must be equal."""
import numpy as np
import pytest

from oracle import oracle as O
from pmsz_anonymous_gb300 import capi, fields as F

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def api():
    from pmsz_anonymous_gb300 import api as A
    return A


def _dev(a, device):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def _case(shape, dtype, comp, eb, seed, octaves=4, base=1 / 16):
    f = F.perlin_field(shape, seed, octaves, base, dtype=dtype)
    return f, F.standin(f, eb, comp, seed)


def _flat_targets(codes, shape, nibble):
    nz, ny, nx = shape
    off = api().rank_offsets()
    r = (codes >> 4) if nibble else (codes & 15)
    r = r.astype(np.int64).ravel()
    i = np.arange(r.size, dtype=np.int64)
    return i + off[r, 0] + nx * (off[r, 1] + ny * off[r, 2])


CASES = [
    ((16, 16, 16), np.float32, "sz3", 1e-3, 0),
    ((16, 16, 16), np.float32, "zfp", 1e-3, 1),
    ((12, 20, 24), np.float64, "zfp", 1e-3, 2),
    ((12, 20, 24), np.float64, "sz3", 2e-3, 3),
    ((5, 17, 33), np.float32, "zfp", 5e-3, 4),     # nx not a multiple of 32
    ((3, 7, 70), np.float64, "sz3", 1e-2, 5),      # three words per row, ragged tail
    ((1, 1, 64), np.float32, "zfp", 5e-2, 6),      # a line
    ((40, 1, 1), np.float64, "zfp", 5e-2, 7),      # a column along z
    ((2, 2, 2), np.float32, "zfp", 1e-1, 8),
    ((32, 32, 32), np.float32, "sz3", 1e-3, 9),
    ((24, 24, 24), np.float64, "zfp", 1e-4, 10),
]


@pytest.mark.parametrize("full", [False, True])
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{np.dtype(c[1]).name}-{c[2]}" if isinstance(c, tuple) else str(c))
def test_correct_matches_oracle(cuda, case, full):
    shape, dtype, comp, eb, seed = case
    f, fh = _case(shape, dtype, comp, eb, seed)
    ref, cnt, st, sw, recs = O.correct(f, fh, eb)
    df, dfh = _dev(f, cuda), _dev(fh, cuda)
    r = api().correct(df, dfh, eb, full_sweeps=full)
    out = dfh.cpu().numpy()
    assert r.status == st
    assert r.sweeps == sw
    assert r.iteration == sw + 1
    np.testing.assert_array_equal(out.view(np.uint8), ref.view(np.uint8))
    np.testing.assert_array_equal(r.log[:, :5], recs)
    assert r.edits == int(recs[:, 3].sum())


def test_active_set_covers_only_a_fraction(cuda):
    f, fh = _case((32, 32, 32), np.float32, "zfp", 1e-3, 21)
    r = api().correct(_dev(f, cuda), _dev(fh, cuda), 1e-3)
    assert r.log[0, 6] == f.size            # sweep 1 is a full pass
    if r.sweeps > 2:
        assert r.log[1:, 6].max() < f.size  # later sweeps examine the active set only


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_codes_match_oracle_labels(cuda, dtype):
    rng = np.random.default_rng(1)
    f = rng.integers(0, 5, size=(9, 11, 37)).astype(dtype)   # plateaus: index tie-breaks
    c = api().codes(_dev(f, cuda)).cpu().numpy()
    asc, desc = O.label(f)
    np.testing.assert_array_equal(_flat_targets(c, f.shape, 0), asc)
    np.testing.assert_array_equal(_flat_targets(c, f.shape, 1), desc)


def test_negative_zero_and_infinities(cuda):
    f = np.array([0.0, -0.0, 0.0, -0.0, np.inf, -np.inf, 1.0, -1.0], np.float64).reshape(2, 2, 2)
    c = api().codes(_dev(f, cuda)).cpu().numpy()
    asc, desc = O.label(f)
    np.testing.assert_array_equal(_flat_targets(c, f.shape, 0), asc)
    np.testing.assert_array_equal(_flat_targets(c, f.shape, 1), desc)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_labels_match_path_compression(cuda, dtype):
    f = F.perlin_field((20, 24, 28), 4, 4, 1 / 8, dtype=dtype)
    c = api().codes(_dev(f, cuda))
    a, d = api().labels(c)
    asc, desc = O.label(f)
    np.testing.assert_array_equal(a.cpu().numpy().ravel(), O.path_compress(asc))
    np.testing.assert_array_equal(d.cpu().numpy().ravel(), O.path_compress(desc))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_verify_matches_oracle(cuda, dtype):
    eb = 1e-3
    f, fh = _case((16, 18, 20), dtype, "zfp", eb, 12)
    got = api().verify(_dev(f, cuda), _dev(fh, cuda), eb)
    ref = O.verify(f, fh, eb)
    assert got["dir_mismatch"] == ref["dir_mismatch"] > 0
    assert got["ext_mismatch"] == ref["ext_mismatch"]
    assert got["as_mismatch"] == ref["as_mismatch"]
    assert got["ds_mismatch"] == ref["ds_mismatch"]
    assert got["bound_strict"] == ref["bound_violations"]
    out, *_ = O.correct(f, fh, eb)
    got = api().verify(_dev(f, cuda), _dev(out, cuda), eb)
    assert got["dir_mismatch"] == got["as_mismatch"] == got["ds_mismatch"] == got["bound_beyond_clamp"] == 0


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_extract_edits_match_oracle(cuda, dtype):
    eb = 1e-3
    f, fh = _case((20, 21, 22), dtype, "sz3", eb, 13)
    out, *_ = O.correct(f, fh, eb)
    d, cl, ec = api().extract_edits(_dev(fh, cuda), _dev(out, cuda), _dev(f, cuda), eb)
    rd, rcl, rec = O.extract_edits(fh, out, f, eb)
    np.testing.assert_array_equal(d.cpu().numpy(), rd)
    np.testing.assert_array_equal(cl.cpu().numpy().view(np.uint8), rcl.view(np.uint8))
    assert ec == rec


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_generators_bit_exact(cuda, dtype):
    shape = (7, 9, 11)
    g = api().gen_perlin(shape, 3, 4, 1 / 8, 0.5, 2.0, dtype=torch.float32 if dtype == np.float32 else torch.float64)
    ref = F.perlin_field(shape, 3, 4, 1 / 8, 0.5, 2.0, dtype=dtype)
    np.testing.assert_array_equal(g.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    for comp in ("sz3", "zfp"):
        s = api().standin(g, 1e-3, comp, seed=5)
        np.testing.assert_array_equal(s.cpu().numpy().view(np.uint8), F.standin(ref, 1e-3, comp, 5).view(np.uint8))


def test_nan_input_is_rejected(cuda):
    f, fh = _case((8, 8, 8), np.float32, "zfp", 1e-3, 14)
    fh[3, 3, 3] = np.nan
    with pytest.raises(capi.PmszError) as e:
        api().correct(_dev(f, cuda), _dev(fh, cuda), 1e-3)
    assert e.value.status == capi.PMSZ_ERR_ARG


def test_sentinel_value_is_rejected_fp64(cuda):
    f, fh = _case((8, 8, 8), np.float64, "zfp", 1e-3, 15)
    f[0, 0, 0] = 1e30
    with pytest.raises(capi.PmszError):
        api().correct(_dev(f, cuda), _dev(fh, cuda), 1e-3)


def test_argument_errors(cuda):
    f, fh = _case((4, 4, 4), np.float32, "zfp", 1e-3, 16)
    with pytest.raises(capi.PmszError) as e:
        api().correct(_dev(f, cuda), _dev(fh, cuda), -1.0)
    assert e.value.status == capi.PMSZ_ERR_ARG
    with pytest.raises(capi.PmszError):
        api().correct(_dev(f, cuda), _dev(fh, cuda), 1e-3, q=0)


def test_isolated_voxel_not_converged(cuda):
    f = np.array([[[0.3]]], np.float64)
    ref, cnt, st, sw, recs = O.correct(f, f.copy(), 0.1)
    d = _dev(f.copy(), cuda)
    r = api().correct(_dev(f, cuda), d, 0.1)
    assert r.status == capi.PMSZ_ERR_NOT_CONVERGED == st
    assert r.sweeps == sw
    np.testing.assert_array_equal(d.cpu().numpy(), ref)


def test_max_sweeps_cap(cuda):
    f, fh = _case((16, 16, 16), np.float32, "zfp", 1e-3, 1)
    r = api().correct(_dev(f, cuda), _dev(fh, cuda), 1e-3, max_sweeps=2)
    assert r.status == capi.PMSZ_ERR_NOT_CONVERGED and r.sweeps == 2


def test_repeat_is_bit_identical(cuda):
    f, fh = _case((24, 24, 24), np.float64, "zfp", 1e-4, 17)
    outs = []
    for _ in range(2):
        d = _dev(fh, cuda)
        api().correct(_dev(f, cuda), d, 1e-4)
        outs.append(d.cpu().numpy())
    np.testing.assert_array_equal(outs[0].view(np.uint8), outs[1].view(np.uint8))


def test_medium_field_against_oracle(cuda):
    """128^3 fp64 through the device generator, checked against the oracle."""
    shape, eb = (128, 128, 128), 1e-4
    df = api().gen_perlin(shape, 1, 5, 1 / 64, dtype=torch.float64)
    dfh = api().standin(df, eb, "zfp", 1)
    f, fh = df.cpu().numpy(), dfh.cpu().numpy()
    ref, cnt, st, sw, recs = O.correct(f, fh, eb)
    r = api().correct(df, dfh, eb)
    assert r.status == st == capi.PMSZ_OK
    np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    np.testing.assert_array_equal(r.log[:, :5], recs)


@pytest.mark.parametrize("dtype,comp", [(torch.float32, "zfp"), (torch.float64, "sz3")])
def test_large_field_through_the_device_sweep_loop(cuda, dtype, comp):
    """256^3: several list sweeps run inside the CUDA-graph loop (the active
    set after the first pass is far above the tail threshold) before the
    cooperative tail; field, sweep count and every per-sweep record equal the
    oracle's, and FULL_SWEEPS (host-driven full sweeps) gives the same."""
    shape, eb = (256, 256, 256), 1e-4
    df = api().gen_perlin(shape, 3, 5, 1 / 64, dtype=dtype)
    dfh = api().standin(df, eb, comp, 3)
    f, fh = df.cpu().numpy(), dfh.cpu().numpy()
    ref, cnt, st, sw, recs = O.correct(f, fh, eb)
    work = dfh.clone()
    r = api().correct(df, work, eb)
    assert r.status == st == capi.PMSZ_OK
    assert r.sweeps == sw
    assert int(r.log[1, 6]) > max(f.size // 32, 1 << 16)  # sweep 2 runs as a list sweep
    np.testing.assert_array_equal(work.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    np.testing.assert_array_equal(r.log[:, :5], recs)
    full = dfh.clone()
    rf = api().correct(df, full, eb, full_sweeps=True)
    assert rf.sweeps == sw
    assert torch.equal(full.view(torch.uint8), work.view(torch.uint8))
    # the same list sweeps enqueued from the host instead of the graph
    host = dfh.clone()
    rh = api().correct(df, host, eb, host_loop=True)
    assert rh.status == st and rh.sweeps == sw
    assert torch.equal(host.view(torch.uint8), work.view(torch.uint8))
    np.testing.assert_array_equal(rh.log[:, :5], recs)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_extract_edits_all_branches_match_oracle(cuda, dtype):
    # synthetic (prev, cur) pairs: unchanged, k whole steps below (subtracted
    # step by step, as the correction does), quotients near half steps (the
    # exact-division fallback), changes below half a step, clamps f - eps,
    # and clamps of value 0 (dropped from the list); dense enough that some
    # warps hold more than 32 changed voxels.  (Values raised other than by a
    # clamp never come out of the correction: their encoding is not pinned.)
    eb, q = 1e-3, 5
    rng = np.random.default_rng(21)
    shape = (40, 64, 66)
    n = int(np.prod(shape))
    f = rng.uniform(0.0, 1.0, n).astype(dtype)
    prev = (f + rng.uniform(-eb, eb, n)).astype(dtype)
    eps, delta = dtype(eb), dtype(eb / q)
    cur = prev.copy()
    kind = rng.integers(0, 10, n)
    for k in range(1, 5):
        sel = kind == k
        for _ in range(k):
            cur[sel] = (cur[sel] - delta).astype(dtype)
    sel = kind == 5
    cur[sel] = (prev[sel] - delta * dtype(2.5) * (1 + rng.uniform(-1e-6, 1e-6, sel.sum()))).astype(dtype)
    sel = kind == 6  # changed by less than half a step: step count 0
    cur[sel] = (prev[sel] - delta * dtype(0.3)).astype(dtype)
    sel = kind == 7
    cur[sel] = (f[sel] - eps).astype(dtype)
    zero = np.flatnonzero(kind == 8)[:50]
    f[zero] = eps
    cur[zero] = (f[zero] - eps).astype(dtype)
    d, cl, ec = api().extract_edits(_dev(prev, cuda), _dev(cur, cuda), _dev(f, cuda), eb, q)
    rd, rcl, rec = O.extract_edits(prev, cur, f, eb, q)
    np.testing.assert_array_equal(d.cpu().numpy(), rd)
    np.testing.assert_array_equal(cl.cpu().numpy().view(np.uint8), rcl.view(np.uint8))
    assert ec == rec


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_dense_active_sets_match_oracle(cuda, dtype):
    # most voxels active after the first pass: the voxel-list compaction
    # expands dense steps word by word
    eb = 3e-2
    f, fh = _case((96, 80, 72), dtype, "sz3", eb, 17)
    ref, cnt, st, sw, recs = O.correct(f, fh, eb)
    dfh = _dev(fh, cuda)
    r = api().correct(_dev(f, cuda), dfh, eb)
    assert r.status == st and r.sweeps == sw
    np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    np.testing.assert_array_equal(r.log[:, :5], recs)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_plateau_field_matches_oracle(cuda, dtype):
    # a decompressed copy quantised to steps of 2*eb: over 90 % of its voxels
    # equal a neighbour, the first pass defers most of them (tied proxies),
    # and the fp32 list sweeps switch to exact keys; many list sweeps run in
    # the CUDA-graph loop before the cooperative tail
    shape, eb = (128, 128, 128), 1e-2
    f = F.perlin_field(shape, 23, 4, 1 / 32, dtype=dtype)
    step = dtype(2 * eb)
    fh = (np.round(f / step) * step).astype(dtype)
    ref, cnt, st, sw, recs = O.correct(f, fh, eb)
    dfh = _dev(fh, cuda)
    r = api().correct(_dev(f, cuda), dfh, eb)
    assert r.status == st and r.sweeps == sw
    assert int(r.log[1, 6]) > (1 << 16)  # sweep 2 runs as a list sweep
    np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    np.testing.assert_array_equal(r.log[:, :5], recs)


def test_c1_plain_64cubed_f32_sz3_matches_oracle(cuda):
    """The CPU-runnable workload exactly as stated: 64^3 fp32 Perlin fBm (seed
    0, 4 octaves, base frequency 1/32, persistence 0.5, lacunarity 2,
    normalised to [0,1]), SZ-like stand-in at eps = 1e-3.  Field, sweep
    count, per-sweep counters and the printed iteration equal the oracle's."""
    shape, eb = (64, 64, 64), 1e-3
    f = F.perlin_field(shape, 0, 4, 1 / 32, 0.5, 2.0, dtype=np.float32)
    fh = F.standin(f, eb, "sz3", 0)
    ref, cnt, st, sw, recs = O.correct(f, fh, eb)
    dfh = _dev(fh, cuda)
    r = api().correct(_dev(f, cuda), dfh, eb)
    assert r.status == st == capi.PMSZ_OK
    assert r.sweeps == sw and r.iteration == sw + 1
    np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    np.testing.assert_array_equal(r.log[:, :5], recs)


def test_c2_plain_512cubed_f64_zfp_matches_oracle(cuda):
    """The headline workload at full size: 512^3 fp64 Perlin fBm (seed 1, 5
    octaves, base frequency 1/64, persistence 0.5), ZFP-like stand-in at
    eps = 1e-4, bit for bit against the oracle (about 10 s of CPU on 16
    cores)."""
    shape, eb = (512, 512, 512), 1e-4
    df = api().gen_perlin(shape, 1, 5, 1 / 64, 0.5, 2.0, dtype=torch.float64)
    dfh = api().standin(df, eb, "zfp", 1)
    f, fh = df.cpu().numpy(), dfh.cpu().numpy()
    ref, cnt, st, sw, recs = O.correct(f, fh, eb)
    r = api().correct(df, dfh, eb)
    assert r.status == st == capi.PMSZ_OK
    assert r.sweeps == sw
    np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint64), ref.view(np.uint64))
    np.testing.assert_array_equal(r.log[:, :5], recs)


@pytest.mark.parametrize("shape,dtype", [
    ((70, 66, 100), np.float64),   # rows of 800 bytes: TMA-fed interior blocks
    ((70, 66, 99), np.float64),    # rows of 792 bytes (not a multiple of 16): threads load every tile
    ((70, 66, 100), np.float32),   # rows of 400 bytes: TMA-fed interior blocks
    ((70, 66, 98), np.float32),    # rows of 392 bytes: threads load every tile
])
def test_first_pass_tile_loaders_match_oracle(cuda, shape, dtype):
    """Ragged fields large enough for interior blocks (tile, halo and planes
    inside the domain), with and without the tensor-map tile loads, against
    the oracle."""
    eb = 1e-3
    f, fh = _case(shape, dtype, "zfp", eb, 41, octaves=4, base=1 / 16)
    ref, cnt, st, sw, recs = O.correct(f, fh, eb)
    dfh = _dev(fh, cuda)
    r = api().correct(_dev(f, cuda), dfh, eb)
    assert r.status == st and r.sweeps == sw
    np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    np.testing.assert_array_equal(r.log[:, :5], recs)


def test_first_pass_unaligned_fields_match_oracle(cuda):
    """Fields that start 8 bytes past a 16-byte boundary (views into larger
    buffers) cannot be described by tensor maps; the threads load the tiles and
    the result is the oracle's."""
    shape, eb = (66, 40, 96), 1e-3
    f, fh = _case(shape, np.float64, "sz3", eb, 43, octaves=4, base=1 / 16)
    ref, cnt, st, sw, recs = O.correct(f, fh, eb)
    n = f.size
    bf = torch.zeros(n + 1, dtype=torch.float64, device=cuda)
    bh = torch.zeros(n + 1, dtype=torch.float64, device=cuda)
    bf[1:] = torch.from_numpy(f.ravel()).to(cuda)
    bh[1:] = torch.from_numpy(fh.ravel()).to(cuda)
    df, dfh = bf[1:].view(shape), bh[1:].view(shape)
    assert df.data_ptr() % 16 == 8
    r = api().correct(df, dfh, eb)
    assert r.status == st and r.sweeps == sw
    np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    np.testing.assert_array_equal(r.log[:, :5], recs)
