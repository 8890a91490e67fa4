"""CPU tests of the oracle: known-answer cases, the padded-grid restatement
(tests/refpy.py) against the unpadded C oracle, and property tests."""
import numpy as np
import pytest

from oracle import oracle as O
from pmsz_anonymous_gb300 import fields as F
from tests import refpy


def _idx(shape, x, y, z):
    nz, ny, nx = shape
    return x + nx * (y + ny * z)


# ---------------------------------------------------------------- labelling KATs

def test_single_peak_and_pit():
    f = np.zeros((3, 3, 3), np.float64)
    f[1, 1, 1] = 1.0
    asc, desc = O.label(f)
    c = _idx(f.shape, 1, 1, 1)
    assert asc[c] == c                      # the peak is its own ascent: a maximum
    # every neighbour of the peak in the 14-stencil ascends to it
    for dx, dy, dz in refpy.DIRS:
        assert asc[_idx(f.shape, 1 + dx, 1 + dy, 1 + dz)] == c
    g = -f
    asc, desc = O.label(g)
    assert desc[c] == c


def test_plateau_ties_break_by_index():
    f = np.zeros((2, 2, 2), np.float32)   # all equal: order is the flat index
    asc, desc = O.label(f)
    n = f.size
    assert (asc[n - 1] == n - 1) and (desc[0] == 0)
    # voxel 0's stencil: +x(1), +y(2), +z(4), (0,1,1)=6, and (-1,*) ones are off-domain
    assert asc[0] == 6 and desc[7] == 1


def test_domain_boundary_has_no_outside_neighbour():
    # a strictly increasing line: the last voxel is the maximum, the first the minimum
    f = np.arange(5, dtype=np.float64).reshape(1, 1, 5)
    asc, desc = O.label(f)
    assert list(asc) == [1, 2, 3, 4, 4]
    assert list(desc) == [0, 0, 1, 2, 3]


def test_label_matches_padded_or_types():
    rng = np.random.default_rng(3)
    f = rng.integers(0, 4, size=(3, 4, 5)).astype(np.float64)  # many ties
    nz, ny, nx = f.shape
    W, H, D = nx + 2, ny + 2, nz + 2
    ot = refpy.or_types(refpy.pad(f), W, H, D)
    asc, desc = O.label(f)
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                p = (x + 1) + W * ((y + 1) + H * (z + 1))
                i = _idx(f.shape, x, y, z)
                t, u = ot[2 * p], ot[2 * p + 1]
                if t == -1:
                    assert asc[i] == i and refpy.unpad_index(u, W, H) == desc[i]
                elif t == -2:
                    assert desc[i] == i and refpy.unpad_index(u, W, H) == asc[i]
                else:
                    assert refpy.unpad_index(t, W, H) == desc[i]
                    assert refpy.unpad_index(u, W, H) == asc[i]


# ---------------------------------------------------------------- correction KATs

def test_false_maximum_is_lowered():
    f = np.arange(27, dtype=np.float64).reshape(3, 3, 3) / 26.0
    fh = f.copy()
    c = _idx(f.shape, 1, 1, 1)
    fh.ravel()[c] = 1.0 + 0.0          # exceeds its neighbours: a false maximum ...
    eb = 1.0                           # ... legal under a generous bound
    out, cnt, st, sw, recs = O.correct(f, fh, eb)
    assert st == O.OK
    assert recs[0][0] >= 1             # fmax counted in the first sweep
    v = O.verify(f, out, eb)
    assert v["dir_mismatch"] == 0 and v["ext_mismatch"] == 0


def test_missing_minimum_is_restored():
    f = np.full((3, 3, 3), 0.5, np.float64)
    f.ravel()[:] += np.arange(27) * 1e-3
    c = _idx(f.shape, 1, 1, 1)
    f.ravel()[c] = 0.0                 # a pit in the original
    fh = f.copy()
    fh.ravel()[c] = 0.6                # decompression filled it in
    eb = 0.7
    out, cnt, st, sw, recs = O.correct(f, fh, eb)
    assert st == O.OK
    assert recs[0][1] >= 1             # fmin counted
    asc, desc = O.label(out)
    assert desc[c] == c


def test_clamp_after_q_minus_one_steps():
    # one voxel that needs a drop larger than (q-1)*delta: four delta steps,
    # then the clamp to f - eps (pMSz.cu:630-638)
    eb, q = 1.0, 5
    f = np.array([0.0, 0.5, 0.0], np.float64).reshape(1, 1, 3)
    fh = np.array([0.0, 0.5, 0.0], np.float64).reshape(1, 1, 3)
    fh[0, 0, 0] = 0.95                 # false max at x=0 (f's max is x=1)
    out, cnt, st, sw, recs = O.correct(f, fh, eb, q=q)
    assert st == O.OK
    d = eb / q
    steps = [0.95]
    for _ in range(q - 1):
        steps.append(steps[-1] - d)
    # the sequence 0.95 -> 0.75 -> 0.55 -> 0.35 ... stops as soon as x=0 < x=1
    assert out[0, 0, 0] < 0.5 and out[0, 0, 0] in steps[1:] + [0.0 - eb]


def test_stuck_clamped_vertex_reports_not_converged():
    # a single voxel is both max and min but is stored as "max" in or_types,
    # so the reference flags a false minimum forever (pMSz.cu:749-836)
    f = np.array([[[0.3]]], np.float64)
    fh = f.copy()
    out, cnt, st, sw, recs = O.correct(f, fh, 0.1)
    assert st == O.ERR_NOT_CONVERGED
    assert out[0, 0, 0] == np.float64(0.3) - np.float64(0.1)   # clamped, then no progress


# ---------------------------------------------------------------- padded restatement parity

@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_matches_padded_restatement(dtype, seed):
    rng = np.random.default_rng(seed)
    shape = (3, 4, 5)
    f = rng.random(shape).astype(dtype)
    eb = 0.05
    fh = np.clip(f + rng.uniform(-eb, eb, shape).astype(dtype), 0, 1).astype(dtype)
    fh = np.where(np.abs(f - fh) <= dtype(eb), fh, f).astype(dtype)
    out, cnt, st, sw, recs = O.correct(f, fh, eb)
    ref_out, ref_log, conv = refpy.correct(f, fh, eb)
    assert conv == (st == O.OK)
    np.testing.assert_array_equal(out.view(np.uint8), ref_out.view(np.uint8))
    np.testing.assert_array_equal(recs[:, :4], ref_log)


# ---------------------------------------------------------------- properties

def _perlin_case(shape, seed, dtype, comp, eb):
    f = F.perlin_field(shape, seed, 3, 1 / 8, dtype=dtype)
    return f, F.standin(f, eb, comp, seed)


@pytest.mark.parametrize("comp", ["sz3", "zfp"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_correction_properties(comp, dtype):
    eb = 1e-2
    f, fh = _perlin_case((12, 10, 14), 5, dtype, comp, eb)
    out, cnt, st, sw, recs = O.correct(f, fh, eb)
    assert st == O.OK
    v = O.verify(f, out, eb)
    assert v["dir_mismatch"] == 0 and v["ext_mismatch"] == 0
    assert v["as_mismatch"] == 0 and v["ds_mismatch"] == 0
    assert np.all(out <= fh)                                  # edits only lower
    assert np.all(out >= (f - dtype(eb)))                     # never below the clamp value
    assert recs[-1][:3].tolist() == [0, 0, 0]
    assert recs[:, 3].sum() == (cnt > 0).sum() or recs[:, 3].sum() >= (cnt > 0).sum()


def test_oracle_is_thread_count_independent():
    eb = 1e-3
    f, fh = _perlin_case((16, 16, 16), 9, np.float32, "zfp", eb)
    outs = []
    for t in (1, 4):
        O.set_threads(t)
        outs.append(O.correct(f, fh, eb)[0])
    O.set_threads(0)
    np.testing.assert_array_equal(outs[0], outs[1])


hyp = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402


@settings(max_examples=25, deadline=None)
@given(nx=st.integers(1, 6), ny=st.integers(1, 5), nz=st.integers(1, 4), seed=st.integers(0, 10_000),
       levels=st.integers(2, 6), f64=st.booleans())
def test_property_random_quantised_fields(nx, ny, nz, seed, levels, f64):
    dtype = np.float64 if f64 else np.float32
    rng = np.random.default_rng(seed)
    f = (rng.integers(0, levels, size=(nz, ny, nx)) / levels).astype(dtype)
    eb = 0.2
    fh = (f + rng.uniform(-eb, eb, f.shape)).astype(dtype)
    fh = np.where(np.abs(f - fh) <= dtype(eb), fh, f).astype(dtype)
    out, cnt, stt, sw, recs = O.correct(f, fh, eb, max_sweeps=5000)
    if f.size == 1:
        assert stt == O.ERR_NOT_CONVERGED   # the isolated-voxel quirk
        return
    ref_out, ref_log, conv = refpy.correct(f, fh, eb, max_sweeps=5000)
    np.testing.assert_array_equal(out.view(np.uint8), ref_out.view(np.uint8))
    if stt == O.OK:
        v = O.verify(f, out, eb)
        assert v["dir_mismatch"] == 0 and v["as_mismatch"] == 0 and v["ds_mismatch"] == 0


# ---------------------------------------------------------------- edit output

@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_extract_and_reconstruct_round_trip(dtype):
    eb = 1e-2
    f, fh = _perlin_case((10, 12, 9), 11, dtype, "sz3", eb)
    out, *_ = O.correct(f, fh, eb)
    deltas, clamp, ec = O.extract_edits(fh, out, f, eb)
    assert ec == int((out < fh).sum())
    assert deltas.max() <= 5
    rec = O.reconstruct(fh, deltas, clamp, eb)
    np.testing.assert_array_equal(rec.view(np.uint8), out.ravel().view(np.uint8))


def test_pack_nbits_round_trip_and_layout():
    sym = np.array([1, 2, 3, 4, 5, 0, 7, 6], np.uint8)
    packed = O.pack_nbits(sym, 3)
    # LSB-first: 1 | 2<<3 | 3<<6 ... first byte = 0b11_010_001
    assert packed[0] == (1 | (2 << 3) | ((3 & 3) << 6))
    assert len(packed) == 3
    np.testing.assert_array_equal(O.unpack_nbits(packed, sym.size, 3), sym)
    assert O.bits_for_max(5) == 3 and O.bits_for_max(0) == 1 and O.bits_for_max(7) == 3 and O.bits_for_max(8) == 4


@pytest.mark.parametrize("comp", ["sz3", "zfp"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_naive_preserves_extrema_and_segmentations(comp, dtype):
    """naive_MSz.cu's loop ends with no false extremum and no label mismatch,
    and its last record is a clean check."""
    eb = 1e-2
    f, fh = _perlin_case((14, 12, 16), 7, dtype, comp, eb)
    out, cnt, st, sw, recs = O.correct_naive(f, fh, eb)
    assert st == O.OK
    v = O.verify(f, out, eb)
    assert v["ext_mismatch"] == 0
    assert v["as_mismatch"] == 0 and v["ds_mismatch"] == 0
    assert np.all(out <= fh)
    assert np.all(out >= (f - dtype(eb)))
    assert recs[-1].tolist() == [0, 0, 0, 0, 0]
    # the first record is an extrema sweep: no direction count
    assert recs[0][2] == 0


def test_naive_record_sequence_structure():
    """Extrema sweeps until one sees no false extremum, then a path repair
    (no extremum counts) and a check (no edits)."""
    eb = 1e-3
    f, fh = _perlin_case((20, 18, 16), 8, np.float32, "zfp", eb)
    out, cnt, st, sw, recs = O.correct_naive(f, fh, eb)
    assert st == O.OK
    prev, i = (1, 1), 0
    while i < len(recs):
        if prev[0] or prev[1]:
            assert recs[i][2] == 0
            prev = (recs[i][0], recs[i][1])
            i += 1
            continue
        assert recs[i][0] == 0 and recs[i][1] == 0      # path repair
        assert recs[i + 1][3] == 0 and recs[i + 1][4] == 0  # check
        prev = (recs[i + 1][0], recs[i + 1][1])
        i += 2
    assert i == len(recs)


def test_naive_is_thread_count_independent():
    eb = 1e-3
    f, fh = _perlin_case((24, 20, 18), 9, np.float64, "sz3", eb)
    n0 = O.num_threads()
    try:
        O.set_threads(1)
        a = O.correct_naive(f, fh, eb)
        O.set_threads(max(2, n0))
        b = O.correct_naive(f, fh, eb)
    finally:
        O.set_threads(n0)
    assert a[0].tobytes() == b[0].tobytes()
    np.testing.assert_array_equal(a[4], b[4])


# ------------------------------------------------ host-core field generator

@pytest.mark.parametrize("shape,seed,octaves,base,pers,dtype", [
    ((24, 20, 36), 0, 4, 1 / 16, 0.5, np.float32),
    ((33, 17, 40), 1, 5, 1 / 64, 0.5, np.float64),
    ((16, 16, 16), 7, 6, 1 / 128, 0.55, np.float32),
    ((64, 64, 64), 0, 4, 1 / 32, 0.5, np.float32),
])
def test_host_generator_matches_numpy(shape, seed, octaves, base, pers, dtype):
    """The oracle's C generator (used by the benchmark's CPU legs so that they
    load no GPU code) gives the numpy generator's bits, fields and stand-ins."""
    a = F.perlin_field(shape, seed, octaves, base, pers, dtype=dtype)
    b = O.perlin_field(shape, seed, octaves, base, pers, dtype=dtype)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    for comp in ("sz3", "zfp"):
        for eb in (1e-3, 1e-4, 3.7e-5):
            x = F.standin(a, eb, comp, seed)
            y = O.standin(a, eb, comp, seed)
            assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), (comp, eb)


def test_host_generator_rejects_bad_arguments():
    with pytest.raises(ValueError):
        O.standin(np.zeros((2, 2, 2), np.float32), 1e-3, "lz4")
    with pytest.raises(ValueError):
        O.standin(np.zeros((2, 2, 2), np.float32), -1.0, "zfp")
