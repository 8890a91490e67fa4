"""The oracle against golden fixtures produced by the REFERENCE's own kernels
(pMSz.cu compiled unmodified, driven at an MPI grid of 1x1x1 by
oracle/ref_harness.cpp; generator: tests/golden/make_reference_fixtures.py)."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixtures(prefix):
    files = sorted(glob.glob(os.path.join(GOLD, f"{prefix}_*.npz")))
    if not files:
        pytest.skip(f"no {prefix} fixtures")
    return files


def _padded_to_flat(p, shape):
    """Padded flat index (reference layout) -> unpadded flat index."""
    nz, ny, nx = shape
    W, H = nx + 2, ny + 2
    x, y, z = p % W, (p // W) % H, p // (W * H)
    return (x - 1) + nx * ((y - 1) + ny * (z - 1))


def _interior(a):
    return a[1:-1, 1:-1, 1:-1]


@pytest.mark.parametrize("path", _fixtures("label") if glob.glob(os.path.join(GOLD, "label_*.npz")) else [None])
def test_labelling_and_detection_directions_match_reference(path):
    if path is None:
        pytest.skip("no fixtures")
    d = np.load(path)
    f, fh, eb = d["f"], d["fh"], float(d["eb"])
    ot = _interior(d["ortypes"]).reshape(-1, 2).astype(np.int64)
    asc, desc = O.label(f)
    i = np.arange(f.size)
    t, u = ot[:, 0], ot[:, 1]
    is_max, is_min = t == -1, t == -2
    other = ~(is_max | is_min)
    # or_types encoding, pMSz.cu:749-783
    assert np.array_equal(is_max, asc == i)
    assert np.array_equal(desc[is_max], _padded_to_flat(u[is_max], f.shape))
    assert np.array_equal(desc[is_min], i[is_min]) and np.array_equal(asc[is_min], _padded_to_flat(u[is_min], f.shape))
    assert np.array_equal(desc[other], _padded_to_flat(t[other], f.shape))
    assert np.array_equal(asc[other], _padded_to_flat(u[other], f.shape))
    # the detect-only pass writes the steepest directions of the decompressed field
    hasc, hdesc = O.label(fh)
    assert np.array_equal(_padded_to_flat(_interior(d["dir_as"]).ravel().astype(np.int64), f.shape), hasc)
    assert np.array_equal(_padded_to_flat(_interior(d["dir_ds"]).ravel().astype(np.int64), f.shape), hdesc)
    # its (racy) counters are zero exactly when the oracle's first sweep is clean
    _, _, _, _, recs = O.correct(f, fh, eb, max_sweeps=1)
    assert (d["counts"] > 0).tolist() == (recs[0, :3] > 0).tolist()


@pytest.mark.parametrize("name", ["pair", "line5"])
def test_single_target_loops_match_reference_bit_for_bit(name):
    path = os.path.join(GOLD, f"correct_{name}.npz")
    if not os.path.exists(path):
        pytest.skip("no fixture")
    d = np.load(path)
    out, cnt, st, sweeps, recs = O.correct(d["f"], d["fh"], float(d["eb"]))
    assert st == O.OK
    np.testing.assert_array_equal(out.view(np.uint8), d["field"].view(np.uint8))
    assert sweeps + 1 == int(d["ite"][0])   # the reference's printed iteration count


def test_racy_reference_loop_is_a_valid_correction_like_the_oracle():
    path = os.path.join(GOLD, "correct_perlin_racy.npz")
    if not os.path.exists(path):
        pytest.skip("no fixture")
    d = np.load(path)
    f, fh, eb = d["f"], d["fh"], float(d["eb"])
    ours, _, st, sweeps, _ = O.correct(f, fh, eb)
    for fp in list(d["fields"]) + [ours]:
        v = O.verify(f, fp, eb)
        assert v["dir_mismatch"] == v["ext_mismatch"] == v["as_mismatch"] == v["ds_mismatch"] == 0
        assert np.all(fp >= f - eb) and np.all(fp <= fh)   # edits only lower, never below fl(f - eps)
    # On this field the reference's scheduling-dependent loop happens to land, in
    # every recorded run, on exactly the snapshot result, in the same number of
    # iterations.
    for fp, ite in zip(d["fields"], d["ites"]):
        np.testing.assert_array_equal(fp.view(np.uint8), ours.view(np.uint8))
        assert int(ite) == sweeps + 1


@pytest.mark.parametrize("name", ["perlin_zfp", "perlin_sz3"])
def test_edit_extraction_matches_reference(name):
    path = os.path.join(GOLD, f"extract_{name}.npz")
    if not os.path.exists(path):
        pytest.skip("no fixture")
    d = np.load(path)
    f, fh, cur, eb = d["f"], d["fh"], d["cur"], float(d["eb"])
    deltas, clamp, ec = O.extract_edits(fh, cur, f, eb)
    ref = d["deltas"]
    raised = (cur > fh).ravel()
    # the reference leaves deltas unwritten where cur > prev; everywhere else: identical
    np.testing.assert_array_equal(deltas[~raised], ref[~raised])
    eo = d["editsout"]
    np.testing.assert_array_equal(eo[eo != 0], clamp)   # copy_if(v != 0) keeps voxel order
    assert int(d["hcount"][0]) == ec


@pytest.mark.parametrize("name", ["perlin_zfp", "perlin_sz3"])
def test_naive_loop_matches_reference_kernels(name):
    """naive_MSz.cu's own kernels (its c_loops restated around them at one
    rank, three runs): the oracle's naive restatement gives the same field
    bit for bit, the same per-pass counts and the same `ite`."""
    path = os.path.join(GOLD, f"naive_{name}.npz")
    d = np.load(path)
    f, fh, eb = d["f"], d["fh"], float(d["eb"])
    out, cnt, st, sw, recs = O.correct_naive(f, fh, eb)
    assert st == O.OK
    for k in range(d["fields"].shape[0]):
        np.testing.assert_array_equal(out.view(np.uint8), d["fields"][k].view(np.uint8))
    # the reference's counters are non-atomic `+= 1` on __device__ globals
    # (naive_MSz.cu:781, 805, 1786, 1826): racy lower bounds of the exact
    # counts, zero exactly when the exact count is zero
    ref = d["recs"].astype(np.uint64)
    assert len(ref) == sw
    for (kind, fmax, fmin, fdir), mine in zip(ref, recs):
        want = {0: (fmax, fmin, 0), 1: (0, 0, fdir), 2: (fmax, fmin, fdir)}[int(kind)]
        got = (mine[0], mine[1], mine[2])
        assert [g > 0 for g in got] == [w > 0 for w in want]
        assert all(g >= w for g, w in zip(got, want))
        if kind == 2:
            assert mine[3] == 0 and mine[4] == 0
    inner, outer = (int(v) for v in d["passes"])
    assert int((ref[:, 0] == 0).sum()) == inner and int((ref[:, 0] == 2).sum()) == outer
    assert all(int(i) == 2 * outer + inner for i in d["ites"])
