"""The autotuner: its choices come from the candidate sets, it records them
for the shape class, and no tile depth or rounds-per-launch count changes any
result (corrected fields, sweep counts, labels, batches) -- all checked
against the oracle through the C ABI."""
import numpy as np
import pytest

from oracle import oracle as O
from pmsz_anonymous_gb300 import fields as F

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def api():
    from pmsz_anonymous_gb300 import api as A
    return A


@pytest.fixture(autouse=True)
def clean_table():
    api().tune_clear()
    yield
    api().tune_clear()


def _dev(a, device):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def _case(shape, dtype, comp, eb, seed):
    f = F.perlin_field(shape, seed, 4, 1 / 16, dtype=dtype)
    return f, F.standin(f, eb, comp, seed)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_autotune_picks_candidates_and_records_them(cuda, dtype):
    f, fh = _case((70, 45, 66), dtype, "sz3", 1e-3, 3)
    df, dfh = _dev(f, cuda), _dev(fh, cuda)
    before = dfh.clone()
    t = api().autotune(df, dfh)
    assert torch.equal(dfh, before)  # tuning leaves the inputs untouched
    assert t["zchunk"] in (8, 16, 32, 64) and t["jump_rounds"] in (1, 2, 4, 8)
    assert set(t["ms_zchunk"]) == {8, 16, 32, 64} and min(t["ms_zchunk"].values()) > 0
    assert t["ms_zchunk"][t["zchunk"]] == min(t["ms_zchunk"].values())
    assert t["ms_rounds"][t["jump_rounds"]] == min(t["ms_rounds"].values())
    known, got = api().tune_get(f.shape, df.dtype)
    assert known and got == {"zchunk": t["zchunk"], "jump_rounds": t["jump_rounds"]}
    # a shape of the same class (same ceil-log2 axes) shares the entry
    assert api().tune_get((65, 33, 127), df.dtype) == (True, got)


def test_shallow_field_tries_one_chunk_depth_only_once(cuda):
    f, fh = _case((6, 40, 50), np.float32, "zfp", 1e-3, 4)
    t = api().autotune(_dev(f, cuda), _dev(fh, cuda))
    assert set(t["ms_zchunk"]) == {8}  # nz = 6: every depth >= 8 is one chunk


@pytest.mark.parametrize("zchunk", [1, 5, 8, 16, 64])
@pytest.mark.parametrize("case", [((77, 45, 70), np.float32, "sz3", 2e-3, 11),
                                  ((40, 33, 37), np.float64, "zfp", 1e-3, 12)],
                         ids=["f32-sz3", "f64-zfp"])
def test_results_do_not_depend_on_tile_depth(cuda, case, zchunk):
    shape, dtype, comp, eb, seed = case
    f, fh = _case(shape, dtype, comp, eb, seed)
    ref, cnt, st, sw, recs = O.correct(f, fh, eb)
    api().tune_set(shape, torch.float32 if dtype == np.float32 else torch.float64, zchunk, 1)
    dfh = _dev(fh, cuda)
    r = api().correct(_dev(f, cuda), dfh, eb)
    assert r.status == st and r.sweeps == sw
    np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    np.testing.assert_array_equal(r.log[:, :5], recs)
    # the host-buffer path slabs its ingest by the same depth
    hfh = torch.from_numpy(fh.copy()).pin_memory()
    api().correct_host(torch.from_numpy(f.copy()).pin_memory(), hfh, eb)
    np.testing.assert_array_equal(hfh.numpy().view(np.uint8), ref.view(np.uint8))


@pytest.mark.parametrize("rounds", [1, 3, 8])
def test_labels_do_not_depend_on_rounds_per_launch(cuda, rounds):
    shape = (30, 41, 67)
    f = F.perlin_field(shape, 5, 4, 1 / 8, dtype=np.float64)
    codes = api().codes(_dev(f, cuda))
    api().tune_set(shape, torch.float64, 32, rounds)
    as_l, ds_l = api().labels(codes)
    asc, desc = O.label(f)
    np.testing.assert_array_equal(as_l.cpu().numpy().ravel(), O.path_compress(asc))
    np.testing.assert_array_equal(ds_l.cpu().numpy().ravel(), O.path_compress(desc))


def test_correct_autotune_flag_tunes_once(cuda):
    f, fh = _case((50, 40, 64), np.float32, "sz3", 1e-3, 6)
    ref = O.correct(f, fh, 1e-3)[0]
    dfh = _dev(fh, cuda)
    assert api().tune_get(f.shape, torch.float32)[0] is False
    api().correct(_dev(f, cuda), dfh, 1e-3, autotune=True)
    assert api().tune_get(f.shape, torch.float32)[0] is True
    np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))


def test_batch_with_autotune_matches_oracle(cuda):
    cases = [((40, 33, 70), np.float32, "sz3", 2e-3, 31), ((20, 64, 20), np.float32, "zfp", 1e-3, 32),
             ((9, 15, 100), np.float32, "sz3", 5e-3, 33)]
    items, refs = [], []
    for shape, dtype, comp, eb, seed in cases:
        f, fh = _case(shape, dtype, comp, eb, seed)
        refs.append(O.correct(f, fh, eb)[0])
        items.append((_dev(f, cuda), _dev(fh, cuda), eb))
    total = sum(int(np.prod(c[0])) for c in cases)
    assert api().tune_batch_get(total, len(cases), torch.float32) == (False, 32)
    res = api().correct_batch(items, autotune=True)
    known, zc = api().tune_batch_get(total, len(cases), torch.float32)
    assert known and zc in (8, 16, 32, 64)
    for (shape, *_), (_, dfh, _), ref, r in zip(cases, items, refs, res):
        assert r.status == 0
        assert api().tune_get(shape, torch.float32)[0] is True
        np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))


@pytest.mark.parametrize("zchunk", [8, 64])
def test_batch_results_do_not_depend_on_batch_tile_depth(cuda, tmp_path, zchunk):
    cases = [((40, 33, 70), np.float32, "sz3", 2e-3, 41), ((20, 64, 20), np.float32, "zfp", 1e-3, 42)]
    total = sum(int(np.prod(c[0])) for c in cases)
    # a recorded batch depth (through the text table) is what the batch runs at
    p = tmp_path / "t.txt"
    p.write_text("pmsz-tune 1\nb 4 %d %d %d\n" % ((total - 1).bit_length(), 1, zchunk))
    api().tune_load(str(p))
    assert api().tune_batch_get(total, 2, torch.float32) == (True, zchunk)
    items, refs = [], []
    for shape, dtype, comp, eb, seed in cases:
        f, fh = _case(shape, dtype, comp, eb, seed)
        refs.append(O.correct(f, fh, eb)[0])
        items.append((_dev(f, cuda), _dev(fh, cuda), eb))
    for r in api().correct_batch(items):
        assert r.status == 0
    for (_, dfh, _), ref in zip(items, refs):
        np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))
