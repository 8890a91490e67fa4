"""Batched correction: every field of a batch must end exactly as it does when
corrected alone (field bits, status, sweep count, per-sweep counters)."""
import numpy as np
import pytest

from pmsz_anonymous_gb300 import capi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _api():
    from pmsz_anonymous_gb300 import api
    return api


def _make(shape, dtype, comp, eb, seed, device):
    A = _api()
    f = A.gen_perlin(shape, seed, 4, 1 / 16, dtype=dtype, device=device)
    return f, A.standin(f, eb, comp, seed)


SPECS = [
    ((40, 36, 48), torch.float32, "zfp", 1e-3),
    ((17, 33, 70), torch.float32, "sz3", 2e-3),   # ragged rows
    ((64, 64, 64), torch.float32, "zfp", 1e-4),
    ((1, 1, 100), torch.float32, "zfp", 5e-2),   # a line
    ((32, 48, 40), torch.float64, "sz3", 1e-3),
    ((24, 24, 24), torch.float64, "zfp", 1e-4),
    ((5, 9, 130), torch.float64, "zfp", 1e-2),
    ((96, 80, 72), torch.float32, "zfp", 1e-3),
]


def test_batch_matches_individual_corrections(cuda):
    A = _api()
    fields = [_make(s, dt, c, eb, 40 + k, cuda) for k, (s, dt, c, eb) in enumerate(SPECS)]
    alone = []
    for (f, fh0), (_, _, _, eb) in zip(fields, SPECS):
        fh = fh0.clone()
        r = A.correct(f, fh, eb)
        alone.append((fh, r))
    work = [fh0.clone() for _, fh0 in fields]
    res = A.correct_batch([(f, w, spec[3]) for (f, _), w, spec in zip(fields, work, SPECS)])
    torch.cuda.synchronize()
    for k, ((fh, r), b, w) in enumerate(zip(alone, res, work)):
        assert b.status == r.status, k
        assert b.sweeps == r.sweeps, k
        np.testing.assert_array_equal(b.log[:, :5], r.log[:, :5], err_msg=f"field {k}")
        assert torch.equal(w.view(torch.uint8), fh.view(torch.uint8)), k


def test_batch_of_one_and_repeat(cuda):
    A = _api()
    f, fh0 = _make((48, 48, 48), torch.float64, "zfp", 1e-4, 7, cuda)
    ref = fh0.clone()
    r = A.correct(f, ref, 1e-4)
    for _ in range(2):
        w = fh0.clone()
        b = A.correct_batch([(f, w, 1e-4)])[0]
        assert b.status == r.status and b.sweeps == r.sweeps
        assert torch.equal(w.view(torch.uint8), ref.view(torch.uint8))


def test_batch_reports_bad_field_and_finishes_the_others(cuda):
    A = _api()
    a, ah = _make((20, 20, 20), torch.float32, "zfp", 1e-3, 1, cuda)
    b, bh = _make((20, 20, 20), torch.float32, "zfp", 1e-3, 2, cuda)
    bh[3, 4, 5] = float("nan")
    ref = ah.clone()
    A.correct(a, ref, 1e-3)
    w = ah.clone()
    res = A.correct_batch([(a, w, 1e-3), (b, bh, 1e-3)])
    assert res[0].status == capi.PMSZ_OK and res[1].status == capi.PMSZ_ERR_ARG
    assert torch.equal(w.view(torch.uint8), ref.view(torch.uint8))


@pytest.mark.parametrize("max_sweeps", [1, 2, 5])
def test_batch_stops_at_max_sweeps_like_alone(cuda, max_sweeps):
    A = _api()
    specs = SPECS[:3] + SPECS[4:6]
    fields = [_make(s, dt, c, eb, 60 + k, cuda) for k, (s, dt, c, eb) in enumerate(specs)]
    for dtype in (torch.float32, torch.float64):
        pick = [(fld, spec) for fld, spec in zip(fields, specs) if spec[1] == dtype]
        alone = []
        for (f, fh0), spec in pick:
            fh = fh0.clone()
            alone.append((fh, A.correct(f, fh, spec[3], max_sweeps=max_sweeps)))
        work = [fh0.clone() for (_, fh0), _ in pick]
        res = A.correct_batch([(f, w, spec[3]) for ((f, _), spec), w in zip(pick, work)], max_sweeps=max_sweeps)
        for k, ((fh, r), b, w) in enumerate(zip(alone, res, work)):
            assert b.status == r.status and b.sweeps == r.sweeps <= max_sweeps, k
            np.testing.assert_array_equal(b.log[:, :5], r.log[:, :5], err_msg=f"field {k}")
            assert torch.equal(w.view(torch.uint8), fh.view(torch.uint8)), k


def test_dense_active_sets_match_alone(cuda):
    # sz3 stand-ins at large eps: plateaus make most voxels active after the
    # first pass, so the batch's compaction takes its dense (word-expanded) form
    A = _api()
    specs = [((64, 64, 64), torch.float32, "sz3", 2e-2), ((96, 48, 40), torch.float32, "sz3", 5e-2),
             ((40, 40, 40), torch.float64, "sz3", 2e-2), ((33, 70, 50), torch.float64, "sz3", 3e-2)]
    fields = [_make(s, dt, c, eb, 80 + k, cuda) for k, (s, dt, c, eb) in enumerate(specs)]
    for dtype in (torch.float32, torch.float64):
        pick = [(fld, spec) for fld, spec in zip(fields, specs) if spec[1] == dtype]
        alone = []
        for (f, fh0), spec in pick:
            fh = fh0.clone()
            alone.append((fh, A.correct(f, fh, spec[3])))
        work = [fh0.clone() for (_, fh0), _ in pick]
        res = A.correct_batch([(f, w, spec[3]) for ((f, _), spec), w in zip(pick, work)])
        for k, ((fh, r), b, w) in enumerate(zip(alone, res, work)):
            assert b.status == r.status and b.sweeps == r.sweeps, k
            np.testing.assert_array_equal(b.log[:, :5], r.log[:, :5], err_msg=f"field {k}")
            assert torch.equal(w.view(torch.uint8), fh.view(torch.uint8)), k
