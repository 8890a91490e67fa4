"""naive-MSz strategy (naive_MSz.cu:1887-2220) through pmsz_correct_naive_*:
bit-identical to the CPU oracle's restatement -- field, every per-pass record
and the reference's iteration count -- and topology-preserving."""
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


def reference_ite(recs) -> int:
    """The reference's `ite` for a converged record sequence: extrema sweeps
    run while the previous extrema sweep or check saw a false extremum
    (initially assumed), then one path repair and one check; +1 per extrema
    sweep, +2 per outer iteration."""
    prev, i, outer, inner = (1, 1), 0, 0, 0
    while i < len(recs):
        if prev[0] or prev[1]:
            inner += 1
            prev = (int(recs[i][0]), int(recs[i][1]))
            i += 1
            continue
        outer += 1
        prev = (int(recs[i + 1][0]), int(recs[i + 1][1]))
        i += 2
    return 2 * outer + inner


CASES = [
    ((16, 16, 16), np.float32, "sz3", 1e-3, 0),
    ((16, 16, 16), np.float32, "zfp", 1e-3, 1),
    ((12, 20, 24), np.float64, "zfp", 1e-3, 2),
    ((12, 20, 24), np.float64, "sz3", 2e-3, 3),
    ((5, 17, 33), np.float32, "zfp", 5e-3, 4),
    ((3, 7, 70), np.float64, "sz3", 1e-2, 5),
    ((1, 1, 64), np.float32, "zfp", 5e-2, 6),
    ((40, 1, 1), np.float64, "zfp", 5e-2, 7),
    ((2, 2, 2), np.float32, "zfp", 1e-1, 8),
    ((32, 32, 32), np.float32, "sz3", 1e-3, 9),
    ((24, 24, 24), np.float64, "zfp", 1e-4, 10),
    ((48, 40, 36), np.float32, "zfp", 1e-3, 11),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{np.dtype(c[1]).name}-{c[2]}")
def test_naive_matches_oracle(cuda, case):
    shape, dtype, comp, eb, seed = case
    f = F.perlin_field(shape, seed, 4, 1 / 16, dtype=dtype)
    fh = F.standin(f, eb, comp, seed)
    ref, cnt, st, sw, recs = O.correct_naive(f, fh, eb)
    df, dfh = _dev(f, cuda), _dev(fh, cuda)
    r = api().correct(df, dfh, eb, strategy="naive")
    out = dfh.cpu().numpy()
    assert r.status == st
    assert r.sweeps == sw
    np.testing.assert_array_equal(out.view(np.uint8), ref.view(np.uint8))
    np.testing.assert_array_equal(r.log[:, :5], recs)
    assert r.edits == int(recs[:, 3].sum())
    assert int(r.log[:, 7].sum()) == 0  # no walk hit its guard
    if st == O.OK:
        assert r.iteration == reference_ite(recs)
        v = api().verify(df, dfh, eb)
        assert v["ext_mismatch"] == 0
        assert v["as_mismatch"] == 0 and v["ds_mismatch"] == 0
        assert v["bound_beyond_clamp"] == 0


def test_naive_repeat_is_deterministic(cuda):
    f = F.perlin_field((40, 36, 30), 12, 4, 1 / 16, dtype=np.float32)
    fh = F.standin(f, 1e-3, "sz3", 12)
    df = _dev(f, cuda)
    outs = []
    for _ in range(2):
        dfh = _dev(fh, cuda)
        r = api().correct(df, dfh, 1e-3, strategy="naive")
        outs.append((r.sweeps, r.edits, dfh.cpu().numpy().tobytes()))
    assert outs[0] == outs[1]


def test_naive_max_sweeps_and_args(cuda):
    f = F.perlin_field((24, 24, 24), 13, 4, 1 / 16, dtype=np.float64)
    fh = F.standin(f, 1e-3, "zfp", 13)
    ref, cnt, st, sw, recs = O.correct_naive(f, fh, 1e-3, max_sweeps=3)
    df, dfh = _dev(f, cuda), _dev(fh, cuda)
    r = api().correct(df, dfh, 1e-3, max_sweeps=3, strategy="naive")
    assert st == O.ERR_NOT_CONVERGED and r.status == capi.PMSZ_ERR_NOT_CONVERGED
    assert r.sweeps == sw == 3
    np.testing.assert_array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8))
    bad = dfh.clone()
    bad.view(-1)[17] = float("nan")
    with pytest.raises(capi.PmszError) as e:
        api().correct(df, bad, 1e-3, strategy="naive")
    assert e.value.status == capi.PMSZ_ERR_ARG
    with pytest.raises(capi.PmszError):
        api().correct(df, dfh, -1.0, strategy="naive")
