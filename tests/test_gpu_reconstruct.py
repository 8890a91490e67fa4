"""GPU reconstruction (pmsz_reconstruct_*): the corrected field rebuilt from
the decompressed field, the delta symbols and the clamp list -- bit-identical
to the correction's output and to the oracle's reconstruction, directly and
through the _deltas.bin / _edits.bin encoders; argument errors leave the
output untouched."""
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


CASES = [
    ((32, 32, 32), np.float32, "sz3", 1e-3, 9),
    ((5, 17, 33), np.float32, "zfp", 5e-3, 4),     # ragged: n not a multiple of 8, 32 or a tile
    ((24, 24, 24), np.float64, "zfp", 1e-4, 10),
    ((40, 48, 56), np.float64, "zfp", 1e-3, 12),   # several tiles, hundreds of clamps
]


def _corrected(case, cuda):
    shape, dtype, comp, eb, seed = case
    f = F.perlin_field(shape, seed, 4, 1 / 16, dtype=dtype)
    fh = F.standin(f, eb, comp, seed)
    df, prev = _dev(f, cuda), _dev(fh, cuda)
    cur = prev.clone()
    api().correct(df, cur, eb)
    return f, fh, df, prev, cur, eb


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{np.dtype(c[1]).name}-{c[2]}")
def test_round_trip_matches_correction_and_oracle(cuda, case):
    f, fh, df, prev, cur, eb = _corrected(case, cuda)
    d, cl, _ = api().extract_edits(prev, cur, df, eb)
    assert cl.numel() > 0 and int((d == 5).sum()) == cl.numel()
    out = api().reconstruct(prev, d, cl, eb)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint8), cur.cpu().numpy().view(np.uint8))
    rec = O.reconstruct(fh, d.cpu().numpy(), cl.cpu().numpy(), eb)
    np.testing.assert_array_equal(out.cpu().numpy().reshape(-1).view(np.uint8), rec.reshape(-1).view(np.uint8))
    inplace = prev.clone()
    assert api().reconstruct(inplace, d, cl, eb, out=inplace) is inplace
    assert torch.equal(inplace.view(torch.uint8), cur.view(torch.uint8))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_round_trip_through_the_output_files(cuda, dtype):
    case = ((40, 48, 56), dtype, "zfp", 1e-3, 12)
    f, fh, df, prev, cur, eb = _corrected(case, cuda)
    d, cl, _ = api().extract_edits(prev, cur, df, eb)
    n = prev.numel()
    blob_d = api().encode_deltas(d.cpu().numpy())
    blob_c = api().encode_clamps(cl.cpu().numpy())
    d2 = api().decode_deltas(blob_d, n)
    c2 = api().decode_clamps(blob_c, dtype)
    out = api().reconstruct(prev, _dev(d2, cuda), _dev(c2, cuda), eb)
    assert torch.equal(out.view(torch.uint8), cur.view(torch.uint8))


def test_no_edits_is_identity(cuda):
    prev = _dev(np.linspace(0.0, 1.0, 3000, dtype=np.float64).reshape(3, 10, 100), cuda)
    d = torch.zeros(prev.numel(), dtype=torch.uint8, device=cuda)
    cl = torch.empty(0, dtype=torch.float64, device=cuda)
    out = api().reconstruct(prev, d, cl, 1e-3)
    assert torch.equal(out.view(torch.uint8), prev.view(torch.uint8))


def test_argument_errors_write_nothing(cuda):
    case = ((32, 32, 32), np.float32, "sz3", 1e-3, 9)
    f, fh, df, prev, cur, eb = _corrected(case, cuda)
    d, cl, _ = api().extract_edits(prev, cur, df, eb)
    sentinel = torch.full_like(prev, 7.0)
    # one clamp value short (as when the reference encoder dropped a 0 clamp)
    with pytest.raises(capi.PmszError) as e:
        api().reconstruct(prev, d, cl[:-1].clone(), eb, out=sentinel)
    assert e.value.status == capi.PMSZ_ERR_ARG
    # a symbol above q
    bad = d.clone()
    bad[17] = 6
    with pytest.raises(capi.PmszError) as e:
        api().reconstruct(prev, bad, cl, eb, out=sentinel)
    assert e.value.status == capi.PMSZ_ERR_ARG
    assert bool((sentinel == 7.0).all())
    # a zero clamp value is dropped by the extraction: its field cannot be rebuilt
    fz = np.full((2, 4, 8), 1e-3, np.float32)
    pz = fz + np.float32(5e-4)
    cz = pz.copy()
    cz[0, 0, 0] = fz[0, 0, 0] - np.float32(1e-3)  # the clamp f - eps == 0
    dz, clz, _ = api().extract_edits(_dev(pz, cuda), _dev(cz, cuda), _dev(fz, cuda), 1e-3)
    assert int(dz[0]) == 5 and clz.numel() == 0
    with pytest.raises(capi.PmszError) as e:
        api().reconstruct(_dev(pz, cuda), dz, clz, 1e-3)
    assert e.value.status == capi.PMSZ_ERR_ARG
    with pytest.raises(capi.PmszError):
        api().reconstruct(prev, d, cl, eb, q=0)
