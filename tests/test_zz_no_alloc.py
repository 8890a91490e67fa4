"""pmsz_correct_noalloc: the allocation-free correction entry point.

It exists for callers that may not allocate device memory while they run --
for example an in-situ pipeline inside a simulation whose memory pool already
owns the GPU, or a service with a fixed memory budget -- so it keeps its
scratch in a fixed array inside the library instead.  These tests call it
through the C ABI and require the same corrected field, sweep count and
per-sweep counters as pmsz_correct_f32 / pmsz_correct_f64 (bit-identical, the
tolerance of every parity test here), on two calls in a row: the second call
finds the first call's leftovers in the shared array and must clear them.
The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

from pmsz_anonymous_gb300 import capi, fields as F

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc(f, fh, eb, max_sweeps=4096):
    L = capi.load()
    nz, ny, nx = f.shape
    opts = capi.Opts(5, 0, max_sweeps)
    log = (capi.SweepRecord * max_sweeps)()
    res = capi.Result()
    res.sweep_log = ctypes.cast(log, ctypes.POINTER(capi.SweepRecord))
    res.sweep_log_cap = max_sweeps
    st = L.pmsz_correct_noalloc(f.data_ptr(), fh.data_ptr(), f.element_size(), nx, ny, nz, float(eb),
                                ctypes.byref(opts), ctypes.byref(res), torch.cuda.current_stream().cuda_stream)
    rows = np.array([[log[i].fmax, log[i].fmin, log[i].fdir, log[i].requested, log[i].changed]
                     for i in range(res.sweeps)], np.uint64)
    _noalloc.ms_total = res.ms_total
    return st, res.sweeps, rows


def _allocating(f, fh, eb):
    from pmsz_anonymous_gb300 import api
    r = api.correct(f, fh, eb)
    return r.status, r.sweeps, r.log[:, :5]


@pytest.mark.parametrize("dtype,comp,shape,eb", [
    (torch.float32, "zfp", (48, 40, 56), 1e-3),
    (torch.float64, "sz3", (64, 64, 64), 1e-3),
    (torch.float32, "sz3", (3, 30, 70), 5e-3),
])
def test_noalloc_matches_allocating_entry_point_twice(cuda, dtype, comp, shape, eb):
    from pmsz_anonymous_gb300 import api
    f = api.gen_perlin(shape, 31, 4, 1 / 16, dtype=dtype, device=cuda)
    fh0 = api.standin(f, eb, comp, 31)
    ref = fh0.clone()
    st_ref, sw_ref, log_ref = _allocating(f, ref, eb)
    assert st_ref == capi.PMSZ_OK
    for _ in range(2):  # the second call starts from the first call's scratch contents
        out = fh0.clone()
        st, sw, log = _noalloc(f, out, eb)
        torch.cuda.synchronize()
        assert st == st_ref
        assert sw == sw_ref
        assert _noalloc.ms_total > 0.0      # the loop's window is measured
        assert torch.equal(out.view(torch.uint8), ref.view(torch.uint8))
        np.testing.assert_array_equal(log, log_ref)


def test_noalloc_call_leaves_device_memory_unchanged(cuda):
    from pmsz_anonymous_gb300 import api
    f = api.gen_perlin((32, 32, 32), 5, 3, 1 / 8, dtype=torch.float32, device=cuda)
    fh0 = api.standin(f, 1e-3, "zfp", 5)
    work = fh0.clone()
    _noalloc(f, work, 1e-3)                      # first call on the device: address set-up
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(cuda)[0]
    work.copy_(fh0)
    st, _, _ = _noalloc(f, work, 1e-3)
    torch.cuda.synchronize()
    assert st == capi.PMSZ_OK
    assert torch.cuda.mem_get_info(cuda)[0] == free_before


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    L = capi.load()
    f = torch.zeros((129, 128, 128), dtype=torch.float32, device=cuda)   # 2^21 + 2^14 voxels
    st = L.pmsz_correct_noalloc(f.data_ptr(), f.data_ptr(), 4, 128, 128, 129, 1e-3, None, None, None)
    assert st == capi.PMSZ_ERR_ARG
    assert b"exceeds its fixed scratch" in L.pmsz_last_error()
    g = torch.zeros((64, 64, 1), dtype=torch.float32, device=cuda)        # 1 voxel per row: 4096 words, fine
    st = L.pmsz_correct_noalloc(g.data_ptr(), g.data_ptr(), 3, 1, 64, 64, 1e-3, None, None, None)
    assert st == capi.PMSZ_ERR_ARG                                        # elem_size must be 4 or 8
