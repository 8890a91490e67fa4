"""Correction server: jobs that arrive while others run are admitted into the
running batch, and every job ends bit-identical to correcting its field alone."""
import threading
import time

import numpy as np
import pytest

from pmsz_anonymous_gb300 import capi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _api():
    from pmsz_anonymous_gb300 import api
    return api


JOBS = [
    ((40, 36, 48), torch.float32, "zfp", 1e-3),
    ((64, 64, 64), torch.float64, "zfp", 1e-4),
    ((17, 33, 70), torch.float32, "sz3", 2e-3),
    ((96, 80, 72), torch.float32, "zfp", 1e-3),
    ((32, 48, 40), torch.float64, "sz3", 1e-3),
    ((1, 1, 100), torch.float32, "zfp", 5e-2),
    ((80, 80, 80), torch.float32, "sz3", 1e-4),
    ((24, 24, 24), torch.float64, "zfp", 1e-4),
]


def _prepare(device):
    A = _api()
    out = []
    for k, (shape, dt, comp, eb) in enumerate(JOBS):
        f = A.gen_perlin(shape, 300 + k, 4, 1 / 16, dtype=dt, device=device)
        fh = A.standin(f, eb, comp, 300 + k)
        ref = fh.clone()
        r = A.correct(f, ref, eb)
        out.append((f, fh, eb, ref, r))
    torch.cuda.synchronize()
    return out


def _check(job, info, work):
    f, fh, eb, ref, r = job
    assert info["done"] == 1
    assert info["status"] == r.status
    assert info["sweeps"] == r.sweeps
    assert info["edits"] == r.edits
    assert torch.equal(work.view(torch.uint8), ref.view(torch.uint8))


def test_jobs_arriving_during_others_match_alone(cuda):
    A = _api()
    jobs = _prepare(cuda)
    work = [j[1].clone() for j in jobs]
    torch.cuda.synchronize()
    with A.Server() as srv:
        ids = []
        for k, (j, w) in enumerate(zip(jobs, work)):
            ids.append(srv.submit(j[0], w, j[2]))
            time.sleep(0.002 * (k % 3))  # later jobs arrive while earlier ones run
        infos = [srv.wait(i) for i in ids]
    torch.cuda.synchronize()
    for j, info, w in zip(jobs, infos, work):
        _check(j, info, w)


def test_submissions_from_several_threads(cuda):
    A = _api()
    jobs = _prepare(cuda)
    work = [j[1].clone() for j in jobs]
    torch.cuda.synchronize()
    infos = [None] * len(jobs)
    with A.Server(max_jobs=3) as srv:
        def client(k):
            jid = srv.submit(jobs[k][0], work[k], jobs[k][2])
            infos[k] = srv.wait(jid)
        threads = [threading.Thread(target=client, args=(k,)) for k in range(len(jobs))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    torch.cuda.synchronize()
    for j, info, w in zip(jobs, infos, work):
        _check(j, info, w)


def test_budget_limits_admission_and_rejects_oversized_jobs(cuda):
    A = _api()
    jobs = _prepare(cuda)
    work = [j[1].clone() for j in jobs]
    torch.cuda.synchronize()
    biggest = max(j[0].numel() * j[0].element_size() for j in jobs)
    budget = 40 * biggest  # room for only a few jobs at a time
    with A.Server(hbm_budget_bytes=budget) as srv:
        ids = [srv.submit(j[0], w, j[2]) for j, w in zip(jobs, work)]
        infos = [srv.wait(i) for i in ids]
        big = torch.zeros((256, 256, 256), dtype=torch.float64, device=cuda)
        with pytest.raises(capi.PmszError) as e:
            srv.submit(big, big.clone(), 1e-3)
        assert e.value.status == capi.PMSZ_ERR_OOM
    for j, info, w in zip(jobs, infos, work):
        _check(j, info, w)
    assert max(i["queue_ms"] for i in infos) >= 0.0


def test_large_group_runs_list_generations_and_matches_alone(cuda):
    # eight 160^3 fields joining together: the running set's estimated active
    # voxels pass 2^20, so the server takes its voxel-list generations
    A = _api()
    jobs = []
    for k in range(8):
        comp, eb = ("sz3", 2e-3) if k % 2 else ("zfp", 1e-3)
        f = A.gen_perlin((160, 160, 160), 500 + k, 4, 1 / 16, dtype=torch.float32, device=cuda)
        fh = A.standin(f, eb, comp, 500 + k)
        ref = fh.clone()
        r = A.correct(f, ref, eb)
        jobs.append((f, fh, eb, ref, r))
    work = [j[1].clone() for j in jobs]
    torch.cuda.synchronize()
    with A.Server() as srv:
        ids = [srv.submit(j[0], w, j[2]) for j, w in zip(jobs, work)]
        infos = [srv.wait(i) for i in ids]
    torch.cuda.synchronize()
    for j, info, w in zip(jobs, infos, work):
        _check(j, info, w)
