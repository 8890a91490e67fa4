"""Side-by-side timing of the REFERENCE's own CUDA kernels and this library on
one GPU, on the same field (test infrastructure: needs the prebuilt
``oracle/_ref/pmsz_ref.cubin`` / ``naive_ref.cubin``, see build_ref.py).

The reference loop runs through ``oracle/_ref/ref_harness`` (its c_loops
restated around its unmodified kernels at an MPI grid of 1x1x1, fp64 only,
device-synchronised time from the original labelling to convergence); this
library's pmsz_correct_f64 / pmsz_correct_naive_f64 runs on the same bytes,
timed with CUDA events over the same window.  Prints one JSON line with both
times and whether the corrected fields are identical.

    python oracle/time_reference.py [--shape 512,512,512] [--strategy pmsz|naive]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this file's folder heads sys.path and its oracle.py would
# shadow the oracle/ folder
sys.path[:] = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--shape", default="512,512,512")
    p.add_argument("--strategy", choices=["pmsz", "naive"], default="pmsz")
    p.add_argument("--eb", type=float, default=1e-4)
    p.add_argument("--comp", default="zfp")
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--octaves", type=int, default=5)
    p.add_argument("--base", type=float, default=1 / 64)
    p.add_argument("--runs", type=int, default=2)
    args = p.parse_args()

    import torch
    from pmsz_anonymous_gb300 import api

    cubin = build_ref.NAIVE_CUBIN if args.strategy == "naive" else build_ref.CUBIN
    if not os.path.exists(cubin):
        print(json.dumps({"unavailable": f"{os.path.basename(cubin)} was not built"}))
        return
    harness = build_ref.build_harness()
    nx, ny, nz = (int(v) for v in args.shape.split(","))
    dev = torch.device("cuda", 0)
    f = api.gen_perlin((nz, ny, nx), args.seed, args.octaves, args.base, dtype=torch.float64, device=dev)
    fh = api.standin(f, args.eb, args.comp, args.seed)
    torch.cuda.synchronize()
    tmp = tempfile.mkdtemp()
    pf, ph = os.path.join(tmp, "f.bin"), os.path.join(tmp, "fh.bin")
    f.cpu().numpy().tofile(pf)
    fh.cpu().numpy().tofile(ph)

    mode = "naive" if args.strategy == "naive" else "correct"
    ref_ms, ref_field, ref_ite = [], None, None
    for k in range(args.runs):
        out = os.path.join(tmp, f"ref{k}")
        subprocess.run([harness, cubin, mode, str(nx), str(ny), str(nz), repr(args.eb), pf, ph, out],
                       check=True, timeout=3600)
        ref_ms.append(float(np.fromfile(out + "_ms.bin", np.float32)[0]))
        ref_ite = int(np.fromfile(out + "_ite.bin", np.int32)[0])
        if k == 0:
            ref_field = np.fromfile(out + "_field.bin", np.float64).reshape(nz + 2, ny + 2, nx + 2)[1:-1, 1:-1, 1:-1]
        for suffix in ("_field.bin", "_ortypes.bin", "_dir_as.bin", "_dir_ds.bin"):
            if os.path.exists(out + suffix):
                os.remove(out + suffix)

    ours_ms, r = [], None
    work = torch.empty_like(fh)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for k in range(args.runs + 1):
        work.copy_(fh)
        torch.cuda.synchronize()
        start.record()
        r = api.correct(f, work, args.eb, strategy=args.strategy)
        stop.record()
        stop.synchronize()
        if k:
            ours_ms.append(start.elapsed_time(stop))
    same = bool(np.array_equal(work.cpu().numpy().view(np.uint8), ref_field.view(np.uint8)))
    n = nx * ny * nz
    print(json.dumps({
        "workload": f"{nx}x{ny}x{nz} f64 Perlin fBm (seed {args.seed}, {args.octaves} octaves, base {args.base}), "
                    f"{args.comp} stand-in, eps={args.eb}",
        "strategy": args.strategy,
        "reference_kernels_ms": statistics.median(ref_ms), "reference_runs_ms": ref_ms, "reference_ite": ref_ite,
        "ours_ms": statistics.median(ours_ms), "ours_runs_ms": ours_ms, "ours_iteration": r.iteration,
        "ours_gvox_s": n / (statistics.median(ours_ms) * 1e-3) / 1e9,
        "reference_gvox_s": n / (statistics.median(ref_ms) * 1e-3) / 1e9,
        "speedup": statistics.median(ref_ms) / statistics.median(ours_ms),
        "identical_fields": same,
    }))


if __name__ == "__main__":
    main()
