"""Benchmark of the correction path (one JSON line on rank 0).

Workload (default): plain single-field correction of a 512^3 fp64 Perlin fBm
field (seed 1, 5 octaves, base frequency 1/64, persistence 0.5, lacunarity 2,
normalised to [0,1]) decompressed through the ZFP-like stand-in at eps = 1e-4
(the reference's per-rank weak-scaling block).  A step = one full correction
(labelling, detection / edit sweeps to convergence) of that field.

value   device-resident throughput, Gvox/s = N / (device time of one
        pmsz_correct call), CUDA events on the launching stream, fhat refreshed
        from a pristine device copy before each step (untimed).
e2e     the same through the host-buffer C ABI (pmsz_correct_host_*): pinned
        host f and fhat copied in, the correction, the edit extraction and the
        copy back of what the reference's main hands to its host encoder --
        the delta symbols (packed at 3 bits) and the clamp list -- all timed.
roofline  the fused labelling + first detection pass k_tiled<T,kFirst> (the
        largest kernel): algorithmic bytes 2*N*(sizeof(T)+1) -- the one-time
        original labelling (read f, write the code byte) plus one detection
        sweep (read fhat and the code byte) -- over its event-timed duration,
        against the measured HBM copy bandwidth; traffic = ncu dram bytes per
        launch of the same kernel.  roofline.per_step: the whole step's
        active-set algorithmic bytes over ms_per_step.
cpu_baseline  the CPU oracle (a restatement of the reference loop, OpenMP on
        all host cores) on the whole field; parity: its corrected field, sweep
        count and per-sweep counters against the GPU's, bit for bit.
batch / serve / reference_kernels  (after the timed region) the batched form
        on 64 mixed fp32 fields against the same fields one by one, the
        served stream's jobs/s and p50/p99 at three arrival rates, and the
        reference's own CUDA kernels timed beside this library on the field.

--impl reference: the reference's path on the host cores -- the reference
itself is CUDA-only with no CPU implementation, so this arm runs the CPU
oracle restatement (kind "port") on the whole field, generated on the host
cores by the oracle library (no GPU code is loaded).
With N > 1 (torchrun) every rank corrects its own replica: no data-path
collective; a barrier brackets the timed region and the max over ranks is taken.
"""
from __future__ import annotations

import argparse
import collections
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gvox/s correction at 512³ fp64 vs ref 1-rank; batched vox/s; p50/p99 latency"


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--no-tune", action="store_true", help="skip the autotuner (default launch parameters)")
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--shape", default="512,512,512", help="nx,ny,nz")
    p.add_argument("--dtype", choices=["f32", "f64"], default="f64")
    p.add_argument("--comp", choices=["sz3", "zfp"], default="zfp")
    p.add_argument("--eb", type=float, default=1e-4)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--octaves", type=int, default=5)
    p.add_argument("--base", type=float, default=1 / 64)
    p.add_argument("--persistence", type=float, default=0.5)
    p.add_argument("--cpu-single-slices", type=int, default=32,
                   help="z-slices of the single-thread CPU sample (0 = none)")
    p.add_argument("--cpu-slices", type=int, default=0,
                   help="z-slices of the CPU sample (0 = the whole field: about 10 s on 16 cores at 512^3 fp64)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--workload", choices=["plain", "batch", "serve", "reconstruct", "hostlink"], default="plain",
                   help="plain: one 512^3 field (the headline); batch: 64 mixed fp32 fields; "
                        "serve: Poisson job stream through the correction server; "
                        "reconstruct: the decoder on the plain workload's field; "
                        "hostlink: host<->device copy rates that bound the e2e number")
    p.add_argument("--serve-jobs", type=int, default=120)
    p.add_argument("--serve-rates", default="100,300,1000,3000", help="arrival rates (jobs/s) to sweep")
    p.add_argument("--batch-fields", type=int, default=64)
    p.add_argument("--host-loop", action="store_true",
                   help="enqueue the list sweeps from the host instead of the CUDA graph (for ncu, which does "
                        "not profile kernels of graphs with conditional nodes)")
    p.add_argument("--no-extra", action="store_true",
                   help="plain workload only: skip the batch, serve and reference-kernel legs")
    return p.parse_args(argv)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                mhz.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(mhz)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def max_over_ranks(value: float, device) -> float:
    """Max of a per-rank scalar over the ranks of the default process group
    (the value itself without one).  device is where the backend reduces:
    the rank's GPU for NCCL, "cpu" for gloo."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(voxels_per_rank: int, world: int, ms: float) -> float:
    """Gvox/s of the whole job: every rank corrects its own replica of
    voxels_per_rank voxels, and the slowest rank's time ms bounds the job."""
    return world * voxels_per_rank / (ms * 1e-3) / 1e9


def profiled_traffic(name: str):
    """dram read+write bytes per launch of `name` from a committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            return json.load(fh).get(name)
    except (OSError, ValueError):
        return None


def cpu_sample(f: np.ndarray, fh: np.ndarray, eb: float, slices: int):
    """Time the CPU oracle on the first `slices` z-slices of the field (0 =
    all of it).  Returns (voxels, seconds, threads, sweeps, (corrected field,
    status, per-sweep records))."""
    from oracle import oracle as O
    slices = slices or f.shape[0]
    fs = np.ascontiguousarray(f[:slices])
    fhs = np.ascontiguousarray(fh[:slices])
    t0 = time.perf_counter()
    out, _, st, sweeps, recs = O.correct(fs, fhs, eb)
    dt = time.perf_counter() - t0
    return fs.size, dt, O.num_threads(), sweeps, (out, st, recs)


def host_fields(args):
    """f and fhat of the workload generated on the host cores by the oracle
    library (bit-identical to the GPU generator; loads no GPU code)."""
    from oracle import oracle as O
    nx, ny, nz = (int(v) for v in args.shape.split(","))
    dt = np.float64 if args.dtype == "f64" else np.float32
    f = O.perlin_field((nz, ny, nx), args.seed, args.octaves, args.base, args.persistence, 2.0, dtype=dt)
    return f, O.standin(f, args.eb, args.comp, args.seed)


def gen_fields(args, torch, device, dtype):
    from pmsz_anonymous_gb300 import api
    nx, ny, nz = (int(v) for v in args.shape.split(","))
    f = api.gen_perlin((nz, ny, nx), args.seed, args.octaves, args.base, args.persistence, 2.0,
                       dtype=dtype, device=device)
    fh = api.standin(f, args.eb, args.comp, args.seed)
    torch.cuda.synchronize()
    return f, fh


def workload_config(args, extra=None):
    nx, ny, nz = (int(v) for v in args.shape.split(","))
    cfg = {"workload": f"plain single-field correction, {nx}x{ny}x{nz} {args.dtype} Perlin fBm "
                       f"(seed {args.seed}, {args.octaves} octaves, base 1/{round(1 / args.base)}, "
                       f"persistence {args.persistence}), {args.comp} stand-in, eps={args.eb:g}",
           "shape": [nx, ny, nz], "dtype": args.dtype, "compressor": f"{args.comp} stand-in (compressor parity unpinned)",
           "eb": args.eb, "q": 5, "l2": f"inputs {nx * ny * nz * (8 if args.dtype == 'f64' else 4) * 2 / 1e9:.2f} GB > 129 MB L2",
           "parallelism": "replicas"}
    if extra:
        cfg.update(extra)
    return cfg


def run_reference(args):
    """The reference's path on the host cores: the reference is CUDA-only, so
    its CPU implementation is the oracle's restatement of c_loops (kind
    "port"), on the whole field the GPU arm corrects, with every host thread.
    Inputs come from the oracle's host generator: nothing here loads the
    CUDA library or initialises a GPU."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    fall, fhall = host_fields(args)
    nz = fall.shape[0]
    nsl = args.cpu_slices or nz
    whole = nsl == nz
    times, n, thr, sweeps = [], 0, 0, 0
    for i in range(args.warmup + args.steps):
        n, dt, thr, sweeps, _ = cpu_sample(fall, fhall, args.eb, nsl)
        if i >= args.warmup:
            times.append(dt)
    v = n / statistics.mean(times) / 1e9
    sample = (f"the whole field ({n} voxels)" if whole else f"first {nsl} z-slices ({n} voxels) of the field") + \
        f", CPU oracle restatement, {sweeps} sweeps"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Gvox/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(times) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
        "data": "synthetic", "config": workload_config(args, {"sample": sample, "same_config": whole}),
        "cpu_baseline": {"value": v, "unit": "Gvox/s", "cores": thr, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "Gvox/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
        "note": "the reference's path is CUDA-only; its CPU arm is the oracle restatement of c_loops "
                "(pMSz.cu:1872-2074), inputs from the oracle's host generator",
    }), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as dist
    from pmsz_anonymous_gb300 import _build, api
    _build.build()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=device)
    dtype = torch.float64 if args.dtype == "f64" else torch.float32
    itemsize = 8 if args.dtype == "f64" else 4
    f, fh0 = gen_fields(args, torch, device, dtype)
    n = f.numel()
    fh = torch.empty_like(fh0)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    first_ms, times, sweeps, launches, last = [], [], [], 0, None
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # tile depth and pointer-jumping rounds per launch for this shape class,
    # measured on the inputs themselves (untimed; the timed calls read the table)
    tune = api.autotune(f, fh0) if not args.no_tune else None
    for _ in range(args.warmup):
        fh.copy_(fh0)
        api.correct(f, fh, args.eb, host_loop=args.host_loop)
    barrier()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            fh.copy_(fh0)
            start.record()
            r = api.correct(f, fh, args.eb, timing=True, host_loop=args.host_loop)
            stop.record()
            stop.synchronize()
            times.append(start.elapsed_time(stop))
            first_ms.append(r.ms_first_pass)
            sweeps.append(r.sweeps)
            launches += r.launches
            last = r
            if r.status != 0:
                raise RuntimeError(f"correction did not converge (status {r.status})")
        barrier()
        wall = time.perf_counter() - wall0
    ms = max_over_ranks(statistics.mean(times), device)
    value = whole_job_rate(n, world, ms)

    # e2e through the host-buffer C ABI (pmsz_correct_host_*): pinned host f and
    # fhat copied in, correction, edit extraction, and the reference main's
    # host output -- the delta symbols and the clamp list -- copied back.
    e2e_times, n_clamp, e2e_res = [], 0, None
    if args.e2e_steps > 0:
        f_h = f.cpu().pin_memory()
        fh_h = fh0.cpu().pin_memory()
        deltas_h = torch.empty(api.packed_len(n), dtype=torch.uint8).pin_memory()
        clamp_h = torch.empty(n, dtype=f.dtype).pin_memory()
    for i in range(1 + args.e2e_steps if args.e2e_steps > 0 else 0):
        barrier()
        start.record()
        e2e_res, extra = api.correct_host(f_h, fh_h, args.eb, deltas=deltas_h, clamp=clamp_h, edits_only=True,
                                          packed_deltas=True)
        stop.record()
        stop.synchronize()
        n_clamp = extra["n_clamp"]
        if i:
            e2e_times.append(start.elapsed_time(stop))
    e2e_ms = max_over_ranks(statistics.mean(e2e_times) if e2e_times else float("nan"), device)
    if e2e_res is not None and (e2e_res.sweeps != last.sweeps or e2e_res.edits != last.edits):
        raise RuntimeError("host-buffer call disagrees with the device-buffer call")
    ok = api.verify(f, fh, args.eb)

    peak, peak_kind = measured_peaks()
    bytes_first = 2 * n * (itemsize + 1)
    achieved = bytes_first / (statistics.mean(first_ms) * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": "Gvox/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.dtype, "data": "synthetic",
        "config": workload_config(args, {"sweeps": int(statistics.median(sweeps)),
                                         "timing": "CUDA events around each pmsz_correct call; fhat refreshed "
                                                   "from a device copy before each step (untimed)",
                                         "wall_s_timed_region": wall,
                                         "ms_first_pass": statistics.mean(first_ms),
                                         "autotune": tune,
                                         "ms_detect_sparse": last.ms_detect, "ms_apply": last.ms_apply,
                                         "active_per_sweep": [int(v) for v in last.log[:, 6]],
                                         "requested_per_sweep": [int(v) for v in last.log[:, 3]]}),
        "e2e": {"value": whole_job_rate(n, world, e2e_ms), "unit": "Gvox/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": 2 * n * itemsize, "d2h_bytes_per_step": api.packed_len(n) + n_clamp * itemsize,
                "path": "pmsz_correct_host with PMSZ_FLAG_EDITS_ONLY | PMSZ_FLAG_PACKED_DELTAS: H2D f and fhat, "
                        "correction, edit extraction, D2H delta symbols packed at 3 bits (the reference's "
                        "pack_nbits) and the clamp list"},
        "roofline": {"bound": "hbm", "kernel": "k_first_tma + k_first_exact (labelling + first detection)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": f"{peak_kind} hbm_gbs", "algorithmic_bytes_per_launch": bytes_first,
                     "ms_per_launch": statistics.mean(first_ms),
                     "traffic": profiled_traffic(f"first_pass_{args.shape.replace(',', 'x')}_{args.dtype}")},
        "gpu_launches": launches,
        "verify": ok,
    }
    # active-set algorithmic bytes of the whole step (one-time labelling, each
    # sweep's examined voxels, each edit), and the same with every sweep
    # counted as a full sweep (what the reference's schedule would move)
    act = [int(v) for v in last.log[:, 6]]
    req = [int(v) for v in last.log[:, 3]]
    step_bytes = n * (itemsize + 1) + sum(act) * (itemsize + 1) + sum(req) * (3 * itemsize + 2)
    full_bytes = n * (itemsize + 1) + len(act) * n * (itemsize + 1) + sum(req) * (3 * itemsize + 2)
    out["roofline"]["per_step"] = {
        "algorithmic_bytes": step_bytes, "achieved": step_bytes / (ms * 1e-3) / 1e9,
        "frac": step_bytes / (ms * 1e-3) / 1e9 / peak,
        "what": "N*(s+1) labelling + sum over sweeps of examined voxels*(s+1) + edits*(3s+2), s = sizeof(T), "
                "over ms_per_step"}
    out["roofline"]["full_sweep_equivalent"] = {
        "algorithmic_bytes": full_bytes, "achieved": full_bytes / (ms * 1e-3) / 1e9,
        "what": "every sweep counted as a full sweep of N*(s+1) bytes (the reference's schedule); credits "
                "skipped work, not a roofline fraction"}
    if rank == 0 and not args.no_cpu:
        nsl = args.cpu_slices or f.shape[0]
        fs = f[:nsl].cpu().numpy()
        fhs = fh0[:nsl].cpu().numpy()
        cn, cdt, thr, csw, (cfield, cst, crecs) = cpu_sample(fs, fhs, args.eb, nsl)
        out["cpu_baseline"] = {"value": cn / cdt / 1e9, "unit": "Gvox/s", "cores": thr, "kind": "port",
                               "sample": (f"the whole field ({cn} voxels)" if nsl == f.shape[0] else
                                          f"first {nsl} z-slices ({cn} voxels) of the same field") + ", "
                                         f"CPU oracle, {cdt:.2f} s"}
        # parity: the oracle's corrected field against the GPU's, bit for bit
        if nsl == f.shape[0]:
            gfield, gres = fh, last
        else:
            gfield = fh0[:nsl].clone()
            gres = api.correct(f[:nsl].contiguous(), gfield, args.eb)
        gnp = gfield.cpu().numpy()
        bits = np.uint64 if itemsize == 8 else np.uint32
        out["parity"] = {
            "checked_against": "CPU oracle (restatement of c_loops, pinned to the reference's kernels)",
            "voxels": int(cn),
            "bit_exact": bool(np.array_equal(gnp.view(np.uint8), cfield.view(np.uint8))),
            "voxels_differing": int(np.count_nonzero(gnp.view(bits) != cfield.view(bits))),
            "sweeps_equal": bool(gres.sweeps == csw), "status_equal": bool(gres.status == cst),
            "records_equal": bool(np.array_equal(gres.log[:, :5], crecs)),
            "sweeps": int(csw)}
        del gnp, cfield
        if args.cpu_single_slices > 0:  # the same oracle on one thread, on a slab of the field
            from oracle import oracle as O
            n1 = min(args.cpu_single_slices, f.shape[0])
            O.set_threads(1)
            try:
                sn, sdt, _, ssw, _ = cpu_sample(f[:n1].cpu().numpy(), fh0[:n1].cpu().numpy(), args.eb, n1)
            finally:
                O.set_threads(thr)
            out["cpu_baseline"]["single_thread"] = {
                "value": sn / sdt / 1e9, "unit": "Gvox/s", "cores": 1,
                "sample": f"first {n1} z-slices ({sn} voxels) of the same field, {ssw} sweeps, CPU oracle, {sdt:.2f} s"}
    out["clocks"] = clk.summary()
    if rank == 0 and not args.no_extra:
        # the rest of the metric: batched vox/s, served p50/p99, and the
        # reference's own CUDA kernels on this GPU (untimed legs after the
        # timed region; none of them changes `value`)
        del fh, fh0
        torch.cuda.empty_cache()
        out["batch"] = batch_measure(args, steps=5, warmup=3)
        out["serve"] = serve_measure(args, rates=[100.0, 1000.0, 3000.0])
        out["reference_kernels"] = reference_kernels_measure(args)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


def batch_specs(count: int, base_seed: int = 100):
    """64 fp32 Perlin fields, seeds 100..163: each axis uniform in 32..256, eps
    log-uniform in [1e-5, 1e-2] of the [0,1] range, first half sz3, second
    half zfp stand-ins."""
    specs = []
    for k in range(count):
        rs = np.random.RandomState(base_seed + k)
        shape = tuple(int(v) for v in rs.randint(32, 257, size=3))
        eb = float(10 ** rs.uniform(-5, -2))
        comp = "sz3" if k < count // 2 else "zfp"
        specs.append((base_seed + k, shape, eb, comp))
    return specs


def batch_measure(args, steps: int, warmup: int) -> dict:
    """Batched form: all fields in one pmsz_correct_batch call vs the same
    fields corrected one by one with pmsz_correct_f32; the batch's fields are
    checked bit for bit against the one-by-one fields."""
    import torch
    from pmsz_anonymous_gb300 import _build, api
    _build.build()
    dev = torch.device("cuda", 0)
    specs = batch_specs(args.batch_fields)
    fields = []
    for seed, shape, eb, comp in specs:
        f = api.gen_perlin(shape, seed, 4, 1 / 32, dtype=torch.float32, device=dev)
        fields.append((f, api.standin(f, eb, comp, seed), eb))
    torch.cuda.synchronize()
    nvox = sum(f.numel() for f, _, _ in fields)
    work = [fh.clone() for _, fh, _ in fields]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def refresh():
        for w, (_, fh, _) in zip(work, fields):
            w.copy_(fh)

    # tune every shape class of the batch on its first field (untimed); both
    # forms below then read the same table
    tune_summary = None
    if not args.no_tune:
        api.correct_batch([(f, fh.clone(), eb) for f, fh, eb in fields], autotune=True)
        chosen = [api.tune_get(f.shape, f.dtype)[1] for f, _, _ in fields]
        classes = {tuple((int(v) - 1).bit_length() for v in f.shape) for f, _, _ in fields}
        tune_summary = {"batch_zchunk": api.tune_batch_get(nvox, len(fields), torch.float32)[1],
                        "shape_classes": len(classes),
                        "one_by_one_fields_per_zchunk": dict(collections.Counter(c["zchunk"] for c in chosen)),
                        "fields_per_jump_rounds": dict(collections.Counter(c["jump_rounds"] for c in chosen))}

    def one_by_one():
        for w, (f, _, eb) in zip(work, fields):
            api.correct(f, w, eb)

    def batched():
        api.correct_batch([(f, w, eb) for w, (f, _, eb) in zip(work, fields)])

    times = {}
    for name, fn in (("plain", one_by_one), ("batch", batched)):
        for _ in range(warmup):
            refresh()
            fn()
        ts = []
        for _ in range(steps):
            refresh()
            torch.cuda.synchronize()
            start.record()
            fn()
            stop.record()
            stop.synchronize()
            ts.append(start.elapsed_time(stop))
        times[name] = statistics.mean(ts)
    refresh()
    alone = [api.correct(f, w, eb) for w, (f, _, eb) in zip(work, fields)]
    alone_fields = [w.clone() for w in work]
    refresh()
    res = api.correct_batch([(f, w, eb) for w, (f, _, eb) in zip(work, fields)])
    same = all(torch.equal(a.view(torch.int32), w.view(torch.int32)) for a, w in zip(alone_fields, work))
    same_sweeps = all(a.sweeps == r.sweeps and a.status == r.status for a, r in zip(alone, res))
    del alone_fields
    return {
        "metric": "batched vox/s (64 mixed fp32 fields, one pmsz_correct_batch call)",
        "value": nvox / (times["batch"] * 1e-3) / 1e9, "unit": "Gvox/s", "n_gpus": 1, "steps": steps,
        "warmup": warmup, "ms_per_step": times["batch"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{len(specs)} fp32 Perlin fBm fields (seeds {specs[0][0]}-{specs[-1][0]}, 4 octaves, "
                               "base 1/32), axes uniform 32-256, eps log-uniform [1e-5,1e-2], half sz3 / half zfp "
                               "stand-ins", "voxels": nvox, "fields": len(specs)},
        "plain_one_by_one": {"value": nvox / (times["plain"] * 1e-3) / 1e9, "unit": "Gvox/s",
                             "ms_per_step": times["plain"]},
        "batch_over_plain": times["plain"] / times["batch"],
        "statuses": sorted(set(r.status for r in res)),
        "sweeps_max": max(r.sweeps for r in res),
        "bit_exact_with_one_by_one": bool(same), "sweeps_equal_one_by_one": bool(same_sweeps),
        "autotune": tune_summary,
    }


def run_batch(args):
    print(json.dumps(batch_measure(args, args.steps, args.warmup)), flush=True)


def run_reconstruct(args):
    """Decoder form: the corrected field rebuilt from the decompressed field,
    the delta symbols and the clamp list (pmsz_reconstruct_*), on the plain
    workload's field; correction and extraction are untimed setup."""
    import torch
    from pmsz_anonymous_gb300 import _build, api
    _build.build()
    dev = torch.device("cuda", 0)
    dtype = torch.float64 if args.dtype == "f64" else torch.float32
    f, prev = gen_fields(args, torch, dev, dtype)
    cur = prev.clone()
    api.correct(f, cur, args.eb)
    deltas, clamp, _ = api.extract_edits(prev, cur, f, args.eb)
    out = torch.empty_like(prev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # 256 MB > L2 between steps
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(args.warmup):
        api.reconstruct(prev, deltas, clamp, args.eb, out=out)
    ts = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        start.record()
        api.reconstruct(prev, deltas, clamp, args.eb, out=out)
        stop.record()
        stop.synchronize()
        ts.append(start.elapsed_time(stop))
    ok = torch.equal(out.view(torch.uint8), cur.view(torch.uint8))
    n = prev.numel()
    ms = statistics.mean(ts)
    item = prev.element_size()
    peak, kind = measured_peaks()
    algo = n * (2 * item + 1) + clamp.numel() * item
    wl = workload_config(args)["workload"].replace("plain single-field correction", "reconstruction from the edit output")
    print(json.dumps({
        "metric": "Gvox/s reconstruction (decompressed field + delta symbols + clamp list -> corrected field)",
        "value": n / (ms * 1e-3) / 1e9, "unit": "Gvox/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
        "data": "synthetic",
        "config": {"workload": wl, "voxels": n, "clamps": clamp.numel(), "l2": "256 MB written between steps",
                   "bit_exact_with_the_correction": ok},
        "roofline": {"bound": "hbm", "kernel": "pmsz_reconstruct call (flags, tile scan, host count check, k_recon_apply)",
                     "achieved": algo / (ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": algo / (ms * 1e-3) / 1e9 / peak, "peak_kind": f"{kind} hbm_gbs",
                     "algorithmic_bytes_per_launch": algo},
        "gpu_launches": 3 * args.steps,
    }), flush=True)
    if not ok:
        raise SystemExit("reconstruction differs from the corrected field")


def run_hostlink(args):
    """Host link rates for the plain workload's inputs: the H2D copy of f and
    fhat (2 * N * sizeof(T) bytes, pinned and pageable host memory, one
    stream and two) and the D2H copy of the packed delta symbols, each timed
    with CUDA events over a 1 GiB buffer; reports the e2e floor the inputs'
    copy sets."""
    import torch
    dev = torch.device("cuda", 0)
    nx, ny, nz = (int(v) for v in args.shape.split(","))
    item = 8 if args.dtype == "f64" else 4
    nbytes = 1 << 30
    pinned = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    pageable = torch.empty(nbytes, dtype=torch.uint8)
    pageable.fill_(1)
    pinned.fill_(1)
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def timed(fn, reps=5):
        best = []
        for r in range(reps + 1):
            torch.cuda.synchronize()
            ev[0].record()
            fn()
            ev[1].record()
            ev[1].synchronize()
            if r:
                best.append(ev[0].elapsed_time(ev[1]))
        return nbytes / (statistics.median(best) * 1e-3) / 1e9

    def two_streams(dst, src):
        h = nbytes // 2
        for k, st in enumerate((s1, s2)):
            st.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(st):
                dst[k * h:(k + 1) * h].copy_(src[k * h:(k + 1) * h], non_blocking=True)
        torch.cuda.current_stream().wait_stream(s1)
        torch.cuda.current_stream().wait_stream(s2)

    rates = {
        "h2d_pinned_gbs": timed(lambda: d.copy_(pinned, non_blocking=True)),
        "h2d_pinned_two_streams_gbs": timed(lambda: two_streams(d, pinned)),
        "h2d_pageable_gbs": timed(lambda: d.copy_(pageable), reps=3),
        "d2h_pinned_gbs": timed(lambda: pinned.copy_(d, non_blocking=True)),
        "d2h_pageable_gbs": timed(lambda: pageable.copy_(d), reps=3),
    }
    inputs = 2 * nx * ny * nz * item
    numa = sorted(n for n in os.listdir("/sys/devices/system/node") if n.startswith("node")) \
        if os.path.isdir("/sys/devices/system/node") else []
    print(json.dumps({
        "metric": "host link GB/s (1 GiB copies, CUDA events)", "value": rates["h2d_pinned_gbs"], "unit": "GB/s",
        "n_gpus": 1, "higher_is_better": True, "data": "synthetic", "rates": rates,
        "config": {"workload": f"host link for {nx}x{ny}x{nz} {args.dtype} inputs", "numa_nodes": numa,
                   "host_cores": os.cpu_count()},
        "e2e_floor_ms": inputs / (max(rates["h2d_pinned_gbs"], rates["h2d_pinned_two_streams_gbs"]) * 1e9) * 1e3,
        "input_bytes": inputs,
    }), flush=True)


def serve_specs(count: int, base_seed: int = 1000):
    """Served stream: per-job seed base+id, 3-6 octaves, each axis log-uniform
    in 32..384, 70% fp32 / 30% fp64, eps log-uniform in [1e-5, 1e-2], sz3 /
    zfp stand-ins 50/50."""
    out = []
    for j in range(count):
        rs = np.random.RandomState(base_seed + j)
        shape = tuple(int(round(np.exp(rs.uniform(np.log(32), np.log(384))))) for _ in range(3))
        out.append({"seed": base_seed + j, "shape": shape, "octaves": int(rs.randint(3, 7)),
                    "f64": bool(rs.uniform() < 0.3), "eb": float(10 ** rs.uniform(-5, -2)),
                    "comp": "sz3" if rs.uniform() < 0.5 else "zfp"})
    return out


def serve_measure(args, rates) -> dict:
    """Continuous-batching server under Poisson arrivals at swept rates."""
    import threading
    import torch
    from pmsz_anonymous_gb300 import _build, api
    _build.build()
    dev = torch.device("cuda", 0)
    specs = serve_specs(args.serve_jobs)
    jobs = []
    for sp in specs:
        dt = torch.float64 if sp["f64"] else torch.float32
        f = api.gen_perlin(sp["shape"], sp["seed"], sp["octaves"], 1 / 32, dtype=dt, device=dev)
        jobs.append((f, api.standin(f, sp["eb"], sp["comp"], sp["seed"]), sp["eb"]))
    work = [fh.clone() for _, fh, _ in jobs]
    torch.cuda.synchronize()
    nvox = sum(f.numel() for f, _, _ in jobs)
    rows = []
    rng = np.random.RandomState(7)
    for rate in rates:
        for w, (_, fh, _) in zip(work, jobs):
            w.copy_(fh)
        torch.cuda.synchronize()
        gaps = rng.exponential(1.0 / rate, size=len(jobs))
        infos = [None] * len(jobs)
        with api.Server(hbm_budget_bytes=120 * 10**9) as srv:
            ids = [None] * len(jobs)
            done = threading.Event()

            def waiter():
                for k in range(len(jobs)):
                    while ids[k] is None:
                        time.sleep(0.0002)
                    infos[k] = srv.wait(ids[k])
                done.set()

            th = threading.Thread(target=waiter)
            th.start()
            t0 = time.perf_counter()
            due = t0
            for k, ((f, _, eb), w) in enumerate(zip(jobs, work)):
                due += gaps[k]
                while time.perf_counter() < due:
                    pass
                ids[k] = srv.submit(f, w, eb)
            done.wait()
            wall = time.perf_counter() - t0
            th.join()
        lat = np.array([i["latency_ms"] for i in infos])
        rows.append({"rate_jobs_s": rate, "jobs_s": len(jobs) / wall, "gvox_s": nvox / wall / 1e9,
                     "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                     "queue_p99_ms": float(np.percentile([i["queue_ms"] for i in infos], 99)),
                     "ok": int(sum(i["status"] == 0 for i in infos))})
    best = max(rows, key=lambda r: r["jobs_s"])
    return {
        "metric": "served correction stream: jobs/s and p50/p99 latency", "value": best["jobs_s"], "unit": "jobs/s",
        "n_gpus": 1, "higher_is_better": True, "dtype": "f32/f64", "data": "synthetic",
        "config": {"workload": f"{len(jobs)} jobs, Poisson arrivals, axes log-uniform 32-384, 70% fp32 / 30% fp64, "
                               "3-6 octaves, eps log-uniform [1e-5,1e-2], sz3/zfp stand-ins 50/50, 120 GB budget",
                   "voxels": nvox},
        "rates": rows}


def run_serve(args):
    print(json.dumps(serve_measure(args, [float(r) for r in args.serve_rates.split(",")])), flush=True)


def reference_kernels_measure(args) -> dict:
    """The reference's own CUDA kernels (pMSz.cu compiled unmodified for
    sm_103a) driven through its c_loops host sequence at an MPI grid of
    1x1x1 on this GPU, beside this library on the same field
    (oracle/time_reference.py, a separate process).  fp64 only: the
    reference hard-codes double."""
    if args.dtype != "f64":
        return {"unavailable": "the reference's kernels are fp64 only"}
    cmd = [sys.executable, os.path.join(ROOT, "oracle", "time_reference.py"), "--shape", args.shape,
           "--eb", repr(args.eb), "--comp", args.comp, "--seed", str(args.seed), "--octaves", str(args.octaves),
           "--base", repr(args.base), "--runs", "2"]
    try:
        p = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
    except subprocess.TimeoutExpired:
        return {"unavailable": "time_reference.py did not finish within 900 s"}
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    if p.returncode != 0 or not lines:
        return {"unavailable": f"time_reference.py exited {p.returncode}: {p.stderr.strip()[-300:]}"}
    return json.loads(lines[-1])


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "reconstruct":
        run_reconstruct(args)
    elif args.workload == "hostlink":
        run_hostlink(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
