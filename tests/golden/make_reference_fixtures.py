"""Generate golden fixtures from the REFERENCE's own kernels.

Runs on a machine with a GPU and the prebuilt ``oracle/_ref/pmsz_ref.cubin``
(compiled from the unmodified pMSz.cu by ``oracle/build_ref.py``).  It drives
the reference kernels through ``oracle/_ref/ref_harness`` (which restates the
host loop of c_loops at an MPI grid of 1x1x1) on small seeded fields and
writes one ``.npz`` per case:

* ``label_*``   or_types of the original field (iscriticle data_type=1) and the
                directions of one detect-only pass on the decompressed field
                (data_type=0, checkFinal=1) -- both deterministic;
* ``correct_*`` the full reference loop on fields where every sweep edits a
                single vertex (so the reference's in-place race cannot change
                the result), plus three runs of the racy loop on a Perlin field;
* ``extract_*`` extract_edits_kernel on (decompressed, oracle-corrected) pairs;
* ``naive_*``   the naive_MSz.cu loop (its own kernels, from
                ``oracle/_ref/naive_ref.cubin``), three runs per field, with the
                per-pass counts.

Usage:  python tests/golden/make_reference_fixtures.py [outdir] [--only naive]
(default outdir ./reference_fixtures; the committed copies live in
tests/golden/).
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build_ref, oracle as O  # noqa: E402
from pmsz_anonymous_gb300 import fields as F  # noqa: E402


def run(harness, cubin, mode, f, fh, eb, tmp, tag, cur=None):
    nz, ny, nx = f.shape
    pf, ph = os.path.join(tmp, f"{tag}_f.bin"), os.path.join(tmp, f"{tag}_fh.bin")
    f.astype(np.float64).tofile(pf)
    fh.astype(np.float64).tofile(ph)
    out = os.path.join(tmp, f"{tag}_{mode}")
    cmd = [harness, cubin, mode, str(nx), str(ny), str(nz), repr(float(eb)), pf, ph, out]
    if cur is not None:
        pc = os.path.join(tmp, f"{tag}_cur.bin")
        cur.astype(np.float64).tofile(pc)
        cmd.append(pc)
    subprocess.run(cmd, check=True, timeout=600)
    W, H, D = nx + 2, ny + 2, nz + 2

    def load(name, dt):
        return np.fromfile(out + name, dtype=dt)

    res = {}
    if mode == "naive":
        res["field"] = load("_field.bin", np.float64).reshape(D, H, W)[1:-1, 1:-1, 1:-1].copy()
        res["ite"] = load("_ite.bin", np.int32)
        res["passes"] = load("_passes.bin", np.int32)
        res["recs"] = load("_recs.bin", np.uint32).reshape(-1, 4)
        return res
    if mode == "extract":
        res["deltas"] = load("_deltas.bin", np.uint8)
        res["editsout"] = load("_editsout.bin", np.float64)
        res["hcount"] = load("_hcount.bin", np.uint32)
        return res
    res["ortypes"] = load("_ortypes.bin", np.int32).reshape(D, H, W, 2)
    res["dir_as"] = load("_dir_as.bin", np.int32).reshape(D, H, W)
    res["dir_ds"] = load("_dir_ds.bin", np.int32).reshape(D, H, W)
    res["counts"] = load("_counts.bin", np.uint32)
    if mode == "correct":
        res["field"] = load("_field.bin", np.float64).reshape(D, H, W)[1:-1, 1:-1, 1:-1].copy()
        res["ite"] = load("_ite.bin", np.int32)
    return res


def naive_fixtures(harness, outdir, tmp):
    if not os.path.exists(build_ref.NAIVE_CUBIN):
        raise SystemExit("oracle/_ref/naive_ref.cubin is missing: build it where the reference sources exist")
    cases = {}
    f = F.perlin_field((20, 20, 20), 6, 4, 1 / 8, dtype=np.float64)
    cases["perlin_zfp"] = (f, F.standin(f, 1e-3, "zfp", 6), 1e-3)
    g = F.perlin_field((14, 16, 18), 7, 4, 1 / 8, dtype=np.float64)
    cases["perlin_sz3"] = (g, F.standin(g, 2e-3, "sz3", 7), 2e-3)
    for name, (f, fh, eb) in cases.items():
        runs = [run(harness, build_ref.NAIVE_CUBIN, "naive", f, fh, eb, tmp, f"naive_{name}{k}") for k in range(3)]
        np.savez_compressed(os.path.join(outdir, f"naive_{name}.npz"), f=f, fh=fh, eb=eb,
                            fields=np.stack([r["field"] for r in runs]),
                            ites=np.concatenate([r["ite"] for r in runs]),
                            passes=runs[0]["passes"], recs=runs[0]["recs"])


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only in args:
        args.remove(only)
    outdir = args[0] if args else os.path.join(os.getcwd(), "reference_fixtures")
    os.makedirs(outdir, exist_ok=True)
    cubin = build_ref.build_cubin()
    if not cubin:
        raise SystemExit("oracle/_ref/pmsz_ref.cubin is missing: build it where the reference sources exist")
    harness = build_ref.build_harness()
    rng = np.random.default_rng(2024)
    tmp = tempfile.mkdtemp()
    if only == "naive":
        naive_fixtures(harness, outdir, tmp)
        print("fixtures written to", outdir)
        return

    label_cases = {}
    f = F.perlin_field((14, 16, 18), 3, 4, 1 / 8, dtype=np.float64)
    label_cases["perlin_zfp"] = (f, F.standin(f, 1e-3, "zfp", 3), 1e-3)
    label_cases["perlin_sz3"] = (f, F.standin(f, 2e-3, "sz3", 3), 2e-3)
    g = (rng.integers(0, 4, size=(11, 7, 9)) / 3.0).astype(np.float64)
    gh = g + rng.uniform(-0.2, 0.2, g.shape)
    label_cases["plateaus"] = (g, np.where(np.abs(g - gh) <= 0.2, gh, g), 0.2)
    line = (np.arange(17, dtype=np.float64) % 5).reshape(1, 1, 17) / 4.0
    label_cases["line"] = (line, line[..., ::-1].copy(), 1.0)
    label_cases["flat2"] = (np.zeros((2, 2, 2)), np.zeros((2, 2, 2)), 0.5)
    pk = np.zeros((3, 3, 3))
    pk[1, 1, 1] = 1.0
    label_cases["peak"] = (pk, -pk, 1.0)
    for name, (f, fh, eb) in label_cases.items():
        lab = run(harness, cubin, "label", f, fh, eb, tmp, name)
        det = run(harness, cubin, "detect", f, fh, eb, tmp, name)
        np.savez_compressed(os.path.join(outdir, f"label_{name}.npz"), f=f, fh=fh, eb=eb,
                            ortypes=lab["ortypes"], dir_as=det["dir_as"], dir_ds=det["dir_ds"],
                            counts=det["counts"])

    # single-target loops: every sweep requests the same single vertex
    single = {
        "pair": (np.array([[[0.0, 1.0]]]), np.array([[[0.9, 0.5]]]), 1.0),
        "line5": (np.arange(5, dtype=np.float64).reshape(1, 1, 5) / 4.0,
                  np.array([[[0.0, 0.25, 0.9, 0.75, 1.0]]]), 0.5),
    }
    for name, (f, fh, eb) in single.items():
        c = run(harness, cubin, "correct", f, fh, eb, tmp, name)
        np.savez_compressed(os.path.join(outdir, f"correct_{name}.npz"), f=f, fh=fh, eb=eb,
                            field=c["field"], ite=c["ite"], ortypes=c["ortypes"])

    # the racy reference loop on a Perlin field, three runs
    f = F.perlin_field((24, 24, 24), 5, 4, 1 / 8, dtype=np.float64)
    fh = F.standin(f, 1e-3, "zfp", 5)
    runs = [run(harness, cubin, "correct", f, fh, 1e-3, tmp, f"racy{k}") for k in range(3)]
    np.savez_compressed(os.path.join(outdir, "correct_perlin_racy.npz"), f=f, fh=fh, eb=1e-3,
                        fields=np.stack([r["field"] for r in runs]),
                        ites=np.concatenate([r["ite"] for r in runs]))

    # extraction on oracle-corrected fields
    for name in ("perlin_zfp", "perlin_sz3"):
        f, fh, eb = label_cases[name]
        cur = O.correct(f, fh, eb)[0]
        e = run(harness, cubin, "extract", f, fh, eb, tmp, name, cur=cur)
        np.savez_compressed(os.path.join(outdir, f"extract_{name}.npz"), f=f, fh=fh, cur=cur, eb=eb,
                            deltas=e["deltas"], editsout=e["editsout"], hcount=e["hcount"])
    naive_fixtures(harness, outdir, tmp)
    print("fixtures written to", outdir)


if __name__ == "__main__":
    main()
