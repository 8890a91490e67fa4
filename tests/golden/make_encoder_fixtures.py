"""Golden vectors of the reference's own edit-file encoder (run in a
container that has the reference's sources; writes encoder_cases.npz).

Each case feeds oracle/_ref/ref_encoder -- the unmodified pMSz.cu built host
side around its compress_symbols_0_N (pMSz.cu:2359-2369: pack_nbits at
bits_for_max(q) bits, zstd level 5; the _deltas.bin payload) and
compress_zstd<T> (pMSz.cu:2261-2277: zstd level 3 of the raw values; the
_edits.bin payload) -- and stores its input and output bytes:

* the delta symbols and clamp lists that the reference's own
  extract_edits_kernel produced in extract_perlin_sz3.npz /
  extract_perlin_zfp.npz (the clamp list = the dense clamp array's non-zero
  entries in voxel order, compact_edits_dense_to_sparse's copy_if);
* a 32^3 fp64 Perlin field corrected by the oracle, then extracted by it;
* synthetic symbol streams for q = 1, 3, 5, 7, 8, 15, 200 and lengths that
  leave 0..7 bits in the last byte, an empty stream, and fp32 / fp64 clamp
  lists (empty included).

    python tests/golden/make_encoder_fixtures.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref, oracle as O  # noqa: E402
from pmsz_anonymous_gb300 import fields as F  # noqa: E402


def run(enc, mode, data: bytes, k: int) -> tuple[bytes, int]:
    with tempfile.TemporaryDirectory() as d:
        src, out = os.path.join(d, "in"), os.path.join(d, "out")
        with open(src, "wb") as fh:
            fh.write(data)
        p = subprocess.run([enc, mode, src, str(k), out], check=True, capture_output=True, text=True)
        with open(out, "rb") as fh:
            return fh.read(), int(p.stdout.split()[-1])


def main():
    enc = build_ref.build_encoder()
    if not enc:
        raise SystemExit("the reference's sources are not available: nothing to generate")
    delta_cases, clamp_cases = [], []
    for name in ("sz3", "zfp"):
        g = np.load(os.path.join(HERE, f"extract_perlin_{name}.npz"))
        delta_cases.append((f"reference_extract_{name}", g["deltas"], 5))
        dense = g["editsout"]
        clamp_cases.append((f"reference_extract_{name}", dense[dense != 0]))
    f = F.perlin_field((32, 32, 32), 5, 4, 1 / 16, dtype=np.float64)
    fh = F.standin(f, 1e-3, "zfp", 5)
    cur, _, _, _, _ = O.correct(f, fh, 1e-3)
    d, c, _ = O.extract_edits(fh, cur, f, 1e-3)
    delta_cases.append(("oracle_32cubed_f64", d, 5))
    clamp_cases.append(("oracle_32cubed_f64", c))
    rng = np.random.default_rng(2024)
    for q in (1, 3, 5, 7, 8, 15, 200):
        for n in (1, 7, 8, 9, 1000, 10007):
            delta_cases.append((f"q{q}_n{n}", rng.integers(0, q + 1, n).astype(np.uint8), q))
    delta_cases.append(("empty", np.zeros(0, np.uint8), 5))
    clamp_cases.append(("random_f32", rng.uniform(-1, 1, 4099).astype(np.float32)))
    clamp_cases.append(("random_f64", rng.uniform(0, 1, 777).astype(np.float64)))
    clamp_cases.append(("empty_f64", np.zeros(0, np.float64)))
    out, version = {}, 0
    for i, (name, sym, q) in enumerate(delta_cases):
        blob, version = run(enc, "deltas", sym.tobytes(), q)
        out[f"d{i}_name"] = np.array(name)
        out[f"d{i}_in"] = sym
        out[f"d{i}_q"] = np.array(q)
        out[f"d{i}_out"] = np.frombuffer(blob, np.uint8)
    for i, (name, vals) in enumerate(clamp_cases):
        blob, version = run(enc, "clamps", vals.tobytes(), vals.itemsize)
        out[f"c{i}_name"] = np.array(name)
        out[f"c{i}_in"] = vals
        out[f"c{i}_out"] = np.frombuffer(blob, np.uint8)
    out["zstd_version"] = np.array(version)
    out["n_delta"] = np.array(len(delta_cases))
    out["n_clamp"] = np.array(len(clamp_cases))
    np.savez_compressed(os.path.join(HERE, "encoder_cases.npz"), **out)
    print(f"{len(delta_cases)} delta cases, {len(clamp_cases)} clamp cases, zstd {version}")


if __name__ == "__main__":
    main()
