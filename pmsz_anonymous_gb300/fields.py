"""Synthetic inputs: seeded Perlin fBm fields and labelled compressor stand-ins.

Noise.  Improved Perlin noise as the reference generator writes it
(generate_perlin.py:17-59: quintic fade 6t^5-15t^4+10t^3, the 16-case
gradient hash, and a permutation made by ``np.random.seed(seed)`` +
``shuffle(arange(256))``, duplicated; generate_perlin.py:105-108).  The
reference emits a single octave at ``scale=64``; the workloads here are fBm:

    v(x,y,z) = sum_{o<octaves} amp_o * perlin(x*fr_o, y*fr_o, z*fr_o)
    amp_o = persistence**o,  fr_o = base_freq * lacunarity**o

then min-max normalised to [0, 1] in double and cast to the field type.
Every operation is an IEEE double operation with no fused multiply-add, so the
CUDA generator (csrc, ``pmsz_gen_perlin``) produces the same bits; the
amplitudes and frequencies are computed here, once, and handed to it.

Fields are C-ordered numpy arrays of shape (nz, ny, nx): x fastest, the raw
layout the reference reads (pMSz.cu:274-313).  The global field is written
row-major; the reference generator's 256^3 sub-block file order
(generate_perlin.py:120-129) is deliberately not reproduced.

Compressor stand-ins.  SZ3 and ZFP are not available, so decompressed inputs
come from two project-written stand-ins, labelled as such wherever used
(compressor parity is unpinned):

* ``sz_standin``  -- SZ-like plateaus: fhat = (2 eps) * round(f / (2 eps)).
* ``zfp_standin`` -- ZFP-like dense error: fhat = f + eps * u, u uniform in
  [-1, 1) from a counter-based hash of (seed, voxel index).

Both then replace any voxel with |f - fhat| > eps (evaluated in the field
type) by f itself, so the bound holds exactly in T.
"""
from __future__ import annotations

import numpy as np

MASK64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def permutation(seed: int) -> np.ndarray:
    """512-entry permutation table (generate_perlin.py:105-108)."""
    perm = np.arange(256, dtype=np.int32)
    rs = np.random.RandomState(seed)
    rs.shuffle(perm)
    return np.concatenate([perm, perm]).astype(np.int32)


def octave_table(octaves: int, base_freq: float, persistence: float,
                 lacunarity: float = 2.0):
    """(amplitudes, frequencies) as float64 arrays, computed once on the host."""
    amps = np.array([persistence ** o for o in range(octaves)], dtype=np.float64)
    freqs = np.array([base_freq * lacunarity ** o for o in range(octaves)], dtype=np.float64)
    return amps, freqs


def _fade(t):
    return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)


def _lerp(a, b, t):
    return a + t * (b - a)


def _grad(h, x, y, z):
    h = h & 15
    u = np.where(h < 8, x, y)
    v = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
    return np.where((h & 1) == 0, u, -u) + np.where((h & 2) == 0, v, -v)


def perlin(x, y, z, p):
    """Vectorised improved Perlin noise (generate_perlin.py:33-59)."""
    fx, fy, fz = np.floor(x), np.floor(y), np.floor(z)
    X = fx.astype(np.int64) & 255
    Y = fy.astype(np.int64) & 255
    Z = fz.astype(np.int64) & 255
    x = x - fx
    y = y - fy
    z = z - fz
    u, v, w = _fade(x), _fade(y), _fade(z)
    A = p[X] + Y
    AA = p[A] + Z
    AB = p[A + 1] + Z
    B = p[X + 1] + Y
    BA = p[B] + Z
    BB = p[B + 1] + Z
    return _lerp(
        _lerp(_lerp(_grad(p[AA], x, y, z), _grad(p[BA], x - 1.0, y, z), u),
              _lerp(_grad(p[AB], x, y - 1.0, z), _grad(p[BB], x - 1.0, y - 1.0, z), u), v),
        _lerp(_lerp(_grad(p[AA + 1], x, y, z - 1.0), _grad(p[BA + 1], x - 1.0, y, z - 1.0), u),
              _lerp(_grad(p[AB + 1], x, y - 1.0, z - 1.0),
                    _grad(p[BB + 1], x - 1.0, y - 1.0, z - 1.0), u), v),
        w)


def fbm_raw(shape, seed: int, octaves: int, base_freq: float,
            persistence: float = 0.5, lacunarity: float = 2.0) -> np.ndarray:
    """Un-normalised fBm in float64, shape (nz, ny, nx)."""
    nz, ny, nx = shape
    p = permutation(seed).astype(np.int64)
    amps, freqs = octave_table(octaves, base_freq, persistence, lacunarity)
    zz, yy, xx = np.meshgrid(np.arange(nz, dtype=np.float64),
                             np.arange(ny, dtype=np.float64),
                             np.arange(nx, dtype=np.float64), indexing="ij")
    total = np.zeros(shape, np.float64)
    for a, fr in zip(amps, freqs):
        total = total + a * perlin(xx * fr, yy * fr, zz * fr, p)
    return total


def normalise(raw: np.ndarray, dtype) -> np.ndarray:
    mn = raw.min()
    mx = raw.max()
    return ((raw - mn) / (mx - mn)).astype(dtype)


def perlin_field(shape, seed: int, octaves: int, base_freq: float,
                 persistence: float = 0.5, lacunarity: float = 2.0,
                 dtype=np.float32) -> np.ndarray:
    """Normalised fBm field in [0, 1] (numpy; use for small and medium sizes)."""
    return normalise(fbm_raw(shape, seed, octaves, base_freq, persistence, lacunarity), dtype)


def _enforce_bound(f: np.ndarray, fh: np.ndarray, eps) -> np.ndarray:
    bad = ~(np.abs(f - fh) <= eps)
    fh[bad] = f[bad]
    return fh


def sz_standin(f: np.ndarray, eb: float) -> np.ndarray:
    """SZ-like quantisation stand-in: plateaus of width 2*eps."""
    step = 2.0 * float(eb)
    fh = (step * np.round(f.astype(np.float64) / step)).astype(f.dtype)
    return _enforce_bound(f, fh, f.dtype.type(eb))


def splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & MASK64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & MASK64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & MASK64
        return z ^ (z >> np.uint64(31))


def zfp_standin(f: np.ndarray, eb: float, seed: int = 0) -> np.ndarray:
    """ZFP-like stand-in: bounded pseudo-random error at every voxel."""
    idx = np.arange(f.size, dtype=np.uint64)
    key = idx ^ (np.uint64(seed & 0xFFFFFFFF) << np.uint64(40))
    h = splitmix64(key)
    u = (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0) * 2.0 - 1.0
    fh = (f.astype(np.float64).ravel() + float(eb) * u).astype(f.dtype).reshape(f.shape)
    return _enforce_bound(f, fh, f.dtype.type(eb))


def standin(f: np.ndarray, eb: float, compressor: str, seed: int = 0) -> np.ndarray:
    """Decompressed copy of f through the stand-in named like the reference's
    compressor argument ("sz3" or "zfp", pMSz.cu:2629)."""
    if compressor == "sz3":
        return sz_standin(f, eb)
    if compressor == "zfp":
        return zfp_standin(f, eb, seed)
    raise ValueError(f"unknown compressor {compressor!r} (expected 'sz3' or 'zfp')")
