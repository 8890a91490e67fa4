"""Pure-Python restatement of the reference kernel logic on the reference's
own PADDED grid, for tiny fields only (test helper).

Where the C oracle uses unpadded indices and in-domain tests, this helper
keeps the reference's data layout literally: a (W+2)(H+2)(D+2) block whose
shell holds INVALID_VAL = 1e30 (pMSz.cu:215, 346-381), ties broken by the
PADDED flat index (pMSz.cu:610-620), neighbours skipped when out of range or
INVALID (pMSz.cu:709), shell voxels never processed (pMSz.cu:673-679), and
or_types stored as the reference's two ints per voxel (pMSz.cu:749-783).
Agreement between the two restatements checks the claim that the padded and
unpadded forms are the same at an MPI grid of 1x1x1.
"""
from __future__ import annotations

import numpy as np

INVALID = 1e30
# directions_host, pMSz.cu:186-193
DIRS = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (-1, 1, 0), (1, -1, 0),
        (-1, 0, 1), (1, 0, -1), (0, 1, 1), (0, -1, -1), (-1, 1, 1), (1, -1, -1)]


def pad(field: np.ndarray) -> np.ndarray:
    """(nz,ny,nx) -> padded flat array with the INVALID shell."""
    nz, ny, nx = field.shape
    p = np.full((nz + 2, ny + 2, nx + 2), INVALID, dtype=field.dtype)
    p[1:-1, 1:-1, 1:-1] = field
    return p.ravel().copy()


def unpad_index(i: int, W: int, H: int) -> int:
    """Padded flat index -> unpadded flat index (W, H = padded sizes)."""
    x = i % W
    y = (i // W) % H
    z = i // (W * H)
    return (x - 1) + (W - 2) * ((y - 1) + (H - 2) * (z - 1))


def scan(dec, i, W, H, D):
    """is_max, is_min, largest, smallest of padded voxel i (pMSz.cu:686-746)."""
    x, y, z = i % W, (i // W) % H, (i // (W * H)) % D
    v = dec[i]
    is_max = is_min = True
    largest, lv = i, v
    smallest, sv = i, v
    for dx, dy, dz in DIRS:
        nx_, ny_, nz_ = x + dx, y + dy, z + dz
        n = nx_ + (ny_ + nz_ * H) * W
        if nx_ < 0 or nx_ >= W or ny_ < 0 or ny_ >= H or nz_ < 0 or nz_ >= D or n >= len(dec) \
                or dec[n] == INVALID:
            continue
        nv = dec[n]
        if nv > v or (nv == v and n > i):
            is_max = False
        if nv < v or (nv == v and n < i):
            is_min = False
        if nv > lv or (nv == lv and n > largest):
            largest, lv = n, nv
        if nv < sv or (nv == sv and n < smallest):
            smallest, sv = n, nv
    return is_max, is_min, largest, smallest


def interior(i, W, H, D):
    x, y, z = i % W, (i // W) % H, (i // (W * H)) % D
    return not (x == 0 or x >= W - 1 or y == 0 or y >= H - 1 or z == 0 or z >= D - 1)


def or_types(f_pad, W, H, D):
    """iscriticle data_type=1 (pMSz.cu:749-783): two ints per padded voxel."""
    ot = np.zeros(2 * len(f_pad), np.int64)
    for i in range(len(f_pad)):
        if not interior(i, W, H, D) or f_pad[i] == INVALID:
            continue
        mx, mn, lg, sm = scan(f_pad, i, W, H, D)
        if mx:
            ot[2 * i], ot[2 * i + 1] = -1, sm
        elif mn:
            ot[2 * i], ot[2 * i + 1] = -2, lg
        else:
            ot[2 * i], ot[2 * i + 1] = sm, lg
    return ot


def correct(f: np.ndarray, fh: np.ndarray, eb: float, q: int = 5, max_sweeps: int = 1000):
    """Snapshot sweeps on the padded grid.  Returns (corrected unpadded field,
    per-sweep [fmax, fmin, fdir, requested] rows, converged flag)."""
    T = f.dtype.type
    nz, ny, nx = f.shape
    W, H, D = nx + 2, ny + 2, nz + 2
    fp, dp = pad(f), pad(fh)
    eps, delta = T(eb), T(eb / q)
    ot = or_types(fp, W, H, D)
    cnt = np.zeros(len(fp), np.int64)
    log = []
    for _ in range(max_sweeps):
        snap = dp.copy()
        req = set()
        cmax = cmin = cdir = 0
        for i in range(len(dp)):
            if not interior(i, W, H, D) or snap[i] == INVALID:
                continue
            is_max, is_min, lg, sm = scan(snap, i, W, H, D)
            t = ot[2 * i]
            r1 = (is_max and t != -1) or (not is_max and t == -1)
            r2 = (is_min and t != -2) or (not is_min and t == -2)
            if r1:
                cmax += 1
                req.add(i if t != -1 else lg)
            if r2:
                cmin += 1
                if t != -2:  # false minimum: lower the original descent neighbour
                    req.add(ot[2 * i + 1] if t == -1 else ot[2 * i])
                else:        # missing minimum: lower the voxel itself
                    req.add(i)
            if r1 or r2:
                cdir += 1
                continue
            o_lg = i if t == -1 else ot[2 * i + 1]
            if lg != o_lg:
                cdir += 1
                req.add(lg)
            o_sm = ot[2 * i + 1] if t == -1 else (i if t == -2 else ot[2 * i])
            if sm != o_sm:
                cdir += 1
                req.add(o_sm)
        for v in req:  # applyDeltaBuffer_local, pMSz.cu:623-645
            low = T(dp[v] - delta)
            if abs(T(fp[v] - low)) <= eps and cnt[v] < q - 1:
                dp[v] = low
                cnt[v] += 1
            else:
                cnt[v] = q
                dp[v] = T(fp[v] - eps)
        log.append([cmax, cmin, cdir, len(req)])
        if cmax == 0 and cmin == 0 and cdir == 0:
            break
    out = dp.reshape(D, H, W)[1:-1, 1:-1, 1:-1].copy()
    return out, np.array(log, np.uint64), log[-1][:3] == [0, 0, 0]
