// helpers.cuh -- device helpers shared by the sweep kernels of correct.cu,
// tiled.cuh and batch.cu: stencil loads, edit requests, per-sweep counters,
// closed-stencil marking of changed vertices, and the edit primitive.
#pragma once
#include "common.cuh"

namespace pmsz {

// ---------------------------------------------------------------------------
// Stencil loads.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void load_keys(const T *__restrict__ v, size_t i, const Geom &g,
                                          uint32_t valid, typename KeyOf<T>::type (&k)[15]) {
    const ptrdiff_t sx = 1, sy = g.nx, sz = static_cast<ptrdiff_t>(g.nx) * g.ny;
#pragma unroll
    for (int r = 0; r < 15; ++r) {
        const ptrdiff_t off = rank_dx(r) * sx + rank_dy(r) * sy + rank_dz(r) * sz;
        k[r] = ((valid >> r) & 1u) ? okey(__ldg(v + (static_cast<ptrdiff_t>(i) + off)))
                                   : typename KeyOf<T>::type(0);
    }
}

__device__ __forceinline__ void request_targets(uint32_t *__restrict__ req, const Geom &g, int x, int y,
                                                int z, uint32_t tm) {
    while (tm) {
        const int r = __ffs(tm) - 1;
        tm &= tm - 1;
        const int tx = x + rank_dx(r), ty = y + rank_dy(r), tz = z + rank_dz(r);
        atomicOr(req + word_of(g, tx, ty, tz), 1u << (tx & 31));
    }
}

__device__ __forceinline__ void flush_counts(SweepSlot *slot, uint32_t cmax, uint32_t cmin,
                                             uint32_t cdir, uint32_t active, uint32_t bad) {
    cmax = warp_sum_u32(cmax);
    cmin = warp_sum_u32(cmin);
    cdir = warp_sum_u32(cdir);
    active = warp_sum_u32(active);
    bad = warp_sum_u32(bad);
    if ((threadIdx.x & 31) == 0) {
        if (cmax) atomicAdd(&slot->fmax, (unsigned long long)cmax);
        if (cmin) atomicAdd(&slot->fmin, (unsigned long long)cmin);
        if (cdir) atomicAdd(&slot->fdir, (unsigned long long)cdir);
        if (active) atomicAdd(&slot->active, (unsigned long long)active);
        if (bad) atomicAdd(&slot->bad, (unsigned long long)bad);
    }
}

// Adds per-thread counters to the 8 fields of a sweep slot (fmax, fmin, fdir,
// requested, changed, progressed, active, bad) with one atomic per non-zero
// field per BLOCK: thousands of warps adding to the same few addresses
// serialise at L2.  Every thread of the block must call it.
__device__ __forceinline__ void block_flush_slot(SweepSlot *slot, const uint32_t (&v)[8]) {
    __shared__ uint32_t s_red[8][32];
    const int nwarps = (blockDim.x * blockDim.y + 31) >> 5;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int w = tid >> 5;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint32_t sum = warp_sum_u32(v[c]);
        if ((tid & 31) == 0) s_red[c][w] = sum;
    }
    __syncthreads();
    if (tid < 8) {
        unsigned long long total = 0;
        for (int k = 0; k < nwarps; ++k) total += s_red[tid][k];
        if (total) atomicAdd(reinterpret_cast<unsigned long long *>(slot) + tid, total);
    }
}

__device__ __forceinline__ void or_word(uint32_t *act, const Geom &g, int wx, int y, int z, uint32_t m) {
    if (!m || wx < 0 || wx >= g.wpr || y < 0 || y >= g.ny || z < 0 || z >= g.nz) return;
    m &= row_tail_mask(g, wx);
    if (m) atomicOr(act + static_cast<size_t>(wx) + static_cast<size_t>(g.wpr) * (static_cast<size_t>(y) + static_cast<size_t>(g.ny) * z), m);
}

// Closed-stencil dilation of the changed bits c of word (wx, y, z).  Rows
// (dy,dz) = (0,0) take x-1..x+1; (1,0),(0,1),(1,1) take x-1,x; (-1,0),(0,-1),
// (-1,-1) take x,x+1 -- the 15 offsets of the stencil.
__device__ __forceinline__ void mark_stencil(uint32_t *act, const Geom &g, int wx, int y, int z, uint32_t c) {
    const uint32_t lo = (c & 1u) << 31;  // x-1 of bit 0 lands in word wx-1
    const uint32_t hi = c >> 31;         // x+1 of bit 31 lands in word wx+1
    or_word(act, g, wx, y, z, c | (c << 1) | (c >> 1));
    or_word(act, g, wx - 1, y, z, lo);
    or_word(act, g, wx + 1, y, z, hi);
    const uint32_t m = c | (c >> 1), p = c | (c << 1);
    or_word(act, g, wx, y + 1, z, m);     or_word(act, g, wx - 1, y + 1, z, lo);
    or_word(act, g, wx, y, z + 1, m);     or_word(act, g, wx - 1, y, z + 1, lo);
    or_word(act, g, wx, y + 1, z + 1, m); or_word(act, g, wx - 1, y + 1, z + 1, lo);
    or_word(act, g, wx, y - 1, z, p);     or_word(act, g, wx + 1, y - 1, z, hi);
    or_word(act, g, wx, y, z - 1, p);     or_word(act, g, wx + 1, y, z - 1, hi);
    or_word(act, g, wx, y - 1, z - 1, p); or_word(act, g, wx + 1, y - 1, z - 1, hi);
}

__device__ __forceinline__ uint64_t bits_of(double v) { return static_cast<uint64_t>(__double_as_longlong(v)); }
__device__ __forceinline__ uint64_t bits_of(float v) { return __float_as_uint(v); }

template <typename T>
__device__ __forceinline__ uint32_t apply_one(const T *__restrict__ f, T *__restrict__ fh, uint8_t *__restrict__ cnt,
                                              size_t v, T eps, T delta, int q, bool &progressed) {
    const T old = fh[v];
    const uint8_t oc = cnt[v];
    const T lowered = old - delta;
    const T fv = f[v];
    T nv;
    uint8_t nc;
    if (fabs(fv - lowered) <= eps && static_cast<int>(oc) < q - 1) {
        nv = lowered;
        nc = static_cast<uint8_t>(oc + 1);
    } else {
        nc = static_cast<uint8_t>(q);
        nv = fv - eps;
    }
    fh[v] = nv;
    cnt[v] = nc;
    const bool vchg = bits_of(old) != bits_of(nv);
    progressed = vchg || nc != oc;
    return vchg ? 1u : 0u;
}

}  // namespace pmsz
