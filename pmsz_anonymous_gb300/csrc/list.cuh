// list.cuh -- voxel-list sweeps for the host-driven part of the correction
// loop, included by correct.cu after tiled.cuh.
//
// The early sweeps of a large field touch millions of voxels each.  Instead
// of compacting and processing a bitmap round by round inside one kernel
// (which keeps the round state and the detection registers live together and
// caps residency at a few blocks per SM), each sweep runs as
//   k_compact       bitmap -> list of flat voxel indices (clears the bitmap);
//                   one atomicAdd per block claims its slice of the list, so
//                   the list order is arbitrary -- every consumer is
//                   order-free (requests and marks are bit ORs, counters sums)
//   k_detect_list   one thread per listed voxel: the 15 proxies, the rules,
//                   the requests, the mismatch bit of the next active set;
//                   failed certificates go to a second list
//   k_detect_exact  the second list on full keys
//   k_compact       request bitmap -> list
//   k_apply_list    one thread per requested voxel: the edit, the proxy
//                   refresh, the closed-stencil marks of the next active set
// The per-voxel kernels are light enough for full residency, so the 15
// gathers of many voxels are in flight at once.  Flat indices are 32-bit:
// the list form is used when the field has fewer than 2^32 voxels.
#pragma once
#include "tiled.cuh"

namespace pmsz {

constexpr int kCompactBlock = 256;
constexpr int kCompactWords = kCompactBlock * 4;  // one uint4 of words per thread per step

// Bitmap -> list.  list[*count ...] receives nx-flat voxel indices.
__global__ void __launch_bounds__(kCompactBlock) k_compact(uint32_t *__restrict__ bm, Geom g,
                                                           uint32_t *__restrict__ list, uint32_t *count) {
    __shared__ uint32_t s_warp[kCompactBlock / 32];
    __shared__ uint32_t s_base;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (size_t base = static_cast<size_t>(blockIdx.x) * kCompactWords; base < g.nwords;
         base += static_cast<size_t>(gridDim.x) * kCompactWords) {
        const size_t w0 = base + static_cast<size_t>(t) * 4;
        uint32_t w[4];
        if (w0 + 4 <= g.nwords) {
            const uint4 v = *reinterpret_cast<const uint4 *>(bm + w0);
            w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
            if (v.x | v.y | v.z | v.w) *reinterpret_cast<uint4 *>(bm + w0) = make_uint4(0, 0, 0, 0);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                w[j] = w0 + j < g.nwords ? bm[w0 + j] : 0u;
                if (w[j]) bm[w0 + j] = 0;
            }
        }
        const uint32_t c = __popc(w[0]) + __popc(w[1]) + __popc(w[2]) + __popc(w[3]);
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) s_warp[warp] = inc;
        __syncthreads();
        if (t == 0) {
            uint32_t run = 0;
            for (int k = 0; k < kCompactBlock / 32; ++k) {
                const uint32_t v = s_warp[k];
                s_warp[k] = run;
                run += v;
            }
            s_base = run ? atomicAdd(count, run) : 0u;
        }
        __syncthreads();
        if (c) {
            uint32_t pos = s_base + s_warp[warp] + inc - c;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (!w[j]) continue;
                const uint32_t wj = static_cast<uint32_t>(w0 + j);
                const uint32_t row = fdiv(wj, g.div_wpr);
                const uint32_t wx = wj - row * static_cast<uint32_t>(g.wpr);
                const uint32_t i0 = row * static_cast<uint32_t>(g.nx) + (wx << 5);
                for (uint32_t bits = w[j]; bits; bits &= bits - 1) list[pos++] = i0 + static_cast<uint32_t>(__ffs(bits) - 1);
            }
        }
        __syncthreads();  // s_warp / s_base are rewritten by the next step
    }
}

// Coordinates of a flat index (n < 2^32).
__device__ __forceinline__ void voxel_coords(const Geom &g, const FastDiv &div_nx, uint32_t i, int &x, int &y, int &z) {
    const uint32_t row = fdiv(i, div_nx);
    x = static_cast<int>(i - row * static_cast<uint32_t>(g.nx));
    const uint32_t zz = fdiv(row, g.div_ny);
    y = static_cast<int>(row - zz * static_cast<uint32_t>(g.ny));
    z = static_cast<int>(zz);
}

// Outcome of one voxel's steepest ranks: the rules, the requests and the
// mismatch bit of the next active set.
__device__ __forceinline__ void detect_outcome(const Geom &g, int x, int y, int z, int asc, int desc, uint8_t c,
                                               uint32_t *__restrict__ req, uint32_t *__restrict__ act_next,
                                               uint32_t &cmax, uint32_t &cmin, uint32_t &cdir) {
    const uint32_t tm = detect_rules(asc, desc, c & 15, c >> 4, cmax, cmin, cdir);
    if (tm) {
        request_targets(req, g, x, y, z, tm);
        atomicOr(act_next + word_of(g, x, y, z), 1u << (x & 31));
    }
}

// Detection of every listed voxel (iscriticle data_type=0) on the proxy
// array.  A voxel whose certificate fails (ties in the truncated proxies) is
// appended to a second list and decided by k_detect_exact on full keys, so
// this loop never runs a one-lane slow path.
constexpr uint32_t kExactCap = 2048;  // failed certificates buffered per block
template <typename T>
__global__ void __launch_bounds__(256, 5) k_detect_list(const uint32_t *__restrict__ list, const uint32_t *count,
                                                     const uint32_t *__restrict__ hp, const uint8_t *__restrict__ codes,
                                                     uint32_t *__restrict__ req, uint32_t *__restrict__ act_next,
                                                     uint32_t *__restrict__ exact_list, uint32_t *exact_count,
                                                     SweepSlot *slot, Geom g, FastDiv div_nx) {
    __shared__ uint32_t s_exact[kExactCap];
    __shared__ uint32_t s_n, s_base;
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    const uint32_t m = *count;
    uint32_t cmax = 0, cmin = 0, cdir = 0, active = 0;
    const ptrdiff_t sy = g.nx, sz = static_cast<ptrdiff_t>(g.nx) * g.ny;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const uint32_t i = __ldg(list + k);
        int x, y, z;
        voxel_coords(g, div_nx, i, x, y, z);
        const bool interior = x >= 1 && x <= g.nx - 2 && y >= 1 && y <= g.ny - 2 && z >= 1 && z <= g.nz - 2;
        const uint32_t valid = interior ? kAllValid : valid_mask(x, y, z, g.nx, g.ny, g.nz);
        const uint32_t *c0 = hp + i;
        uint32_t t[15];
#pragma unroll
        for (int r = 0; r < 15; ++r) {
            const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
            t[r] = ((valid >> r) & 1u) ? __ldg(c0 + off) : 0u;
        }
        const uint8_t c = __ldg(codes + i);
        const Ext ex = interior ? proxy_ext_interior(t) : proxy_ext(t);
        ++active;
        if (ex.exact) {
            detect_outcome(g, x, y, z, ex.asc, ex.desc, c, req, act_next, cmax, cmin, cdir);
        } else {  // buffered in shared memory; a full buffer spills straight to the list
            const uint32_t pos = atomicAdd(&s_n, 1u);
            if (pos < kExactCap) s_exact[pos] = i;
            else exact_list[atomicAdd(exact_count, 1u)] = i;
        }
    }
    flush_counts(slot, cmax, cmin, cdir, active, 0);
    __syncthreads();
    const uint32_t nb = min(s_n, kExactCap);
    if (threadIdx.x == 0) s_base = nb ? atomicAdd(exact_count, nb) : 0u;  // one global atomic per block
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < nb; j += blockDim.x) exact_list[s_base + j] = s_exact[j];
}

// The voxels whose certificate failed: steepest ranks on the 15 exact keys of
// fhat (loaded together), then the same outcome.
template <typename T>
__global__ void __launch_bounds__(256) k_detect_exact(const uint32_t *__restrict__ exact_list, const uint32_t *count,
                                                      const T *__restrict__ fh, const uint8_t *__restrict__ codes,
                                                      uint32_t *__restrict__ req, uint32_t *__restrict__ act_next,
                                                      SweepSlot *slot, Geom g, FastDiv div_nx) {
    const uint32_t m = *count;
    uint32_t cmax = 0, cmin = 0, cdir = 0;
    const ptrdiff_t sy = g.nx, sz = static_cast<ptrdiff_t>(g.nx) * g.ny;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const uint32_t i = __ldg(exact_list + k);
        int x, y, z;
        voxel_coords(g, div_nx, i, x, y, z);
        const uint32_t valid = valid_mask(x, y, z, g.nx, g.ny, g.nz);
        using K = typename KeyOf<T>::type;
        K kk[15];
#pragma unroll
        for (int r = 0; r < 15; ++r) {
            const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
            kk[r] = ((valid >> r) & 1u) ? okey(__ldg(fh + (static_cast<ptrdiff_t>(i) + off))) : K(0);
        }
        int asc, desc;
        arg_ext(kk, valid, asc, desc);
        detect_outcome(g, x, y, z, asc, desc, __ldg(codes + i), req, act_next, cmax, cmin, cdir);
    }
    flush_counts(slot, cmax, cmin, cdir, 0, 0);
}

// The edit of every listed voxel (applyDeltaBuffer_local, pMSz.cu:623-645),
// the proxy refresh, and for a changed value the closed stencil of the voxel
// in the next active set.
template <typename T>
__global__ void __launch_bounds__(256) k_apply_list(const uint32_t *__restrict__ list, const uint32_t *count,
                                                    const T *__restrict__ f, T *__restrict__ fh,
                                                    uint8_t *__restrict__ cnt, uint32_t *__restrict__ hp,
                                                    uint32_t *__restrict__ act_next, SweepSlot *slot, Geom g,
                                                    FastDiv div_nx, T eps, T delta, int q) {
    const uint32_t m = *count;
    uint32_t nreq = 0, nchg = 0, nprog = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const uint32_t v = __ldg(list + k);
        const T old = fh[v];
        const uint8_t oc = cnt[v];
        const T fv = __ldg(f + v);
        const T lowered = old - delta;
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
        const bool chg = bits_of(old) != bits_of(nv);
        ++nreq;
        nprog += (chg || nc != oc) ? 1u : 0u;
        if (chg) {
            ++nchg;
            hp[v] = proxy_of(nv);
            int x, y, z;
            voxel_coords(g, div_nx, v, x, y, z);
            mark_stencil(act_next, g, x >> 5, y, z, 1u << (x & 31));
        }
    }
    flush_apply_counts(slot, nreq, nchg, nprog);
}

inline unsigned compact_grid(const Geom &g) {
    const size_t need = (g.nwords + kCompactWords - 1) / kCompactWords;
    return static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>(need, 152 * 8)));
}

}  // namespace pmsz
