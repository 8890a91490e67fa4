// list.cuh -- voxel-list sweeps for the host-driven part of the correction
// loop, included by correct.cu after tiled.cuh.
//
// The early sweeps of a large field touch millions of voxels each.  Instead
// of compacting and processing a bitmap round by round inside one kernel
// (which keeps the round state and the detection registers live together and
// caps residency at a few blocks per SM), each sweep runs as
//   compaction      bitmap -> list of flat voxel indices in voxel order
//                   (clears the bitmap); every consumer is order-free anyway
//                   (requests and marks are bit ORs, counters sums)
//   k_detect_list   one thread per listed voxel: the 15 proxies, the rules,
//                   the requests, the mismatch bit of the next active set;
//                   failed certificates are decided on full keys by the
//                   block after its list loop (a full buffer spills)
//   k_detect_exact  the spilled ones, on full keys
//   compaction      request bitmap -> list
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

// Bitmap -> list in two passes with a deterministic order and no contended
// atomics: k_count_words sums the set bits of each block's contiguous range of
// words; k_write_list derives its block's offset from the counts before it,
// writes the flat indices of its range in order and clears the words.  Block b
// of both kernels covers words [b * per, (b + 1) * per), per a multiple of 4.

// Words per block of a compaction launched with `blocks` blocks.
__host__ __device__ __forceinline__ size_t compact_per(const Geom &g, size_t blocks) {
    return ((g.nwords + blocks - 1) / blocks + 3) & ~static_cast<size_t>(3);
}

__device__ __forceinline__ uint32_t block_sum_u32(uint32_t v, uint32_t *s_warp) {
    const int t = threadIdx.x;
    v = warp_sum_u32(v);
    if ((t & 31) == 0) s_warp[t >> 5] = v;
    __syncthreads();
    uint32_t tot = 0;
    for (int k = 0; k < kCompactBlock / 32; ++k) tot += s_warp[k];
    __syncthreads();
    return tot;
}

// Both compaction kernels read g.nwords words from bm; a z-range of a bitmap
// is passed as bm + wbase (wbase a multiple of 4, for the 16-byte loads) with
// g.nwords the range's length from there, and `skip` (< 4) words at its start
// that belong to the plane before the range: they are neither listed nor
// cleared.  List entries are absolute voxel indices.  The block count is the
// launch's (compact_per).
static __global__ void __launch_bounds__(kCompactBlock) k_count_words(const uint32_t *__restrict__ bm, Geom g,
                                                               uint32_t *__restrict__ counts, const int *run,
                                                               uint32_t skip = 0) {
    __shared__ uint32_t s_warp[kCompactBlock / 32];
    if (run && *run == 0) return;
    const size_t per = compact_per(g, gridDim.x);
    const size_t lo = static_cast<size_t>(blockIdx.x) * per, hi = min(g.nwords, lo + per);
    uint32_t c = 0;
    for (size_t w0 = lo + static_cast<size_t>(threadIdx.x) * 4; w0 < hi; w0 += kCompactWords) {
        if (w0 + 4 <= hi && w0 >= skip) {
            const uint4 v = *reinterpret_cast<const uint4 *>(bm + w0);
            c += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
        } else {
            for (size_t w = w0; w < hi && w < w0 + 4; ++w)
                if (w >= skip) c += __popc(bm[w]);
        }
    }
    c = block_sum_u32(c, s_warp);
    if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

// Writes the entries of one compaction step (the block's kCompactWords
// bitmap words, four per thread in w) to out[0 .. step) in word order; base(j)
// gives the entry of bit 0 of the thread's word j (a word's entries are base
// + bit), lane_ex is the thread's exclusive prefix of bit counts within its
// warp and wbase its warp's offset in the step.  Block-uniform choice:
//  - the step fits the staging buffer: every thread writes its own
//    entries into shared memory at their ranks, then the block copies the
//    step out with coalesced stores;
//  - denser steps: the words and their bases are staged per warp and the
//    warp visits its non-zero words in order, every lane writing the entry of
//    its own bit of the word at the bit's rank, so each word's entries go out
//    as one contiguous store and no thread loops over more than its bit.
// 24 KB: nine compaction blocks fit on an SM, so the 8-per-SM grid runs in one
// wave (32 KB allowed seven: 1.14 waves, 7 % slower at 512^3); a step of the
// first list sweeps (about 5000 entries) still fits.
constexpr uint32_t kStageBytes = 24576;
template <typename E, class Base>
__device__ __forceinline__ void write_step_entries(const uint32_t (&w)[4], uint32_t lane_ex, uint32_t wbase,
                                                   uint32_t step, unsigned char *raw, E *out, Base &&base) {
    constexpr uint32_t kCap = kStageBytes / sizeof(E);
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (step <= kCap) {
        E *st = reinterpret_cast<E *>(raw);
        uint32_t p = wbase + lane_ex;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (!w[j]) continue;
            const E b0 = base(j);
            for (uint32_t bits = w[j]; bits; bits &= bits - 1) st[p++] = b0 + static_cast<E>(__ffs(bits) - 1);
        }
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < step; e += blockDim.x) out[e] = st[e];
        __syncthreads();  // the buffer is reused by the next step
        return;
    }
    uint32_t *sw = reinterpret_cast<uint32_t *>(raw) + warp * 128;
    E *sb = reinterpret_cast<E *>(raw + 4 * kCompactWords) + warp * 128;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        sw[lane * 4 + j] = w[j];
        sb[lane * 4 + j] = w[j] ? base(j) : E(0);
    }
    __syncwarp();
    const uint32_t below = (1u << lane) - 1u;
    E *wo = out + wbase;
    uint32_t run = 0;
#pragma unroll
    for (int gi = 0; gi < 4; ++gi) {
        for (uint32_t nz = __ballot_sync(0xFFFFFFFFu, sw[gi * 32 + lane] != 0u); nz; nz &= nz - 1) {
            const int k = gi * 32 + __ffs(nz) - 1;
            const uint32_t word = sw[k];
            if ((word >> lane) & 1u) wo[run + __popc(word & below)] = sb[k] + static_cast<E>(lane);
            run += __popc(word);
        }
    }
    __syncthreads();  // the buffer is reused by the next step
}

// Four words per thread per step (one 16-byte load), written with
// write_step_entries.
static __global__ void __launch_bounds__(kCompactBlock) k_write_list(uint32_t *__restrict__ bm, Geom g,
                                                              const uint32_t *__restrict__ counts,
                                                              uint32_t *__restrict__ list, uint32_t *total,
                                                              const int *run, uint32_t wbase = 0,
                                                              uint32_t skip = 0) {
    __shared__ uint32_t s_warp[kCompactBlock / 32];
    __shared__ __align__(16) unsigned char s_raw[kStageBytes];
    if (run && *run == 0) return;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t before = 0, all = 0;
    for (int b = t; b < static_cast<int>(gridDim.x); b += kCompactBlock) {
        const uint32_t c = counts[b];
        all += c;
        if (b < static_cast<int>(blockIdx.x)) before += c;
    }
    uint32_t pos = block_sum_u32(before, s_warp);
    all = block_sum_u32(all, s_warp);
    if (blockIdx.x == 0 && t == 0) *total = all;
    const size_t per = compact_per(g, gridDim.x);
    const size_t lo = static_cast<size_t>(blockIdx.x) * per, hi = min(g.nwords, lo + per);
    for (size_t base = lo; base < hi; base += kCompactWords) {
        const size_t w0 = base + static_cast<size_t>(t) * 4;
        uint32_t w[4] = {0u, 0u, 0u, 0u};
        if (w0 + 4 <= hi && w0 >= skip) {
            const uint4 v = *reinterpret_cast<const uint4 *>(bm + w0);
            w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
            if (v.x | v.y | v.z | v.w) *reinterpret_cast<uint4 *>(bm + w0) = make_uint4(0, 0, 0, 0);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (w0 + j < hi && w0 + j >= skip) {
                    w[j] = bm[w0 + j];
                    if (w[j]) bm[w0 + j] = 0;
                }
            }
        }
        const uint32_t c = __popc(w[0]) + __popc(w[1]) + __popc(w[2]) + __popc(w[3]);
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += u;
        }
        if (lane == 31) s_warp[warp] = inc;
        __syncthreads();
        uint32_t wbase_warp = 0, step = 0;
        for (int k = 0; k < kCompactBlock / 32; ++k) {
            const uint32_t u = s_warp[k];
            if (k < warp) wbase_warp += u;
            step += u;
        }
        const uint32_t mine = wbase + static_cast<uint32_t>(w0);  // nwords < 2^27 in the list form
        write_step_entries(w, inc - c, wbase_warp, step, s_raw, list + pos, [&](int j) {
            const uint32_t wj = mine + static_cast<uint32_t>(j);
            const uint32_t row = fdiv(wj, g.div_wpr);
            const uint32_t wx = wj - row * static_cast<uint32_t>(g.wpr);
            return row * static_cast<uint32_t>(g.nx) + (wx << 5);
        });
        pos += step;  // write_step_entries ends with a barrier: s_warp is free
    }
}

// Lanes whose voxels share a bitmap word carry the same key; in a list in
// voxel order they are consecutive lanes.  ORs the changed bits cb over each
// group (a suffix OR within the group) and returns true on the group's lowest
// lane when the merged bits are non-zero: that lane marks the word's closed
// stencil once for the whole group.
template <typename K>
__device__ __forceinline__ bool warp_merge_word(K key, uint32_t &cb) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t grp = __match_any_sync(0xFFFFFFFFu, key);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_down_sync(0xFFFFFFFFu, cb, o);
        if (lane + o < 32 && ((grp >> (lane + o)) & 1u)) cb |= u;
    }
    return cb && lane == static_cast<uint32_t>(__ffs(grp) - 1);
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
// buffered in shared memory and decided on full keys by the whole block after
// its list loop, so the loop never runs a one-lane slow path; a full buffer
// spills to a second list that k_detect_exact decides.  *deferred (or null)
// counts the buffered and spilled voxels.
constexpr uint32_t kExactCap = 2048;  // failed certificates buffered per block
template <typename T>
__global__ void __launch_bounds__(256, 5) k_detect_list(const uint32_t *__restrict__ list, const uint32_t *count,
                                                     const T *__restrict__ fh,
                                                     const uint32_t *__restrict__ hp, const uint8_t *__restrict__ codes,
                                                     uint32_t *__restrict__ req, uint32_t *__restrict__ act_next,
                                                     uint32_t *__restrict__ exact_list, uint32_t *exact_count,
                                                     SweepSlot *slot, Geom g, FastDiv div_nx, const int *run,
                                                     const int *exact_keys, uint32_t *deferred = nullptr) {
    __shared__ uint32_t s_exact[kExactCap];
    __shared__ uint32_t s_n;
    if (run && *run == 0) return;
    // fp32 with exact_keys set (k_pick_detection, k_loop_gate): the 4-byte keys
    // of fhat, gathered as the proxies would be, decide every voxel (no
    // certificates, nothing deferred)
    const bool keys = sizeof(T) == 4 && exact_keys && *exact_keys;
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
        const uint8_t c = __ldg(codes + i);
        ++active;
        if (keys) {
            uint32_t kk[15];
#pragma unroll
            for (int r = 0; r < 15; ++r) {
                const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
                kk[r] = ((valid >> r) & 1u) ? static_cast<uint32_t>(okey(__ldg(fh + (static_cast<ptrdiff_t>(i) + off))))
                                            : 0u;
            }
            int asc, desc;
            arg_ext(kk, valid, asc, desc);
            detect_outcome(g, x, y, z, asc, desc, c, req, act_next, cmax, cmin, cdir);
            continue;
        }
        const uint32_t *c0 = hp + i;
        uint32_t t[15];
#pragma unroll
        for (int r = 0; r < 15; ++r) {
            const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
            t[r] = ((valid >> r) & 1u) ? __ldg(c0 + off) : 0u;
        }
        const Ext ex = interior ? proxy_ext_interior<true>(t) : proxy_ext<true>(t);
        if (ex.exact) {
            detect_outcome(g, x, y, z, ex.asc, ex.desc, c, req, act_next, cmax, cmin, cdir);
        } else {  // buffered in shared memory; a full buffer spills straight to the list
            const uint32_t pos = atomicAdd(&s_n, 1u);
            if (pos < kExactCap) s_exact[pos] = i;
            else spill_append(exact_list, exact_count, i);
        }
    }
    __syncthreads();  // s_n is final
    const uint32_t nd = s_n, nb = min(nd, kExactCap);
    if (deferred && threadIdx.x == 0 && nd) atomicAdd(deferred, nd);
    // the buffered voxels on the 15 exact keys of fhat, one per thread; the
    // keys are scanned one at a time (rank order, arg_ext's rule) so that this
    // rare path adds no registers to the list loop
    for (uint32_t j = threadIdx.x; j < nb; j += blockDim.x) {
        const uint32_t i = s_exact[j];
        int x, y, z;
        voxel_coords(g, div_nx, i, x, y, z);
        const uint32_t valid = valid_mask(x, y, z, g.nx, g.ny, g.nz);
        using K = typename KeyOf<T>::type;
        K bmax = 0, bmin = ~K(0);
        int asc = kSelf, desc = kSelf;
#pragma unroll 1
        for (int r = 0; r < 15; ++r) {
            if (!((valid >> r) & 1u)) continue;
            const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
            const K k = okey(__ldg(fh + (static_cast<ptrdiff_t>(i) + off)));
            if (k >= bmax) { bmax = k; asc = r; }
            if (k < bmin) { bmin = k; desc = r; }
        }
        detect_outcome(g, x, y, z, asc, desc, __ldg(codes + i), req, act_next, cmax, cmin, cdir);
    }
    const uint32_t v[8] = {cmax, cmin, cdir, 0u, 0u, 0u, active, 0u};
    block_flush_slot(slot, v);
}

// The voxels whose certificate failed: steepest ranks on the 15 exact keys of
// fhat (loaded together), then the same outcome.
template <typename T>
__global__ void __launch_bounds__(256) k_detect_exact(const uint32_t *__restrict__ exact_list, const uint32_t *count,
                                                      const T *__restrict__ fh, const uint8_t *__restrict__ codes,
                                                      uint32_t *__restrict__ req, uint32_t *__restrict__ act_next,
                                                      SweepSlot *slot, Geom g, FastDiv div_nx, const int *run) {
    if (run && *run == 0) return;
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
    const uint32_t v[8] = {cmax, cmin, cdir, 0u, 0u, 0u, 0u, 0u};
    block_flush_slot(slot, v);
}

// Voxels the first pass deferred (a failed certificate in f or fhat): the
// first detection on the full keys of fhat, and the original code byte on the
// full keys of f where the first pass left it unset (kCodeUnset: f's own
// certificate failed).
template <typename T>
__global__ void __launch_bounds__(256) k_first_exact(const uint32_t *__restrict__ xlist, const uint32_t *count,
                                                     const T *__restrict__ f, const T *__restrict__ fh,
                                                     uint8_t *__restrict__ codes, uint32_t *__restrict__ req,
                                                     uint32_t *__restrict__ act_next, SweepSlot *slot, Geom g,
                                                     FastDiv div_nx, const uint32_t *start = nullptr) {
    const uint32_t m = *count, m0 = start ? *start : 0u;  // entries m0 .. m-1
    uint32_t cmax = 0, cmin = 0, cdir = 0;
    const ptrdiff_t sy = g.nx, sz = static_cast<ptrdiff_t>(g.nx) * g.ny;
    using K = typename KeyOf<T>::type;
    for (uint32_t k = m0 + blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const uint32_t i = __ldg(xlist + k);
        int x, y, z;
        voxel_coords(g, div_nx, i, x, y, z);
        const uint32_t valid = valid_mask(x, y, z, g.nx, g.ny, g.nz);
        K kk[15];
        int asc, desc;
        uint8_t c = codes[i];
        if (c == kCodeUnset) {
            int oasc, odesc;
#pragma unroll
            for (int r = 0; r < 15; ++r) {
                const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
                kk[r] = ((valid >> r) & 1u) ? okey(__ldg(f + (static_cast<ptrdiff_t>(i) + off))) : K(0);
            }
            arg_ext(kk, valid, oasc, odesc);
            c = static_cast<uint8_t>(oasc | (odesc << 4));
            codes[i] = c;
        }
#pragma unroll
        for (int r = 0; r < 15; ++r) {
            const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
            kk[r] = ((valid >> r) & 1u) ? okey(__ldg(fh + (static_cast<ptrdiff_t>(i) + off))) : K(0);
        }
        arg_ext(kk, valid, asc, desc);
        detect_outcome(g, x, y, z, asc, desc, c, req, act_next, cmax, cmin, cdir);
    }
    const uint32_t v[8] = {cmax, cmin, cdir, 0u, 0u, 0u, 0u, 0u};
    block_flush_slot(slot, v);
}

// The edit of every listed voxel (applyDeltaBuffer_local, pMSz.cu:623-645),
// the proxy refresh, and for a changed value the closed stencil of the voxel
// in the next active set.
template <typename T>
__global__ void __launch_bounds__(256) k_apply_list(const uint32_t *__restrict__ list, const uint32_t *count,
                                                    const T *__restrict__ f, T *__restrict__ fh,
                                                    uint8_t *__restrict__ cnt, uint32_t *__restrict__ hp,
                                                    uint32_t *__restrict__ act_next, SweepSlot *slot, Geom g,
                                                    FastDiv div_nx, T eps, T delta, int q, const int *run) {
    if (run && *run == 0) return;
    const uint32_t m = *count;
    uint32_t nreq = 0, nchg = 0, nprog = 0;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t k0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); k0 < m; k0 += gridDim.x * blockDim.x) {
        const uint32_t k = k0 + lane;  // k0 is warp-uniform
        uint32_t key = 0xFFFFFFFFu, cb = 0;
        int x = 0, y = 0, z = 0;
        if (k < m) {
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
            voxel_coords(g, div_nx, v, x, y, z);
            key = v - static_cast<uint32_t>(x & 31);
            if (chg) {
                ++nchg;
                hp[v] = proxy_of(nv);
                cb = 1u << (x & 31);
            }
        }
        if (warp_merge_word(key, cb)) mark_stencil(act_next, g, x >> 5, y, z, cb);
    }
    const uint32_t v[8] = {0u, 0u, 0u, nreq, nchg, nprog, 0u, 0u};
    block_flush_slot(slot, v);
}

// Bitmap -> list (k_count_words, k_write_list); counts: kCompactBlocks words of
// scratch; *total receives the list length.  run (or null): the sweep's gate.
inline void compact_bitmap(uint32_t *bm, const Geom &g, uint32_t *counts, uint32_t *list, uint32_t *total,
                           const int *run, cudaStream_t s) {
    k_count_words<<<kCompactBlocks, kCompactBlock, 0, s>>>(bm, g, counts, run);
    k_write_list<<<kCompactBlocks, kCompactBlock, 0, s>>>(bm, g, counts, list, total, run);
}

// The same over the planes [z0, z1) of the bitmap (z0 < z1), with at most a
// block per step of words (a z-range is often a small part of the bitmap).
inline void compact_bitmap_planes(uint32_t *bm, const Geom &g, int z0, int z1, uint32_t *counts, uint32_t *list,
                                  uint32_t *total, cudaStream_t s) {
    const size_t wpp = static_cast<size_t>(g.wpr) * g.ny;  // words per plane
    const size_t first = static_cast<size_t>(z0) * wpp, base = first & ~static_cast<size_t>(3);
    Geom r = g;
    r.nwords = static_cast<size_t>(z1) * wpp - base;
    const uint32_t skip = static_cast<uint32_t>(first - base);
    const unsigned blocks = static_cast<unsigned>(
        std::min<size_t>(kCompactBlocks, (r.nwords + kCompactWords - 1) / kCompactWords));
    k_count_words<<<blocks, kCompactBlock, 0, s>>>(bm + base, r, counts, nullptr, skip);
    k_write_list<<<blocks, kCompactBlock, 0, s>>>(bm + base, r, counts, list, total, nullptr,
                                                   static_cast<uint32_t>(base), skip);
}

// State of the device-side sweep loop: the index of the sweep that runs
// next, its gate, its list lengths and its counters (copied to the sweep's
// slot by k_loop_gate).
struct LoopState {
    long long k;
    int go;
    int tail;        // the loop stopped only because the next active set is small: the cooperative tail runs
    int exact_keys;  // fp32 list detection on exact keys (k_pick_detection)
    uint32_t lc[4];  // active list, request list, exact list (spills), first-pass deferrals
    uint32_t deferred;  // voxels of the current list sweep decided on exact keys
    uint32_t err;    // set by the first pass when a tensor copy did not arrive
    uint32_t xdone;  // first-pass deferrals already decided (the host-buffer wavefront)
    SweepSlot cur;
};

// Before the first list sweep (after sweep 0's edits): fp32 fields run the
// list detection on exact keys when the first pass deferred more than a
// tenth of the voxels (plateaus of quantised values: each such voxel would
// be detected twice), or when the first list -- estimated as 15 * changed +
// fdir of sweep 0 -- would defer, at the first pass's rate, more than half
// of every detection block's buffer (a list of a billion voxels would
// otherwise spill its deferrals through one global counter).  k_loop_gate
// makes the first switch later when a list sweep defers more than a tenth.
static __global__ void k_pick_detection(LoopState *ls, unsigned long long n, unsigned long long blocks) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const unsigned long long deferred = ls->lc[3];
    const unsigned long long est = 15ull * ls->cur.changed + ls->cur.fdir;
    const double spill = static_cast<double>(deferred) * static_cast<double>(est) / static_cast<double>(n);
    if (10ull * deferred > n || spill > 0.5 * kExactCap * static_cast<double>(blocks)) ls->exact_keys = 1;
}

// After sweep ls->k: store its counters, decide whether the next sweep runs
// (not converged, not stuck, no NaN input at sweep 0, sweeps left, and an
// active set still too large for the cooperative tail: 15 * changed + fdir >
// tail_at), advance k, clear the per-sweep state, and, in the loop body, set
// the condition of the graph's while node.
static __global__ void k_loop_gate(LoopState *ls, SweepSlot *slots, long long max_sweeps, unsigned long long tail_at,
                            cudaGraphConditionalHandle cond, int set_cond) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (ls->go) {
        const SweepSlot c = ls->cur;
        const long long k = ls->k;
        slots[k] = c;
        // a list sweep that deferred more than a tenth of its voxels (failed
        // certificates) switches the following ones to exact keys, for good
        if (10ull * ls->deferred > ls->lc[0]) ls->exact_keys = 1;
        const bool stop = (k == 0 && c.bad) || (c.fmax == 0 && c.fmin == 0 && c.fdir == 0) || c.progressed == 0 ||
                          k + 1 >= max_sweeps;
        const bool tail = 15ull * c.changed + c.fdir <= tail_at;
        ls->go = (!stop && !tail) ? 1 : 0;
        ls->tail = (!stop && tail) ? 1 : 0;
        ls->k = k + 1;
        ls->cur = SweepSlot{};
        ls->lc[0] = ls->lc[1] = ls->lc[2] = ls->lc[3] = 0;
        ls->deferred = 0;
    }
    if (set_cond) cudaGraphSetConditional(cond, ls->go ? 1u : 0u);
}

// The graph node ahead of the while node: the loop's first body runs only if
// the gate before the graph let the next sweep run.
static __global__ void k_loop_enter(const LoopState *ls, cudaGraphConditionalHandle cond) {
    if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(cond, ls->go ? 1u : 0u);
}

// After the host-buffer wavefront has run sweeps 0 .. K to the end: the loop
// state that k_loop_gate would have left after sweep K, or after the first of
// those sweeps that stops the loop (the sweeps after a stopping one changed
// nothing: they found an empty active set, or repeated a sweep whose edits
// changed no value and no counter, or follow a NaN input whose call fails),
// and k_pick_detection's choice from sweep 0.
static __global__ void k_wave_gate(LoopState *ls, const SweepSlot *slots, long long K, long long max_sweeps,
                                   unsigned long long tail_at, unsigned long long n, unsigned long long blocks) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    long long k = 0;
    bool stop = false;
    for (; k <= K; ++k) {
        const SweepSlot c = slots[k];
        stop = (k == 0 && c.bad) || (c.fmax == 0 && c.fmin == 0 && c.fdir == 0) || c.progressed == 0 ||
               k + 1 >= max_sweeps;
        if (stop) break;
    }
    if (stop) {
        ls->k = k + 1;
        ls->go = 0;
        ls->tail = 0;
    } else {
        const SweepSlot c = slots[K];
        ls->k = K + 1;
        ls->go = 15ull * c.changed + c.fdir <= tail_at ? 0 : 1;
        ls->tail = 1 - ls->go;
    }
    const unsigned long long deferred = ls->lc[3];
    const unsigned long long est = 15ull * slots[0].changed + slots[0].fdir;
    const double spill = static_cast<double>(deferred) * static_cast<double>(est) / static_cast<double>(n);
    if (10ull * deferred > n || spill > 0.5 * kExactCap * static_cast<double>(blocks)) ls->exact_keys = 1;
    ls->cur = SweepSlot{};
    ls->lc[0] = ls->lc[1] = ls->lc[2] = ls->lc[3] = 0;
    ls->deferred = 0;
}

}  // namespace pmsz
