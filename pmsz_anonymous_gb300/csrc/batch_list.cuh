// batch_list.cuh -- voxel-list sweeps over a table of fields: the host-driven
// generations of pmsz_correct_batch and of the server.  Included by batch.cu.
//
// The words of every field's bitmap are laid end to end in one global word
// space (field i owns [wpre[i], wpre[i+1]), each field's share rounded up to
// a multiple of 4 words so that 16-byte loads never straddle two fields).
// A generation compacts the active bitmaps of the fields that run detection
// into one list of entries (field << 48 | flat voxel index), in voxel order,
// detects every listed voxel (failed certificates go to a second list decided
// on full keys), then compacts the request bitmaps of every running field and
// edits every listed voxel -- the single-field list sweeps of list.cuh over a
// whole batch in a fixed number of launches.  Each field keeps its own sweep
// index, bitmaps and slots.  Entries are processed in block chunks of
// consecutive entries, so a chunk almost always belongs to one field and its
// counters are summed per block before one atomic per counter.
#pragma once
#include "batch.h"
#include "list.cuh"

namespace pmsz {

constexpr int kMultiPerThread = 16;
constexpr uint32_t kMultiChunk = kCompactBlock * kMultiPerThread;  // entries per block step
constexpr int kFieldShift = 48;
constexpr uint64_t kVoxelMask = (1ull << kFieldShift) - 1;

__device__ __forceinline__ int seg_of(const uint32_t *__restrict__ pre, int n, uint64_t w) {
    int lo = 0, hi = n - 1;  // largest i with pre[i] <= w
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(pre + mid) <= w) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Does field I take part in phase P (0: detection, 1: edits), and its bitmap.
template <typename T, int P>
__device__ __forceinline__ uint32_t *phase_bitmap(const Inst<T> &I) {
    if (!I.active) return nullptr;
    if (P == 0) return I.first ? nullptr : ((I.k & 1) ? I.act1 : I.act0);
    return I.req;
}

__host__ __device__ __forceinline__ uint64_t multi_per(uint64_t total_words) {
    return ((total_words + kCompactBlocks - 1) / kCompactBlocks + 3) & ~static_cast<uint64_t>(3);
}

template <typename T, int P>
__global__ void __launch_bounds__(kCompactBlock) k_count_words_multi(const Inst<T> *__restrict__ inst,
                                                                     const uint32_t *__restrict__ wpre, int n,
                                                                     uint64_t total_words, uint32_t *__restrict__ counts,
                                                                     const int *run) {
    __shared__ uint32_t s_warp[kCompactBlock / 32];
    if (run && *run == 0) return;
    const uint64_t per = multi_per(total_words);
    const uint64_t lo = static_cast<uint64_t>(blockIdx.x) * per, hi = min(total_words, lo + per);
    uint32_t c = 0;
    for (uint64_t w0 = lo + static_cast<uint64_t>(threadIdx.x) * 4; w0 < hi; w0 += kCompactWords) {
        const int i = seg_of(wpre, n, w0);
        const uint32_t *bm = phase_bitmap<T, P>(inst[i]);
        if (!bm) continue;
        const uint4 v = *reinterpret_cast<const uint4 *>(bm + (w0 - __ldg(wpre + i)));
        c += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
    }
    c = block_sum_u32(c, s_warp);
    if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

template <typename T, int P>
__global__ void __launch_bounds__(kCompactBlock) k_write_list_multi(const Inst<T> *__restrict__ inst,
                                                                    const uint32_t *__restrict__ wpre, int n,
                                                                    uint64_t total_words,
                                                                    const uint32_t *__restrict__ counts,
                                                                    uint64_t *__restrict__ list, uint32_t *total,
                                                                    const int *run) {
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
    const uint64_t per = multi_per(total_words);
    const uint64_t lo = static_cast<uint64_t>(blockIdx.x) * per, hi = min(total_words, lo + per);
    for (uint64_t base = lo; base < hi; base += kCompactWords) {
        const uint64_t w0 = base + static_cast<uint64_t>(t) * 4;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        int fi = 0;
        uint32_t local = 0;  // the word's index within its field (< 2^27); a thread's 4 words share a field
        if (w0 < hi) {
            fi = seg_of(wpre, n, w0);
            uint32_t *bm = phase_bitmap<T, P>(inst[fi]);
            if (bm) {
                local = static_cast<uint32_t>(w0 - __ldg(wpre + fi));
                v = *reinterpret_cast<const uint4 *>(bm + local);
                if (v.x | v.y | v.z | v.w) *reinterpret_cast<uint4 *>(bm + local) = make_uint4(0, 0, 0, 0);
            }
        }
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
        const uint32_t c = __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += u;
        }
        if (lane == 31) s_warp[warp] = inc;
        __syncthreads();
        uint32_t wbase = 0, step = 0;
        for (int k = 0; k < kCompactBlock / 32; ++k) {
            const uint32_t u = s_warp[k];
            if (k < warp) wbase += u;
            step += u;
        }
        write_step_entries(w, inc - c, wbase, step, s_raw, list + pos, [&](int j) {
            const Geom &g = inst[fi].g;
            const uint32_t wj = local + static_cast<uint32_t>(j);
            const uint32_t row = fdiv(wj, g.div_wpr);
            const uint32_t wx = wj - row * static_cast<uint32_t>(g.wpr);
            return (static_cast<uint64_t>(fi) << kFieldShift) |
                   (static_cast<uint64_t>(row) * static_cast<uint32_t>(g.nx) + (wx << 5));
        });
        pos += step;  // write_step_entries ends with a barrier: s_warp is free
    }
}

// Flat index -> coordinates for a field of the table (n < 2^32 per field:
// the list form is used only when all fields together have fewer voxels).
__device__ __forceinline__ void field_coords(const Geom &g, uint64_t i, int &x, int &y, int &z) {
    voxel_coords(g, g.div_nx, static_cast<uint32_t>(i), x, y, z);
}

template <typename T>
__device__ __forceinline__ SweepSlot *slot_of_k(const Inst<T> &I) {
    return I.slots + I.k * I.stride;
}

// Adds per-thread counters to a field's slot: once per block when the whole
// chunk belongs to that field (single), else thread by thread.
__device__ __forceinline__ void multi_flush(SweepSlot *slot, const uint32_t (&v)[8], bool single) {
    if (single) {
        block_flush_slot(slot, v);
        return;
    }
#pragma unroll
    for (int c = 0; c < 8; ++c)
        if (v[c]) atomicAdd(reinterpret_cast<unsigned long long *>(slot) + c, static_cast<unsigned long long>(v[c]));
}

// Detection of the listed voxels.  fp32 fields decide on the exact keys of
// fhat (a 4-byte gather, the same bytes as the proxies, so no certificate is
// needed); fp64 fields decide on the proxies and append failed certificates
// to xlist for k_detect_exact_multi.
template <typename T>
__global__ void __launch_bounds__(256, 4) k_detect_list_multi(const Inst<T> *__restrict__ inst,
                                                             const uint64_t *__restrict__ list, const uint32_t *count,
                                                             uint64_t *__restrict__ xlist, uint32_t *xcount,
                                                             const int *run) {
    constexpr bool kExactKeys = sizeof(T) == 4;
    __shared__ uint64_t s_x[kExactKeys ? 1 : kMultiChunk];
    __shared__ uint32_t s_n, s_base;
    if (run && *run == 0) return;
    const uint32_t m = *count;
    for (uint32_t c0 = blockIdx.x * kMultiChunk; c0 < m; c0 += gridDim.x * kMultiChunk) {
        const uint32_t c1 = min(m, c0 + kMultiChunk);
        const int f0 = static_cast<int>(__ldg(list + c0) >> kFieldShift);
        const bool single = f0 == static_cast<int>(__ldg(list + c1 - 1) >> kFieldShift);  // block-uniform
        if (!kExactKeys) {
            if (threadIdx.x == 0) s_n = 0;
            __syncthreads();
        }
        uint32_t v[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        for (uint32_t e = c0 + threadIdx.x; e < c1; e += blockDim.x) {
            const uint64_t ent = __ldg(list + e);
            const int fi = static_cast<int>(ent >> kFieldShift);
            const uint64_t i = ent & kVoxelMask;
            const Inst<T> &I = inst[fi];
            const Geom &g = I.g;
            int x, y, z;
            field_coords(g, i, x, y, z);
            const bool interior = x >= 1 && x <= g.nx - 2 && y >= 1 && y <= g.ny - 2 && z >= 1 && z <= g.nz - 2;
            const uint32_t valid = interior ? kAllValid : valid_mask(x, y, z, g.nx, g.ny, g.nz);
            const ptrdiff_t sy = g.nx, sz = static_cast<ptrdiff_t>(g.nx) * g.ny;
            const uint8_t c = __ldg(I.codes + i);
            uint32_t w[8] = {0u, 0u, 0u, 0u, 0u, 0u, 1u, 0u};  // active
            uint32_t *nxt = ((I.k + 1) & 1) ? I.act1 : I.act0;
            if (kExactKeys) {
                const T *c0p = I.fh + i;
                uint32_t kk[15];
#pragma unroll
                for (int r = 0; r < 15; ++r) {
                    const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
                    kk[r] = ((valid >> r) & 1u) ? static_cast<uint32_t>(okey(__ldg(c0p + off))) : 0u;
                }
                int asc, desc;
                arg_ext(kk, valid, asc, desc);
                detect_outcome(g, x, y, z, asc, desc, c, I.req, nxt, w[0], w[1], w[2]);
            } else {
                const uint32_t *c0p = I.hp + i;
                uint32_t t[15];
#pragma unroll
                for (int r = 0; r < 15; ++r) {
                    const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
                    t[r] = ((valid >> r) & 1u) ? __ldg(c0p + off) : 0u;
                }
                const Ext ex = interior ? proxy_ext_interior<true>(t) : proxy_ext<true>(t);
                if (ex.exact) detect_outcome(g, x, y, z, ex.asc, ex.desc, c, I.req, nxt, w[0], w[1], w[2]);
                else s_x[atomicAdd(&s_n, 1u)] = ent;  // at most kMultiChunk per step: no overflow
            }
            if (single) {
#pragma unroll
                for (int k = 0; k < 8; ++k) v[k] += w[k];
            } else {
                multi_flush(slot_of_k(I), w, false);
            }
        }
        if (single) multi_flush(slot_of_k(inst[f0]), v, true);  // every thread: contains a barrier
        if (!kExactKeys) {
            __syncthreads();
            const uint32_t nb = s_n;
            if (threadIdx.x == 0) s_base = nb ? atomicAdd(xcount, nb) : 0u;
            __syncthreads();
            for (uint32_t j = threadIdx.x; j < nb; j += blockDim.x) xlist[s_base + j] = s_x[j];
            __syncthreads();
        }
    }
}

// fp64 voxels whose proxy certificate failed: steepest ranks on the exact
// keys.  xlist holds each detecting block's failures as one run, so a chunk
// almost always belongs to one field and its counters are summed per block.
template <typename T>
__global__ void __launch_bounds__(256) k_detect_exact_multi(const Inst<T> *__restrict__ inst,
                                                            const uint64_t *__restrict__ xlist, const uint32_t *count,
                                                            const int *run) {
    if (run && *run == 0) return;
    const uint32_t m = *count;
    using K = typename KeyOf<T>::type;
    for (uint32_t c0 = blockIdx.x * kMultiChunk; c0 < m; c0 += gridDim.x * kMultiChunk) {
        const uint32_t c1 = min(m, c0 + kMultiChunk);
        const int f0 = static_cast<int>(__ldg(xlist + c0) >> kFieldShift);
        // block-uniform: every field in [c0, c1) equal to the first and last is
        // not implied (runs are unordered), so check the whole chunk
        const bool single = __syncthreads_and([&] {
            for (uint32_t e = c0 + threadIdx.x; e < c1; e += blockDim.x)
                if (static_cast<int>(__ldg(xlist + e) >> kFieldShift) != f0) return 0;
            return 1;
        }());
        uint32_t v[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        for (uint32_t e = c0 + threadIdx.x; e < c1; e += blockDim.x) {
            const uint64_t ent = __ldg(xlist + e);
            const Inst<T> &I = inst[static_cast<int>(ent >> kFieldShift)];
            const uint64_t i = ent & kVoxelMask;
            const Geom &g = I.g;
            int x, y, z;
            field_coords(g, i, x, y, z);
            const uint32_t valid = valid_mask(x, y, z, g.nx, g.ny, g.nz);
            const ptrdiff_t sy = g.nx, sz = static_cast<ptrdiff_t>(g.nx) * g.ny;
            K kk[15];
#pragma unroll
            for (int r = 0; r < 15; ++r) {
                const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
                kk[r] = ((valid >> r) & 1u) ? okey(__ldg(I.fh + (static_cast<ptrdiff_t>(i) + off))) : K(0);
            }
            int asc, desc;
            arg_ext(kk, valid, asc, desc);
            uint32_t w[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
            uint32_t *nxt = ((I.k + 1) & 1) ? I.act1 : I.act0;
            detect_outcome(g, x, y, z, asc, desc, __ldg(I.codes + i), I.req, nxt, w[0], w[1], w[2]);
            if (single) {
#pragma unroll
                for (int k = 0; k < 8; ++k) v[k] += w[k];
            } else {
                multi_flush(slot_of_k(I), w, false);
            }
        }
        if (single) multi_flush(slot_of_k(inst[f0]), v, true);
    }
}

// Edits of the listed voxels.  The list is in (field, voxel) order, so the
// lanes of a warp whose voxels share a bitmap word are consecutive: their
// changed bits are OR-ed across the group and its lowest lane marks the
// closed stencil of the whole word once (15 atomics per word, not per voxel).
template <typename T>
__global__ void __launch_bounds__(256) k_apply_list_multi(const Inst<T> *__restrict__ inst,
                                                          const uint64_t *__restrict__ list, const uint32_t *count,
                                                          const int *run) {
    if (run && *run == 0) return;
    const uint32_t m = *count;
    const int lane = threadIdx.x & 31;
    for (uint32_t c0 = blockIdx.x * kMultiChunk; c0 < m; c0 += gridDim.x * kMultiChunk) {
        const uint32_t c1 = min(m, c0 + kMultiChunk);
        const int f0 = static_cast<int>(__ldg(list + c0) >> kFieldShift);
        const bool single = f0 == static_cast<int>(__ldg(list + c1 - 1) >> kFieldShift);  // block-uniform
        uint32_t v[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        for (uint32_t e0 = c0 + (threadIdx.x & ~31u); e0 < c1; e0 += blockDim.x) {  // warp-uniform
            const uint32_t e = e0 + lane;
            uint64_t key = ~0ull;  // lanes past the end form the last group
            uint32_t cb = 0;
            int fi = 0, x = 0, y = 0, z = 0;
            if (e < c1) {
                const uint64_t ent = __ldg(list + e);
                fi = static_cast<int>(ent >> kFieldShift);
                const Inst<T> &I = inst[fi];
                const uint64_t vx = ent & kVoxelMask;
                const T old = I.fh[vx];
                const uint8_t oc = I.cnt[vx];
                const T fv = __ldg(I.f + vx);
                const T lowered = old - I.delta;
                T nv;
                uint8_t nc;
                if (fabs(fv - lowered) <= I.eps && static_cast<int>(oc) < I.q - 1) {
                    nv = lowered;
                    nc = static_cast<uint8_t>(oc + 1);
                } else {
                    nc = static_cast<uint8_t>(I.q);
                    nv = fv - I.eps;
                }
                I.fh[vx] = nv;
                I.cnt[vx] = nc;
                const bool chg = bits_of(old) != bits_of(nv);
                uint32_t w[8] = {0u, 0u, 0u, 1u, chg ? 1u : 0u, (chg || nc != oc) ? 1u : 0u, 0u, 0u};
                if (chg) I.hp[vx] = proxy_of(nv);
                field_coords(I.g, vx, x, y, z);
                key = (static_cast<uint64_t>(fi) << kFieldShift) | (vx - (x & 31));  // the word's first voxel
                cb = chg ? 1u << (x & 31) : 0u;
                if (single) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) v[k] += w[k];
                } else {
                    multi_flush(slot_of_k(I), w, false);
                }
            }
            if (warp_merge_word(key, cb)) {
                const Inst<T> &I = inst[fi];
                uint32_t *nxt = ((I.k + 1) & 1) ? I.act1 : I.act0;
                mark_stencil(nxt, I.g, x >> 5, y, z, cb);
            }
        }
        if (single) multi_flush(slot_of_k(inst[f0]), v, true);
    }
}

// Detection of every running field that does not start now, then the edits of
// every running field, as voxel-list passes.  run: a device flag that turns
// every kernel into a no-op when zero (the gated graph loop), or null.
template <typename T>
int launch_list_sweep(const Inst<T> *dinst, int n, const MultiLists &ml, cudaStream_t s, const int *run = nullptr) {
    PMSZ_CUDA(cudaMemsetAsync(ml.lc, 0, 4 * sizeof(uint32_t), s));
    const unsigned blocks = 152 * 4;
    k_count_words_multi<T, 0><<<kCompactBlocks, kCompactBlock, 0, s>>>(dinst, ml.wpre, n, ml.total_words, ml.counts,
                                                                       run);
    k_write_list_multi<T, 0><<<kCompactBlocks, kCompactBlock, 0, s>>>(dinst, ml.wpre, n, ml.total_words, ml.counts,
                                                                      ml.list, ml.lc, run);
    k_detect_list_multi<T><<<blocks, 256, 0, s>>>(dinst, ml.list, ml.lc, ml.xlist, ml.lc + 2, run);
    k_detect_exact_multi<T><<<blocks, 256, 0, s>>>(dinst, ml.xlist, ml.lc + 2, run);
    k_count_words_multi<T, 1><<<kCompactBlocks, kCompactBlock, 0, s>>>(dinst, ml.wpre, n, ml.total_words, ml.counts,
                                                                       run);
    k_write_list_multi<T, 1><<<kCompactBlocks, kCompactBlock, 0, s>>>(dinst, ml.wpre, n, ml.total_words, ml.counts,
                                                                      ml.list, ml.lc + 1, run);
    k_apply_list_multi<T><<<blocks, 256, 0, s>>>(dinst, ml.list, ml.lc + 1, run);
    PMSZ_CUDA(cudaGetLastError());
    return PMSZ_OK;
}

// After generation st->k of a batch: every running field's stop rule on its
// slot of that sweep (NaN input at sweep 0, converged, stuck, max_sweeps), the
// survivors advance to sweep k + 1; the next generation runs (st->go) while
// some field runs and their estimated next active sets exceed tail_at (below
// it the cooperative tail takes over).  In the graph body it also sets the
// condition of the while node.  One block; table rows are the fields.
template <typename T>
__global__ void __launch_bounds__(256) k_batch_gate(Inst<T> *inst, int n, BatchState *st, long long max_sweeps,
                                                    unsigned long long tail_at, cudaGraphConditionalHandle cond,
                                                    int set_cond) {
    __shared__ unsigned long long s_est;
    __shared__ int s_live;
    const int go = st->go;  // block-uniform
    if (go) {
        if (threadIdx.x == 0) {
            s_est = 0;
            s_live = 0;
        }
        __syncthreads();
        const long long k = st->k;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            Inst<T> &I = inst[i];
            if (!I.active) continue;
            const SweepSlot h = *slot_of_k(I);
            if ((k == 0 && h.bad) || sweep_stops(h.fmax, h.fmin, h.fdir, h.progressed, k + 1, I.max_sweeps)) {
                I.active = 0;
                continue;
            }
            I.k = k + 1;
            I.first = 0;
            atomicAdd(&s_est, 15ull * h.changed + h.fdir);
            atomicAdd(&s_live, 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            st->k = k + 1;
            st->live = s_live;
            st->est = s_est;
            st->go = (s_live > 0 && s_est > tail_at && k + 1 < max_sweeps) ? 1 : 0;
        }
    }
    if (set_cond && threadIdx.x == 0) cudaGraphSetConditional(cond, st->go ? 1u : 0u);
}

}  // namespace pmsz
