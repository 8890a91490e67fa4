// tail.cuh -- the last sweeps of the correction loop in one cooperative
// launch, over two-level bitmaps; included by correct.cu after list.cuh.
//
// Once the active set has shrunk to thousands of voxels, scanning a whole
// one-bit-per-voxel bitmap per phase (67 MB at 512^3) costs far more than the
// work.  Each bitmap of the tail therefore has a SUMMARY with one bit per
// word (1/32 of the bitmap).  Every writer sets the summary bit of each word
// it touches; a phase scans only the summary and visits the marked words,
// clearing word and summary bits as it consumes them.  Phases are separated by grid barriers; every block reads the same
// sweep counters after the second one and takes the same stop decision.
#pragma once
#include "list.cuh"

namespace pmsz {

constexpr int kTailBlock = 256;
constexpr int kSumPerThread = 8;                       // summary words per thread and step
constexpr int kSumStep = kTailBlock * kSumPerThread;   // 2048 summary words = 65536 bitmap words
constexpr uint32_t kGroupCap = 2048;                   // marked words staged per pass

__host__ __device__ __forceinline__ size_t summary_words(const Geom &g) { return (g.nwords + 31) / 32; }

__device__ __forceinline__ void summary_mark(uint32_t *sum, size_t w) {
    atomicOr(sum + (w >> 5), 1u << (w & 31u));
}

// or_word / mark_stencil / request_targets that also mark the summary.
__device__ __forceinline__ void or_word_s(uint32_t *act, uint32_t *sum, const Geom &g, int wx, int y, int z,
                                          uint32_t m) {
    if (!m || wx < 0 || wx >= g.wpr || y < 0 || y >= g.ny || z < 0 || z >= g.nz) return;
    m &= row_tail_mask(g, wx);
    if (!m) return;
    const size_t w = static_cast<size_t>(wx) + static_cast<size_t>(g.wpr) * (static_cast<size_t>(y) + static_cast<size_t>(g.ny) * z);
    atomicOr(act + w, m);
    summary_mark(sum, w);
}

__device__ __forceinline__ void mark_stencil_s(uint32_t *act, uint32_t *sum, const Geom &g, int wx, int y, int z,
                                               uint32_t c) {
    const uint32_t lo = (c & 1u) << 31, hi = c >> 31;
    or_word_s(act, sum, g, wx, y, z, c | (c << 1) | (c >> 1));
    or_word_s(act, sum, g, wx - 1, y, z, lo);
    or_word_s(act, sum, g, wx + 1, y, z, hi);
    const uint32_t m = c | (c >> 1), p = c | (c << 1);
    or_word_s(act, sum, g, wx, y + 1, z, m);     or_word_s(act, sum, g, wx - 1, y + 1, z, lo);
    or_word_s(act, sum, g, wx, y, z + 1, m);     or_word_s(act, sum, g, wx - 1, y, z + 1, lo);
    or_word_s(act, sum, g, wx, y + 1, z + 1, m); or_word_s(act, sum, g, wx - 1, y + 1, z + 1, lo);
    or_word_s(act, sum, g, wx, y - 1, z, p);     or_word_s(act, sum, g, wx + 1, y - 1, z, hi);
    or_word_s(act, sum, g, wx, y, z - 1, p);     or_word_s(act, sum, g, wx + 1, y, z - 1, hi);
    or_word_s(act, sum, g, wx, y - 1, z - 1, p); or_word_s(act, sum, g, wx + 1, y - 1, z - 1, hi);
}

__device__ __forceinline__ void request_targets_s(uint32_t *req, uint32_t *sum, const Geom &g, int x, int y, int z,
                                                  uint32_t tm) {
    while (tm) {
        const int r = __ffs(tm) - 1;
        tm &= tm - 1;
        const int tx = x + rank_dx(r), ty = y + rank_dy(r), tz = z + rank_dz(r);
        const size_t w = word_of(g, tx, ty, tz);
        atomicOr(req + w, 1u << (tx & 31));
        summary_mark(sum, w);
    }
}

// Summary of a plain bitmap (at the hand-over to the tail): one warp per
// summary word, lane j testing word j of its 32.
__device__ __forceinline__ void build_summary(const uint32_t *__restrict__ bm, const Geom &g, uint32_t *__restrict__ sum) {
    const size_t ns = summary_words(g);
    const int lane = threadIdx.x & 31;
    const size_t warps = static_cast<size_t>(gridDim.x) * (blockDim.x >> 5);
    for (size_t s = static_cast<size_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); s < ns; s += warps) {
        const size_t w = s * 32 + static_cast<size_t>(lane);
        const uint32_t bits = __ballot_sync(0xFFFFFFFFu, w < g.nwords && bm[w] != 0);
        if (lane == 0) sum[s] = bits;
    }
}
static __global__ void __launch_bounds__(256) k_build_summary(const uint32_t *__restrict__ bm, Geom g,
                                                       uint32_t *__restrict__ sum) {
    build_summary(bm, g, sum);
}
// The same for a tail launched ahead of the host's decision: nothing unless
// *run_if, and the bitmap of sweep *k_at (act0 / sum0 for even sweeps).
static __global__ void __launch_bounds__(256) k_build_summary_at(const uint32_t *act0, const uint32_t *act1, Geom g,
                                                          uint32_t *sum0, uint32_t *sum1, const long long *k_at,
                                                          const int *run_if) {
    if (!*run_if) return;
    const bool odd = (*k_at & 1) != 0;
    build_summary(odd ? act1 : act0, g, odd ? sum1 : sum0);
}

constexpr uint32_t kTailListCap = 4096;

struct TailSmem {
    uint32_t groups[kGroupCap];       // marked words of the current summary step
    uint32_t list[kTailListCap];      // (word slot << 5) | bit of the current step
    uint32_t mask[kTailBlock];         // result bits per word slot
    uint32_t warp_tot[kTailBlock / 32];
    uint32_t total;
};

// Visits every set bit of a two-level bitmap (bm, sum), clearing both.  Block b
// owns summary words [b * per, (b + 1) * per), read kSumStep at a time (an
// empty step costs one barrier) and ranked into a list of marked words.  Those are taken 256 at a time (one per thread):
// their set bits are ranked by a block scan into a shared list that all
// threads share (visit(x, y, z) returns the voxel's result bit), and
// flush(w, results) runs once per word by its owner thread.
template <class Visit, class Flush>
__device__ __forceinline__ void for_each_set_bit_2l(TailSmem &sm, uint32_t *__restrict__ bm, uint32_t *__restrict__ sum,
                                                    const Geom &g, Visit &visit, Flush &flush) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    auto block_scan = [&](uint32_t c, uint32_t &first) -> uint32_t {  // exclusive rank of c; returns the total
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) sm.warp_tot[warp] = inc;
        __syncthreads();
        if (t == 0) {
            uint32_t run = 0;
            for (int k = 0; k < kTailBlock / 32; ++k) {
                const uint32_t v = sm.warp_tot[k];
                sm.warp_tot[k] = run;
                run += v;
            }
            sm.total = run;
        }
        __syncthreads();
        first = sm.warp_tot[warp] + inc - c;
        return sm.total;
    };
    const size_t ns = summary_words(g);
    const size_t per = (ns + gridDim.x - 1) / gridDim.x;
    const size_t lo = static_cast<size_t>(blockIdx.x) * per, hi = min(ns, lo + per);
    for (size_t base = lo; base < hi; base += kSumStep) {
        // kSumPerThread summary words per thread; an empty step costs one barrier
        uint32_t sw[kSumPerThread];
        uint32_t c = 0;
#pragma unroll
        for (int j = 0; j < kSumPerThread; ++j) {
            const size_t si = base + static_cast<size_t>(t) * kSumPerThread + j;
            sw[j] = si < hi ? __ldcg(sum + si) : 0u;
            if (sw[j]) sum[si] = 0;
            c += __popc(sw[j]);
        }
        if (!__syncthreads_or(c != 0)) continue;
        uint32_t first;
        const uint32_t nmarked = block_scan(c, first);
        for (uint32_t lo1 = 0; lo1 < nmarked; lo1 += kGroupCap) {  // marked words, kGroupCap per pass
            const uint32_t hi1 = lo1 + kGroupCap;
            uint32_t r = first;
#pragma unroll
            for (int j = 0; j < kSumPerThread; ++j) {
                const size_t si = base + static_cast<size_t>(t) * kSumPerThread + j;
                for (uint32_t bits = sw[j]; bits; bits &= bits - 1, ++r)
                    if (r >= lo1 && r < hi1)
                        sm.groups[r - lo1] = static_cast<uint32_t>(si * 32 + static_cast<size_t>(__ffs(bits) - 1));
            }
            __syncthreads();
            const uint32_t ng = min(kGroupCap, nmarked - lo1);
            // the marked words, 256 per step
            for (uint32_t g0 = 0; g0 < ng; g0 += kTailBlock) {
                const uint32_t gi = g0 + static_cast<uint32_t>(t);
                size_t w = 0;
                uint32_t m = 0;
                if (gi < ng) {
                    w = sm.groups[gi];
                    m = __ldcg(bm + w);
                    if (m) bm[w] = 0;
                }
                sm.mask[t] = 0;
                uint32_t rank;
                const uint32_t total = block_scan(__popc(m), rank);
                for (uint32_t lo2 = 0; lo2 < total; lo2 += kTailListCap) {
                    const uint32_t hi2 = lo2 + kTailListCap;
                    uint32_t rr = rank;
                    for (uint32_t bits = m; bits; bits &= bits - 1, ++rr)
                        if (rr >= lo2 && rr < hi2)
                            sm.list[rr - lo2] = (static_cast<uint32_t>(t) << 5) | static_cast<uint32_t>(__ffs(bits) - 1);
                    __syncthreads();
                    const uint32_t n = min(kTailListCap, total - lo2);
                    for (uint32_t k = t; k < n; k += kTailBlock) {
                        const uint32_t e = sm.list[k];
                        const uint32_t slot = e >> 5;
                        const int b = static_cast<int>(e & 31u);
                        const size_t ww = sm.groups[g0 + slot];
                        int wx, y, z;
                        word_coords(g, ww, wx, y, z);
                        if (visit(wx * 32 + b, y, z)) atomicOr(&sm.mask[slot], 1u << b);
                    }
                    __syncthreads();
                }
                const uint32_t res = sm.mask[t];
                if (m && res) flush(w, res);
                __syncthreads();  // mask / list are rewritten by the next step
            }
        }
    }
}

template <typename T>
struct TailDetect {
    const T *fh;
    const uint32_t *hp;
    const uint8_t *codes;
    uint32_t *req, *sum_req;
    Geom g;
    uint32_t cmax = 0, cmin = 0, cdir = 0, active = 0;
    __device__ __forceinline__ bool operator()(int x, int y, int z) {
        const ptrdiff_t sy = g.nx, sz = static_cast<ptrdiff_t>(g.nx) * g.ny;
        const size_t i = flat(g, x, y, z);
        const bool interior = x >= 1 && x <= g.nx - 2 && y >= 1 && y <= g.ny - 2 && z >= 1 && z <= g.nz - 2;
        const uint32_t valid = interior ? kAllValid : valid_mask(x, y, z, g.nx, g.ny, g.nz);
        uint32_t t[15];
#pragma unroll
        for (int r = 0; r < 15; ++r) {
            const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
            t[r] = ((valid >> r) & 1u) ? __ldcg(hp + (static_cast<ptrdiff_t>(i) + off)) : 0u;
        }
        Ext ex = interior ? proxy_ext_interior<true>(t) : proxy_ext<true>(t);
        if (!ex.exact) {
            typename KeyOf<T>::type kk[15];
#pragma unroll
            for (int r = 0; r < 15; ++r) {
                const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
                kk[r] = ((valid >> r) & 1u) ? okey(__ldcg(fh + (static_cast<ptrdiff_t>(i) + off)))
                                            : typename KeyOf<T>::type(0);
            }
            arg_ext(kk, valid, ex.asc, ex.desc);
        }
        const uint8_t c = __ldg(codes + i);
        const uint32_t tm = detect_rules(ex.asc, ex.desc, c & 15, c >> 4, cmax, cmin, cdir);
        ++active;
        if (tm) request_targets_s(req, sum_req, g, x, y, z, tm);
        return tm != 0;
    }
};

struct TailDetectFlush {
    uint32_t *act_next, *sum_next;
    __device__ __forceinline__ void operator()(size_t w, uint32_t m) {
        act_next[w] = m;  // one owner per word; the apply phase ORs in after the grid barrier
        summary_mark(sum_next, w);
    }
};

template <typename T>
struct TailApply {
    const T *f;
    T *fh;
    uint8_t *cnt;
    uint32_t *hp;
    Geom g;
    T eps, delta;
    int q;
    uint32_t nreq = 0, nprog = 0;
    __device__ __forceinline__ bool operator()(int x, int y, int z) {
        const size_t v = flat(g, x, y, z);
        const T old = __ldcg(fh + v);
        const uint8_t oc = __ldcg(cnt + v);
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
        if (chg) hp[v] = proxy_of(nv);
        ++nreq;
        nprog += (chg || nc != oc) ? 1u : 0u;
        return chg;
    }
};

struct TailApplyFlush {
    uint32_t *act_next, *sum_next;
    Geom g;
    uint32_t nchg = 0;
    __device__ __forceinline__ void operator()(size_t w, uint32_t m) {
        nchg += __popc(m);
        int wx, y, z;
        word_coords(g, w, wx, y, z);
        mark_stencil_s(act_next, sum_next, g, wx, y, z, m);
    }
};

template <typename T>
struct TailArgs {
    const T *f;
    T *fh;
    const uint8_t *codes;
    uint8_t *cnt;
    uint32_t *hp, *req, *act0, *act1, *sum_req, *sum0, *sum1;
    SweepSlot *slots;
    int64_t first;       // index of the first sweep this launch runs
    int64_t max_sweeps;
    long long *sweeps_out;
    Geom g;
    T eps, delta;
    int q;
    // launched ahead of the host's decision (run_if not null): the first
    // sweep is *first_at, and nothing runs unless *run_if
    const long long *first_at = nullptr;
    const int *run_if = nullptr;
};

// Sweep k reads (act[k & 1], sum[k & 1]) and fills (act[(k + 1) & 1], ...).
template <typename T>
__global__ void __launch_bounds__(kTailBlock, 2) k_tail_loop(TailArgs<T> a) {
    __shared__ TailSmem sm;
    cg::grid_group grid = cg::this_grid();
    int64_t k = a.first;
    if (a.run_if) {  // every block reads the same flag: all return, or none
        k = __ldcg(a.first_at);
        if (!__ldcg(a.run_if)) {
            if (blockIdx.x == 0 && threadIdx.x == 0) *a.sweeps_out = k;
            return;
        }
    }
    while (true) {
        const SweepSlot *p = a.slots + (k - 1);
        if (sweep_stops(__ldcg(&p->fmax), __ldcg(&p->fmin), __ldcg(&p->fdir), __ldcg(&p->progressed), k,
                        a.max_sweeps))
            break;
        uint32_t *cur = (k & 1) ? a.act1 : a.act0, *nxt = (k & 1) ? a.act0 : a.act1;
        uint32_t *scur = (k & 1) ? a.sum1 : a.sum0, *snxt = (k & 1) ? a.sum0 : a.sum1;
        {
            TailDetect<T> visit{a.fh, a.hp, a.codes, a.req, a.sum_req, a.g};
            TailDetectFlush flush{nxt, snxt};
            for_each_set_bit_2l(sm, cur, scur, a.g, visit, flush);
            const uint32_t v[8] = {visit.cmax, visit.cmin, visit.cdir, 0u, 0u, 0u, visit.active, 0u};
            block_flush_slot(a.slots + k, v);
        }
        grid.sync();
        {
            TailApply<T> visit{a.f, a.fh, a.cnt, a.hp, a.g, a.eps, a.delta, a.q};
            TailApplyFlush flush{nxt, snxt, a.g};
            for_each_set_bit_2l(sm, a.req, a.sum_req, a.g, visit, flush);
            const uint32_t v[8] = {0u, 0u, 0u, visit.nreq, flush.nchg, visit.nprog, 0u, 0u};
            block_flush_slot(a.slots + k, v);
        }
        grid.sync();
        ++k;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.sweeps_out = k;
}

}  // namespace pmsz
