// batch.cu -- many independent fields corrected together.
//
// pmsz_correct_batch runs the correction of every field of a batch with one
// set of launches: the fused labelling + first-detection pass covers the
// tiles of all fields in one grid (a global tile index is mapped to its field
// by binary search over per-field prefix counts), the heavy early sweeps are
// multi-field launches over the bitmap rounds of all fields, and the light
// tail runs in one cooperative persistent launch that keeps a per-field stop
// decision on the device.  Each field keeps its own scratch, sweep index and
// stop state, so its result is bit-identical to correcting it alone
// (pmsz_correct_f32 / pmsz_correct_f64).  The same kernels serve the
// continuous-batching server (server.cpp), where fields join and leave between
// sweeps.
#include "batch.h"
#include "batch_list.cuh"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace pmsz {

__device__ __forceinline__ int find_seg(const uint32_t *__restrict__ pre, int n, uint32_t r) {
    int lo = 0, hi = n - 1;  // largest i with pre[i] <= r (pre[0] = 0, segments non-empty)
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(pre + mid) <= r) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 5) k_first_multi(const Inst<T> *__restrict__ inst,
                                                            const uint32_t *__restrict__ tpre, int n) {
    __shared__ TileOf<T, kFirst, false> sm;
    const int i = find_seg(tpre, n, blockIdx.x);
    const Inst<T> &I = inst[i];
    if (!I.first) return;  // uniform: only fields that start now
    const uint32_t lt = blockIdx.x - __ldg(tpre + i);
    const uint32_t bx = lt % I.tiles_x, rest = lt / I.tiles_x;
    const uint32_t by = rest % I.tiles_y, bz = rest / I.tiles_y;
    // fp32 blocks whose tile, halo and planes zb-1 .. ze lie inside their
    // field run the check-free body, as in k_tiled (21.8 against 21.97 ms on
    // the 64-field batch; for fp64 the second body raises the spills)
    const int x0 = static_cast<int>(bx) * kTX, y0 = static_cast<int>(by) * kTY, zb = static_cast<int>(bz) * I.g.zc;
    const bool inside = x0 >= 1 && x0 + kTX + 1 <= I.g.nx && y0 >= 1 && y0 + kTY + 1 <= I.g.ny && zb >= 1 &&
                        zb + I.g.zc + 1 <= I.g.nz;
    if (sizeof(T) == 4 && inside)
        tiled_body<T, kFirst, false, true>(sm, I.f, I.fh, I.codes, I.hp, I.req, I.act1, I.slots, I.g,
                                           static_cast<int>(bx), static_cast<int>(by), static_cast<int>(bz));
    else
        tiled_body<T, kFirst>(sm, I.f, I.fh, I.codes, I.hp, I.req, I.act1, I.slots, I.g, static_cast<int>(bx),
                              static_cast<int>(by), static_cast<int>(bz));
}

template <typename T>
__device__ __forceinline__ SweepSlot *slot_of(const Inst<T> &I, int64_t k) {
    return I.slots + k * I.stride;
}

// One detect (PHASE 0) or apply (PHASE 1) pass over the rounds of every
// active field; `it` is added to each field's sweep index (0 outside the
// persistent loop).
template <class L, typename T, int PHASE>
__device__ __forceinline__ void multi_phase(ListSmem &sm, const Inst<T> *__restrict__ inst,
                                            const uint32_t *__restrict__ rpre, int n, uint32_t total_rounds,
                                            const uint32_t *active_mask, int64_t it) {
    for (uint32_t r = blockIdx.x; r < total_rounds; r += gridDim.x) {
        const int i = find_seg(rpre, n, r);
        if (!((active_mask[i >> 5] >> (i & 31)) & 1u)) continue;  // uniform
        const Inst<T> &I = inst[i];
        const int64_t s = I.k + it;
        uint32_t *cur = (s & 1) ? I.act1 : I.act0;
        uint32_t *nxt = (s & 1) ? I.act0 : I.act1;
        const size_t base = static_cast<size_t>(r - __ldg(rpre + i)) * kRoundWords;
        if (PHASE == 0) {
            DetectWork<L, T> work{I.fh, I.hp, I.codes, I.req, I.g};
            DetectFlush flush{nxt};
            process_round<L>(sm, cur, I.g, base, work, flush);
            work.flush_to(slot_of(I, s));
        } else {
            ApplyWork<L, T> work{I.f, I.fh, I.cnt, I.hp, I.g, I.eps, I.delta, I.q};
            ApplyFlush flush{nxt, I.g};
            process_round<L>(sm, I.req, I.g, base, work, flush);
            flush_apply_counts(slot_of(I, s), work.nreq, flush.nchg, work.nprog);
        }
    }
}

// Host-driven multi-field sweep phase; the active mask is the `active` flags
// of the table, gathered into shared memory.
template <typename T, int PHASE>
__global__ void __launch_bounds__(kListBlock) k_phase_multi(const Inst<T> *__restrict__ inst,
                                                          const uint32_t *__restrict__ rpre, int n,
                                                          uint32_t total_rounds) {
    __shared__ ListSmem sm;
    __shared__ uint32_t mask[kMaxBatch / 32];
    for (int w = threadIdx.x; w < (n + 31) / 32; w += blockDim.x) mask[w] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)  // detection skips fields that start now
        if (inst[i].active && (PHASE == 1 || !inst[i].first)) atomicOr(&mask[i >> 5], 1u << (i & 31));
    __syncthreads();
    multi_phase<LdgLoads, T, PHASE>(sm, inst, rpre, n, total_rounds, mask, 0);
}

// The light tail of every field in one cooperative launch.  Each iteration:
// every block evaluates the stop rule of every field from the field's last
// sweep slot (fields stop for good: an unrun sweep leaves its slot zeroed,
// which reads as "stop"), then detect, grid barrier, apply, grid barrier.
// Bounded by each field's max_sweeps; *iters receives the iteration count.
template <typename T>
__global__ void __launch_bounds__(kListBlock, 2) k_loop_multi(const Inst<T> *__restrict__ inst,
                                                             const uint32_t *__restrict__ rpre, int n,
                                                             uint32_t total_rounds, long long *iters) {
    __shared__ ListSmem sm;
    __shared__ uint32_t mask[kMaxBatch / 32];
    cg::grid_group grid = cg::this_grid();
    int64_t it = 0;
    while (true) {
        for (int w = threadIdx.x; w < (n + 31) / 32; w += blockDim.x) mask[w] = 0;
        __syncthreads();
        bool any = false;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const Inst<T> &I = inst[i];
            if (!I.active) continue;
            const int64_t s = I.k + it;
            const SweepSlot *p = slot_of(I, s - 1);
            if (!sweep_stops(__ldcg(&p->fmax), __ldcg(&p->fmin), __ldcg(&p->fdir), __ldcg(&p->progressed), s,
                             I.max_sweeps)) {
                atomicOr(&mask[i >> 5], 1u << (i & 31));
                any = true;
            }
        }
        if (!__syncthreads_or(any)) break;
        multi_phase<CgLoads, T, 0>(sm, inst, rpre, n, total_rounds, mask, it);
        grid.sync();
        multi_phase<CgLoads, T, 1>(sm, inst, rpre, n, total_rounds, mask, it);
        grid.sync();
        ++it;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *iters = it;
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
template <typename T>
int MultiRun<T>::setup(const std::vector<FieldSpec<T>> &specs, int64_t max_sweeps_, int q_, cudaStream_t s_) {
    s = s_;
    n = static_cast<int>(specs.size());
    max_sweeps = max_sweeps_;
    q = q_;
    if (n < 1 || n > kMaxBatch) return set_error(PMSZ_ERR_ARG, "batch size must be in 1..4096");
    host.assign(n, Inst<T>{});
    size_t zero_bytes = 0, other_bytes = 0;
    std::vector<size_t> o_cnt(n), o_req(n), o_a0(n), o_a1(n), o_codes(n), o_hp(n);
    auto take = [](size_t &acc, size_t bytes) {
        const size_t off = acc;
        acc += (bytes + 255) & ~static_cast<size_t>(255);
        return off;
    };
    tpre.assign(n + 1, 0);
    rpre.assign(n + 1, 0);
    uint64_t tiles = 0, rounds = 0;
    voxels = 0;
    for (const FieldSpec<T> &sp : specs) voxels += sp.nx * sp.ny * sp.nz;
    const int zc = tuned_batch_zchunk(voxels, n, sizeof(T));  // one first-pass launch covers the batch
    for (int i = 0; i < n; ++i) {
        Geom g = make_geom(specs[i].nx, specs[i].ny, specs[i].nz);
        g.zc = zc;
        o_cnt[i] = take(zero_bytes, g.n);
        o_req[i] = take(zero_bytes, 4 * g.nwords);
        o_a0[i] = take(zero_bytes, 4 * g.nwords);
        o_a1[i] = take(zero_bytes, 4 * g.nwords);
        o_codes[i] = take(other_bytes, g.n);
        o_hp[i] = take(other_bytes, 4 * g.n);
        Inst<T> &I = host[i];
        I.f = specs[i].f;
        I.fh = specs[i].fh;
        I.g = g;
        I.eps = static_cast<T>(specs[i].eb);
        I.delta = static_cast<T>(specs[i].eb / static_cast<double>(q));  // pMSz.cu:2814
        I.q = q;
        I.max_sweeps = max_sweeps;
        I.k = 0;
        I.active = 0;
        I.first = 1;
        I.stride = n;
        I.tiles_x = static_cast<uint32_t>(g.wpr);
        I.tiles_y = static_cast<uint32_t>((g.ny + kTY - 1) / kTY);
        const uint64_t tz = static_cast<uint64_t>((g.nz + g.zc - 1) / g.zc);
        tpre[i] = static_cast<uint32_t>(tiles);
        rpre[i] = static_cast<uint32_t>(rounds);
        tiles += static_cast<uint64_t>(I.tiles_x) * I.tiles_y * tz;
        rounds += (g.nwords + kRoundWords - 1) / kRoundWords;
        if (tiles >= (1ull << 31) || rounds >= (1ull << 31)) return set_error(PMSZ_ERR_ARG, "batch too large");
    }
    tpre[n] = static_cast<uint32_t>(tiles);
    rpre[n] = static_cast<uint32_t>(rounds);
    total_tiles = static_cast<uint32_t>(tiles);
    total_rounds = static_cast<uint32_t>(rounds);
    const size_t slot_bytes = sizeof(SweepSlot) * static_cast<size_t>(max_sweeps) * n;
    const size_t o_zero = ws.reserve<unsigned char>(zero_bytes + slot_bytes);
    const size_t o_other = ws.reserve<unsigned char>(other_bytes);
    const size_t o_inst = ws.reserve<Inst<T>>(n);
    const size_t o_pre = ws.reserve<uint32_t>(2 * (n + 1));
    const size_t o_iters = ws.reserve<long long>(1);
    std::vector<Geom> geoms(n);
    for (int i = 0; i < n; ++i) geoms[i] = host[i].g;
    std::vector<uint32_t> wpre;
    uint64_t total_voxels = 0;
    for (const Geom &g : geoms) total_voxels += g.n;
    lists = list_prefixes(geoms, wpre, ml.total_words);
    const size_t o_wpre = ws.reserve<uint32_t>(lists ? n + 1 : 0);
    const size_t o_cnts = ws.reserve<uint32_t>(lists ? kCompactBlocks : 0);
    const size_t o_list = ws.reserve<uint64_t>(lists ? total_voxels : 0);
    const size_t o_xlist = ws.reserve<uint64_t>(lists ? total_voxels : 0);
    const size_t o_lc = ws.reserve<uint32_t>(lists ? 4 : 0);
    const size_t o_state = ws.reserve<BatchState>(lists ? 1 : 0);
    int rc = ws.commit();
    if (rc) return rc;
    if (lists) {
        ml.wpre = ws.at<uint32_t>(o_wpre);
        ml.counts = ws.at<uint32_t>(o_cnts);
        ml.list = ws.at<uint64_t>(o_list);
        ml.xlist = ws.at<uint64_t>(o_xlist);
        ml.lc = ws.at<uint32_t>(o_lc);
        ml.state = ws.at<BatchState>(o_state);
        PMSZ_CUDA(cudaMemcpyAsync(ml.wpre, wpre.data(), wpre.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    }
    unsigned char *zero = ws.at<unsigned char>(o_zero), *other = ws.at<unsigned char>(o_other);
    slots = reinterpret_cast<SweepSlot *>(zero + zero_bytes);
    for (int i = 0; i < n; ++i) {
        Inst<T> &I = host[i];
        I.cnt = zero + o_cnt[i];
        I.req = reinterpret_cast<uint32_t *>(zero + o_req[i]);
        I.act0 = reinterpret_cast<uint32_t *>(zero + o_a0[i]);
        I.act1 = reinterpret_cast<uint32_t *>(zero + o_a1[i]);
        I.codes = other + o_codes[i];
        I.hp = reinterpret_cast<uint32_t *>(other + o_hp[i]);
        I.slots = slots + i;
    }
    dinst = ws.at<Inst<T>>(o_inst);
    dtpre = ws.at<uint32_t>(o_pre);
    drpre = dtpre + (n + 1);
    diters = ws.at<long long>(o_iters);
    zero_base = zero;
    zero_total = zero_bytes + slot_bytes;
    PMSZ_CUDA(cudaMemsetAsync(zero, 0, zero_bytes + slot_bytes, s));
    std::vector<uint32_t> pre(tpre);
    pre.insert(pre.end(), rpre.begin(), rpre.end());
    PMSZ_CUDA(cudaMemcpyAsync(dtpre, pre.data(), pre.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    return PMSZ_OK;
}

template <typename T>
int MultiRun<T>::push_table() {
    if (!pin) PMSZ_CUDA(cudaMallocHost(reinterpret_cast<void **>(&pin), 2 * host.size() * sizeof(Inst<T>)));
    Inst<T> *dst = pin + static_cast<size_t>(pin_next) * host.size();
    pin_next ^= 1;
    std::copy(host.begin(), host.end(), dst);
    PMSZ_CUDA(cudaMemcpyAsync(dinst, dst, host.size() * sizeof(Inst<T>), cudaMemcpyHostToDevice, s));
    return PMSZ_OK;
}

template <typename T>
int MultiRun<T>::set_zchunk(int zc) {
    uint64_t tiles = 0;
    for (int i = 0; i < n; ++i) {
        Inst<T> &I = host[i];
        I.g.zc = zc;
        tpre[i] = static_cast<uint32_t>(tiles);
        tiles += static_cast<uint64_t>(I.tiles_x) * I.tiles_y * static_cast<uint64_t>((I.g.nz + zc - 1) / zc);
        if (tiles >= (1ull << 31)) return set_error(PMSZ_ERR_ARG, "batch too large");
    }
    tpre[n] = static_cast<uint32_t>(tiles);
    total_tiles = static_cast<uint32_t>(tiles);
    PMSZ_CUDA(cudaMemcpyAsync(dtpre, tpre.data(), tpre.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    PMSZ_CUDA(cudaStreamSynchronize(s));  // tpre may change again right after
    return PMSZ_OK;
}

template <typename T>
int MultiRun<T>::tune_zchunk() {
    int m = 0;
    const int *cands = zchunk_candidates(&m);
    int maxnz = 1;
    for (const Inst<T> &I : host) maxnz = std::max(maxnz, I.g.nz);
    EventTimer et;
    int rc = et.init();
    if (rc) return rc;
    for (Inst<T> &I : host) {
        I.active = 1;
        I.first = 1;
        I.k = 0;
    }
    int best = cands[0];
    float best_ms = 0.f;
    for (int c = 0; c < m; ++c) {
        if ((rc = set_zchunk(cands[c]))) return rc;
        if ((rc = push_table())) return rc;
        float t_best = 0.f;
        for (int rep = 0; rep < 3; ++rep) {  // the first run of each candidate is a warm-up
            PMSZ_CUDA(cudaMemsetAsync(zero_base, 0, zero_total, s));
            PMSZ_CUDA(cudaEventRecord(et.ev[0], s));
            k_first_multi<T><<<total_tiles, dim3(kTX, kTY, 1), 0, s>>>(dinst, dtpre, n);
            PMSZ_CUDA(cudaGetLastError());
            PMSZ_CUDA(cudaEventRecord(et.ev[1], s));
            PMSZ_CUDA(cudaEventSynchronize(et.ev[1]));
            float t = 0.f;
            PMSZ_CUDA(cudaEventElapsedTime(&t, et.ev[0], et.ev[1]));
            if (rep > 0 && (t_best == 0.f || t < t_best)) t_best = t;
        }
        if (c == 0 || t_best < best_ms) {
            best_ms = t_best;
            best = cands[c];
        }
        if (cands[c] >= maxnz) break;  // deeper columns are one chunk for every field
    }
    record_batch_zchunk(voxels, n, sizeof(T), best);
    if ((rc = set_zchunk(best))) return rc;
    PMSZ_CUDA(cudaMemsetAsync(zero_base, 0, zero_total, s));
    return PMSZ_OK;
}

template <typename T>
int MultiRun<T>::read_rows(int64_t k, int64_t count, std::vector<SweepSlot> &out) {
    out.resize(static_cast<size_t>(count) * n);
    if (count > 0)
        PMSZ_CUDA(cudaMemcpyAsync(out.data(), slots + k * n, out.size() * sizeof(SweepSlot), cudaMemcpyDeviceToHost,
                                  s));
    PMSZ_CUDA(cudaStreamSynchronize(s));
    return PMSZ_OK;
}

template <typename T>
int MultiRun<T>::read_row(int64_t k, std::vector<SweepSlot> &row) {
    row.resize(n);
    PMSZ_CUDA(cudaMemcpyAsync(row.data(), slots + k * n, n * sizeof(SweepSlot), cudaMemcpyDeviceToHost, s));
    PMSZ_CUDA(cudaStreamSynchronize(s));
    return PMSZ_OK;
}

// Gathers the slot of each field's current sweep (index k) into out[i].
template <typename T>
__global__ void k_gather_slots(const Inst<T> *__restrict__ inst, int n, SweepSlot *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = *slot_of(inst[i], inst[i].k);
}

template <typename T>
int launch_generation(const Inst<T> *dinst, const uint32_t *dtpre, const uint32_t *drpre, int n,
                      uint32_t total_tiles, uint32_t total_rounds, bool any_first, cudaStream_t s,
                      const MultiLists *ml) {
    if (any_first) k_first_multi<T><<<total_tiles, dim3(kTX, kTY, 1), 0, s>>>(dinst, dtpre, n);
    if (ml) return launch_list_sweep<T>(dinst, n, *ml, s);
    const unsigned grid = static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>(total_rounds, 152 * 16)));
    k_phase_multi<T, 0><<<grid, kListBlock, 0, s>>>(dinst, drpre, n, total_rounds);
    k_phase_multi<T, 1><<<grid, kListBlock, 0, s>>>(dinst, drpre, n, total_rounds);
    PMSZ_CUDA(cudaGetLastError());
    return PMSZ_OK;
}

template <typename T>
int launch_gather(const Inst<T> *dinst, int n, SweepSlot *out, cudaStream_t s) {
    k_gather_slots<T><<<(n + 127) / 128, 128, 0, s>>>(dinst, n, out);
    PMSZ_CUDA(cudaGetLastError());
    return PMSZ_OK;
}

template int launch_generation<float>(const Inst<float> *, const uint32_t *, const uint32_t *, int, uint32_t,
                                      uint32_t, bool, cudaStream_t, const MultiLists *);
template int launch_generation<double>(const Inst<double> *, const uint32_t *, const uint32_t *, int, uint32_t,
                                       uint32_t, bool, cudaStream_t, const MultiLists *);
template int launch_gather<float>(const Inst<float> *, int, SweepSlot *, cudaStream_t);
template int launch_gather<double>(const Inst<double> *, int, SweepSlot *, cudaStream_t);

template <typename T>
int MultiRun<T>::generation() {
    int rc = push_table();
    if (rc) return rc;
    bool any_first = false;
    for (const Inst<T> &I : host) any_first |= I.first != 0;
    if ((rc = launch_generation<T>(dinst, dtpre, drpre, n, total_tiles, total_rounds, any_first, s,
                                   lists ? &ml : nullptr)))
        return rc;
    for (Inst<T> &I : host) I.first = 0;
    return PMSZ_OK;
}

template <typename T>
int MultiRun<T>::loop(int64_t *iters) {
    int rc = push_table();
    if (rc) return rc;
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    PMSZ_CUDA(cudaGetDevice(&dev));
    PMSZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PMSZ_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return set_error(PMSZ_ERR_CUDA, "device does not support cooperative launches");
    PMSZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_loop_multi<T>, kListBlock, 0));
    if (per_sm < 1) return set_error(PMSZ_ERR_CUDA, "loop kernel does not fit on an SM");
    const unsigned grid = static_cast<unsigned>(
        std::max<size_t>(1, std::min<size_t>(total_rounds, static_cast<size_t>(per_sm) * sms)));
    const Inst<T> *a0 = dinst;
    const uint32_t *a1 = drpre;
    int a2 = n;
    uint32_t a3 = total_rounds;
    long long *a4 = diters;
    void *args[] = {&a0, &a1, &a2, &a3, &a4};
    PMSZ_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(k_loop_multi<T>), dim3(grid),
                                          dim3(kListBlock), args, 0, s));
    long long h = 0;
    PMSZ_CUDA(cudaMemcpyAsync(&h, diters, sizeof(h), cudaMemcpyDeviceToHost, s));
    PMSZ_CUDA(cudaStreamSynchronize(s));
    *iters = h;
    return PMSZ_OK;
}

template <typename T>
int MultiRun<T>::enqueue_loop(long long *hiters) {
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    PMSZ_CUDA(cudaGetDevice(&dev));
    PMSZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PMSZ_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return set_error(PMSZ_ERR_CUDA, "device does not support cooperative launches");
    PMSZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_loop_multi<T>, kListBlock, 0));
    if (per_sm < 1) return set_error(PMSZ_ERR_CUDA, "loop kernel does not fit on an SM");
    const unsigned grid = static_cast<unsigned>(
        std::max<size_t>(1, std::min<size_t>(total_rounds, static_cast<size_t>(per_sm) * sms)));
    const Inst<T> *a0 = dinst;
    const uint32_t *a1 = drpre;
    int a2 = n;
    uint32_t a3 = total_rounds;
    long long *a4 = diters;
    void *args[] = {&a0, &a1, &a2, &a3, &a4};
    PMSZ_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(k_loop_multi<T>), dim3(grid),
                                          dim3(kListBlock), args, 0, s));
    PMSZ_CUDA(cudaMemcpyAsync(hiters, diters, sizeof(long long), cudaMemcpyDeviceToHost, s));
    return PMSZ_OK;
}

template struct MultiRun<float>;
template struct MultiRun<double>;

// The list form of a batch: generation 0 (first passes and the first edits)
// on the stream, then the generations as a CUDA graph whose while node
// repeats one generation and k_batch_gate until the gate stops it -- no host
// round trip per generation; the graph is built while generation 0 runs.
// What the gate leaves (small active sets) goes to the cooperative tail.  The
// sweep logs and statuses are rebuilt afterwards from the slot rows, with the
// stop rule the gate and the tail applied.
template <typename T>
static int run_gated(MultiRun<T> &run, int64_t max_sweeps, std::vector<BatchOutcome> &out) {
    const int n = run.n;
    cudaStream_t s = run.s;
    size_t total_n = 0;
    for (const Inst<T> &I : run.host) total_n += I.g.n;
    const unsigned long long tail_at = std::max<unsigned long long>(total_n / 32, 1ull << 16);
    BatchState *st = run.ml.state;
    PMSZ_CUDA(cudaMemsetAsync(st, 0, sizeof(BatchState), s));
    PMSZ_CUDA(cudaMemsetAsync(&st->go, 1, 1, s));  // generation 0 runs (little-endian int 1)
    int rc = run.generation();
    if (rc) return rc;
    k_batch_gate<T><<<1, 256, 0, s>>>(run.dinst, n, st, max_sweeps, tail_at, cudaGraphConditionalHandle{}, 0);
    PMSZ_CUDA(cudaGetLastError());

    struct GraphGuard {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaStream_t cs = nullptr;
        ~GraphGuard() {
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            if (cs) cudaStreamDestroy(cs);
        }
    } gg;
    PMSZ_CUDA(cudaGraphCreate(&gg.graph, 0));
    cudaGraphConditionalHandle cond;
    PMSZ_CUDA(cudaGraphConditionalHandleCreate(&cond, gg.graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode;
    PMSZ_CUDA(cudaGraphAddNode(&wnode, gg.graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    PMSZ_CUDA(cudaStreamCreateWithFlags(&gg.cs, cudaStreamNonBlocking));
    PMSZ_CUDA(cudaStreamBeginCaptureToGraph(gg.cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    // the body runs once even when generation 0's gate stopped: its kernels
    // then see go == 0 and return at once
    if ((rc = launch_list_sweep<T>(run.dinst, n, run.ml, gg.cs, &st->go))) {
        cudaStreamEndCapture(gg.cs, &body);
        return rc;
    }
    k_batch_gate<T><<<1, 256, 0, gg.cs>>>(run.dinst, n, st, max_sweeps, tail_at, cond, 1);
    PMSZ_CUDA(cudaStreamEndCapture(gg.cs, &body));
    PMSZ_CUDA(cudaGraphInstantiate(&gg.exec, gg.graph, 0));
    PMSZ_CUDA(cudaGraphLaunch(gg.exec, s));

    // The rest of the live fields in the cooperative tail, enqueued at once:
    // it reads the table the last gate left on the device and, with no field
    // left running, ends at its first iteration.  One read-back follows.
    unsigned char *hb = static_cast<unsigned char *>(host_pinned(128 + sizeof(BatchState)));
    if (!hb) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
    long long *hiters = reinterpret_cast<long long *>(hb);
    BatchState *hs = reinterpret_cast<BatchState *>(hb + 128);
    if ((rc = run.enqueue_loop(hiters))) return rc;
    PMSZ_CUDA(cudaMemcpyAsync(hs, st, sizeof(BatchState), cudaMemcpyDeviceToHost, s));
    PMSZ_CUDA(cudaStreamSynchronize(s));
    const int64_t total = hs->k + *hiters;  // generations 0 .. hs->k - 1, then the tail's iterations
    std::vector<SweepSlot> rows;
    if ((rc = run.read_rows(0, total, rows))) return rc;
    for (int i = 0; i < n; ++i) {
        for (int64_t k = 0; k < total; ++k) {
            const SweepSlot &h = rows[static_cast<size_t>(k) * n + i];
            out[i].log.push_back(h);
            if (k == 0 && h.bad) {
                out[i].status = PMSZ_ERR_ARG;
                out[i].message = "input contains NaN or the value 1e30 (the reference's halo sentinel)";
                break;
            }
            if (sweep_stops(h.fmax, h.fmin, h.fdir, h.progressed, k + 1, max_sweeps)) break;
        }
    }
    return PMSZ_OK;
}

// Corrects a batch of same-type fields: first pass, host-driven sweeps while
// the batch's next active sets are large, then the cooperative tail loop.
template <typename T>
int batch_impl(const std::vector<FieldSpec<T>> &specs, const pmsz_opts *opts, std::vector<BatchOutcome> &out,
               cudaStream_t s) {
    const int q = opts ? opts->q : 5;
    const int64_t max_sweeps = opts && opts->max_sweeps > 0 ? opts->max_sweeps : 10000;
    if (q < 1 || q > 255) return set_error(PMSZ_ERR_ARG, "q must be in 1..255");
    int rc = PMSZ_OK;
    const bool tune = opts && (opts->flags & PMSZ_FLAG_AUTOTUNE);
    if (tune)  // the first field of each untuned shape class tunes it (its single-call parameters)
        for (const FieldSpec<T> &sp : specs)
            if (!tune_known(sp.nx, sp.ny, sp.nz, sizeof(T)) &&
                (rc = autotune_impl<T>(sp.f, sp.fh, sp.nx, sp.ny, sp.nz, nullptr, s)))
                return rc;
    MultiRun<T> run(s);
    rc = run.setup(specs, max_sweeps, q, s);
    if (rc) return rc;
    if (tune && !batch_tune_known(run.voxels, run.n, sizeof(T)) && (rc = run.tune_zchunk())) return rc;
    const int n = run.n;
    out.assign(n, BatchOutcome{});
    for (Inst<T> &I : run.host) {
        I.active = 1;
        I.first = 1;
        I.k = 0;
    }
    if (run.lists) {
        if ((rc = run_gated<T>(run, max_sweeps, out))) return rc;
    } else {
        if ((rc = run.generation())) return rc;
        std::vector<SweepSlot> row;
        int64_t k = 0;
        size_t total_n = 0;
        for (const Inst<T> &I : run.host) total_n += I.g.n;
        // decisions after each host-driven sweep
        while (true) {
            if ((rc = run.read_row(k, row))) return rc;
            unsigned long long est = 0;
            int live = 0;
            for (int i = 0; i < n; ++i) {
                Inst<T> &I = run.host[i];
                if (!I.active) continue;
                const SweepSlot &h = row[i];
                out[i].log.push_back(h);
                if (k == 0 && h.bad) {
                    I.active = 0;
                    out[i].status = PMSZ_ERR_ARG;
                    out[i].message = "input contains NaN or the value 1e30 (the reference's halo sentinel)";
                    continue;
                }
                if (sweep_stops(h.fmax, h.fmin, h.fdir, h.progressed, k + 1, max_sweeps)) {
                    I.active = 0;
                    continue;
                }
                I.k = k + 1;
                est += 15ull * h.changed + h.fdir;
                ++live;
            }
            ++k;
            if (!live) break;
            if (est <= std::max<unsigned long long>(total_n / 32, 1ull << 16)) {
                int64_t iters = 0;
                if ((rc = run.loop(&iters))) return rc;
                // rebuild each live field's tail from the slot rows
                std::vector<SweepSlot> rows;
                if ((rc = run.read_rows(k, iters, rows))) return rc;
                for (int i = 0; i < n; ++i) {
                    Inst<T> &I = run.host[i];
                    if (!I.active) continue;
                    for (int64_t j = 0; j < iters; ++j) {
                        const SweepSlot &h = rows[static_cast<size_t>(j) * n + i];
                        out[i].log.push_back(h);
                        if (sweep_stops(h.fmax, h.fmin, h.fdir, h.progressed, k + j + 1, max_sweeps)) break;
                    }
                    I.active = 0;
                }
                break;
            }
            if ((rc = run.generation())) return rc;
        }
    }
    for (int i = 0; i < n; ++i) {
        BatchOutcome &o = out[i];
        if (o.status == PMSZ_ERR_ARG) continue;
        const SweepSlot &last = o.log.back();
        if (last.fmax == 0 && last.fmin == 0 && last.fdir == 0) {
            o.status = PMSZ_OK;
        } else {
            o.status = PMSZ_ERR_NOT_CONVERGED;
            o.message = last.progressed == 0 ? "a sweep requested edits that changed nothing (all requested vertices clamped)"
                                             : "max_sweeps reached before convergence";
        }
    }
    return run.ws.release();
}

template int batch_impl<float>(const std::vector<FieldSpec<float>> &, const pmsz_opts *, std::vector<BatchOutcome> &,
                               cudaStream_t);
template int batch_impl<double>(const std::vector<FieldSpec<double>> &, const pmsz_opts *,
                                std::vector<BatchOutcome> &, cudaStream_t);

static void fill_result(const BatchOutcome &o, pmsz_result *res) {
    if (!res) return;
    res->sweeps = static_cast<int64_t>(o.log.size());
    res->iteration = res->sweeps + 1;
    uint64_t e = 0;
    for (const SweepSlot &h : o.log) e += h.requested;
    res->edits = e;
    if (res->sweep_log && res->sweep_log_cap > 0) {
        const size_t m = std::min<size_t>(o.log.size(), static_cast<size_t>(res->sweep_log_cap));
        std::memcpy(res->sweep_log, o.log.data(), m * sizeof(SweepSlot));
    }
    res->ms_first_pass = res->ms_detect = res->ms_apply = res->ms_total = 0.0;
    res->launches = 0;
}

int correct_batch(const pmsz_field *fields, int count, const pmsz_opts *opts, pmsz_result *results, int *statuses,
                  cudaStream_t s) {
    if (!fields || count < 1) return set_error(PMSZ_ERR_ARG, "empty batch");
    std::vector<int> st(count, PMSZ_OK);
    std::vector<FieldSpec<float>> f32;
    std::vector<FieldSpec<double>> f64;
    std::vector<int> i32, i64;
    for (int i = 0; i < count; ++i) {
        const pmsz_field &F = fields[i];
        int rc = check_geom(F.nx, F.ny, F.nz);
        if (!rc && (!F.f || !F.fhat)) rc = set_error(PMSZ_ERR_ARG, "null field pointer");
        if (!rc && (!(F.eb > 0.0) || !(F.eb < 1e300))) rc = set_error(PMSZ_ERR_ARG, "error bound must be positive and finite");
        if (!rc && F.elem_size != 4 && F.elem_size != 8) rc = set_error(PMSZ_ERR_ARG, "elem_size must be 4 or 8");
        if (rc) {
            st[i] = rc;
            continue;
        }
        if (F.elem_size == 4) {
            f32.push_back({static_cast<const float *>(F.f), static_cast<float *>(F.fhat), F.nx, F.ny, F.nz, F.eb});
            i32.push_back(i);
        } else {
            f64.push_back({static_cast<const double *>(F.f), static_cast<double *>(F.fhat), F.nx, F.ny, F.nz, F.eb});
            i64.push_back(i);
        }
    }
    std::vector<BatchOutcome> o32, o64;
    int rc = PMSZ_OK;
    if (!f32.empty() && (rc = batch_impl<float>(f32, opts, o32, s))) return rc;
    if (!f64.empty() && (rc = batch_impl<double>(f64, opts, o64, s))) return rc;
    for (size_t j = 0; j < i32.size(); ++j) {
        st[i32[j]] = o32[j].status;
        fill_result(o32[j], results ? results + i32[j] : nullptr);
    }
    for (size_t j = 0; j < i64.size(); ++j) {
        st[i64[j]] = o64[j].status;
        fill_result(o64[j], results ? results + i64[j] : nullptr);
    }
    int worst = PMSZ_OK;
    for (int i = 0; i < count; ++i) {
        if (statuses) statuses[i] = st[i];
        if (st[i] != PMSZ_OK && worst == PMSZ_OK) worst = st[i];
    }
    for (const auto *o : {&o32, &o64})
        for (const BatchOutcome &b : *o)
            if (b.status != PMSZ_OK && !b.message.empty()) set_error(b.status, b.message);
    return worst;
}

}  // namespace pmsz

using namespace pmsz;

extern "C" int pmsz_correct_batch(const pmsz_field *fields, int count, const pmsz_opts *opts, pmsz_result *results,
                                  int *statuses, void *stream) {
    return guarded([&] { return correct_batch(fields, count, opts, results, statuses, as_stream(stream)); });
}
