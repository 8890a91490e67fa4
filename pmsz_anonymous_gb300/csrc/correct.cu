// correct.cu -- labelling, detection and edit kernels and the correction loop.
//
// Replaces iscriticle (pMSz.cu:649-899), applyDeltaBuffer_local
// (pMSz.cu:623-645), init_edits / init_counter (pMSz.cu:902-906, 1745-1749) and
// the host loop c_loops (pMSz.cu:1872-2074) at an MPI grid of 1x1x1.
//
// Sweep k (snapshot semantics):
//   detect   every voxel u of the active set A_k reads fhat on its closed
//            stencil N[u] and the original direction code of u, applies the
//            reference rules, ORs the vertices it wants lowered into the
//            request bitmap R, and sets u in M_k (the next active bitmap) if
//            it mismatched.
//   apply    every vertex in R is edited once (applyDeltaBuffer_local); R is
//            cleared; the closed stencil of every vertex whose value changed
//            is ORed into the next active bitmap.
// A voxel whose stencil did not change keeps its previous outcome, so
// A_{k+1} = M_k U N[C_k] (C_k = changed vertices) yields exactly the requests
// and counters of a full sweep over all voxels.  Sweep 1 is a full pass fused
// with the original labelling: it reads f and fhat once and writes the codes.
// PMSZ_FLAG_FULL_SWEEPS replaces the active set by the whole field.
#include "common.cuh"
#include "../../include/pmsz.h"
#include "helpers.cuh"
#include "internal.h"

#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled

#include <algorithm>
#include <cstring>
#include <chrono>
#include <mutex>
#include <string>
#include <vector>

namespace pmsz {

// ---------------------------------------------------------------------------
// Full detection pass over a 3-D grid: block (32, 8), one warp per 32-voxel
// x-segment, which is exactly one bitmap word.  FIRST: also label the
// original field f and store the code byte (iscriticle data_type=1 fused with
// the first data_type=0 pass).
// ---------------------------------------------------------------------------
template <typename T, bool FIRST>
__global__ void __launch_bounds__(256) k_detect_full(const T *__restrict__ f, const T *__restrict__ fh,
                                                     uint8_t *__restrict__ codes, uint32_t *__restrict__ req,
                                                     uint32_t *__restrict__ act_next, SweepSlot *slot, Geom g) {
    using K = typename KeyOf<T>::type;
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    const bool in = x < g.nx && y < g.ny;
    uint32_t cmax = 0, cmin = 0, cdir = 0, bad = 0;
    uint32_t tm = 0;
    if (in) {
        const size_t i = flat(g, x, y, z);
        const uint32_t valid = valid_mask(x, y, z, g.nx, g.ny, g.nz);
        int oasc, odesc;
        K k[15];
        if (FIRST) {
            load_keys(f, i, g, valid, k);
            arg_ext(k, valid, oasc, odesc);
            codes[i] = static_cast<uint8_t>(oasc | (odesc << 4));
            bad = bad_value(f[i]) || bad_value(fh[i]);
        } else {
            const uint8_t c = codes[i];
            oasc = c & 15;
            odesc = c >> 4;
        }
        int asc, desc;
        load_keys(fh, i, g, valid, k);
        arg_ext(k, valid, asc, desc);
        tm = detect_rules(asc, desc, oasc, odesc, cmax, cmin, cdir);
        if (tm) request_targets(req, g, x, y, z, tm);
    }
    const uint32_t mism = __ballot_sync(0xFFFFFFFFu, tm != 0);
    if (threadIdx.x == 0 && y < g.ny && mism) act_next[word_of(g, blockIdx.x * 32, y, z)] = mism;
    flush_counts(slot, cmax, cmin, cdir, in ? 1u : 0u, bad);
}

// ---------------------------------------------------------------------------
// Sparse detection over the active bitmap (grid-stride over words).  The
// word's bits are consumed and cleared; mismatching voxels go to act_next
// (only this thread touches that word of act_next in this kernel).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_detect_sparse(const T *__restrict__ fh, const uint8_t *__restrict__ codes,
                                                       uint32_t *__restrict__ act_cur, uint32_t *__restrict__ act_next,
                                                       uint32_t *__restrict__ req, SweepSlot *slot, Geom g) {
    using K = typename KeyOf<T>::type;
    uint32_t cmax = 0, cmin = 0, cdir = 0, active = 0;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t w = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; w < g.nwords; w += stride) {
        uint32_t bits = act_cur[w];
        if (!bits) continue;
        act_cur[w] = 0;
        const size_t row = w / g.wpr;
        const int wx = static_cast<int>(w - row * g.wpr);
        const int y = static_cast<int>(row % g.ny);
        const int z = static_cast<int>(row / g.ny);
        uint32_t mism = 0;
        active += __popc(bits);
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            const int x = wx * 32 + b;
            const size_t i = flat(g, x, y, z);
            const uint32_t valid = valid_mask(x, y, z, g.nx, g.ny, g.nz);
            K k[15];
            load_keys(fh, i, g, valid, k);
            int asc, desc;
            arg_ext(k, valid, asc, desc);
            const uint8_t c = codes[i];
            const uint32_t tm = detect_rules(asc, desc, c & 15, c >> 4, cmax, cmin, cdir);
            if (tm) {
                request_targets(req, g, x, y, z, tm);
                mism |= 1u << b;
            }
        }
        if (mism) act_next[w] = mism;
    }
    flush_counts(slot, cmax, cmin, cdir, active, 0);
}

// ---------------------------------------------------------------------------
// Apply: applyDeltaBuffer_local (pMSz.cu:623-645) on every requested vertex,
// in T:  if |f - (fhat - delta)| <= eps && cnt < q-1 { fhat -= delta; cnt++ }
//        else { cnt = q; fhat = f - eps }
// then mark the closed stencil of every vertex whose value changed.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_apply(const T *__restrict__ f, T *__restrict__ fh, uint8_t *__restrict__ cnt,
                                               uint32_t *__restrict__ req, uint32_t *__restrict__ act_next,
                                               SweepSlot *slot, Geom g, T eps, T delta, int q) {
    uint32_t nreq = 0, nchg = 0, nprog = 0;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t w = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; w < g.nwords; w += stride) {
        uint32_t bits = req[w];
        if (!bits) continue;
        req[w] = 0;
        const size_t row = w / g.wpr;
        const int wx = static_cast<int>(w - row * g.wpr);
        const int y = static_cast<int>(row % g.ny);
        const int z = static_cast<int>(row / g.ny);
        nreq += __popc(bits);
        uint32_t changed = 0;
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            bool prog;
            const uint32_t c = apply_one(f, fh, cnt, flat(g, wx * 32 + b, y, z), eps, delta, q, prog);
            changed |= c << b;
            nprog += prog ? 1u : 0u;
        }
        nchg += __popc(changed);
        if (changed) mark_stencil(act_next, g, wx, y, z, changed);
    }
    nreq = warp_sum_u32(nreq);
    nchg = warp_sum_u32(nchg);
    nprog = warp_sum_u32(nprog);
    if ((threadIdx.x & 31) == 0) {
        if (nreq) atomicAdd(&slot->requested, (unsigned long long)nreq);
        if (nchg) atomicAdd(&slot->changed, (unsigned long long)nchg);
        if (nprog) atomicAdd(&slot->progressed, (unsigned long long)nprog);
    }
}

// Codes only (pmsz_codes): the labelling half of the first pass.
template <typename T>
__global__ void __launch_bounds__(256) k_codes(const T *__restrict__ v, uint8_t *__restrict__ codes, Geom g) {
    using K = typename KeyOf<T>::type;
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= g.nx || y >= g.ny) return;
    const size_t i = flat(g, x, y, z);
    const uint32_t valid = valid_mask(x, y, z, g.nx, g.ny, g.nz);
    K k[15];
    load_keys(v, i, g, valid, k);
    int a, d;
    arg_ext(k, valid, a, d);
    codes[i] = static_cast<uint8_t>(a | (d << 4));
}

}  // namespace pmsz

#include "tail.cuh"

namespace pmsz {

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
static inline dim3 grid3(const Geom &g) {
    return dim3(static_cast<unsigned>(g.wpr), static_cast<unsigned>((g.ny + 7) / 8), static_cast<unsigned>(g.nz));
}

static inline unsigned stride_grid(size_t items) {
    const size_t want = (items + 255) / 256;
    return static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>(want, 152 * 16)));
}

// Tensor maps of f and fhat for the TMA-fed first pass (k_first_tma): 3-D
// (nx, ny, nz) maps with a box of one tile plane.  The encoder is the driver's
// cuTensorMapEncodeTiled, reached through the runtime (the library does not
// link libcuda).  Not available (ok = false: the first pass loads its tiles
// itself) when the encoder is missing, the fields are not 16-byte aligned or
// a row is not a multiple of 16 bytes.
struct FirstMaps {
    CUtensorMap f, fh;
    bool ok = false;
};

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

template <typename T>
static FirstMaps first_maps(const T *f, const T *fh, const Geom &g) {
    FirstMaps m;
    const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || (static_cast<size_t>(g.nx) * sizeof(T)) % 16 || reinterpret_cast<uintptr_t>(f) % 16 ||
        reinterpret_cast<uintptr_t>(fh) % 16)
        return m;
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(g.nx), static_cast<cuuint64_t>(g.ny),
                                static_cast<cuuint64_t>(g.nz)};
    const cuuint64_t strides[2] = {static_cast<cuuint64_t>(g.nx) * sizeof(T),
                                   static_cast<cuuint64_t>(g.nx) * g.ny * sizeof(T)};
    const cuuint32_t box[3] = {static_cast<cuuint32_t>(RawBox<T>::kX), static_cast<cuuint32_t>(kHY), 1u};
    const cuuint32_t es[3] = {1u, 1u, 1u};
    const CUtensorMapDataType dt = sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    for (int k = 0; k < 2; ++k)
        if (enc(k ? &m.fh : &m.f, dt, 3, const_cast<T *>(k ? fh : f), dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return m;
    m.ok = true;
    return m;
}

// The deferring first pass over the z-chunks bz0 .. bz0+grid.z-1: TMA-fed
// interior blocks when the maps exist; *err is set if a plane's copy did not
// arrive within the bounded wait.
template <typename T>
static void launch_first_pass(const FirstMaps &m, dim3 grid, cudaStream_t s, const T *f, T *fh, uint8_t *codes,
                              uint32_t *hp, uint32_t *req, uint32_t *act, SweepSlot *slot, const Geom &g, int bz0,
                              uint32_t *xl, uint32_t *xc, uint32_t *err) {
    const dim3 blk(kTX, kTY, 1);
    if (m.ok)
        k_first_tma<T><<<grid, blk, 0, s>>>(m.f, m.fh, f, fh, codes, hp, req, act, slot, g, bz0, xl, xc, err);
    else
        k_tiled<T, kFirst, true><<<grid, blk, 0, s>>>(f, fh, codes, hp, req, act, slot, g, bz0, xl, xc);
}

// Runs sweeps first.. in one cooperative launch of k_tail_loop (grid = the
// number of co-resident blocks) after summarising the active bitmap of sweep
// `first`; *done receives the total number of sweeps.
template <typename T>
static int run_sweep_loop(const T *f, T *fh, const uint8_t *codes, uint8_t *cnt, uint32_t *hp, uint32_t *req,
                          uint32_t *const act[2], SweepSlot *slots, int64_t first, int64_t max_sweeps, const Geom &g,
                          T eps, T delta, int q, cudaStream_t s, EventTimer *et, double *ms_acc, int64_t *done) {
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    PMSZ_CUDA(cudaGetDevice(&dev));
    PMSZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PMSZ_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return set_error(PMSZ_ERR_CUDA, "device does not support cooperative launches");
    PMSZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tail_loop<T>, kTailBlock, 0));
    if (per_sm < 1) return set_error(PMSZ_ERR_CUDA, "sweep loop kernel does not fit on an SM");
    const size_t ns = summary_words(g);
    const unsigned grid = static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>(ns, static_cast<size_t>(per_sm) * sms)));
    long long *d_done = nullptr;
    Workspace ws(s);
    const size_t o_done = ws.reserve<long long>(1);
    const size_t o_sum = ws.reserve<uint32_t>(3 * ns);
    int rc = ws.commit();
    if (rc) return rc;
    d_done = ws.at<long long>(o_done);
    uint32_t *sum = ws.at<uint32_t>(o_sum);  // summaries of act[0], act[1], req
    if (et) PMSZ_CUDA(cudaEventRecord(et->ev[0], s));
    PMSZ_CUDA(cudaMemsetAsync(sum, 0, 3 * ns * sizeof(uint32_t), s));
    const int c = static_cast<int>(first & 1);
    k_build_summary<<<static_cast<unsigned>(std::min<size_t>((ns + 7) / 8, 152 * 16)), 256, 0, s>>>(
        act[c], g, sum + static_cast<size_t>(c) * ns);
    PMSZ_CUDA(cudaGetLastError());
    TailArgs<T> a{f,    fh,        codes, cnt, hp,    req, act[0], act[1], sum + 2 * ns, sum, sum + ns,
                  slots, first, max_sweeps, d_done, g,  eps, delta,  q};
    void *args[] = {&a};
    PMSZ_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(k_tail_loop<T>), dim3(grid), dim3(kTailBlock),
                                          args, 0, s));
    if (et) PMSZ_CUDA(cudaEventRecord(et->ev[1], s));
    long long h = 0;
    PMSZ_CUDA(cudaMemcpyAsync(&h, d_done, sizeof(h), cudaMemcpyDeviceToHost, s));
    PMSZ_CUDA(cudaStreamSynchronize(s));
    if (et) {
        float ms = 0;
        PMSZ_CUDA(cudaEventElapsedTime(&ms, et->ev[0], et->ev[1]));
        *ms_acc += ms;
    }
    *done = h;
    return ws.release();
}

// The cooperative tail behind the list sweeps, enqueued without waiting for
// the host: it starts at sweep ls->k and runs only if the last gate handed
// over to it (ls->tail); *hdone (pinned host memory) receives the total
// number of sweeps once the stream gets there.
template <typename T>
static int enqueue_gated_tail(const T *f, T *fh, const uint8_t *codes, uint8_t *cnt, uint32_t *hp, uint32_t *req,
                              uint32_t *const act[2], SweepSlot *slots, const LoopState *ls, int64_t max_sweeps,
                              const Geom &g, T eps, T delta, int q, cudaStream_t s, EventTimer *et, long long *hdone) {
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    PMSZ_CUDA(cudaGetDevice(&dev));
    PMSZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PMSZ_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return set_error(PMSZ_ERR_CUDA, "device does not support cooperative launches");
    PMSZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tail_loop<T>, kTailBlock, 0));
    if (per_sm < 1) return set_error(PMSZ_ERR_CUDA, "sweep loop kernel does not fit on an SM");
    const size_t ns = summary_words(g);
    const unsigned grid = static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>(ns, static_cast<size_t>(per_sm) * sms)));
    Workspace ws(s);
    const size_t o_done = ws.reserve<long long>(1);
    const size_t o_sum = ws.reserve<uint32_t>(3 * ns);
    int rc = ws.commit();
    if (rc) return rc;
    long long *d_done = ws.at<long long>(o_done);
    uint32_t *sum = ws.at<uint32_t>(o_sum);  // summaries of act[0], act[1], req
    if (et) PMSZ_CUDA(cudaEventRecord(et->ev[0], s));
    PMSZ_CUDA(cudaMemsetAsync(sum, 0, 3 * ns * sizeof(uint32_t), s));
    k_build_summary_at<<<static_cast<unsigned>(std::min<size_t>((ns + 7) / 8, 152 * 16)), 256, 0, s>>>(
        act[0], act[1], g, sum, sum + ns, &ls->k, &ls->tail);
    PMSZ_CUDA(cudaGetLastError());
    TailArgs<T> a{f,    fh,        codes, cnt, hp,    req, act[0], act[1], sum + 2 * ns, sum, sum + ns,
                  slots, 0, max_sweeps, d_done, g,  eps, delta,  q};
    a.first_at = &ls->k;
    a.run_if = &ls->tail;
    void *args[] = {&a};
    PMSZ_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(k_tail_loop<T>), dim3(grid), dim3(kTailBlock),
                                          args, 0, s));
    if (et) PMSZ_CUDA(cudaEventRecord(et->ev[1], s));
    PMSZ_CUDA(cudaMemcpyAsync(hdone, d_done, sizeof(long long), cudaMemcpyDeviceToHost, s));
    return ws.release();
}

// Grid of the list-compaction kernels: one block per 2048-word round, at most
// 16 blocks per SM (grid-stride beyond).
static inline unsigned list_grid(const Geom &g) {
    const size_t want = (g.nwords + kRoundWords - 1) / kRoundWords;
    return static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>(want, 152 * 16)));
}

int check_geom(size_t nx, size_t ny, size_t nz) {
    if (nx == 0 || ny == 0 || nz == 0) return set_error(PMSZ_ERR_ARG, "field dimensions must be positive");
    if (nx > (1u << 30) || ny > 65535 * 8 || nz > 65535)
        return set_error(PMSZ_ERR_ARG, "field dimensions exceed the supported range (nz <= 65535)");
    if (((nx + 31) / 32) * ny * nz >= (static_cast<size_t>(1) << 32))
        return set_error(PMSZ_ERR_ARG, "field too large: ceil(nx/32)*ny*nz must stay below 2^32");
    return PMSZ_OK;
}

// Slabs of the host-buffer copy: whole z-chunks, about 64 MiB of f + fhat.
// The copy of slab j ends one plane past its chunks (planes b_j .. b_{j+1} - 1
// with b_j = j * cps * zc + 1, b_0 = 0, the last ending at nz), so the first
// pass of slab j's chunks, whose tiles read one plane beyond them, waits for
// the copy of slab j only: once the host link delivers the last slab, one
// slab's first pass is left, not two.
struct IngestSlabs {
    int cps, nchunks, nslabs;
};
static IngestSlabs ingest_slabs(const Geom &g, size_t elem) {
    const size_t plane = static_cast<size_t>(g.nx) * g.ny;
    const size_t chunk_bytes = 2 * plane * static_cast<size_t>(g.zc) * elem;
    IngestSlabs r;
    r.nchunks = (g.nz + g.zc - 1) / g.zc;
    r.cps = static_cast<int>(std::max<size_t>(1, (static_cast<size_t>(64) << 20) / chunk_bytes));
    r.nslabs = (r.nchunks + r.cps - 1) / r.cps;
    return r;
}
static size_t slab_begin(int j, int cps, int nslabs, int zc, size_t nz) {
    if (j <= 0) return 0;
    if (j >= nslabs) return nz;
    return std::min(nz, static_cast<size_t>(j) * cps * zc + 1);  // j * cps * zc < nz for j < nslabs
}

template <typename T>
int enqueue_ingest(const T *hf, const T *hfh, T *df, T *dfh, T *dprev, size_t nx, size_t ny, size_t nz,
                   cudaStream_t s, IngestCopies &c) {
    int rc = check_geom(nx, ny, nz);
    if (rc) return rc;
    Geom g = make_geom(nx, ny, nz);
    g.zc = tuned_zchunk(nx, ny, nz, sizeof(T));  // the tile depth correct_impl will use
    const IngestSlabs sl = ingest_slabs(g, sizeof(T));
    c.cps = sl.cps;
    c.nchunks = sl.nchunks;
    c.nslabs = sl.nslabs;
    c.zc = g.zc;
    const size_t plane = static_cast<size_t>(g.nx) * g.ny;
    // cs: host copies; ds: device copies of fhat into dprev (kept off cs so
    // the host link never idles behind them)
    PMSZ_CUDA(cudaStreamCreateWithFlags(&c.cs, cudaStreamNonBlocking));
    PMSZ_CUDA(cudaStreamCreateWithFlags(&c.ds, cudaStreamNonBlocking));
    c.ev.assign(static_cast<size_t>(c.nslabs) + 1, nullptr);
    c.evp.assign(static_cast<size_t>(c.nslabs), nullptr);
    for (cudaEvent_t &e : c.ev) PMSZ_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (cudaEvent_t &e : c.evp) PMSZ_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    PMSZ_CUDA(cudaEventRecord(c.ev[c.nslabs], s));  // the destinations are allocated
    PMSZ_CUDA(cudaStreamWaitEvent(c.cs, c.ev[c.nslabs], 0));
    for (int j = 0; j < c.nslabs; ++j) {
        const size_t z0 = slab_begin(j, c.cps, c.nslabs, g.zc, g.nz);
        const size_t z1 = slab_begin(j + 1, c.cps, c.nslabs, g.zc, g.nz);
        const size_t off = z0 * plane, bytes = (z1 - z0) * plane * sizeof(T);
        if (bytes) {
            PMSZ_CUDA(cudaMemcpyAsync(df + off, hf + off, bytes, cudaMemcpyHostToDevice, c.cs));
            PMSZ_CUDA(cudaMemcpyAsync(dfh + off, hfh + off, bytes, cudaMemcpyHostToDevice, c.cs));
        }
        PMSZ_CUDA(cudaEventRecord(c.ev[j], c.cs));
        if (dprev) {  // the pre-correction copy of fhat, before any edit of the slab
            PMSZ_CUDA(cudaStreamWaitEvent(c.ds, c.ev[j], 0));
            if (bytes)
                PMSZ_CUDA(cudaMemcpyAsync(dprev + off, dfh + off, bytes, cudaMemcpyDeviceToDevice, c.ds));
            PMSZ_CUDA(cudaEventRecord(c.evp[j], c.ds));
        } else {
            PMSZ_CUDA(cudaEventRecord(c.evp[j], c.cs));
        }
    }
    return PMSZ_OK;
}

// The fused first pass over a field that is still being copied in from the
// host (the copies of enqueue_ingest): the first pass of a slab's chunks waits
// for that slab's event (its copy includes the plane beyond the chunks).
template <typename T>
int first_pass_ingest(const HostIngest<T> &in, const T *f, T *fh, uint8_t *codes, uint32_t *hp, uint32_t *req,
                      uint32_t *a_next, SweepSlot *slot, const Geom &g, cudaStream_t s, int64_t *launches,
                      uint32_t *xlist, uint32_t *xcount, const FirstMaps *maps = nullptr, uint32_t *err = nullptr) {
    if (in.df != f || !in.copies || in.copies->zc != g.zc)
        return set_error(PMSZ_ERR_ARG, "ingest copies do not match the field");
    const IngestCopies &r = *in.copies;
    const int cps = r.cps, nchunks = r.nchunks, nslabs = r.nslabs;
    const dim3 blk3(kTX, kTY, 1);
    for (int j = 0; j < nslabs; ++j) {
        PMSZ_CUDA(cudaStreamWaitEvent(s, r.ev[j], 0));
        dim3 grid = tiled_grid(g);
        grid.z = static_cast<unsigned>(std::min(cps, nchunks - j * cps));
        if (xlist)  // deferring first pass (see k_first_exact)
            launch_first_pass<T>(*maps, grid, s, f, fh, codes, hp, req, a_next, slot, g, j * cps, xlist, xcount, err);
        else
            k_tiled<T, kFirst><<<grid, blk3, 0, s>>>(f, fh, codes, hp, req, a_next, slot, g, j * cps);
        PMSZ_CUDA(cudaGetLastError());
        ++*launches;
    }
    PMSZ_CUDA(cudaStreamWaitEvent(s, r.evp[nslabs - 1], 0));  // dprev complete before the first edit
    return PMSZ_OK;
}

// Sweeps pipelined behind the host copy (even: the graph's two-sweep body
// starts at an odd sweep), and the fractions of the slabs after which they
// advance: every piece of a sweep costs two compaction kernels and five more
// launches whatever its size, so the early waves are large and the late
// ones, whose remainder is all that is left once the copy ends, small (a
// wave per slab piled these fixed costs up behind the copy).
constexpr int kWaveSweeps = 6;
// in sixteenths of the slabs; fp32 slabs cross the link in half the time of
// fp64 slabs of as many voxels, while the sweeps cost about the same
constexpr int kWaveAt8[] = {4, 8, 12, 14, 16};
constexpr int kWaveAt4[] = {4, 8, 12, 16};

// One-thread bookkeeping between the pieces of the wavefront (kernels rather
// than small copies or memsets: a device-to-device copy may queue behind the
// host copies on the copy engine).
static __global__ void k_wave_mark(LoopState *ls) {
    if (threadIdx.x == 0 && blockIdx.x == 0) ls->xdone = ls->lc[3];
}
static __global__ void k_wave_clear_spills(LoopState *ls) {
    if (threadIdx.x == 0 && blockIdx.x == 0) ls->lc[2] = 0;
}

// The host-buffer wavefront.  The copy of slab j releases the first pass
// of slab j (sweep 0's detection, complete below plane Z = (j + 1) * slab
// depth, or nz after the last slab); after the slabs of kWaveAt8 / kWaveAt4
// follows a wave: on the planes already final, the pieces of sweeps 0 .. K that those
// planes allow:
//   sweep k's detection covers planes below D_k, its edits planes below A_k,
//   with D_0 = Z, A_k = D_k - 1 and D_k = A_{k-1} - 1 (k >= 1),
// every front reaching nz after the last slab.  Sweep k's detection reads
// planes up to D_k = A_{k-1} - 1, all edited by sweep k - 1 already; its
// edits stop one plane below D_k, so no later detection of sweep k reads an
// edited plane or requests an edit below A_k; the active set of sweep k + 1
// below D_{k+1} is final once sweep k has edited planes up to D_{k+1} + 1.
// Each sweep thus sees exactly the field, codes and active set of the
// snapshot schedule, and sweeps that run while the rest of the field is still
// crossing the host link leave little to do after it.  Counters go straight
// to slots[k]; k_wave_gate then sets the loop state as after sweep K.
template <typename T>
static int first_pass_waves(const HostIngest<T> &in, const T *f, T *fh, uint8_t *codes, uint8_t *cnt, uint32_t *hp,
                            uint32_t *req, uint32_t *const act[2], SweepSlot *slots, LoopState *ls, const Geom &g,
                            const FirstMaps &maps, uint32_t *list, uint32_t *xlist, uint32_t *slist, uint32_t *bcnt,
                            const FastDiv &div_nx, T eps, T delta, int q, int K, cudaStream_t s, int64_t *launches) {
    if (in.df != f || !in.copies || in.copies->zc != g.zc)
        return set_error(PMSZ_ERR_ARG, "ingest copies do not match the field");
    const IngestCopies &r = *in.copies;
    const int cps = r.cps, nchunks = r.nchunks, nslabs = r.nslabs;
    const unsigned lb = 152 * 8;
    std::vector<int> Dp(static_cast<size_t>(K) + 1, 0), Ap(static_cast<size_t>(K) + 1, 0);  // fronts so far
    std::vector<char> wave_after(static_cast<size_t>(nslabs), 0);
    auto mark = [&](int e) { wave_after[static_cast<size_t>(std::max(1, (nslabs * e + 15) / 16) - 1)] = 1; };
    if (sizeof(T) == 8)
        for (int e : kWaveAt8) mark(e);
    else
        for (int e : kWaveAt4) mark(e);
    for (int j = 0; j < nslabs; ++j) {
        const bool last = j == nslabs - 1;
        PMSZ_CUDA(cudaStreamWaitEvent(s, r.ev[j], 0));
        dim3 grid = tiled_grid(g);
        grid.z = static_cast<unsigned>(std::min(cps, nchunks - j * cps));
        launch_first_pass<T>(maps, grid, s, f, fh, codes, hp, req, act[1], &slots[0], g, j * cps, xlist, &ls->lc[3],
                             &ls->err);
        ++*launches;
        if (!wave_after[static_cast<size_t>(j)]) continue;
        // the first pass's deferred voxels so far (all below Z), then mark them done
        k_first_exact<T><<<lb, 256, 0, s>>>(xlist, &ls->lc[3], f, fh, codes, req, act[1], &slots[0], g, div_nx,
                                            &ls->xdone);
        k_wave_mark<<<1, 32, 0, s>>>(ls);
        PMSZ_CUDA(cudaGetLastError());
        *launches += 2;
        PMSZ_CUDA(cudaStreamWaitEvent(s, r.evp[j], 0));  // fhat's pre-correction copy of slabs 0 .. j
        const int Z = last ? g.nz : std::min(g.nz, (j + 1) * cps * g.zc);
        for (int k = 0; k <= K; ++k) {
            const int D = k == 0 ? Z : (last ? g.nz : std::max(0, Ap[k - 1] - 1));
            uint32_t *a_next = act[(k + 1) & 1];
            if (k > 0 && D > Dp[k]) {
                compact_bitmap_planes(act[k & 1], g, Dp[k], D, bcnt, list, &ls->lc[0], s);
                k_detect_list<T><<<lb, 256, 0, s>>>(list, &ls->lc[0], fh, hp, codes, req, a_next, slist, &ls->lc[2],
                                                    &slots[k], g, div_nx, nullptr, &ls->exact_keys, nullptr);
                k_detect_exact<T><<<lb, 256, 0, s>>>(slist, &ls->lc[2], fh, codes, req, a_next, &slots[k], g, div_nx,
                                                     nullptr);
                k_wave_clear_spills<<<1, 32, 0, s>>>(ls);
                *launches += 5;
            }
            Dp[k] = std::max(Dp[k], D);
            const int A = last ? g.nz : std::max(0, D - 1);
            if (A > Ap[k]) {
                compact_bitmap_planes(req, g, Ap[k], A, bcnt, list, &ls->lc[1], s);
                k_apply_list<T><<<lb, 256, 0, s>>>(list, &ls->lc[1], f, fh, cnt, hp, a_next, &slots[k], g, div_nx, eps,
                                                   delta, q, nullptr);
                *launches += 3;
                Ap[k] = A;
            }
            PMSZ_CUDA(cudaGetLastError());
        }
    }
    return PMSZ_OK;
}

template int enqueue_ingest<float>(const float *, const float *, float *, float *, float *, size_t, size_t, size_t,
                                   cudaStream_t, IngestCopies &);
template int enqueue_ingest<double>(const double *, const double *, double *, double *, double *, size_t, size_t,
                                    size_t, cudaStream_t, IngestCopies &);

template <typename T>
int correct_impl(const T *f, T *fh, size_t nx, size_t ny, size_t nz, double eb, const pmsz_opts *opts,
                 pmsz_result *res, cudaStream_t s, const HostIngest<T> *ingest) {
    if (!f || !fh) return set_error(PMSZ_ERR_ARG, "null field pointer");
    int rc = check_geom(nx, ny, nz);
    if (rc) return rc;
    const int q = opts ? opts->q : 5;
    const uint32_t flags = opts ? opts->flags : 0u;
    const int64_t max_sweeps = opts && opts->max_sweeps > 0 ? opts->max_sweeps : 10000;
    if (!(eb > 0.0) || !(eb < 1e300)) return set_error(PMSZ_ERR_ARG, "error bound must be positive and finite");
    if (q < 1 || q > 255) return set_error(PMSZ_ERR_ARG, "q must be in 1..255");
    if ((flags & PMSZ_FLAG_AUTOTUNE) && !ingest && !tune_known(nx, ny, nz, sizeof(T)) &&
        (rc = autotune_impl<T>(f, fh, nx, ny, nz, nullptr, s)))
        return rc;
    Geom g = make_geom(nx, ny, nz);
    g.zc = tuned_zchunk(nx, ny, nz, sizeof(T));
    const T eps = static_cast<T>(eb);
    const T delta = static_cast<T>(eb / static_cast<double>(q));  // pMSz.cu:2814

    // Scratch: codes (n), counters (n), request + two active bitmaps, sweep slots.
    Workspace ws(s);
    const size_t o_codes = ws.reserve<uint8_t>(g.n);
    const bool own_cnt = !(ingest && ingest->cnt);
    const size_t o_cnt = ws.reserve<uint8_t>(own_cnt ? g.n : 0);
    const size_t o_req = ws.reserve<uint32_t>(g.nwords);
    const size_t o_a0 = ws.reserve<uint32_t>(g.nwords);
    const size_t o_a1 = ws.reserve<uint32_t>(g.nwords);
    const size_t o_slots = ws.reserve<SweepSlot>(static_cast<size_t>(max_sweeps));
    const size_t o_hp = ws.reserve<uint32_t>(g.n);
    // voxel-list sweeps (list.cuh) for fields of fewer than 2^32 voxels
    const bool use_list = !(flags & PMSZ_FLAG_FULL_SWEEPS) && g.n < (static_cast<size_t>(1) << 32);
    const size_t o_list = ws.reserve<uint32_t>(use_list ? g.n : 0);
    const size_t o_xlist = ws.reserve<uint32_t>(use_list ? g.n : 0);
    const size_t o_bcnt = ws.reserve<uint32_t>(use_list ? kCompactBlocks : 0);
    const size_t o_ls = ws.reserve<LoopState>(use_list ? 1 : 0);
    // host-buffer calls of several slabs run sweeps 1 .. K behind the copy
    // (first_pass_waves; K even, below max_sweeps); their detection spills go
    // to a list of their own (xlist still collects the first pass's deferrals)
    const int wave_k = static_cast<int>(std::min<int64_t>(kWaveSweeps, max_sweeps - 1)) & ~1;
    const bool waves = ingest && use_list && wave_k >= 2 && ingest->copies && ingest->copies->nslabs >= 2;
    const size_t o_slist = ws.reserve<uint32_t>(waves ? g.n : 0);
    if ((rc = ws.commit())) return rc;
    uint32_t *hp = ws.at<uint32_t>(o_hp);
    uint8_t *codes = ws.at<uint8_t>(o_codes);
    uint8_t *cnt = own_cnt ? ws.at<uint8_t>(o_cnt) : ingest->cnt;
    uint32_t *req = ws.at<uint32_t>(o_req);
    uint32_t *act[2] = {ws.at<uint32_t>(o_a0), ws.at<uint32_t>(o_a1)};
    SweepSlot *slots = ws.at<SweepSlot>(o_slots);
    uint32_t *list = use_list ? ws.at<uint32_t>(o_list) : nullptr;
    uint32_t *xlist = use_list ? ws.at<uint32_t>(o_xlist) : nullptr;
    uint32_t *bcnt = use_list ? ws.at<uint32_t>(o_bcnt) : nullptr;  // per-block counts of a compaction
    LoopState *ls = use_list ? ws.at<LoopState>(o_ls) : nullptr;
    uint32_t *slist = waves ? ws.at<uint32_t>(o_slist) : nullptr;
    const FastDiv div_nx = make_fastdiv(static_cast<uint32_t>(g.nx));
    const unsigned list_blocks = 152 * 8;
    const FirstMaps maps = use_list ? first_maps<T>(f, fh, g) : FirstMaps{};
    EventTimer et;
    if ((rc = et.init())) return rc;
    PMSZ_CUDA(cudaEventRecord(et.ev[3], s));  // start of the loop's device window

    PMSZ_CUDA(cudaMemsetAsync(cnt, 0, g.n, s));  // init_counter, pMSz.cu:1745-1749
    PMSZ_CUDA(cudaMemsetAsync(req, 0, g.nwords * 4, s));
    PMSZ_CUDA(cudaMemsetAsync(act[0], 0, g.nwords * 4, s));
    PMSZ_CUDA(cudaMemsetAsync(act[1], 0, g.nwords * 4, s));
    PMSZ_CUDA(cudaMemsetAsync(slots, 0, sizeof(SweepSlot) * static_cast<size_t>(max_sweeps), s));
    if (use_list) {
        PMSZ_CUDA(cudaMemsetAsync(ls, 0, sizeof(LoopState), s));
        PMSZ_CUDA(cudaMemsetAsync(&ls->go, 1, 1, s));  // sweep 0 runs (little-endian int 1)
    }

    SweepSlot *hslot = static_cast<SweepSlot *>(host_pinned(sizeof(SweepSlot)));
    if (!hslot) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
    const bool timing = (flags & PMSZ_FLAG_TIMING) != 0;
    double ms_first = 0, ms_detect = 0, ms_apply = 0;
    int64_t launches = 0;
    const dim3 blk3(32, 8, 1);
    int cur = 0;  // act[cur] = active set of the coming sweep; act[cur^1] receives the next one
    int64_t sweeps = 0;
    uint64_t edits = 0;
    int status = PMSZ_ERR_NOT_CONVERGED;
    bool end_recorded = false;  // et.ev[0] marks the end of the correction's device window
    std::vector<SweepSlot> log;
    // The cooperative tail takes over once the next active set is estimated
    // below N/32, but never above kTailCap voxels: its barrier-separated
    // phases serve millions of active voxels worse than list sweeps do, and at
    // 1536^3 N/32 is 113 M.
    constexpr unsigned long long kTailCap = 1ull << 20;
    const unsigned long long tail_at = std::max<unsigned long long>(std::min<unsigned long long>(g.n / 32, kTailCap), 1ull << 16);
    if (use_list) {
        // Sweep 0 (the fused first pass and its edits) on the stream; then the
        // voxel-list sweeps as a CUDA graph whose while node repeats a body of
        // two sweeps (odd: act[1] -> act[0], even: act[0] -> act[1]) for as
        // long as k_loop_gate lets the next sweep run: no host round trip
        // between sweeps.  The graph is built on the host while sweep 0 runs.
        // What the gate leaves (a small active set) goes to the cooperative
        // tail.
        EventTimer lt;  // sweep 0 start, first pass done, sweep 0 done, list sweeps done
        if (timing) {
            if ((rc = lt.init())) return rc;
            PMSZ_CUDA(cudaEventRecord(lt.ev[0], s));
        }
        if (waves) {  // sweeps 0 .. wave_k behind the host copy, then the state after them
            if ((rc = first_pass_waves<T>(*ingest, f, fh, codes, cnt, hp, req, act, slots, ls, g, maps, list, xlist,
                                          slist, bcnt, div_nx, eps, delta, q, wave_k, s, &launches)))
                return rc;
            if (timing) PMSZ_CUDA(cudaEventRecord(lt.ev[1], s));
            k_wave_gate<<<1, 32, 0, s>>>(ls, slots, wave_k, max_sweeps, tail_at, static_cast<unsigned long long>(g.n),
                                         list_blocks);
            ++launches;
            PMSZ_CUDA(cudaGetLastError());
            if (timing) PMSZ_CUDA(cudaEventRecord(lt.ev[2], s));
        } else {
            if (ingest) {
                if ((rc = first_pass_ingest<T>(*ingest, f, fh, codes, hp, req, act[1], &ls->cur, g, s, &launches,
                                               xlist, &ls->lc[3], &maps, &ls->err)))
                    return rc;
            } else {
                launch_first_pass<T>(maps, tiled_grid(g), s, f, fh, codes, hp, req, act[1], &ls->cur, g, 0, xlist,
                                     &ls->lc[3], &ls->err);
                ++launches;
            }
            k_first_exact<T><<<list_blocks, 256, 0, s>>>(xlist, &ls->lc[3], f, fh, codes, req, act[1], &ls->cur, g,
                                                         div_nx);
            ++launches;
            if (timing) PMSZ_CUDA(cudaEventRecord(lt.ev[1], s));
            compact_bitmap(req, g, bcnt, list, &ls->lc[1], &ls->go, s);
            k_apply_list<T><<<list_blocks, 256, 0, s>>>(list, &ls->lc[1], f, fh, cnt, hp, act[1], &ls->cur, g, div_nx,
                                                        eps, delta, q, &ls->go);
            k_pick_detection<<<1, 32, 0, s>>>(ls, static_cast<unsigned long long>(g.n), list_blocks);
            k_loop_gate<<<1, 32, 0, s>>>(ls, slots, max_sweeps, tail_at, cudaGraphConditionalHandle{}, 0);
            launches += 5;
            PMSZ_CUDA(cudaGetLastError());
            if (timing) PMSZ_CUDA(cudaEventRecord(lt.ev[2], s));
        }

        // One body: two list sweeps (odd: act[1] -> act[0], even: act[0] ->
        // act[1]), each ending with k_loop_gate; with set_cond the second gate
        // also sets the graph's while condition.
        auto enqueue_body = [&](cudaStream_t bs, cudaGraphConditionalHandle cond, bool set_cond) {
            for (int half = 0; half < 2; ++half) {
                uint32_t *a_cur = act[half == 0 ? 1 : 0], *a_next = act[half == 0 ? 0 : 1];
                compact_bitmap(a_cur, g, bcnt, list, &ls->lc[0], &ls->go, bs);
                k_detect_list<T><<<list_blocks, 256, 0, bs>>>(list, &ls->lc[0], fh, hp, codes, req, a_next, xlist,
                                                              &ls->lc[2], &ls->cur, g, div_nx, &ls->go,
                                                              &ls->exact_keys, &ls->deferred);
                k_detect_exact<T><<<list_blocks, 256, 0, bs>>>(xlist, &ls->lc[2], fh, codes, req, a_next, &ls->cur, g,
                                                               div_nx, &ls->go);
                compact_bitmap(req, g, bcnt, list, &ls->lc[1], &ls->go, bs);
                k_apply_list<T><<<list_blocks, 256, 0, bs>>>(list, &ls->lc[1], f, fh, cnt, hp, a_next, &ls->cur, g,
                                                             div_nx, eps, delta, q, &ls->go);
                k_loop_gate<<<1, 32, 0, bs>>>(ls, slots, max_sweeps, tail_at, cond, set_cond && half == 1 ? 1 : 0);
            }
        };
        int64_t bodies = 0;
        if (flags & PMSZ_FLAG_HOST_LOOP) {
            // the same sweeps enqueued from the host, two per round trip to the
            // device gate (tools that cannot look into conditional graph nodes)
            int *hgo = static_cast<int *>(host_pinned(sizeof(int)));
            if (!hgo) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
            for (;;) {
                PMSZ_CUDA(cudaMemcpyAsync(hgo, &ls->go, sizeof(int), cudaMemcpyDeviceToHost, s));
                PMSZ_CUDA(cudaStreamSynchronize(s));
                if (!*hgo) break;
                enqueue_body(s, cudaGraphConditionalHandle{}, false);
                PMSZ_CUDA(cudaGetLastError());
                ++bodies;
            }
        } else {
            // The graph: k_loop_enter, then one conditional while node whose
            // body is enqueue_body, captured while sweep 0 runs; no host round
            // trip between sweeps.
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
            // k_loop_enter sets the condition before the while node is reached
            const LoopState *cls = ls;
            void *eargs[] = {&cls, &cond};
            cudaGraphNodeParams ep = {};
            ep.type = cudaGraphNodeTypeKernel;
            ep.kernel.func = reinterpret_cast<void *>(k_loop_enter);
            ep.kernel.gridDim = dim3(1);
            ep.kernel.blockDim = dim3(32);
            ep.kernel.kernelParams = eargs;
            cudaGraphNode_t enode, wnode;
            PMSZ_CUDA(cudaGraphAddNode(&enode, gg.graph, nullptr, nullptr, 0, &ep));
            PMSZ_CUDA(cudaGraphAddNode(&wnode, gg.graph, &enode, nullptr, 1, &cp));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            PMSZ_CUDA(cudaStreamCreateWithFlags(&gg.cs, cudaStreamNonBlocking));
            PMSZ_CUDA(cudaStreamBeginCaptureToGraph(gg.cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
            enqueue_body(gg.cs, cond, true);
            PMSZ_CUDA(cudaStreamEndCapture(gg.cs, &body));
            PMSZ_CUDA(cudaGraphInstantiate(&gg.exec, gg.graph, 0));
            PMSZ_CUDA(cudaGraphLaunch(gg.exec, s));
        }
        if (timing) PMSZ_CUDA(cudaEventRecord(lt.ev[3], s));

        // The cooperative tail follows without a host round trip (it reads
        // the gate's decision), then the caller's work on the result; one
        // read-back brings the loop state, the sweep count and the first
        // slots of the sweep log.
        constexpr int64_t kLogAhead = 64;
        const int64_t pre = std::min<int64_t>(max_sweeps, kLogAhead);
        const size_t ls_bytes = (sizeof(LoopState) + 63) / 64 * 64;
        unsigned char *hb =
            static_cast<unsigned char *>(host_pinned(ls_bytes + 64 + static_cast<size_t>(pre) * sizeof(SweepSlot)));
        if (!hb) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
        LoopState *hls = reinterpret_cast<LoopState *>(hb);
        long long *hdone = reinterpret_cast<long long *>(hb + ls_bytes);
        const SweepSlot *hlog = reinterpret_cast<const SweepSlot *>(hb + ls_bytes + 64);
        EventTimer tt;
        if (timing && (rc = tt.init())) return rc;
        if ((rc = enqueue_gated_tail<T>(f, fh, codes, cnt, hp, req, act, slots, ls, max_sweeps, g, eps, delta, q, s,
                                        timing ? &tt : nullptr, hdone)))
            return rc;
        launches += 2;
        PMSZ_CUDA(cudaEventRecord(et.ev[0], s));  // end of the correction's device window
        end_recorded = true;
        PMSZ_CUDA(cudaMemcpyAsync(hls, ls, sizeof(LoopState), cudaMemcpyDeviceToHost, s));
        PMSZ_CUDA(cudaMemcpyAsync(hb + ls_bytes + 64, slots, static_cast<size_t>(pre) * sizeof(SweepSlot),
                                  cudaMemcpyDeviceToHost, s));
        if (ingest && ingest->after && ingest->after->fn) {
            ingest->after->done = true;
            if ((rc = ingest->after->fn(s))) return rc;
        }
        PMSZ_CUDA(cudaStreamSynchronize(s));
        if (hls->err)
            return set_error(PMSZ_ERR_CUDA, "first pass: a tile plane's tensor copy did not arrive within the bounded wait");
        const int64_t gdone = hls->k;  // sweeps 0 .. gdone-1 ran before the tail
        const int64_t done = std::max<int64_t>(*hdone, gdone);  // and 0 .. done-1 in all
        const int64_t nloop = std::max<int64_t>(gdone - (waves ? wave_k + 1 : 1), 0);  // sweeps of the loop
        // graph: k_loop_enter and one body (16 kernels) per two sweeps that ran
        launches += (flags & PMSZ_FLAG_HOST_LOOP) ? 16 * bodies : 1 + 16 * ((nloop + 1) / 2);
        if (timing) {  // the list sweeps' edits run inside the graph and count as detection time
            float a = 0, b = 0, c = 0;
            PMSZ_CUDA(cudaEventElapsedTime(&a, lt.ev[0], lt.ev[1]));
            PMSZ_CUDA(cudaEventElapsedTime(&b, lt.ev[1], lt.ev[2]));
            PMSZ_CUDA(cudaEventElapsedTime(&c, lt.ev[2], lt.ev[3]));
            ms_first += a;
            ms_apply += b;
            ms_detect += c;
            if (hls->tail) {
                PMSZ_CUDA(cudaEventElapsedTime(&a, tt.ev[0], tt.ev[1]));
                ms_detect += a;
            }
        }
        log.assign(hlog, hlog + std::min(done, pre));
        if (done > pre) {
            log.resize(static_cast<size_t>(done));
            PMSZ_CUDA(cudaMemcpyAsync(log.data() + pre, slots + pre, static_cast<size_t>(done - pre) * sizeof(SweepSlot),
                                      cudaMemcpyDeviceToHost, s));
            PMSZ_CUDA(cudaStreamSynchronize(s));
        }
        for (const SweepSlot &t : log) edits += t.requested;
        sweeps = done;
        const SweepSlot h = log[static_cast<size_t>(gdone - 1)];  // the sweep the last gate decided on
        if (gdone == 1 && h.bad) {
            status = set_error(PMSZ_ERR_ARG, "input contains NaN or the value 1e30 (the reference's halo sentinel)");
        } else if (h.fmax == 0 && h.fmin == 0 && h.fdir == 0) {
            status = PMSZ_OK;
        } else if (h.progressed == 0) {
            set_error(PMSZ_ERR_NOT_CONVERGED, "a sweep requested edits that changed nothing (all requested vertices clamped)");
        } else if (done > gdone) {  // the cooperative tail ran sweeps gdone .. done-1
            const SweepSlot &last = log.back();
            if (last.fmax == 0 && last.fmin == 0 && last.fdir == 0) status = PMSZ_OK;
            else if (last.progressed == 0)
                set_error(PMSZ_ERR_NOT_CONVERGED, "a sweep requested edits that changed nothing (all requested vertices clamped)");
        }
    }
    while (!use_list && sweeps < max_sweeps) {
        SweepSlot *slot = slots + sweeps;
        uint32_t *a_next = act[cur ^ 1];
        if (timing) PMSZ_CUDA(cudaEventRecord(et.ev[0], s));
        if (sweeps == 0 && ingest) {
            if ((rc = first_pass_ingest<T>(*ingest, f, fh, codes, hp, req, a_next, slot, g, s, &launches, nullptr,
                                           nullptr)))
                return rc;
        } else if (sweeps == 0) {
            k_tiled<T, kFirst><<<tiled_grid(g), blk3, 0, s>>>(f, fh, codes, hp, req, a_next, slot, g, 0);
            ++launches;
        } else if (flags & PMSZ_FLAG_FULL_SWEEPS) {
            k_tiled<T, kDetect><<<tiled_grid(g), blk3, 0, s>>>(fh, nullptr, codes, nullptr, req, a_next, slot, g, 0);
            ++launches;
        } else {
            k_sparse_px<T><<<list_grid(g), kListBlock, 0, s>>>(fh, hp, codes, act[cur], a_next, req, slot, g);
            ++launches;
        }
        if (timing) PMSZ_CUDA(cudaEventRecord(et.ev[1], s));
        k_apply_px<T><<<list_grid(g), kListBlock, 0, s>>>(f, fh, cnt, hp, req, a_next, slot, g, eps, delta, q);
        ++launches;
        if (timing) PMSZ_CUDA(cudaEventRecord(et.ev[2], s));
        PMSZ_CUDA(cudaGetLastError());
        PMSZ_CUDA(cudaMemcpyAsync(hslot, slot, sizeof(SweepSlot), cudaMemcpyDeviceToHost, s));
        PMSZ_CUDA(cudaStreamSynchronize(s));
        if (timing) {
            float a = 0, b = 0;
            PMSZ_CUDA(cudaEventElapsedTime(&a, et.ev[0], et.ev[1]));
            PMSZ_CUDA(cudaEventElapsedTime(&b, et.ev[1], et.ev[2]));
            (sweeps == 0 ? ms_first : ms_detect) += a;
            ms_apply += b;
        }
        ++sweeps;
        const SweepSlot h = *hslot;
        log.push_back(h);
        edits += h.requested;
        if (sweeps == 1 && h.bad) {
            status = set_error(PMSZ_ERR_ARG, "input contains NaN or the value 1e30 (the reference's halo sentinel)");
            break;
        }
        if (h.fmax == 0 && h.fmin == 0 && h.fdir == 0) { status = PMSZ_OK; break; }
        if (h.progressed == 0) {
            set_error(PMSZ_ERR_NOT_CONVERGED, "a sweep requested edits that changed nothing (all requested vertices clamped)");
            break;
        }
        cur ^= 1;
        // Once the next active set is small, per-sweep launches and host round
        // trips dominate: hand the remaining sweeps to one cooperative launch.
        const unsigned long long est_next = 15ull * h.changed + h.fdir;
        if (!(flags & PMSZ_FLAG_FULL_SWEEPS) && sweeps < max_sweeps && est_next <= tail_at) {
            int64_t done = 0;
            if ((rc = run_sweep_loop<T>(f, fh, codes, cnt, hp, req, act, slots, sweeps, max_sweeps, g, eps, delta, q,
                                        s, timing ? &et : nullptr, &ms_detect, &done)))
                return rc;
            ++launches;
            const size_t m = static_cast<size_t>(done - sweeps);
            if (m) {
                std::vector<SweepSlot> tail(m);
                PMSZ_CUDA(cudaMemcpyAsync(tail.data(), slots + sweeps, m * sizeof(SweepSlot), cudaMemcpyDeviceToHost, s));
                PMSZ_CUDA(cudaStreamSynchronize(s));
                for (const SweepSlot &t : tail) {
                    log.push_back(t);
                    edits += t.requested;
                }
                const SweepSlot &last = tail.back();
                if (last.fmax == 0 && last.fmin == 0 && last.fdir == 0) status = PMSZ_OK;
                else if (last.progressed == 0)
                    set_error(PMSZ_ERR_NOT_CONVERGED, "a sweep requested edits that changed nothing (all requested vertices clamped)");
            }
            sweeps = done;
            break;
        }
    }
    float ms_total = 0;
    if (!end_recorded) PMSZ_CUDA(cudaEventRecord(et.ev[0], s));
    PMSZ_CUDA(cudaEventSynchronize(et.ev[0]));
    PMSZ_CUDA(cudaEventElapsedTime(&ms_total, et.ev[3], et.ev[0]));
    if (status == PMSZ_ERR_NOT_CONVERGED && sweeps >= max_sweeps)
        set_error(PMSZ_ERR_NOT_CONVERGED, "max_sweeps reached before convergence");
    if (res) {
        res->sweeps = sweeps;
        res->iteration = sweeps + 1;
        res->edits = edits;
        res->ms_first_pass = ms_first;
        res->ms_detect = ms_detect;
        res->ms_apply = ms_apply;
        res->launches = launches;
        res->ms_total = ms_total;
        if (res->sweep_log && res->sweep_log_cap > 0) {
            const size_t m = std::min<size_t>(log.size(), static_cast<size_t>(res->sweep_log_cap));
            static_assert(sizeof(SweepSlot) == sizeof(pmsz_sweep_record), "record layout");
            std::memcpy(res->sweep_log, log.data(), m * sizeof(SweepSlot));
        }
    }
    rc = ws.release();
    return status != PMSZ_OK ? status : rc;
}

template <typename T>
int codes_impl(const T *v, size_t nx, size_t ny, size_t nz, uint8_t *codes, cudaStream_t s) {
    if (!v || !codes) return set_error(PMSZ_ERR_ARG, "null pointer");
    int rc = check_geom(nx, ny, nz);
    if (rc) return rc;
    const Geom g = make_geom(nx, ny, nz);
    k_tiled<T, kCodes><<<tiled_grid(g), dim3(kTX, kTY, 1), 0, s>>>(v, nullptr, codes, nullptr, nullptr, nullptr, nullptr, g, 0);
    PMSZ_CUDA(cudaGetLastError());
    return PMSZ_OK;
}

// The tuner's first-pass timing: the fused first pass (deferring form) of
// f / fhat at each tile depth zcs[k] on scratch of its own; ms[k] is the best
// of two timed launches after a warm-up.  The code bytes (independent of the
// depth) go to the caller's buffer, completed by k_first_exact for the voxels
// the last run deferred, so every byte is a valid pair of ranks.
template <typename T>
int time_first_pass(const T *f, const T *fh, size_t nx, size_t ny, size_t nz, uint8_t *codes, const int *zcs, int m,
                    float *ms, cudaStream_t s) {
    Geom g = make_geom(nx, ny, nz);
    const bool defer = g.n < (static_cast<size_t>(1) << 32);
    Workspace ws(s);
    const size_t o_hp = ws.reserve<uint32_t>(g.n), o_req = ws.reserve<uint32_t>(g.nwords),
                 o_act = ws.reserve<uint32_t>(g.nwords), o_slot = ws.reserve<SweepSlot>(1),
                 o_x = ws.reserve<uint32_t>(defer ? g.n : 0), o_xc = ws.reserve<uint32_t>(2);
    int rc = ws.commit();
    if (rc) return rc;
    const FirstMaps maps = defer ? first_maps<T>(f, fh, g) : FirstMaps{};
    uint32_t *hp = ws.at<uint32_t>(o_hp), *req = ws.at<uint32_t>(o_req), *act = ws.at<uint32_t>(o_act);
    uint32_t *xl = ws.at<uint32_t>(o_x), *xc = ws.at<uint32_t>(o_xc), *err = xc + 1;
    SweepSlot *slot = ws.at<SweepSlot>(o_slot);
    PMSZ_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), s));
    EventTimer et;
    if ((rc = et.init())) return rc;
    const dim3 blk3(kTX, kTY, 1);
    for (int k = 0; k < m; ++k) {
        g.zc = zcs[k];
        float best = 0.f;
        for (int rep = 0; rep < 3; ++rep) {  // the first run of each candidate is a warm-up
            PMSZ_CUDA(cudaMemsetAsync(req, 0, g.nwords * 4, s));
            PMSZ_CUDA(cudaMemsetAsync(act, 0, g.nwords * 4, s));
            PMSZ_CUDA(cudaMemsetAsync(slot, 0, sizeof(SweepSlot), s));
            PMSZ_CUDA(cudaMemsetAsync(xc, 0, sizeof(uint32_t), s));
            PMSZ_CUDA(cudaEventRecord(et.ev[0], s));
            if (defer)
                launch_first_pass<T>(maps, tiled_grid(g), s, f, const_cast<T *>(fh), codes, hp, req, act, slot, g, 0, xl,
                                     xc, err);
            else
                k_tiled<T, kFirst><<<tiled_grid(g), blk3, 0, s>>>(f, fh, codes, hp, req, act, slot, g, 0);
            PMSZ_CUDA(cudaGetLastError());
            PMSZ_CUDA(cudaEventRecord(et.ev[1], s));
            PMSZ_CUDA(cudaEventSynchronize(et.ev[1]));
            float t = 0.f;
            PMSZ_CUDA(cudaEventElapsedTime(&t, et.ev[0], et.ev[1]));
            if (rep > 0 && (best == 0.f || t < best)) best = t;
        }
        ms[k] = best;
    }
    if (defer) {
        uint32_t herr = 0;
        PMSZ_CUDA(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, s));
        PMSZ_CUDA(cudaStreamSynchronize(s));
        if (herr)
            return set_error(PMSZ_ERR_CUDA, "first pass: a tile plane's tensor copy did not arrive within the bounded wait");
    }
    if (defer) {  // the deferred voxels' code bytes: codes is complete for the caller
        k_first_exact<T><<<152 * 8, 256, 0, s>>>(xl, xc, f, fh, codes, req, act, slot, g, g.div_nx);
        PMSZ_CUDA(cudaGetLastError());
    }
    return ws.release();
}

template int time_first_pass<float>(const float *, const float *, size_t, size_t, size_t, uint8_t *, const int *, int,
                                    float *, cudaStream_t);
template int time_first_pass<double>(const double *, const double *, size_t, size_t, size_t, uint8_t *, const int *,
                                     int, float *, cudaStream_t);

template int codes_impl<float>(const float *, size_t, size_t, size_t, uint8_t *, cudaStream_t);
template int codes_impl<double>(const double *, size_t, size_t, size_t, uint8_t *, cudaStream_t);

template int correct_impl<float>(const float *, float *, size_t, size_t, size_t, double, const pmsz_opts *, pmsz_result *, cudaStream_t, const HostIngest<float> *);
template int correct_impl<double>(const double *, double *, size_t, size_t, size_t, double, const pmsz_opts *, pmsz_result *, cudaStream_t, const HostIngest<double> *);

}  // namespace pmsz

using namespace pmsz;

extern "C" int pmsz_correct_f32(const float *f, float *fhat, size_t nx, size_t ny, size_t nz, double eb,
                                const pmsz_opts *opts, pmsz_result *res, void *stream) {
    return guarded([&] { return correct_impl<float>(f, fhat, nx, ny, nz, eb, opts, res, as_stream(stream)); });
}
extern "C" int pmsz_correct_f64(const double *f, double *fhat, size_t nx, size_t ny, size_t nz, double eb,
                                const pmsz_opts *opts, pmsz_result *res, void *stream) {
    return guarded([&] { return correct_impl<double>(f, fhat, nx, ny, nz, eb, opts, res, as_stream(stream)); });
}
extern "C" int pmsz_codes_f32(const float *v, size_t nx, size_t ny, size_t nz, uint8_t *codes, void *stream) {
    return guarded([&] { return codes_impl<float>(v, nx, ny, nz, codes, as_stream(stream)); });
}
extern "C" int pmsz_codes_f64(const double *v, size_t nx, size_t ny, size_t nz, uint8_t *codes, void *stream) {
    return guarded([&] { return codes_impl<double>(v, nx, ny, nz, codes, as_stream(stream)); });
}
extern "C" int pmsz_rank_offset(int r, int *dx, int *dy, int *dz) {
    if (r < 0 || r > 14 || !dx || !dy || !dz) return PMSZ_ERR_ARG;
    *dx = rank_dx(r);
    *dy = rank_dy(r);
    *dz = rank_dz(r);
    return PMSZ_OK;
}

// ---------------------------------------------------------------------------
// pmsz_correct_noalloc: the correction loop with its scratch in a fixed
// device array instead of per-call allocations, for callers that must not
// allocate device memory -- code that runs while another component owns the
// GPU's memory through its own pool or arena (a simulation that reserved HBM
// up front for in-situ compression, a serving process with a fixed budget),
// or that cannot afford an allocator call on its path.  The array below is
// part of the library image: every GPU that loads the library holds its
// PMSZ_NOALLOC_SCRATCH_BYTES until the process exits, and all calls on a
// device share it.
// ---------------------------------------------------------------------------
namespace pmsz {
namespace noalloc {

constexpr size_t kMaxVoxels = PMSZ_NOALLOC_MAX_VOXELS;
constexpr size_t kMaxWords = PMSZ_NOALLOC_MAX_WORDS;
constexpr size_t kMaxSweeps = PMSZ_NOALLOC_MAX_SWEEPS;
constexpr size_t kOffCodes = 0;
constexpr size_t kOffCnt = kOffCodes + kMaxVoxels;
constexpr size_t kOffReq = kOffCnt + kMaxVoxels;
constexpr size_t kOffAct0 = kOffReq + 4 * kMaxWords;
constexpr size_t kOffAct1 = kOffAct0 + 4 * kMaxWords;
constexpr size_t kOffSlots = kOffAct1 + 4 * kMaxWords;
constexpr size_t kBytes = kOffSlots + sizeof(SweepSlot) * kMaxSweeps;
static_assert(kBytes == PMSZ_NOALLOC_SCRATCH_BYTES, "header constant out of date");
static_assert(kOffReq % 256 == 0 && kOffSlots % 256 == 0, "sub-arrays stay 256-byte aligned");

// codes | edit counters | request bitmap | two active bitmaps | sweep slots
static __device__ __align__(256) unsigned char g_scratch[kBytes];

// Device address of g_scratch in the calling thread's current context.  The
// host-side symbol is only a stand-in for the array, so the address is looked
// up with cudaGetSymbolAddress (which allocates nothing) on every call: a
// cached address would go stale after cudaDeviceReset or in another context
// on the same device, where the library's device code is loaded again.
static int scratch_address(unsigned char **out) {
    void *p = nullptr;
    PMSZ_CUDA(cudaGetSymbolAddress(&p, g_scratch));
    *out = static_cast<unsigned char *>(p);
    return PMSZ_OK;
}

template <typename T>
int run(const T *f, T *fh, size_t nx, size_t ny, size_t nz, double eb, const pmsz_opts *opts, pmsz_result *res,
        cudaStream_t s) {
    if (!f || !fh) return set_error(PMSZ_ERR_ARG, "null field pointer");
    int rc = check_geom(nx, ny, nz);
    if (rc) return rc;
    const int q = opts ? opts->q : 5;
    const uint32_t flags = opts ? opts->flags : 0u;
    const int64_t max_sweeps = opts && opts->max_sweeps > 0 ? opts->max_sweeps : static_cast<int64_t>(kMaxSweeps);
    if (!(eb > 0.0) || !(eb < 1e300)) return set_error(PMSZ_ERR_ARG, "error bound must be positive and finite");
    if (q < 1 || q > 255) return set_error(PMSZ_ERR_ARG, "q must be in 1..255");
    const Geom g = make_geom(nx, ny, nz);
    if (g.n > kMaxVoxels)
        return set_error(PMSZ_ERR_ARG, "pmsz_correct_noalloc: field of " + std::to_string(g.n) +
                                           " voxels exceeds its fixed scratch (at most " + std::to_string(kMaxVoxels) +
                                           " voxels); use pmsz_correct_f32/f64");
    if (g.nwords > kMaxWords)
        return set_error(PMSZ_ERR_ARG, "pmsz_correct_noalloc: ceil(nx/32)*ny*nz = " + std::to_string(g.nwords) +
                                           " exceeds its fixed bitmap scratch (at most " + std::to_string(kMaxWords) + ")");
    if (max_sweeps > static_cast<int64_t>(kMaxSweeps))
        return set_error(PMSZ_ERR_ARG, "pmsz_correct_noalloc: max_sweeps above " + std::to_string(kMaxSweeps));
    unsigned char *base = nullptr;
    if ((rc = scratch_address(&base))) return rc;
    uint8_t *codes = base + kOffCodes;
    uint8_t *cnt = base + kOffCnt;
    uint32_t *req = reinterpret_cast<uint32_t *>(base + kOffReq);
    uint32_t *act[2] = {reinterpret_cast<uint32_t *>(base + kOffAct0), reinterpret_cast<uint32_t *>(base + kOffAct1)};
    SweepSlot *slots = reinterpret_cast<SweepSlot *>(base + kOffSlots);

    // The array keeps the previous call's contents: clear everything that
    // the loop expects to start at zero (codes are fully rewritten by sweep 1).
    PMSZ_CUDA(cudaMemsetAsync(cnt, 0, g.n, s));
    PMSZ_CUDA(cudaMemsetAsync(req, 0, g.nwords * 4, s));
    PMSZ_CUDA(cudaMemsetAsync(act[0], 0, g.nwords * 4, s));
    PMSZ_CUDA(cudaMemsetAsync(act[1], 0, g.nwords * 4, s));
    PMSZ_CUDA(cudaMemsetAsync(slots, 0, sizeof(SweepSlot) * static_cast<size_t>(max_sweeps), s));
    // ms_total: host clock from here to the last sweep's read-back; the loop
    // synchronises the stream after every sweep, so this is the device window
    // of the loop (timing events are not created: they are driver resources)
    PMSZ_CUDA(cudaStreamSynchronize(s));
    const auto t0 = std::chrono::steady_clock::now();

    const T eps = static_cast<T>(eb);
    const T delta = static_cast<T>(eb / static_cast<double>(q));
    const dim3 blk3(32, 8, 1);
    int cur = 0;
    int64_t sweeps = 0;
    uint64_t edits = 0;
    int status = PMSZ_ERR_NOT_CONVERGED;
    while (sweeps < max_sweeps) {
        SweepSlot *slot = slots + sweeps;
        uint32_t *a_next = act[cur ^ 1];
        if (sweeps == 0) {
            k_detect_full<T, true><<<grid3(g), blk3, 0, s>>>(f, fh, codes, req, a_next, slot, g);
        } else if (flags & PMSZ_FLAG_FULL_SWEEPS) {
            k_detect_full<T, false><<<grid3(g), blk3, 0, s>>>(nullptr, fh, codes, req, a_next, slot, g);
        } else {
            k_detect_sparse<T><<<stride_grid(g.nwords), 256, 0, s>>>(fh, codes, act[cur], a_next, req, slot, g);
        }
        k_apply<T><<<stride_grid(g.nwords), 256, 0, s>>>(f, fh, cnt, req, a_next, slot, g, eps, delta, q);
        PMSZ_CUDA(cudaGetLastError());
        SweepSlot h;  // read back into the caller's stack: no pinned buffer
        PMSZ_CUDA(cudaMemcpyAsync(&h, slot, sizeof(SweepSlot), cudaMemcpyDeviceToHost, s));
        PMSZ_CUDA(cudaStreamSynchronize(s));
        if (res && res->sweep_log && sweeps < res->sweep_log_cap)
            std::memcpy(res->sweep_log + sweeps, &h, sizeof(SweepSlot));
        ++sweeps;
        edits += h.requested;
        if (sweeps == 1 && h.bad) {
            status = set_error(PMSZ_ERR_ARG, "input contains NaN or the value 1e30 (the reference's halo sentinel)");
            break;
        }
        if (h.fmax == 0 && h.fmin == 0 && h.fdir == 0) { status = PMSZ_OK; break; }
        if (h.progressed == 0) {
            set_error(PMSZ_ERR_NOT_CONVERGED, "a sweep requested edits that changed nothing (all requested vertices clamped)");
            break;
        }
        cur ^= 1;
    }
    if (status == PMSZ_ERR_NOT_CONVERGED && sweeps >= max_sweeps)
        set_error(PMSZ_ERR_NOT_CONVERGED, "max_sweeps reached before convergence");
    if (res) {
        res->sweeps = sweeps;
        res->iteration = sweeps + 1;
        res->edits = edits;
        res->ms_first_pass = res->ms_detect = res->ms_apply = 0.0;
        res->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        res->launches = 2 * sweeps;
    }
    return status;
}

}  // namespace noalloc
}  // namespace pmsz

extern "C" int pmsz_correct_noalloc(const void *f, void *fhat, size_t elem_size, size_t nx, size_t ny, size_t nz,
                                    double eb, const pmsz_opts *opts, pmsz_result *res, void *stream) {
    return guarded([&] {
        if (elem_size == sizeof(float))
            return noalloc::run<float>(static_cast<const float *>(f), static_cast<float *>(fhat), nx, ny, nz, eb,
                                       opts, res, as_stream(stream));
        if (elem_size == sizeof(double))
            return noalloc::run<double>(static_cast<const double *>(f), static_cast<double *>(fhat), nx, ny, nz, eb,
                                        opts, res, as_stream(stream));
        return set_error(PMSZ_ERR_ARG, "elem_size must be 4 (float) or 8 (double)");
    });
}
