// edits.cu -- edit-output extraction with an order-preserving compaction.
//
// Replaces extract_edits_kernel + run_extract_edits (pMSz.cu:2090-2226) and
// the thrust::copy_if compaction of compact_edits_dense_to_sparse
// (pMSz.cu:227-250).  Per voxel, x fastest, comparing the corrected field cur
// with the decompressed field prev (pMSz.cu:2104-2137):
//   cur == prev              -> delta 0
//   cur == f - eps           -> delta q, clamp value f - eps (dropped if == 0,
//                               as copy_if(v != 0) drops it)
//   otherwise                -> delta round((prev - cur) / delta_step)
// The reference leaves deltas undefined where cur > prev (only a clamp can
// raise a value; its `currentV < previousV` branch is skipped); those voxels
// take the same encoding as any other changed voxel here.  "Edit count" is
// the number of voxels with cur < prev (pMSz.cu:2114).
//
// Three kernels: (1) deltas + one clamp flag bit per voxel + per-tile clamp
// and edit counts; (2) one-block exclusive scan of the tile clamp counts and
// sum of the edit counts; (3) one warp per tile writes its clamp values at
// the tile's offset in voxel order.
#include "common.cuh"
#include "internal.h"

#include <algorithm>

namespace pmsz {

constexpr int kTile = 2048;  // voxels per tile: 256 threads x 8

// Step count of an edited voxel, round((p - c) / delta) as the reference
// computes it.  fp64 division is slow on this GPU (its FP64 pipe runs two
// operations per SM per cycle), so a candidate k -- the voxel's edit counter
// when the correction left it, else rint((p - c) * inv) -- is accepted when
// one fma shows |p - c - k*delta| <= delta/4: then the correctly rounded
// quotient lies within k +- 0.25 (plus one rounding), and round() gives k.
// Anything else takes the division.  fp32 divides directly.
__device__ __forceinline__ uint8_t edit_steps(double p, double c, double delta, double inv, double quarter, int hint) {
    const double diff = p - c;
    const double k = hint >= 0 ? static_cast<double>(hint) : rint(diff * inv);
    if (fabs(k) < 1048576.0 && fabs(fma(-k, delta, diff)) <= quarter) return static_cast<uint8_t>(k);
    return static_cast<uint8_t>(round(diff / delta));
}
__device__ __forceinline__ uint8_t edit_steps(float p, float c, float delta, float, float, int) {
    return static_cast<uint8_t>(round((p - c) / delta));
}

// IEEE equality and order of two values on the integer pipe (NaN equals
// nothing and orders below nothing; +0 and -0 are equal): the tests every
// voxel takes stay off the slow fp64 pipe.
__device__ __forceinline__ uint64_t fp_bits(double v) { return static_cast<uint64_t>(__double_as_longlong(v)); }
__device__ __forceinline__ uint32_t fp_bits(float v) { return __float_as_uint(v); }
__device__ __forceinline__ bool fp_nan(uint64_t x) { return (x & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull; }
__device__ __forceinline__ bool fp_nan(uint32_t x) { return (x & 0x7FFFFFFFu) > 0x7F800000u; }
template <typename T>
__device__ __forceinline__ bool fp_eq(T a, T b) {
    const auto x = fp_bits(a), y = fp_bits(b);
    using U = decltype(x);
    const U mag = ~(U(1) << (sizeof(U) * 8 - 1));
    return !fp_nan(x) && !fp_nan(y) && (x == y || ((x | y) & mag) == 0);
}
template <typename T>
__device__ __forceinline__ bool fp_lt(T a, T b) {
    const auto x = fp_bits(a), y = fp_bits(b);
    using U = decltype(x);
    const U sign = U(1) << (sizeof(U) * 8 - 1);
    if (fp_nan(x) || fp_nan(y) || ((x | y) & ~sign) == 0) return false;
    const U kx = (x & sign) ? ~x : (x | sign), ky = (y & sign) ? ~y : (y | sign);  // order-preserving keys
    return kx < ky;
}

// cnt (optional): the correction's edit counters; a voxel whose counter is 0
// was never edited, so cur == prev there and its three values need not be read.
// The block first lists the voxels of its tile whose value changed (in shared
// memory, voxel order), then decides them 256 at a time, so the fp64 work of
// the decision runs on full warps (GB300's fp64 pipe issues a warp's
// instruction at the same cost whether 32 lanes or 4 are active; listed per
// warp, a few percent of changed voxels filled about a third of the lanes).  Per
// tile: the clamp flags (one word per 32 voxels, set in shared memory), the
// clamp count and the edit count, combined in shared memory (no global
// atomics: one counter shared by every warp serialises at L2).
// PACK: the symbols are not stored one byte per voxel but staged in shared
// memory and written packed at nbits bits each (thread t of the grid: symbols
// 8t .. 8t+7 in bytes nbits*t .. nbits*t + nbits - 1, pack_nbits' layout, as
// k_pack_deltas writes it from the unpacked array).
template <typename T, bool PACK>
__global__ void __launch_bounds__(256) k_extract(const T *__restrict__ prev, const T *__restrict__ cur,
                                                 const T *__restrict__ f, const uint8_t *__restrict__ cnt, size_t n,
                                                 T eps, T delta, T inv, T quarter, int q, uint8_t *__restrict__ deltas,
                                                 uint32_t *__restrict__ flags, uint32_t *__restrict__ tile_count,
                                                 uint32_t *__restrict__ tile_edits, int nbits, size_t packed_len,
                                                 uint32_t tile0) {
    __shared__ uint32_t s_cnt, s_edits;
    __shared__ uint32_t s_fl[kTile / 32];
    __shared__ uint16_t s_list[kTile];  // the tile's changed voxels (offsets), in voxel order
    __shared__ uint32_t s_wtot[8];
    __shared__ __align__(8) uint8_t s_sym[PACK ? kTile : 8];  // PACK: the tile's symbols
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_cnt = s_edits = 0;
    if (threadIdx.x < kTile / 32) s_fl[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t tile = tile0 + blockIdx.x;
    const size_t base = static_cast<size_t>(tile) * kTile;
    // each thread: 8 consecutive voxels (one 8-byte counter load, one 8-byte
    // delta store); the values of the touched ones are loaded together
    const uint32_t off0 = static_cast<uint32_t>(threadIdx.x) * 8;
    const size_t i0 = base + off0;
    const bool full = i0 + 8 <= n && (PACK || (reinterpret_cast<uintptr_t>(deltas + i0) & 7) == 0) &&
                      (!cnt || (reinterpret_cast<uintptr_t>(cnt + i0) & 7) == 0);
    uint8_t cv[8];
    if (full && cnt) {
        const uint2 u = *reinterpret_cast<const uint2 *>(cnt + i0);
#pragma unroll
        for (int j = 0; j < 8; ++j) cv[j] = static_cast<uint8_t>(((j < 4 ? u.x : u.y) >> ((j & 3) * 8)) & 0xFFu);
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) cv[j] = (i0 + j < n) ? (cnt ? cnt[i0 + j] : uint8_t(1)) : uint8_t(0);
    }
    // with counters, every counted voxel is listed and the decision below
    // compares its two values (loaded there anyway); without, the values of
    // every voxel are compared here
    uint32_t needm = 0;
    if (cnt) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (cv[j]) needm |= 1u << j;
    } else {
        T c8[8], p8[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            c8[j] = cv[j] ? cur[i0 + j] : T(0);
            p8[j] = cv[j] ? prev[i0 + j] : T(0);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (cv[j] && !fp_eq(c8[j], p8[j])) needm |= 1u << j;
    }
    if (PACK) {  // voxels not listed: symbol 0 (the listed ones are written below)
        *reinterpret_cast<uint2 *>(s_sym + off0) = make_uint2(0u, 0u);
    } else if (full) {  // unchanged voxels: delta 0; changed ones are written below
        if (needm != 0xFFu) *reinterpret_cast<uint2 *>(deltas + i0) = make_uint2(0u, 0u);
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (i0 + j < n && !((needm >> j) & 1u)) deltas[i0 + j] = 0;
    }
    const uint32_t cnt8 = __popc(needm);
    uint32_t inc = cnt8;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) s_wtot[w] = inc;
    __syncthreads();
    uint32_t pos = inc - cnt8, nt = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t u = s_wtot[k];
        if (k < w) pos += u;
        nt += u;
    }
    for (uint32_t m = needm; m; m &= m - 1) s_list[pos++] = static_cast<uint16_t>(off0 + (__ffs(m) - 1));
    __syncthreads();
    uint32_t clamps = 0, edits = 0;
    for (uint32_t k0 = 0; k0 < nt; k0 += 256) {  // full warps: the tile's changed voxels, 256 at a time
        const uint32_t k = k0 + static_cast<uint32_t>(threadIdx.x);
        if (k < nt) {
            const uint32_t off = s_list[k];
            const size_t i = base + off;
            const T c = cur[i], p = prev[i];
            edits += fp_lt(c, p);
            const T cv = f[i] - eps;
            uint8_t d;
            if (fp_eq(c, p)) {  // counted but unchanged (only listed when counters are given)
                d = 0;
            } else if (!fp_eq(c, cv)) {
                d = edit_steps(p, c, delta, inv, quarter, cnt ? static_cast<int>(cnt[i]) : -1);
            } else {
                d = static_cast<uint8_t>(q);
                if (!fp_eq(cv, T(0))) {
                    atomicOr(&s_fl[off >> 5], 1u << (off & 31));
                    ++clamps;
                }
            }
            if (PACK) s_sym[off] = d;
            else deltas[i] = d;
        }
    }
    if (PACK) {  // this thread's 8 symbols -> nbits bytes
        __syncthreads();
        if (i0 < n) {
            const uint2 u = *reinterpret_cast<const uint2 *>(s_sym + off0);
            const uint64_t mask = (1ull << nbits) - 1ull;
            uint64_t v = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const uint64_t sym = ((j < 4 ? u.x : u.y) >> ((j & 3) * 8)) & 0xFFu;
                if (i0 + j < n) v |= (sym & mask) << (j * nbits);
            }
            const size_t b0 = (i0 >> 3) * static_cast<size_t>(nbits);
            for (int b = 0; b < nbits && b0 + b < packed_len; ++b) deltas[b0 + b] = static_cast<uint8_t>(v >> (8 * b));
        }
    }
    clamps = warp_sum_u32(clamps);
    edits = warp_sum_u32(edits);
    if (lane == 0) {
        if (clamps) atomicAdd(&s_cnt, clamps);
        if (edits) atomicAdd(&s_edits, edits);
    }
    __syncthreads();
    if (threadIdx.x < kTile / 32 && base + static_cast<size_t>(threadIdx.x) * 32 < n)
        flags[(base >> 5) + threadIdx.x] = s_fl[threadIdx.x];
    if (threadIdx.x == 0) {
        tile_count[tile] = s_cnt;
        tile_edits[tile] = s_edits;
    }
}

// Exclusive scan of the `m` tile clamp counts in two levels: k_scan_part
// scans chunks of 1024 tiles in place (one block each) and stores each
// chunk's clamp and edit sums; k_scan_chunks scans the chunk sums in one
// block (offsets in part[0 .. nc), the clamp total in total[0], the edit total
// in total[1]); a tile's offset is then counts[t] + part[t >> 10].
constexpr int kScanChunk = 1024;
__global__ void __launch_bounds__(kScanChunk) k_scan_part(uint32_t *__restrict__ counts,
                                                          const uint32_t *__restrict__ edits, size_t m,
                                                          uint32_t *__restrict__ part, unsigned long long *epart) {
    __shared__ uint32_t s_warp[32];
    __shared__ unsigned long long s_e[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t i = static_cast<size_t>(blockIdx.x) * kScanChunk + threadIdx.x;
    const uint32_t v = i < m ? counts[i] : 0u;
    unsigned long long e = i < m ? edits[i] : 0ull;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xFFFFFFFFu, e, o);
    if (lane == 31) s_warp[warp] = inc;
    if (lane == 0) s_e[warp] = e;
    __syncthreads();
    if (warp == 0) {
        const uint32_t wv = s_warp[lane];
        uint32_t winc = wv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, winc, o);
            if (lane >= o) winc += t;
        }
        s_warp[lane] = winc - wv;  // exclusive offsets of the warps
        unsigned long long es = s_e[lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) es += __shfl_xor_sync(0xFFFFFFFFu, es, o);
        if (lane == 31) {
            part[blockIdx.x] = winc;  // the chunk's clamp sum
            epart[blockIdx.x] = es;
        }
    }
    __syncthreads();
    if (i < m) counts[i] = s_warp[warp] + inc - v;
}

__global__ void __launch_bounds__(1024) k_scan_chunks(uint32_t *__restrict__ part,
                                                      const unsigned long long *__restrict__ epart, size_t nc,
                                                      unsigned long long *total) {
    __shared__ unsigned long long s_warp[32];
    __shared__ unsigned long long s_run;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_run = 0;
    unsigned long long esum = 0;
    for (size_t c0 = 0; c0 < nc; c0 += 1024) {  // at most 2^32 / 2^21 = 2048 chunks: two rounds
        const size_t i = c0 + threadIdx.x;
        const unsigned long long v = i < nc ? part[i] : 0ull;
        if (i < nc) esum += epart[i];
        unsigned long long inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += t;
        }
        __syncthreads();  // s_warp / s_run of the previous round are consumed
        if (lane == 31) s_warp[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            const unsigned long long wv = s_warp[lane];
            unsigned long long winc = wv;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long t = __shfl_up_sync(0xFFFFFFFFu, winc, o);
                if (lane >= o) winc += t;
            }
            s_warp[lane] = winc - wv;
        }
        __syncthreads();
        const unsigned long long run = s_run;
        if (i < nc) part[i] = static_cast<uint32_t>(run + s_warp[warp] + inc - v);  // at most n < 2^32 clamps
        __syncthreads();
        if (threadIdx.x == 1023) s_run = run + s_warp[31] + inc;
    }
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) esum += __shfl_xor_sync(0xFFFFFFFFu, esum, o);
    if (lane == 0) s_warp[warp] = esum;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long e = 0;
        for (int w = 0; w < 32; ++w) e += s_warp[w];
        total[0] = s_run;
        total[1] = e;
    }
}

// One warp per tile: the 64 flag words of the tile (two per lane), a warp scan
// of their popcounts, then every set flag writes its clamp value (cur) at the
// tile's offset plus its rank: clamp values in voxel order.
template <typename T>
__global__ void __launch_bounds__(256) k_scatter_clamps(const T *__restrict__ cur, const uint32_t *__restrict__ flags,
                                                        const uint32_t *__restrict__ tile_off,
                                                        const uint32_t *__restrict__ part, size_t n, size_t tiles,
                                                        T *__restrict__ clamp) {
    const size_t tile = static_cast<size_t>(blockIdx.x) * 8 + (threadIdx.x >> 5);
    if (tile >= tiles) return;
    const int lane = threadIdx.x & 31;
    const size_t base = tile * kTile;
    const size_t nw = (std::min(n - base, static_cast<size_t>(kTile)) + 31) / 32;
    const size_t w0 = static_cast<size_t>(lane) * 2;
    const uint32_t a = w0 < nw ? flags[(base >> 5) + w0] : 0u;
    const uint32_t b = w0 + 1 < nw ? flags[(base >> 5) + w0 + 1] : 0u;
    const uint32_t c = __popc(a) + __popc(b);
    uint32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += t;
    }
    uint32_t pos = tile_off[tile] + part[tile / kScanChunk] + inc - c;
    for (uint32_t bits = a; bits; bits &= bits - 1) clamp[pos++] = cur[base + w0 * 32 + (__ffs(bits) - 1)];
    for (uint32_t bits = b; bits; bits &= bits - 1) clamp[pos++] = cur[base + (w0 + 1) * 32 + (__ffs(bits) - 1)];
}

// Scratch of the two-level tile scan.
struct TileScan {
    size_t chunks;
    size_t o_part, o_epart;
};
static TileScan reserve_tile_scan(Workspace &ws, size_t tiles) {
    TileScan t;
    t.chunks = (tiles + kScanChunk - 1) / kScanChunk;
    t.o_part = ws.reserve<uint32_t>(t.chunks);
    t.o_epart = ws.reserve<unsigned long long>(t.chunks);
    return t;
}
static void launch_tile_scan(Workspace &ws, const TileScan &t, uint32_t *counts, const uint32_t *second, size_t tiles,
                             unsigned long long *tot, cudaStream_t s) {
    k_scan_part<<<static_cast<unsigned>(t.chunks), kScanChunk, 0, s>>>(counts, second, tiles, ws.at<uint32_t>(t.o_part),
                                                                        ws.at<unsigned long long>(t.o_epart));
    k_scan_chunks<<<1, 1024, 0, s>>>(ws.at<uint32_t>(t.o_part), ws.at<unsigned long long>(t.o_epart), t.chunks, tot);
}

// Enqueues the extraction on s; the clamp and edit totals land in host[0]
// and host[1] (pinned) once the stream reaches that point.  packed (or
// null): the symbols packed at nbits bits each instead of one byte per voxel
// in deltas; with packed_host as well, the tiles are extracted in four
// ranges and each range's packed symbols are copied to packed_host on a
// second stream while the next range is extracted (s waits for the copies).
// The scratch is released stream-ordered before return.
constexpr int kExtractRanges = 4;
template <typename T>
int extract_enqueue(const T *prev, const T *cur, const T *f, size_t n, double eb, int q, uint8_t *deltas,
                    uint8_t *packed, int nbits, T *clamp, unsigned long long *host, cudaStream_t s,
                    const uint8_t *cnt, uint8_t *packed_host) {
    if (!prev || !cur || !f || !(deltas || packed) || !clamp || !host) return set_error(PMSZ_ERR_ARG, "null pointer");
    if (n == 0 || n >= (static_cast<size_t>(1) << 32)) return set_error(PMSZ_ERR_ARG, "n must be in 1..2^32-1");
    if (q < 1 || q > 255) return set_error(PMSZ_ERR_ARG, "q must be in 1..255");
    if (!(eb > 0.0)) return set_error(PMSZ_ERR_ARG, "error bound must be positive");
    if (packed && (nbits < 1 || nbits > 8)) return set_error(PMSZ_ERR_ARG, "symbol width must be 1..8 bits");
    const size_t tiles = (n + kTile - 1) / kTile;
    Workspace ws(s);
    const size_t o_flags = ws.reserve<uint32_t>(tiles * (kTile / 32));
    const size_t o_tiles = ws.reserve<uint32_t>(tiles), o_tedits = ws.reserve<uint32_t>(tiles);
    const size_t o_tot = ws.reserve<unsigned long long>(2);
    const TileScan ts = reserve_tile_scan(ws, tiles);
    int rc = ws.commit();
    if (rc) return rc;
    uint32_t *flags = ws.at<uint32_t>(o_flags), *tc = ws.at<uint32_t>(o_tiles), *te = ws.at<uint32_t>(o_tedits);
    unsigned long long *tot = ws.at<unsigned long long>(o_tot);
    const T eps = static_cast<T>(eb);
    const T delta = static_cast<T>(eb / static_cast<double>(q));
    const T inv = static_cast<T>(1.0 / static_cast<double>(delta)), quarter = static_cast<T>(0.25 * static_cast<double>(delta));
    const size_t plen = (n * static_cast<size_t>(nbits) + 7) / 8;
    struct Copies {  // released once their work completes
        cudaStream_t cs = nullptr;
        cudaEvent_t ev[kExtractRanges + 1] = {};
        ~Copies() {
            for (cudaEvent_t e : ev)
                if (e) cudaEventDestroy(e);
            if (cs) cudaStreamDestroy(cs);
        }
    } cp;
    if (packed && packed_host) {
        PMSZ_CUDA(cudaStreamCreateWithFlags(&cp.cs, cudaStreamNonBlocking));
        for (cudaEvent_t &e : cp.ev) PMSZ_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        for (int r = 0; r < kExtractRanges; ++r) {
            const size_t t0 = tiles * r / kExtractRanges, t1 = tiles * (r + 1) / kExtractRanges;
            if (t1 > t0)
                k_extract<T, true><<<static_cast<unsigned>(t1 - t0), 256, 0, s>>>(
                    prev, cur, f, cnt, n, eps, delta, inv, quarter, q, packed, flags, tc, te, nbits, plen,
                    static_cast<uint32_t>(t0));
            PMSZ_CUDA(cudaEventRecord(cp.ev[r], s));
            PMSZ_CUDA(cudaStreamWaitEvent(cp.cs, cp.ev[r], 0));
            const size_t b0 = std::min(plen, t0 * kTile / 8 * static_cast<size_t>(nbits));
            const size_t b1 = std::min(plen, t1 * kTile / 8 * static_cast<size_t>(nbits));
            if (b1 > b0)
                PMSZ_CUDA(cudaMemcpyAsync(packed_host + b0, packed + b0, b1 - b0, cudaMemcpyDeviceToHost, cp.cs));
        }
        PMSZ_CUDA(cudaEventRecord(cp.ev[kExtractRanges], cp.cs));
    } else if (packed) {
        k_extract<T, true><<<static_cast<unsigned>(tiles), 256, 0, s>>>(
            prev, cur, f, cnt, n, eps, delta, inv, quarter, q, packed, flags, tc, te, nbits, plen, 0u);
    } else {
        k_extract<T, false><<<static_cast<unsigned>(tiles), 256, 0, s>>>(prev, cur, f, cnt, n, eps, delta, inv,
                                                                         quarter, q, deltas, flags, tc, te, 8, 0, 0u);
    }
    launch_tile_scan(ws, ts, tc, te, tiles, tot, s);
    k_scatter_clamps<T><<<static_cast<unsigned>((tiles + 7) / 8), 256, 0, s>>>(cur, flags, tc, ws.at<uint32_t>(ts.o_part),
                                                                              n, tiles, clamp);
    PMSZ_CUDA(cudaGetLastError());
    PMSZ_CUDA(cudaMemcpyAsync(host, tot, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    if (cp.cs) PMSZ_CUDA(cudaStreamWaitEvent(s, cp.ev[kExtractRanges], 0));  // the symbols' copies, too
    return ws.release();
}

template <typename T>
int extract_impl(const T *prev, const T *cur, const T *f, size_t n, double eb, int q, uint8_t *deltas, T *clamp,
                 uint64_t *n_clamp, uint64_t *edit_count, cudaStream_t s, const uint8_t *cnt) {
    if (!deltas || !n_clamp || !edit_count) return set_error(PMSZ_ERR_ARG, "null pointer");
    unsigned long long *h = static_cast<unsigned long long *>(host_pinned(2 * sizeof(unsigned long long)));
    if (!h) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
    int rc = extract_enqueue<T>(prev, cur, f, n, eb, q, deltas, nullptr, 8, clamp, h, s, cnt, nullptr);
    if (rc) return rc;
    PMSZ_CUDA(cudaStreamSynchronize(s));
    *n_clamp = h[0];
    *edit_count = h[1];
    return PMSZ_OK;
}

// Thread t packs symbols 8t .. 8t+7 (8 * nbits bits = nbits whole bytes).
__global__ void __launch_bounds__(256) k_pack_deltas(const uint8_t *__restrict__ deltas, size_t n, int nbits,
                                                     uint8_t *__restrict__ out, size_t out_len) {
    const size_t t = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t i0 = t * 8;
    if (i0 >= n) return;
    const uint64_t mask = (1ull << nbits) - 1ull;
    uint64_t v = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (i0 + j < n) v |= (static_cast<uint64_t>(deltas[i0 + j]) & mask) << (j * nbits);
    const size_t b0 = t * static_cast<size_t>(nbits);
    for (int b = 0; b < nbits && b0 + b < out_len; ++b) out[b0 + b] = static_cast<uint8_t>(v >> (8 * b));
}

int bits_for_symbols(int q) {
    int b = 1;
    while ((1 << b) < q + 1) ++b;
    return b;
}

int pack_deltas_impl(const uint8_t *deltas, size_t n, int nbits, uint8_t *out, cudaStream_t s) {
    if (nbits < 1 || nbits > 8) return set_error(PMSZ_ERR_ARG, "symbol width must be 1..8 bits");
    const size_t len = (n * static_cast<size_t>(nbits) + 7) / 8, threads = (n + 7) / 8;
    if (!threads) return PMSZ_OK;
    k_pack_deltas<<<static_cast<unsigned>((threads + 255) / 256), 256, 0, s>>>(deltas, n, nbits, out, len);
    PMSZ_CUDA(cudaGetLastError());
    return PMSZ_OK;
}

// ---------------------------------------------------------------------------
// Reconstruction: the decoder the reference lacks (validateResult,
// pMSz.cu:2545-2584, only decompresses).  The inverse of the extraction per
// voxel: delta k < q lowers the decompressed value k times by delta_step in T
// -- the correction's own repeated subtraction (applyDeltaBuffer_local,
// pMSz.cu:631), so the result is bit-identical to the corrected field -- and
// delta q takes the next value of the clamp list (voxel order).  A symbol
// above q, or a count of q symbols other than the list's length (the
// reference encoder drops clamp values equal to 0, so such a field cannot be
// rebuilt from its files), is an argument error found before anything is
// written.  Kernels: per-tile q flags and counts, the tile scan of the
// extraction, then every voxel's value.
// ---------------------------------------------------------------------------

// Per tile: one flag word per 32 voxels (bit set where the symbol is q), the
// number of q symbols and of symbols above q.  Each thread reads 8 symbols;
// the four lanes whose symbols share a flag word OR their bytes together.
__global__ void __launch_bounds__(256) k_recon_flags(const uint8_t *__restrict__ deltas, size_t n, int q,
                                                     uint32_t *__restrict__ flags, uint32_t *__restrict__ tile_count,
                                                     uint32_t *__restrict__ tile_bad) {
    __shared__ uint32_t s_cnt, s_bad;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0) s_cnt = s_bad = 0;
    __syncthreads();
    const size_t base = static_cast<size_t>(blockIdx.x) * kTile;
    const size_t i0 = base + static_cast<size_t>(threadIdx.x) * 8;
    uint32_t qm = 0, bad = 0;
    uint8_t d8[8];
    if (i0 + 8 <= n && (reinterpret_cast<uintptr_t>(deltas + i0) & 7) == 0) {  // one 8-byte load
        const uint2 u = *reinterpret_cast<const uint2 *>(deltas + i0);
#pragma unroll
        for (int j = 0; j < 8; ++j) d8[j] = static_cast<uint8_t>(((j < 4 ? u.x : u.y) >> ((j & 3) * 8)) & 0xFFu);
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) d8[j] = i0 + j < n ? deltas[i0 + j] : uint8_t(0);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (d8[j] == q && i0 + j < n) qm |= 1u << j;
        bad += d8[j] > q;
    }
    uint32_t word = qm << ((lane & 3) * 8);
    word |= __shfl_xor_sync(0xFFFFFFFFu, word, 1);
    word |= __shfl_xor_sync(0xFFFFFFFFu, word, 2);
    if ((lane & 3) == 0 && i0 < n) flags[i0 >> 5] = word;
    const uint32_t cnt = warp_sum_u32(__popc(qm)), nbad = warp_sum_u32(bad);
    if (lane == 0) {
        if (cnt) atomicAdd(&s_cnt, cnt);
        if (nbad) atomicAdd(&s_bad, nbad);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        tile_count[blockIdx.x] = s_cnt;
        tile_bad[blockIdx.x] = s_bad;
    }
}

// Every voxel of a tile: its clamp rank is the tile's offset, the q flags of
// the tile's earlier words (a prefix over the 64 words in shared memory) and
// the flags below it in its own word.  out may alias prev.
template <typename T>
__global__ void __launch_bounds__(256) k_recon_apply(const T *prev, const uint8_t *__restrict__ deltas,
                                                     const T *__restrict__ clamp, const uint32_t *__restrict__ flags,
                                                     const uint32_t *__restrict__ tile_off,
                                                     const uint32_t *__restrict__ part, size_t n, T delta, int q,
                                                     T *out) {
    __shared__ uint32_t s_fl[kTile / 32], s_pre[kTile / 32];
    const size_t base = static_cast<size_t>(blockIdx.x) * kTile;
    const size_t nw = (std::min(n - base, static_cast<size_t>(kTile)) + 31) / 32;
    if (threadIdx.x < kTile / 32) s_fl[threadIdx.x] = threadIdx.x < nw ? flags[(base >> 5) + threadIdx.x] : 0u;
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive prefix of the popcounts, two words per lane
        const int lane = threadIdx.x;
        const uint32_t a = __popc(s_fl[2 * lane]), b = __popc(s_fl[2 * lane + 1]);
        uint32_t inc = a + b;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += t;
        }
        s_pre[2 * lane] = inc - a - b;
        s_pre[2 * lane + 1] = inc - b;
    }
    __syncthreads();
    const uint32_t t0 = tile_off[blockIdx.x] + part[blockIdx.x / kScanChunk];
    // consecutive threads, consecutive voxels; all eight symbols and values
    // are loaded before any is used, so their loads are in flight together
    int d8[8];
    T v8[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const size_t i = base + static_cast<size_t>(j) * 256 + threadIdx.x;
        d8[j] = i < n ? deltas[i] : 0;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const size_t i = base + static_cast<size_t>(j) * 256 + threadIdx.x;
        v8[j] = i < n ? prev[i] : T(0);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint32_t off = static_cast<uint32_t>(j) * 256 + threadIdx.x;
        const size_t i = base + off;
        if (i >= n) break;
        T v = v8[j];
        if (d8[j] == q) {
            const uint32_t w = off >> 5;
            v = clamp[t0 + s_pre[w] + __popc(s_fl[w] & ((1u << (off & 31)) - 1u))];
        } else {
            for (int k = 0; k < d8[j]; ++k) v = v - delta;
        }
        out[i] = v;
    }
}

template <typename T>
int reconstruct_impl(const T *prev, const uint8_t *deltas, const T *clamp, uint64_t n_clamp, size_t n, double eb,
                     int q, T *out, cudaStream_t s) {
    if (!prev || !deltas || !out || (n_clamp && !clamp)) return set_error(PMSZ_ERR_ARG, "null pointer");
    if (n == 0 || n >= (static_cast<size_t>(1) << 32)) return set_error(PMSZ_ERR_ARG, "n must be in 1..2^32-1");
    if (q < 1 || q > 255) return set_error(PMSZ_ERR_ARG, "q must be in 1..255");
    if (!(eb > 0.0)) return set_error(PMSZ_ERR_ARG, "error bound must be positive");
    const size_t tiles = (n + kTile - 1) / kTile;
    Workspace ws(s);
    const size_t o_flags = ws.reserve<uint32_t>(tiles * (kTile / 32));
    const size_t o_tiles = ws.reserve<uint32_t>(tiles), o_bad = ws.reserve<uint32_t>(tiles);
    const size_t o_tot = ws.reserve<unsigned long long>(2);
    const TileScan ts = reserve_tile_scan(ws, tiles);
    int rc = ws.commit();
    if (rc) return rc;
    uint32_t *flags = ws.at<uint32_t>(o_flags), *tc = ws.at<uint32_t>(o_tiles), *tb = ws.at<uint32_t>(o_bad);
    unsigned long long *tot = ws.at<unsigned long long>(o_tot);
    k_recon_flags<<<static_cast<unsigned>(tiles), 256, 0, s>>>(deltas, n, q, flags, tc, tb);
    launch_tile_scan(ws, ts, tc, tb, tiles, tot, s);
    PMSZ_CUDA(cudaGetLastError());
    unsigned long long *h = static_cast<unsigned long long *>(host_pinned(2 * sizeof(unsigned long long)));
    if (!h) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
    PMSZ_CUDA(cudaMemcpyAsync(h, tot, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    PMSZ_CUDA(cudaStreamSynchronize(s));
    if (h[1]) {
        ws.release();
        return set_error(PMSZ_ERR_ARG, std::to_string(h[1]) + " delta symbols above q");
    }
    if (h[0] != n_clamp) {
        ws.release();
        return set_error(PMSZ_ERR_ARG, "the deltas hold " + std::to_string(h[0]) + " clamp symbols, the clamp list " +
                                           std::to_string(n_clamp) + " values");
    }
    const T delta = static_cast<T>(eb / static_cast<double>(q));
    k_recon_apply<T><<<static_cast<unsigned>(tiles), 256, 0, s>>>(prev, deltas, clamp, flags, tc,
                                                                  ws.at<uint32_t>(ts.o_part), n, delta, q, out);
    PMSZ_CUDA(cudaGetLastError());
    return ws.release();
}

template int extract_enqueue<float>(const float *, const float *, const float *, size_t, double, int, uint8_t *,
                                    uint8_t *, int, float *, unsigned long long *, cudaStream_t, const uint8_t *,
                                    uint8_t *);
template int extract_enqueue<double>(const double *, const double *, const double *, size_t, double, int, uint8_t *,
                                     uint8_t *, int, double *, unsigned long long *, cudaStream_t, const uint8_t *,
                                     uint8_t *);
template int extract_impl<float>(const float *, const float *, const float *, size_t, double, int, uint8_t *, float *,
                                 uint64_t *, uint64_t *, cudaStream_t, const uint8_t *);
template int extract_impl<double>(const double *, const double *, const double *, size_t, double, int, uint8_t *,
                                  double *, uint64_t *, uint64_t *, cudaStream_t, const uint8_t *);
template int reconstruct_impl<float>(const float *, const uint8_t *, const float *, uint64_t, size_t, double, int,
                                     float *, cudaStream_t);
template int reconstruct_impl<double>(const double *, const uint8_t *, const double *, uint64_t, size_t, double, int,
                                      double *, cudaStream_t);

}  // namespace pmsz

using namespace pmsz;

extern "C" int pmsz_extract_edits_f32(const float *prev, const float *cur, const float *f, size_t n, double eb,
                                      int q, uint8_t *deltas, float *clamp, uint64_t *n_clamp,
                                      uint64_t *edit_count, void *stream) {
    return guarded([&] {
        return extract_impl<float>(prev, cur, f, n, eb, q, deltas, clamp, n_clamp, edit_count, as_stream(stream));
    });
}
extern "C" int pmsz_extract_edits_f64(const double *prev, const double *cur, const double *f, size_t n, double eb,
                                      int q, uint8_t *deltas, double *clamp, uint64_t *n_clamp,
                                      uint64_t *edit_count, void *stream) {
    return guarded([&] {
        return extract_impl<double>(prev, cur, f, n, eb, q, deltas, clamp, n_clamp, edit_count, as_stream(stream));
    });
}
extern "C" int pmsz_reconstruct_f32(const float *prev, const uint8_t *deltas, const float *clamp, uint64_t n_clamp,
                                    size_t n, double eb, int q, float *out, void *stream) {
    return guarded([&] {
        return reconstruct_impl<float>(prev, deltas, clamp, n_clamp, n, eb, q, out, as_stream(stream));
    });
}
extern "C" int pmsz_reconstruct_f64(const double *prev, const uint8_t *deltas, const double *clamp, uint64_t n_clamp,
                                    size_t n, double eb, int q, double *out, void *stream) {
    return guarded([&] {
        return reconstruct_impl<double>(prev, deltas, clamp, n_clamp, n, eb, q, out, as_stream(stream));
    });
}
