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

// cnt (optional): the correction's edit counters; a voxel whose counter is 0
// was never edited, so cur == prev there and its three values need not be read.
// Per tile: the clamp flags (one ballot word per 32 voxels), the clamp count
// and the edit count, combined in shared memory (no global atomics: one
// counter shared by every warp serialises at L2).
template <typename T>
__global__ void __launch_bounds__(256) k_extract(const T *__restrict__ prev, const T *__restrict__ cur,
                                                 const T *__restrict__ f, const uint8_t *__restrict__ cnt, size_t n,
                                                 T eps, T delta, int q, uint8_t *__restrict__ deltas,
                                                 uint32_t *__restrict__ flags, uint32_t *__restrict__ tile_count,
                                                 uint32_t *__restrict__ tile_edits) {
    __shared__ uint32_t s_cnt, s_edits;
    if (threadIdx.x == 0) s_cnt = s_edits = 0;
    __syncthreads();
    const size_t base = static_cast<size_t>(blockIdx.x) * kTile;
    uint32_t clamps = 0, edits = 0;
#pragma unroll
    for (int j = 0; j < kTile / 256; ++j) {
        const size_t i = base + static_cast<size_t>(j) * 256 + threadIdx.x;
        bool cl = false;
        if (i < n) {
            uint8_t d = 0;
            const bool touched = !cnt || cnt[i] != 0;
            const T c = touched ? cur[i] : T(0), p = touched ? prev[i] : T(0);
            if (touched && c != p) {
                edits += c < p;
                const T cv = f[i] - eps;
                if (c != cv) {
                    d = static_cast<uint8_t>(round((p - c) / delta));
                } else {
                    d = static_cast<uint8_t>(q);
                    cl = cv != T(0);
                }
            }
            deltas[i] = d;
        }
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, cl);
        if ((threadIdx.x & 31) == 0 && (base + static_cast<size_t>(j) * 256 + (threadIdx.x & ~31u)) < n)
            flags[(base + static_cast<size_t>(j) * 256 + threadIdx.x) >> 5] = bal;
        clamps += cl;
    }
    clamps = warp_sum_u32(clamps);
    edits = warp_sum_u32(edits);
    if ((threadIdx.x & 31) == 0) {
        if (clamps) atomicAdd(&s_cnt, clamps);
        if (edits) atomicAdd(&s_edits, edits);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        tile_count[blockIdx.x] = s_cnt;
        tile_edits[blockIdx.x] = s_edits;
    }
}

// Exclusive scan of `m` tile clamp counts in one block of 1024 threads (total
// in total[0]) and the sum of the tile edit counts (total[1]).
__global__ void __launch_bounds__(1024) k_scan_tiles(uint32_t *__restrict__ counts,
                                                     const uint32_t *__restrict__ edits, size_t m,
                                                     unsigned long long *total) {
    __shared__ unsigned long long s_part[1024];
    __shared__ unsigned long long s_edits[32];
    const size_t per = (m + 1023) / 1024;
    const size_t lo = threadIdx.x * per, hi = std::min(m, lo + per);
    unsigned long long sum = 0, esum = 0;
#pragma unroll 8
    for (size_t i = lo; i < hi; ++i) {
        sum += counts[i];
        esum += edits[i];
    }
    for (int o = 16; o > 0; o >>= 1) esum += __shfl_xor_sync(0xFFFFFFFFu, esum, o);
    if ((threadIdx.x & 31) == 0) s_edits[threadIdx.x >> 5] = esum;
    s_part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
        const unsigned long long v = threadIdx.x >= static_cast<unsigned>(o) ? s_part[threadIdx.x - o] : 0ull;
        __syncthreads();
        s_part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = s_part[threadIdx.x] - sum;
#pragma unroll 8
    for (size_t i = lo; i < hi; ++i) {
        const uint32_t c = counts[i];
        counts[i] = static_cast<uint32_t>(run);  // offsets fit: at most n clamp values, n < 2^32 per call
        run += c;
    }
    if (threadIdx.x == 1023) total[0] = s_part[1023];
    if (threadIdx.x == 0) {
        unsigned long long e = 0;
        for (int w = 0; w < 32; ++w) e += s_edits[w];
        total[1] = e;
    }
}

// One warp per tile: the 64 flag words of the tile (two per lane), a warp scan
// of their popcounts, then every set flag writes its clamp value (cur) at the
// tile's offset plus its rank: clamp values in voxel order.
template <typename T>
__global__ void __launch_bounds__(256) k_scatter_clamps(const T *__restrict__ cur, const uint32_t *__restrict__ flags,
                                                        const uint32_t *__restrict__ tile_off, size_t n, size_t tiles,
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
    uint32_t pos = tile_off[tile] + inc - c;
    for (uint32_t bits = a; bits; bits &= bits - 1) clamp[pos++] = cur[base + w0 * 32 + (__ffs(bits) - 1)];
    for (uint32_t bits = b; bits; bits &= bits - 1) clamp[pos++] = cur[base + (w0 + 1) * 32 + (__ffs(bits) - 1)];
}

template <typename T>
int extract_impl(const T *prev, const T *cur, const T *f, size_t n, double eb, int q, uint8_t *deltas, T *clamp,
                 uint64_t *n_clamp, uint64_t *edit_count, cudaStream_t s, const uint8_t *cnt) {
    if (!prev || !cur || !f || !deltas || !clamp || !n_clamp || !edit_count)
        return set_error(PMSZ_ERR_ARG, "null pointer");
    if (n == 0 || n >= (static_cast<size_t>(1) << 32)) return set_error(PMSZ_ERR_ARG, "n must be in 1..2^32-1");
    if (q < 1 || q > 255) return set_error(PMSZ_ERR_ARG, "q must be in 1..255");
    if (!(eb > 0.0)) return set_error(PMSZ_ERR_ARG, "error bound must be positive");
    const size_t tiles = (n + kTile - 1) / kTile;
    Workspace ws(s);
    const size_t o_flags = ws.reserve<uint32_t>(tiles * (kTile / 32));
    const size_t o_tiles = ws.reserve<uint32_t>(tiles), o_tedits = ws.reserve<uint32_t>(tiles);
    const size_t o_tot = ws.reserve<unsigned long long>(2);
    int rc = ws.commit();
    if (rc) return rc;
    uint32_t *flags = ws.at<uint32_t>(o_flags), *tc = ws.at<uint32_t>(o_tiles), *te = ws.at<uint32_t>(o_tedits);
    unsigned long long *tot = ws.at<unsigned long long>(o_tot);
    const T eps = static_cast<T>(eb);
    const T delta = static_cast<T>(eb / static_cast<double>(q));
    k_extract<T><<<static_cast<unsigned>(tiles), 256, 0, s>>>(prev, cur, f, cnt, n, eps, delta, q, deltas, flags, tc,
                                                              te);
    k_scan_tiles<<<1, 1024, 0, s>>>(tc, te, tiles, tot);
    k_scatter_clamps<T><<<static_cast<unsigned>((tiles + 7) / 8), 256, 0, s>>>(cur, flags, tc, n, tiles, clamp);
    PMSZ_CUDA(cudaGetLastError());
    unsigned long long *h = static_cast<unsigned long long *>(host_pinned(2 * sizeof(unsigned long long)));
    if (!h) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
    PMSZ_CUDA(cudaMemcpyAsync(h, tot, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    PMSZ_CUDA(cudaStreamSynchronize(s));
    *n_clamp = h[0];
    *edit_count = h[1];
    return ws.release();
}

template int extract_impl<float>(const float *, const float *, const float *, size_t, double, int, uint8_t *, float *,
                                 uint64_t *, uint64_t *, cudaStream_t, const uint8_t *);
template int extract_impl<double>(const double *, const double *, const double *, size_t, double, int, uint8_t *,
                                  double *, uint64_t *, uint64_t *, cudaStream_t, const uint8_t *);

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
