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
// counts; (2) one-block exclusive scan of the tile counts; (3) each tile
// writes its clamp values at its offset in voxel order.
#include "common.cuh"
#include "internal.h"

#include <algorithm>

namespace pmsz {

constexpr int kTile = 2048;  // voxels per tile: 256 threads x 8

template <typename T>
__global__ void __launch_bounds__(256) k_extract(const T *__restrict__ prev, const T *__restrict__ cur,
                                                 const T *__restrict__ f, size_t n, T eps, T delta, int q,
                                                 uint8_t *__restrict__ deltas, uint32_t *__restrict__ flags,
                                                 uint32_t *__restrict__ tile_count, unsigned long long *edit_count) {
    __shared__ uint32_t s_cnt;
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    const size_t base = static_cast<size_t>(blockIdx.x) * kTile;
    uint32_t clamps = 0, edits = 0;
#pragma unroll
    for (int j = 0; j < kTile / 256; ++j) {
        const size_t i = base + static_cast<size_t>(j) * 256 + threadIdx.x;
        bool cl = false;
        if (i < n) {
            const T c = cur[i], p = prev[i];
            uint8_t d = 0;
            if (c != p) {
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
        if (edits) atomicAdd(edit_count, (unsigned long long)edits);
    }
    __syncthreads();
    if (threadIdx.x == 0) tile_count[blockIdx.x] = s_cnt;
}

// Exclusive scan of `m` tile counts in one block of 1024 threads; total in *total.
__global__ void __launch_bounds__(1024) k_scan_tiles(uint32_t *__restrict__ counts, size_t m,
                                                     unsigned long long *total) {
    __shared__ unsigned long long s_part[1024];
    const size_t per = (m + 1023) / 1024;
    const size_t lo = threadIdx.x * per, hi = std::min(m, lo + per);
    unsigned long long sum = 0;
    for (size_t i = lo; i < hi; ++i) sum += counts[i];
    s_part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
        const unsigned long long v = threadIdx.x >= static_cast<unsigned>(o) ? s_part[threadIdx.x - o] : 0ull;
        __syncthreads();
        s_part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = s_part[threadIdx.x] - sum;
    for (size_t i = lo; i < hi; ++i) {
        const uint32_t c = counts[i];
        counts[i] = static_cast<uint32_t>(run);  // offsets fit: at most n clamp values, n < 2^32 per call
        run += c;
    }
    if (threadIdx.x == 1023) *total = s_part[1023];
}

template <typename T>
__global__ void __launch_bounds__(256) k_scatter_clamps(const T *__restrict__ cur, const uint32_t *__restrict__ flags,
                                                        const uint32_t *__restrict__ tile_off, size_t n,
                                                        T *__restrict__ clamp) {
    __shared__ uint32_t s_warp[kTile / 32];
    const size_t base = static_cast<size_t>(blockIdx.x) * kTile;
    const size_t nw = (std::min(n - base, static_cast<size_t>(kTile)) + 31) / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // popcount of each flag word of the tile, then an exclusive scan over words
    for (size_t w = threadIdx.x; w < kTile / 32; w += 256) s_warp[w] = w < nw ? __popc(flags[(base >> 5) + w]) : 0u;
    __syncthreads();
    if (warp == 0) {
        uint32_t run = 0;
        for (int c = 0; c < kTile / 32; c += 32) {
            const uint32_t v = s_warp[c + lane];
            uint32_t inc = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
                if (lane >= o) inc += t;
            }
            s_warp[c + lane] = run + inc - v;
            run += __shfl_sync(0xFFFFFFFFu, inc, 31);
        }
    }
    __syncthreads();
    const uint32_t off = tile_off[blockIdx.x];
    for (size_t w = warp; w < nw; w += 8) {
        const uint32_t bits = flags[(base >> 5) + w];
        if ((bits >> lane) & 1u) {
            const uint32_t pos = off + s_warp[w] + __popc(bits & ((1u << lane) - 1u));
            clamp[pos] = cur[base + w * 32 + lane];
        }
    }
}

template <typename T>
int extract_impl(const T *prev, const T *cur, const T *f, size_t n, double eb, int q, uint8_t *deltas, T *clamp,
                 uint64_t *n_clamp, uint64_t *edit_count, cudaStream_t s) {
    if (!prev || !cur || !f || !deltas || !clamp || !n_clamp || !edit_count)
        return set_error(PMSZ_ERR_ARG, "null pointer");
    if (n == 0 || n >= (static_cast<size_t>(1) << 32)) return set_error(PMSZ_ERR_ARG, "n must be in 1..2^32-1");
    if (q < 1 || q > 255) return set_error(PMSZ_ERR_ARG, "q must be in 1..255");
    if (!(eb > 0.0)) return set_error(PMSZ_ERR_ARG, "error bound must be positive");
    const size_t tiles = (n + kTile - 1) / kTile;
    Workspace ws(s);
    const size_t o_flags = ws.reserve<uint32_t>(tiles * (kTile / 32));
    const size_t o_tiles = ws.reserve<uint32_t>(tiles);
    const size_t o_tot = ws.reserve<unsigned long long>(2);
    int rc = ws.commit();
    if (rc) return rc;
    uint32_t *flags = ws.at<uint32_t>(o_flags), *tc = ws.at<uint32_t>(o_tiles);
    unsigned long long *tot = ws.at<unsigned long long>(o_tot);
    PMSZ_CUDA(cudaMemsetAsync(tot, 0, 2 * sizeof(unsigned long long), s));
    const T eps = static_cast<T>(eb);
    const T delta = static_cast<T>(eb / static_cast<double>(q));
    k_extract<T><<<static_cast<unsigned>(tiles), 256, 0, s>>>(prev, cur, f, n, eps, delta, q, deltas, flags, tc, tot + 1);
    k_scan_tiles<<<1, 1024, 0, s>>>(tc, tiles, tot);
    k_scatter_clamps<T><<<static_cast<unsigned>(tiles), 256, 0, s>>>(cur, flags, tc, n, clamp);
    PMSZ_CUDA(cudaGetLastError());
    unsigned long long *h = static_cast<unsigned long long *>(host_pinned(2 * sizeof(unsigned long long)));
    if (!h) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
    PMSZ_CUDA(cudaMemcpyAsync(h, tot, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    PMSZ_CUDA(cudaStreamSynchronize(s));
    *n_clamp = h[0];
    *edit_count = h[1];
    return ws.release();
}

template int extract_impl<float>(const float *, const float *, const float *, size_t, double, int, uint8_t *, float *, uint64_t *, uint64_t *, cudaStream_t);
template int extract_impl<double>(const double *, const double *, const double *, size_t, double, int, uint8_t *, double *, uint64_t *, uint64_t *, cudaStream_t);

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
