// verify.cu -- manifold labels by pointer jumping, and re-verification.
//
// Replaces PathCompression (pMSz.cu:255-271): the reference walks every
// vertex's pointer chain to its root one step at a time.  Here every round
// replaces L[i] by L[L[L[i]]] in place (a vertex's pointer only ever moves to
// another vertex of its own chain, so concurrent readers see valid ancestors)
// and the rounds stop when one changes nothing: O(log path length) rounds of
// coalesced work instead of one unbounded walk per thread.  A launch gives
// every vertex up to `rounds` such jumps (the tuned pointer-jumping rounds per
// launch) before the host reads the convergence flag; a launch that changes
// nothing reads a static array, so it certifies the fixpoint.
//
// Verification replaces the reference's disabled check_consistency block
// (pMSz.cu:3038-3126) and count_false_cases (pMSz.cu:1852-1870).
#include "common.cuh"
#include "internal.h"

#include <algorithm>

namespace pmsz {

__global__ void __launch_bounds__(256) k_init_ptr(const uint8_t *__restrict__ codes, uint32_t *__restrict__ as,
                                                  uint32_t *__restrict__ ds, Geom g) {
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= g.nx || y >= g.ny) return;
    const size_t i = flat(g, x, y, z);
    const uint8_t c = codes[i];
    const int a = c & 15, d = c >> 4;
    if (as) as[i] = static_cast<uint32_t>(flat(g, x + rank_dx(a), y + rank_dy(a), z + rank_dz(a)));
    if (ds) ds[i] = static_cast<uint32_t>(flat(g, x + rank_dx(d), y + rank_dy(d), z + rank_dz(d)));
}

__global__ void __launch_bounds__(256) k_jump(uint32_t *__restrict__ L, size_t n, unsigned int *changed,
                                              int rounds) {
    bool any = false;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint32_t l = L[i];
        bool moved = false;
        for (int r = 0; r < rounds; ++r) {
            const uint32_t ll = L[l];
            if (ll == l) break;
            // three hops: a pointer spanning d chain steps now spans at least 3d
            l = L[ll];
            moved = true;
        }
        if (moved) {
            L[i] = l;
            any = true;
        }
    }
    if (__any_sync(0xFFFFFFFFu, any) && (threadIdx.x & 31) == 0) atomicOr(changed, 1u);
}

static inline unsigned grid_for(size_t n) {
    return static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 152 * 16)));
}

static int jump_to_roots(uint32_t *L, size_t n, unsigned int *d_flag, cudaStream_t s, int rounds) {
    unsigned int *h = static_cast<unsigned int *>(host_pinned(sizeof(unsigned int)));
    if (!h) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
    for (int launch = 0; launch < 64; ++launch) {
        PMSZ_CUDA(cudaMemsetAsync(d_flag, 0, sizeof(unsigned int), s));
        k_jump<<<grid_for(n), 256, 0, s>>>(L, n, d_flag, rounds);
        PMSZ_CUDA(cudaGetLastError());
        PMSZ_CUDA(cudaMemcpyAsync(h, d_flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        PMSZ_CUDA(cudaStreamSynchronize(s));
        if (*h == 0) return PMSZ_OK;
    }
    return set_error(PMSZ_ERR_CUDA, "pointer jumping did not reach its fixpoint");
}

int labels_impl(const uint8_t *codes, size_t nx, size_t ny, size_t nz, uint32_t *as, uint32_t *ds, cudaStream_t s) {
    if (!codes) return set_error(PMSZ_ERR_ARG, "null codes pointer");
    int rc = check_geom(nx, ny, nz);
    if (rc) return rc;
    const Geom g = make_geom(nx, ny, nz);
    if (g.n >= (static_cast<size_t>(1) << 32)) return set_error(PMSZ_ERR_ARG, "labels need fewer than 2^32 voxels");
    Workspace ws(s);
    const size_t o_flag = ws.reserve<unsigned int>(1);
    if ((rc = ws.commit())) return rc;
    const dim3 grid(static_cast<unsigned>(g.wpr), static_cast<unsigned>((g.ny + 7) / 8), static_cast<unsigned>(g.nz));
    k_init_ptr<<<grid, dim3(32, 8, 1), 0, s>>>(codes, as, ds, g);
    PMSZ_CUDA(cudaGetLastError());
    const int rounds = tuned_jump_rounds(nx, ny, nz);
    if (as && (rc = jump_to_roots(as, g.n, ws.at<unsigned int>(o_flag), s, rounds))) return rc;
    if (ds && (rc = jump_to_roots(ds, g.n, ws.at<unsigned int>(o_flag), s, rounds))) return rc;
    return ws.release();
}

int time_jump_rounds(const uint8_t *codes, size_t nx, size_t ny, size_t nz, const int *rounds, int m, float *ms,
                     cudaStream_t s) {
    const Geom g = make_geom(nx, ny, nz);
    for (int k = 0; k < m; ++k) ms[k] = 0.f;
    if (g.n >= (static_cast<size_t>(1) << 32)) return PMSZ_OK;  // no labels at this size
    Workspace ws(s);
    const size_t o_l = ws.reserve<uint32_t>(g.n), o_flag = ws.reserve<unsigned int>(1);
    int rc = ws.commit();
    if (rc) return rc;
    uint32_t *L = ws.at<uint32_t>(o_l);
    EventTimer et;
    if ((rc = et.init())) return rc;
    const dim3 grid(static_cast<unsigned>(g.wpr), static_cast<unsigned>((g.ny + 7) / 8), static_cast<unsigned>(g.nz));
    for (int k = 0; k < m; ++k) {
        float best = 0.f;
        for (int rep = 0; rep < 3; ++rep) {  // the first run of each candidate is a warm-up
            k_init_ptr<<<grid, dim3(32, 8, 1), 0, s>>>(codes, L, nullptr, g);
            PMSZ_CUDA(cudaEventRecord(et.ev[0], s));
            if ((rc = jump_to_roots(L, g.n, ws.at<unsigned int>(o_flag), s, rounds[k]))) return rc;
            PMSZ_CUDA(cudaEventRecord(et.ev[1], s));
            PMSZ_CUDA(cudaEventSynchronize(et.ev[1]));
            float t = 0.f;
            PMSZ_CUDA(cudaEventElapsedTime(&t, et.ev[0], et.ev[1]));
            if (rep > 0 && (best == 0.f || t < best)) best = t;
        }
        ms[k] = best;
    }
    return ws.release();
}

template <typename T>
__global__ void __launch_bounds__(256) k_verify_cmp(const T *__restrict__ f, const T *__restrict__ fp,
                                                    const uint8_t *__restrict__ c0, const uint8_t *__restrict__ c1,
                                                    size_t n, T eps, unsigned long long *out) {
    uint32_t dm = 0, em = 0, bs = 0, bc = 0;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint8_t a = c0[i], b = c1[i];
        dm += a != b;
        em += (((a & 15) == kSelf) != ((b & 15) == kSelf)) || (((a >> 4) == kSelf) != ((b >> 4) == kSelf));
        const T fv = f[i], pv = fp[i];
        bs += !(fabs(pv - fv) <= eps);
        bc += !(pv >= fv - eps && pv <= fv + eps);
    }
    dm = warp_sum_u32(dm);
    em = warp_sum_u32(em);
    bs = warp_sum_u32(bs);
    bc = warp_sum_u32(bc);
    if ((threadIdx.x & 31) == 0) {
        if (dm) atomicAdd(out + 0, (unsigned long long)dm);
        if (em) atomicAdd(out + 1, (unsigned long long)em);
        if (bs) atomicAdd(out + 4, (unsigned long long)bs);
        if (bc) atomicAdd(out + 5, (unsigned long long)bc);
    }
}

__global__ void __launch_bounds__(256) k_count_diff(const uint32_t *__restrict__ a, const uint32_t *__restrict__ b,
                                                    size_t n, unsigned long long *out) {
    uint32_t c = 0;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) c += a[i] != b[i];
    c = warp_sum_u32(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, (unsigned long long)c);
}

template <typename T>
int verify_impl(const T *f, const T *fp, size_t nx, size_t ny, size_t nz, double eb, pmsz_verify_result *out,
                cudaStream_t s) {
    if (!f || !fp || !out) return set_error(PMSZ_ERR_ARG, "null pointer");
    int rc = check_geom(nx, ny, nz);
    if (rc) return rc;
    const Geom g = make_geom(nx, ny, nz);
    const bool with_labels = g.n < (static_cast<size_t>(1) << 32);
    Workspace ws(s);
    const size_t o_c0 = ws.reserve<uint8_t>(g.n), o_c1 = ws.reserve<uint8_t>(g.n);
    const size_t o_l0 = ws.reserve<uint32_t>(with_labels ? g.n : 0), o_l1 = ws.reserve<uint32_t>(with_labels ? g.n : 0);
    const size_t o_cnt = ws.reserve<unsigned long long>(6);
    if ((rc = ws.commit())) return rc;
    uint8_t *c0 = ws.at<uint8_t>(o_c0), *c1 = ws.at<uint8_t>(o_c1);
    uint32_t *l0 = ws.at<uint32_t>(o_l0), *l1 = ws.at<uint32_t>(o_l1);
    unsigned long long *cnt = ws.at<unsigned long long>(o_cnt);
    PMSZ_CUDA(cudaMemsetAsync(cnt, 0, 6 * sizeof(unsigned long long), s));
    if ((rc = codes_impl<T>(f, nx, ny, nz, c0, s))) return rc;
    if ((rc = codes_impl<T>(fp, nx, ny, nz, c1, s))) return rc;
    k_verify_cmp<T><<<grid_for(g.n), 256, 0, s>>>(f, fp, c0, c1, g.n, static_cast<T>(eb), cnt);
    PMSZ_CUDA(cudaGetLastError());
    if (with_labels) {
        if ((rc = labels_impl(c0, nx, ny, nz, l0, nullptr, s))) return rc;
        if ((rc = labels_impl(c1, nx, ny, nz, l1, nullptr, s))) return rc;
        k_count_diff<<<grid_for(g.n), 256, 0, s>>>(l0, l1, g.n, cnt + 2);
        if ((rc = labels_impl(c0, nx, ny, nz, nullptr, l0, s))) return rc;
        if ((rc = labels_impl(c1, nx, ny, nz, nullptr, l1, s))) return rc;
        k_count_diff<<<grid_for(g.n), 256, 0, s>>>(l0, l1, g.n, cnt + 3);
        PMSZ_CUDA(cudaGetLastError());
    }
    unsigned long long *h = static_cast<unsigned long long *>(host_pinned(6 * sizeof(unsigned long long)));
    if (!h) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
    PMSZ_CUDA(cudaMemcpyAsync(h, cnt, 6 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    PMSZ_CUDA(cudaStreamSynchronize(s));
    out->dir_mismatch = h[0];
    out->ext_mismatch = h[1];
    out->as_mismatch = with_labels ? h[2] : UINT64_MAX;
    out->ds_mismatch = with_labels ? h[3] : UINT64_MAX;
    out->bound_strict = h[4];
    out->bound_beyond_clamp = h[5];
    return ws.release();
}

template int verify_impl<float>(const float *, const float *, size_t, size_t, size_t, double, pmsz_verify_result *, cudaStream_t);
template int verify_impl<double>(const double *, const double *, size_t, size_t, size_t, double, pmsz_verify_result *, cudaStream_t);

}  // namespace pmsz

using namespace pmsz;

extern "C" int pmsz_labels(const uint8_t *codes, size_t nx, size_t ny, size_t nz, uint32_t *as_label,
                           uint32_t *ds_label, void *stream) {
    return guarded([&] { return labels_impl(codes, nx, ny, nz, as_label, ds_label, as_stream(stream)); });
}
extern "C" int pmsz_verify_f32(const float *f, const float *fp, size_t nx, size_t ny, size_t nz, double eb,
                               pmsz_verify_result *out, void *stream) {
    return guarded([&] { return verify_impl<float>(f, fp, nx, ny, nz, eb, out, as_stream(stream)); });
}
extern "C" int pmsz_verify_f64(const double *f, const double *fp, size_t nx, size_t ny, size_t nz, double eb,
                               pmsz_verify_result *out, void *stream) {
    return guarded([&] { return verify_impl<double>(f, fp, nx, ny, nz, eb, out, as_stream(stream)); });
}
