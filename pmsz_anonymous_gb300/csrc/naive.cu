// naive.cu -- the naive-MSz correction strategy (naive_MSz.cu c_loops,
// 1887-2220): extrema-only sweeps to a fixpoint, then one repair of the
// integral paths whose segmentation labels differ from the original's
// (extract_false_path, naive_MSz.cu:1767-1864), then a check, repeated until
// the check finds no false extremum and no label mismatch.
//
// Layout: the original and current code bytes (steepest ascent rank in the
// low nibble, descent rank in the high nibble; rank 7 = the voxel itself),
// four uint32 label arrays (AS/DS of the original and of the current field,
// roots found by pointer jumping), one request byte per voxel, and the edit
// counters.  Every kernel is a coalesced grid-stride pass over flat indices;
// the only gathers are the path walks, which run for mismatched voxels only.
//
// Semantics per pass are the snapshot ones of the pMSz loop: an extrema sweep
// reads the codes of fhat at its start and applies the union of its requests
// once per voxel, the same outcome as one legal interleaving of the
// reference's in-place kernel; extract_false_path reads only the codes and the
// labels, which it never writes, so its requests are the reference's exactly.
#include "common.cuh"
#include "helpers.cuh"
#include "internal.h"

#include <algorithm>
#include <vector>

namespace pmsz {

namespace {

struct Offsets {
    long long o[15];  // flat offset of every stencil rank
};

Offsets make_offsets(const Geom &g) {
    Offsets t;
    const long long sy = g.nx, sz = static_cast<long long>(g.nx) * g.ny;
    for (int r = 0; r < 15; ++r) t.o[r] = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
    return t;
}

inline unsigned grid_for(size_t n) {
    return static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 152 * 16)));
}

__device__ __forceinline__ void flush_slot(SweepSlot *slot, uint32_t a, uint32_t b, uint32_t c, uint32_t d,
                                           uint32_t e, uint32_t p, uint32_t act, uint32_t bad) {
    a = warp_sum_u32(a);
    b = warp_sum_u32(b);
    c = warp_sum_u32(c);
    d = warp_sum_u32(d);
    e = warp_sum_u32(e);
    p = warp_sum_u32(p);
    act = warp_sum_u32(act);
    bad = warp_sum_u32(bad);
    if ((threadIdx.x & 31) == 0) {
        if (a) atomicAdd(&slot->fmax, (unsigned long long)a);
        if (b) atomicAdd(&slot->fmin, (unsigned long long)b);
        if (c) atomicAdd(&slot->fdir, (unsigned long long)c);
        if (d) atomicAdd(&slot->requested, (unsigned long long)d);
        if (e) atomicAdd(&slot->changed, (unsigned long long)e);
        if (p) atomicAdd(&slot->progressed, (unsigned long long)p);
        if (act) atomicAdd(&slot->active, (unsigned long long)act);
        if (bad) atomicAdd(&slot->bad, (unsigned long long)bad);
    }
}

}  // namespace

// NaN or the 1e30 sentinel in f or fhat (the reference treats 1e30 as a ghost
// cell, pMSz.cu:215): rejected before the loop.
template <typename T>
__global__ void __launch_bounds__(256) k_naive_bad(const T *__restrict__ a, const T *__restrict__ b, size_t n,
                                                   SweepSlot *slot) {
    uint32_t bad = 0;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        bad += (bad_value(a[i]) || bad_value(b[i])) ? 1u : 0u;
    flush_slot(slot, 0, 0, 0, 0, 0, 0, 0, bad);
}

// Extrema-only detection (iscriticle with data_type=0 in naive_MSz.cu:776-826):
// a false or missing maximum requests the voxel itself (false) or its current
// ascent neighbour (missing); a false or missing minimum requests its
// original descent neighbour (false) or the voxel itself (missing).  No
// direction rule.
__global__ void __launch_bounds__(256) k_naive_extrema(const uint8_t *__restrict__ oc, const uint8_t *__restrict__ cc,
                                                       uint8_t *__restrict__ req, size_t n, Offsets off,
                                                       SweepSlot *slot) {
    uint32_t cmax = 0, cmin = 0;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint8_t o = oc[i], c = cc[i];
        const int oa = o & 15, od = o >> 4, ca = c & 15, cd = c >> 4;
        const bool omax = oa == kSelf, omin = !omax && od == kSelf;
        const bool is_max = ca == kSelf, is_min = cd == kSelf;
        if (is_max != omax) {
            ++cmax;
            req[omax ? static_cast<size_t>(static_cast<long long>(i) + off.o[ca]) : i] = 1;
        }
        if (is_min != omin) {
            ++cmin;
            req[omin ? i : static_cast<size_t>(static_cast<long long>(i) + off.o[od])] = 1;
        }
    }
    flush_slot(slot, cmax, cmin, 0, 0, 0, 0, 0, 0);
}

// The integral-path repair (extract_false_path, fix = 0).  For a voxel whose
// DS label differs: follow the original descent while the current descent
// agrees with it and the vertex is not an original extremum; at the stop
// vertex request its original descent neighbour if the current one differs
// (nothing at an original minimum, whose or_types slot is the -2 marker).
// For an AS label mismatch: follow or_types[2c+1] (the original ascent, or the
// original descent at an original maximum) while the current ascent equals
// it; at the stop vertex request its current ascent neighbour if the two
// differ.  Each walk follows a strictly monotone chain of the original order,
// so it ends within n steps; the bound is a guard, counted in `bad` if hit.
__global__ void __launch_bounds__(256) k_naive_paths(const uint8_t *__restrict__ oc, const uint8_t *__restrict__ cc,
                                                     const uint32_t *__restrict__ as0, const uint32_t *__restrict__ ds0,
                                                     const uint32_t *__restrict__ as1, const uint32_t *__restrict__ ds1,
                                                     uint8_t *__restrict__ req, size_t n, Offsets off,
                                                     SweepSlot *slot) {
    uint32_t fdir = 0, guard = 0;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (ds0[i] != ds1[i]) {
            ++fdir;
            long long cur = static_cast<long long>(i);
            bool ok = true;
            for (size_t steps = 0;; ++steps) {
                const uint8_t o = oc[cur];
                const int oa = o & 15, od = o >> 4, cd = cc[cur] >> 4;
                const bool omax = oa == kSelf, omin = !omax && od == kSelf;
                if (omax || omin || od != cd) break;
                if (steps >= n) {
                    ok = false;
                    break;
                }
                cur += off.o[od];
            }
            if (ok) {
                const uint8_t o = oc[cur];
                const int oa = o & 15, od = o >> 4, cd = cc[cur] >> 4;
                const bool omin = oa != kSelf && od == kSelf;
                if (!omin && od != cd) req[cur + off.o[od]] = 1;
            } else {
                ++guard;
            }
        }
        if (as0[i] != as1[i]) {
            ++fdir;
            long long cur = static_cast<long long>(i);
            bool ok = true, skip = false;
            for (size_t steps = 0;; ++steps) {
                const uint8_t o = oc[cur];
                const int oa = o & 15, od = o >> 4, ca = cc[cur] & 15;
                const int r1 = oa == kSelf ? od : oa;
                if (r1 != ca) break;
                if (r1 == kSelf) {  // a vertex that is its own successor in both fields
                    skip = true;
                    break;
                }
                if (steps >= n) {
                    ok = false;
                    break;
                }
                cur += off.o[r1];
            }
            if (!ok) {
                ++guard;
            } else if (!skip) {
                const uint8_t o = oc[cur];
                const int oa = o & 15, od = o >> 4, ca = cc[cur] & 15;
                const int r1 = oa == kSelf ? od : oa;
                if (r1 != ca) req[cur + off.o[ca]] = 1;
            }
        }
    }
    flush_slot(slot, 0, 0, fdir, 0, 0, 0, 0, guard);
}

// The edits of one pass: every requested voxel once (applyDeltaBuffer_local,
// naive_MSz.cu:620-641), the request cleared.
template <typename T>
__global__ void __launch_bounds__(256) k_naive_apply(const T *__restrict__ f, T *__restrict__ fh,
                                                     uint8_t *__restrict__ cnt, uint8_t *__restrict__ req, size_t n,
                                                     T eps, T delta, int q, SweepSlot *slot) {
    uint32_t rq = 0, ch = 0, pr = 0;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (!req[i]) continue;
        req[i] = 0;
        bool progressed = false;
        ch += apply_one(f, fh, cnt, i, eps, delta, q, progressed);
        pr += progressed ? 1u : 0u;
        ++rq;
    }
    flush_slot(slot, 0, 0, 0, rq, ch, pr, 0, 0);
}

// The check (iscriticle with checkFinal = 1, then extract_false_path with
// fix = 1): false/missing extrema, and per voxel one count for a DS label
// mismatch, else one for an AS label mismatch.
__global__ void __launch_bounds__(256) k_naive_check(const uint8_t *__restrict__ oc, const uint8_t *__restrict__ cc,
                                                     const uint32_t *__restrict__ as0, const uint32_t *__restrict__ ds0,
                                                     const uint32_t *__restrict__ as1, const uint32_t *__restrict__ ds1,
                                                     size_t n, SweepSlot *slot) {
    uint32_t cmax = 0, cmin = 0, cdir = 0;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint8_t o = oc[i], c = cc[i];
        const int oa = o & 15, od = o >> 4, ca = c & 15, cd = c >> 4;
        const bool omax = oa == kSelf, omin = !omax && od == kSelf;
        cmax += (ca == kSelf) != omax;
        cmin += (cd == kSelf) != omin;
        cdir += (ds0[i] != ds1[i]) || (as0[i] != as1[i]);
    }
    flush_slot(slot, cmax, cmin, cdir, 0, 0, 0, 0, 0);
}

template <typename T>
int naive_impl(const T *f, T *fh, size_t nx, size_t ny, size_t nz, double eb, const pmsz_opts *opts,
               pmsz_result *res, cudaStream_t s) {
    if (!f || !fh) return set_error(PMSZ_ERR_ARG, "null field pointer");
    int rc = check_geom(nx, ny, nz);
    if (rc) return rc;
    const int q = opts ? opts->q : 5;
    const int64_t max_sweeps = opts ? opts->max_sweeps : 10000;
    if (!(eb > 0.0) || q < 1 || q > 255 || max_sweeps < 1)
        return set_error(PMSZ_ERR_ARG, "need eb > 0, 1 <= q <= 255 and max_sweeps >= 1");
    const Geom g = make_geom(nx, ny, nz);
    if (g.n >= (static_cast<size_t>(1) << 32))
        return set_error(PMSZ_ERR_ARG, "the naive strategy's labels need fewer than 2^32 voxels");
    const size_t n = g.n;
    const T eps = static_cast<T>(eb), delta = static_cast<T>(eb / q);
    const Offsets off = make_offsets(g);
    const unsigned grid = grid_for(n);

    Workspace ws(s);
    const size_t o_oc = ws.reserve<uint8_t>(n), o_cc = ws.reserve<uint8_t>(n), o_cnt = ws.reserve<uint8_t>(n),
                 o_req = ws.reserve<uint8_t>(n);
    const size_t o_as0 = ws.reserve<uint32_t>(n), o_ds0 = ws.reserve<uint32_t>(n), o_as1 = ws.reserve<uint32_t>(n),
                 o_ds1 = ws.reserve<uint32_t>(n);
    const size_t o_slot = ws.reserve<SweepSlot>(1);
    if ((rc = ws.commit())) return rc;
    uint8_t *oc = ws.at<uint8_t>(o_oc), *cc = ws.at<uint8_t>(o_cc), *cnt = ws.at<uint8_t>(o_cnt),
            *req = ws.at<uint8_t>(o_req);
    uint32_t *as0 = ws.at<uint32_t>(o_as0), *ds0 = ws.at<uint32_t>(o_ds0), *as1 = ws.at<uint32_t>(o_as1),
             *ds1 = ws.at<uint32_t>(o_ds1);
    SweepSlot *slot = ws.at<SweepSlot>(o_slot);
    SweepSlot *hs = static_cast<SweepSlot *>(host_pinned(sizeof(SweepSlot)));
    if (!hs) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");

    EventTimer et;
    if ((rc = et.init())) return rc;
    PMSZ_CUDA(cudaEventRecord(et.ev[0], s));
    int64_t launches = 0;
    auto read_slot = [&]() -> int {
        PMSZ_CUDA(cudaMemcpyAsync(hs, slot, sizeof(SweepSlot), cudaMemcpyDeviceToHost, s));
        PMSZ_CUDA(cudaStreamSynchronize(s));
        return PMSZ_OK;
    };
    auto clear_slot = [&]() -> int {
        PMSZ_CUDA(cudaMemsetAsync(slot, 0, sizeof(SweepSlot), s));
        return PMSZ_OK;
    };

    PMSZ_CUDA(cudaMemsetAsync(cnt, 0, n, s));
    PMSZ_CUDA(cudaMemsetAsync(req, 0, n, s));
    if ((rc = clear_slot())) return rc;
    k_naive_bad<T><<<grid, 256, 0, s>>>(f, fh, n, slot);
    PMSZ_CUDA(cudaGetLastError());
    ++launches;
    if ((rc = read_slot())) return rc;
    if (hs->bad) return set_error(PMSZ_ERR_ARG, "input holds NaN or the 1e30 ghost sentinel");

    // original codes and labels (iscriticle data_type=1 + PathCompression,
    // naive_MSz.cu:1910-1917)
    if ((rc = codes_impl<T>(f, nx, ny, nz, oc, s))) return rc;
    if ((rc = labels_impl(oc, nx, ny, nz, as0, ds0, s))) return rc;

    std::vector<SweepSlot> log;
    int status = PMSZ_ERR_NOT_CONVERGED;
    std::string why = "max_sweeps reached";
    uint64_t hmax = 1, hmin = 1, edits = 0;
    int64_t outer = 0, inner = 0;
    bool labels_current = false;  // as1/ds1 and cc describe the current fhat
    auto record = [&](const SweepSlot &r) { log.push_back(r); };
    auto full = [&]() { return static_cast<int64_t>(log.size()) >= max_sweeps; };
    auto apply_pass = [&]() -> int {
        k_naive_apply<T><<<grid, 256, 0, s>>>(f, fh, cnt, req, n, eps, delta, q, slot);
        PMSZ_CUDA(cudaGetLastError());
        ++launches;
        return PMSZ_OK;
    };

    for (;;) {
        ++outer;
        uint64_t progressed_outer = 0;
        bool stuck = false;
        while (hmax || hmin) {  // extrema-only sweeps
            if (full()) goto done;
            ++inner;
            if ((rc = codes_impl<T>(fh, nx, ny, nz, cc, s))) return rc;
            if ((rc = clear_slot())) return rc;
            k_naive_extrema<<<grid, 256, 0, s>>>(oc, cc, req, n, off, slot);
            PMSZ_CUDA(cudaGetLastError());
            ++launches;
            if ((rc = apply_pass())) return rc;
            if ((rc = read_slot())) return rc;
            record(*hs);
            edits += hs->requested;
            progressed_outer += hs->progressed;
            hmax = hs->fmax;
            hmin = hs->fmin;
            labels_current = false;
            if ((hmax || hmin) && hs->progressed == 0) {
                stuck = true;
                break;
            }
        }
        if (stuck) {
            why = "a sweep changed nothing";
            goto done;
        }
        // path repair
        if (full()) goto done;
        // cc is current here: the last extrema sweep found nothing to edit,
        // or none ran and the previous check left cc and the labels current
        if (!labels_current && (rc = labels_impl(cc, nx, ny, nz, as1, ds1, s))) return rc;
        if ((rc = clear_slot())) return rc;
        k_naive_paths<<<grid, 256, 0, s>>>(oc, cc, as0, ds0, as1, ds1, req, n, off, slot);
        PMSZ_CUDA(cudaGetLastError());
        ++launches;
        if ((rc = apply_pass())) return rc;
        if ((rc = read_slot())) return rc;
        if (hs->bad) {
            status = PMSZ_ERR_CUDA;
            why = "an integral-path walk exceeded its bound";
            goto done;
        }
        record(*hs);
        edits += hs->requested;
        progressed_outer += hs->progressed;
        // check
        if (full()) goto done;
        if ((rc = codes_impl<T>(fh, nx, ny, nz, cc, s))) return rc;
        if ((rc = labels_impl(cc, nx, ny, nz, as1, ds1, s))) return rc;
        labels_current = true;
        if ((rc = clear_slot())) return rc;
        k_naive_check<<<grid, 256, 0, s>>>(oc, cc, as0, ds0, as1, ds1, n, slot);
        PMSZ_CUDA(cudaGetLastError());
        ++launches;
        if ((rc = read_slot())) return rc;
        record(*hs);
        if (!hs->fmax && !hs->fmin && !hs->fdir) {
            status = PMSZ_OK;
            goto done;
        }
        if (!progressed_outer) {
            why = "an outer iteration changed nothing";
            goto done;
        }
        hmax = hs->fmax;
        hmin = hs->fmin;
    }
done:
    PMSZ_CUDA(cudaEventRecord(et.ev[1], s));
    PMSZ_CUDA(cudaEventSynchronize(et.ev[1]));
    float ms_total = 0;
    PMSZ_CUDA(cudaEventElapsedTime(&ms_total, et.ev[0], et.ev[1]));
    if (res) {
        res->sweeps = static_cast<int64_t>(log.size());
        res->iteration = 2 * outer + inner;
        res->edits = edits;
        if (res->sweep_log)
            for (int64_t k = 0; k < std::min<int64_t>(res->sweeps, res->sweep_log_cap); ++k) {
                const SweepSlot &r = log[static_cast<size_t>(k)];
                res->sweep_log[k] = pmsz_sweep_record{r.fmax, r.fmin, r.fdir, r.requested,
                                                      r.changed, r.progressed, r.active, r.bad};
            }
        res->ms_first_pass = res->ms_detect = res->ms_apply = 0.0;
        res->launches = launches;
        res->ms_total = ms_total;
    }
    if ((rc = ws.release())) return rc;
    if (status == PMSZ_ERR_NOT_CONVERGED) return set_error(status, "naive strategy did not converge: " + why);
    if (status != PMSZ_OK) return set_error(status, why);
    return PMSZ_OK;
}

template int naive_impl<float>(const float *, float *, size_t, size_t, size_t, double, const pmsz_opts *,
                               pmsz_result *, cudaStream_t);
template int naive_impl<double>(const double *, double *, size_t, size_t, size_t, double, const pmsz_opts *,
                                pmsz_result *, cudaStream_t);

}  // namespace pmsz

using namespace pmsz;

extern "C" int pmsz_correct_naive_f32(const float *f, float *fhat, size_t nx, size_t ny, size_t nz, double eb,
                                      const pmsz_opts *opts, pmsz_result *res, void *stream) {
    return guarded([&] { return naive_impl<float>(f, fhat, nx, ny, nz, eb, opts, res, as_stream(stream)); });
}
extern "C" int pmsz_correct_naive_f64(const double *f, double *fhat, size_t nx, size_t ny, size_t nz, double eb,
                                      const pmsz_opts *opts, pmsz_result *res, void *stream) {
    return guarded([&] { return naive_impl<double>(f, fhat, nx, ny, nz, eb, opts, res, as_stream(stream)); });
}
