// host.cu -- host-buffer entry points: the reference's main-program pipeline
// for one rank (pMSz.cu:2855-2987) behind one call.  The caller hands HOST
// arrays; the call copies f and fhat to the device, keeps the pre-correction
// copy the reference keeps in device_decp_copy (pMSz.cu:2898), runs the
// correction loop, and returns the corrected field plus, on request, the edit
// output of gather_cost_sparse / run_extract_edits (pMSz.cu:2429-2543,
// 2140-2226) and a re-verification.  Device buffers are stream-ordered
// allocations on `stream`, freed before return.
#include "internal.h"

#include <cstring>

namespace pmsz {

template <typename T>
int host_impl(const T *f, T *fhat, size_t nx, size_t ny, size_t nz, double eb, const pmsz_opts *opts,
              pmsz_result *res, pmsz_host_outputs *outs, cudaStream_t s) {
    if (!f || !fhat) return set_error(PMSZ_ERR_ARG, "null field pointer");
    if (nx == 0 || ny == 0 || nz == 0) return set_error(PMSZ_ERR_ARG, "field dimensions must be positive");
    const size_t n = nx * ny * nz;
    const bool want_edits = outs && (outs->deltas || outs->clamp);
    const bool want_verify = outs && outs->verify;
    const int q = opts ? opts->q : 5;
    Workspace ws(s);
    const bool packed = opts && (opts->flags & PMSZ_FLAG_PACKED_DELTAS) && outs && outs->deltas;
    const size_t o_f = ws.reserve<T>(n), o_fh = ws.reserve<T>(n);
    const size_t o_prev = ws.reserve<T>(want_edits ? n : 0);
    const size_t o_d = ws.reserve<uint8_t>(want_edits && !packed ? n : 0);
    const size_t o_c = ws.reserve<T>(want_edits ? n : 0);
    const size_t o_cnt = ws.reserve<uint8_t>(want_edits ? n : 0);
    const int nbits = q >= 1 && q <= 255 ? bits_for_symbols(q) : 8;  // q is checked by the correction
    const size_t plen = packed ? (n * static_cast<size_t>(nbits) + 7) / 8 : 0;
    const size_t o_pack = ws.reserve<uint8_t>(plen);
    int rc = ws.commit();
    if (rc) return rc;
    T *df = ws.at<T>(o_f), *dfh = ws.at<T>(o_fh), *dprev = ws.at<T>(o_prev), *dclamp = ws.at<T>(o_c);
    uint8_t *dd = ws.at<uint8_t>(o_d);
    uint8_t *dcnt = want_edits ? ws.at<uint8_t>(o_cnt) : nullptr;
    // the edit output: enqueued by the correction right behind its last
    // kernel where it can (no host round trip in between), else below.  The
    // symbols (packed on the GPU at nbits bits, the reference's pack_nbits,
    // when asked: n * nbits / 8 bytes cross the host link) go back during the
    // extraction; the clamp and edit totals land in h.
    const bool counted = !(opts && (opts->flags & PMSZ_FLAG_NAIVE));  // the pMSz loop leaves its counters in dcnt
    unsigned long long *h = nullptr;
    AfterCorrection after;
    if (want_edits) {
        h = static_cast<unsigned long long *>(host_pinned(2 * sizeof(unsigned long long), 1));
        if (!h) return set_error(PMSZ_ERR_OOM, "pinned host allocation failed");
        uint8_t *dp = packed ? ws.at<uint8_t>(o_pack) : nullptr;
        after.fn = [=](cudaStream_t st) -> int {
            int r = extract_enqueue<T>(dprev, dfh, df, n, eb, q, dd, dp, nbits, dclamp, h, st, counted ? dcnt : nullptr,
                                       packed ? static_cast<uint8_t *>(outs->deltas) : nullptr);
            if (r) return r;
            if (!packed && outs->deltas) PMSZ_CUDA(cudaMemcpyAsync(outs->deltas, dd, n, cudaMemcpyDeviceToHost, st));
            return PMSZ_OK;
        };
    }
    int st;
    if (opts && (opts->flags & PMSZ_FLAG_NAIVE)) {
        PMSZ_CUDA(cudaMemcpyAsync(df, f, n * sizeof(T), cudaMemcpyHostToDevice, s));
        PMSZ_CUDA(cudaMemcpyAsync(dfh, fhat, n * sizeof(T), cudaMemcpyHostToDevice, s));
        if (want_edits) PMSZ_CUDA(cudaMemcpyAsync(dprev, dfh, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
        st = naive_impl<T>(df, dfh, nx, ny, nz, eb, opts, res, s);
    } else {
        // the copies in start now and overlap the fused first pass (slab by
        // slab) and the sweeps behind it
        IngestCopies copies;
        if ((rc = enqueue_ingest<T>(f, fhat, df, dfh, want_edits ? dprev : nullptr, nx, ny, nz, s, copies))) return rc;
        const HostIngest<T> in{f, fhat, df, want_edits ? dprev : nullptr, dcnt, &copies, want_edits ? &after : nullptr};
        st = correct_impl<T>(df, dfh, nx, ny, nz, eb, opts, res, s, &in);
    }
    if (st != PMSZ_OK && st != PMSZ_ERR_NOT_CONVERGED) return st;
    std::string keep = st == PMSZ_ERR_NOT_CONVERGED ? pmsz_last_error() : std::string();
    if (want_edits) {
        if (!after.done && (rc = after.fn(s))) return rc;
        PMSZ_CUDA(cudaStreamSynchronize(s));
        const uint64_t nc = h[0];
        outs->n_clamp = nc;
        outs->edit_count = h[1];
        if (outs->clamp && nc) PMSZ_CUDA(cudaMemcpyAsync(outs->clamp, dclamp, nc * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    if (want_verify && (rc = verify_impl<T>(df, dfh, nx, ny, nz, eb, outs->verify, s))) return rc;
    if (!(opts && (opts->flags & PMSZ_FLAG_EDITS_ONLY)))
        PMSZ_CUDA(cudaMemcpyAsync(fhat, dfh, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    PMSZ_CUDA(cudaStreamSynchronize(s));
    if ((rc = ws.release())) return rc;
    if (st == PMSZ_ERR_NOT_CONVERGED) set_error(st, keep);
    return st;
}

}  // namespace pmsz

using namespace pmsz;

extern "C" int pmsz_correct_host_f32(const float *f, float *fhat, size_t nx, size_t ny, size_t nz, double eb,
                                     const pmsz_opts *opts, pmsz_result *res, pmsz_host_outputs *outs,
                                     void *stream) {
    return guarded([&] { return host_impl<float>(f, fhat, nx, ny, nz, eb, opts, res, outs, as_stream(stream)); });
}
extern "C" int pmsz_correct_host_f64(const double *f, double *fhat, size_t nx, size_t ny, size_t nz, double eb,
                                     const pmsz_opts *opts, pmsz_result *res, pmsz_host_outputs *outs,
                                     void *stream) {
    return guarded([&] { return host_impl<double>(f, fhat, nx, ny, nz, eb, opts, res, outs, as_stream(stream)); });
}
