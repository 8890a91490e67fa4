// internal.h -- host-side plumbing shared by the C-ABI translation units:
// thread-local error messages, exception fencing, stream-ordered scratch.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <new>
#include <string>
#include <functional>
#include <vector>

#include "../../include/pmsz.h"
#include "../../include/pmsz_host.h"

namespace pmsz {

// Records `msg` as the calling thread's last error and returns `status`.
int set_error(int status, const std::string &msg);

#define PMSZ_CUDA(expr)                                                                       \
    do {                                                                                      \
        cudaError_t e_ = (expr);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return ::pmsz::set_error(PMSZ_ERR_CUDA, std::string(#expr " failed: ") +         \
                                                        cudaGetErrorString(e_));              \
    } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// No exception crosses the C ABI.
template <class F>
int guarded(F &&fn) noexcept {
    try {
        return fn();
    } catch (const std::bad_alloc &) {
        return set_error(PMSZ_ERR_OOM, "host allocation failed");
    } catch (const std::exception &e) {
        return set_error(PMSZ_ERR_ARG, e.what());
    } catch (...) {
        return set_error(PMSZ_ERR_ARG, "unknown exception");
    }
}

// Keeps the device's default memory pool from returning freed blocks to the
// driver, so repeated calls reuse scratch without new allocations.
void retain_pool_once();

// Stream-ordered scratch: reserve() sizes, commit() makes one cudaMallocAsync
// on the call's stream, at<T>() hands out 256-byte aligned sub-ranges, the
// destructor frees stream-ordered.
class Workspace {
public:
    explicit Workspace(cudaStream_t s) : s_(s) {}
    ~Workspace() { release(); }
    Workspace(const Workspace &) = delete;
    Workspace &operator=(const Workspace &) = delete;

    template <class T>
    size_t reserve(size_t count) {
        const size_t off = total_;
        total_ += (count * sizeof(T) + 255) & ~static_cast<size_t>(255);
        return off;
    }
    int commit();
    template <class T>
    T *at(size_t off) const { return reinterpret_cast<T *>(base_ + off); }
    int release();

private:
    cudaStream_t s_;
    size_t total_ = 0;
    char *base_ = nullptr;
};

// A few CUDA events for per-kernel timing, destroyed with the object.
struct EventTimer {
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    int init() {
        for (auto &e : ev)
            if (cudaEventCreate(&e) != cudaSuccess) return set_error(PMSZ_ERR_CUDA, "cudaEventCreate failed");
        return PMSZ_OK;
    }
    ~EventTimer() {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
};

// Pinned host memory for per-sweep counter read-back: per thread, one block
// per slot (0: the correction's read-back, 1: the edit output's totals).
void *host_pinned(size_t bytes, int slot = 0);

// Implementations behind the C entry points (explicitly instantiated for
// float and double in their translation units).
int check_geom(size_t nx, size_t ny, size_t nz);
// Host-resident inputs of pmsz_correct_host_*: f and fhat are copied in slab
// by slab on a second stream while the fused first pass already runs on the
// slabs that have arrived (the host link, not HBM, bounds that phase).
// df is the device destination of f (the f of correct_impl; fhat goes to its
// fh); dprev, if not null, receives a device copy of the input fhat; cnt, if
// not null, is a caller buffer of n bytes the correction uses as its edit
// counters (left holding them for the edit extraction).
// The slab copies of a host-buffer call (enqueue_ingest): slab j's f and
// fhat go up on cs, then ev[j]; the pre-correction copy of slab j's fhat
// into dprev follows on ds, then evp[j] (without dprev, evp[j] marks ev[j]'s
// point).  Slabs are whole z-chunks of the tile depth, about 64 MiB of f +
// fhat each (cps chunks).  Events and streams are released once their work
// completes.
struct IngestCopies {
    cudaStream_t cs = nullptr, ds = nullptr;
    std::vector<cudaEvent_t> ev, evp;
    int cps = 0, nchunks = 0, nslabs = 0, zc = 0;
    IngestCopies() = default;
    IngestCopies(const IngestCopies &) = delete;
    IngestCopies &operator=(const IngestCopies &) = delete;
    ~IngestCopies() {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : evp)
            if (e) cudaEventDestroy(e);
        if (cs) cudaStreamDestroy(cs);
        if (ds) cudaStreamDestroy(ds);
    }
};
// Enqueues the copies of a host-buffer call as soon as the destinations df,
// dfh (and dprev) exist on s: the copy stream waits for s only up to here,
// not for the correction's own setup.
template <typename T>
int enqueue_ingest(const T *hf, const T *hfh, T *df, T *dfh, T *dprev, size_t nx, size_t ny, size_t nz,
                   cudaStream_t s, IngestCopies &c);

// Work the caller wants on the stream right behind the correction's last
// kernel and ahead of its read-back (the host-buffer edit output): fn is
// called once, by correct_impl where its path allows (done is then set),
// else by the caller after it.
struct AfterCorrection {
    std::function<int(cudaStream_t)> fn;
    bool done = false;
};
template <typename T>
struct HostIngest {
    const T *hf, *hfh;
    T *df, *dprev;
    uint8_t *cnt;
    const IngestCopies *copies;  // enqueued by enqueue_ingest
    AfterCorrection *after;      // or null
};
template <typename T>
int correct_impl(const T *f, T *fh, size_t nx, size_t ny, size_t nz, double eb, const pmsz_opts *opts,
                 pmsz_result *res, cudaStream_t s, const HostIngest<T> *ingest = nullptr);
// AS / DS labels (roots of the steepest-ascent / descent forests) of a code
// array; n < 2^32.
int labels_impl(const uint8_t *codes, size_t nx, size_t ny, size_t nz, uint32_t *as, uint32_t *ds, cudaStream_t s);
// Tuning table (tune.cu): the tile depth (planes per tile column) and the
// pointer-jumping rounds per launch recorded for a shape class, or the
// defaults; tune_known says whether the class has an entry.
int tuned_zchunk(size_t nx, size_t ny, size_t nz, size_t elem);
int tuned_jump_rounds(size_t nx, size_t ny, size_t nz);
bool tune_known(size_t nx, size_t ny, size_t nz, size_t elem);
// The batch tile depth of a batch's size class (voxels, field count, element
// size), tuned over the whole table; and the candidate depths.
int tuned_batch_zchunk(size_t voxels, int nfields, size_t elem);
bool batch_tune_known(size_t voxels, int nfields, size_t elem);
void record_batch_zchunk(size_t voxels, int nfields, size_t elem, int zc);
const int *zchunk_candidates(int *count);
template <typename T>
int autotune_impl(const T *f, const T *fh, size_t nx, size_t ny, size_t nz, pmsz_tune *out, cudaStream_t s);
// The tuner's measurements: the fused first pass at each tile depth
// (correct.cu), and the AS labels of a code array at each rounds-per-launch
// count (verify.cu).
template <typename T>
int time_first_pass(const T *f, const T *fh, size_t nx, size_t ny, size_t nz, uint8_t *codes, const int *zcs, int m,
                    float *ms, cudaStream_t s);
int time_jump_rounds(const uint8_t *codes, size_t nx, size_t ny, size_t nz, const int *rounds, int m, float *ms,
                     cudaStream_t s);
template <typename T>
int naive_impl(const T *f, T *fh, size_t nx, size_t ny, size_t nz, double eb, const pmsz_opts *opts,
               pmsz_result *res, cudaStream_t s);
template <typename T>
int codes_impl(const T *v, size_t nx, size_t ny, size_t nz, uint8_t *codes, cudaStream_t s);
template <typename T>
int verify_impl(const T *f, const T *fp, size_t nx, size_t ny, size_t nz, double eb, pmsz_verify_result *out,
                cudaStream_t s);
// Delta symbols packed LSB-first at nbits bits each (pack_nbits,
// pMSz.cu:2328-2348) into ceil(n * nbits / 8) bytes; bits_for_max(q) is
// ceil(log2(q + 1)) (pMSz.cu:2352-2356).
int bits_for_symbols(int q);
int pack_deltas_impl(const uint8_t *deltas, size_t n, int nbits, uint8_t *out, cudaStream_t s);
// cnt (optional): edit counters of the correction that turned prev into cur;
// voxels with counter 0 are then known unchanged and not read.
template <typename T>
int extract_impl(const T *prev, const T *cur, const T *f, size_t n, double eb, int q, uint8_t *deltas, T *clamp,
                 uint64_t *n_clamp, uint64_t *edit_count, cudaStream_t s, const uint8_t *cnt = nullptr);
// The same without the synchronisation: the clamp and edit totals land in
// host[0], host[1] (pinned) once the stream reaches them; with packed set the
// symbols go there at nbits bits each (pack_nbits' layout) instead of deltas,
// and with packed_host as well they are also copied there, range by range,
// overlapping the extraction (complete when s reaches the end).
template <typename T>
int extract_enqueue(const T *prev, const T *cur, const T *f, size_t n, double eb, int q, uint8_t *deltas,
                    uint8_t *packed, int nbits, T *clamp, unsigned long long *host, cudaStream_t s,
                    const uint8_t *cnt, uint8_t *packed_host);

}  // namespace pmsz
