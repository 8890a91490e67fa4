/*
 * pmsz.h -- C ABI of the GB300-native pMSz correction path.
 *
 * Plain pointers and sizes only.  Field pointers are DEVICE pointers owned by
 * the caller; `stream` is a cudaStream_t passed as void* (NULL = the legacy
 * default stream).  Every entry point returns a status code (PMSZ_OK = 0) and
 * never aborts the process or the CUDA context; pmsz_last_error() describes
 * the most recent failure on the calling thread.
 *
 * Fields are x-fastest, then y, then z: the raw layout the reference reads
 * (read_subblock, pMSz.cu:274-313), without the reference's one-voxel padding
 * -- the domain boundary is handled by in-domain tests, which is what the
 * reference's INVALID_VAL halo encodes at an MPI grid of 1x1x1
 * (pMSz.cu:346-381, 673-679, 709).
 */
#ifndef PMSZ_H
#define PMSZ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PMSZ_OK 0
#define PMSZ_ERR_ARG 1            /* bad sizes / eb / q, NaN input, null pointer */
#define PMSZ_ERR_OOM 2            /* device or host allocation failed */
#define PMSZ_ERR_NOT_CONVERGED 3  /* max_sweeps reached, or a sweep changed nothing */
#define PMSZ_ERR_CUDA 4           /* a CUDA runtime call failed */
#define PMSZ_ERR_IO 5             /* file read / write failed (host helpers) */

/* Sweep schedule flags. */
#define PMSZ_FLAG_FULL_SWEEPS 1u  /* every detection sweep scans the whole field
                                     (the reference's schedule) instead of only
                                     voxels whose neighbourhood changed */
#define PMSZ_FLAG_TIMING 2u       /* record CUDA events around every kernel on
                                     `stream` and report per-kernel device time
                                     in pmsz_result */
#define PMSZ_FLAG_EDITS_ONLY 4u   /* pmsz_correct_host_*: hand back only the
                                     edit output (deltas, clamp list) the
                                     reference's main copies to the host
                                     (pMSz.cu:2429-2543) and leave the host
                                     fhat unchanged */
#define PMSZ_FLAG_NAIVE 8u        /* pmsz_correct_host_*: run the naive-MSz
                                     strategy (pmsz_correct_naive_*) instead of
                                     the pMSz loop */
#define PMSZ_FLAG_PACKED_DELTAS 32u /* pmsz_correct_host_*: outs->deltas receives
                                     the delta symbols packed on the GPU as
                                     the reference's pack_nbits does
                                     (pMSz.cu:2328-2348): LSB-first,
                                     bits_for_max(q) bits each (3 for q = 5),
                                     ceil(n * bits / 8) bytes -- what
                                     pmsz_encode_packed_deltas compresses */
#define PMSZ_FLAG_AUTOTUNE 16u    /* pmsz_correct_{f32,f64} and
                                     pmsz_correct_batch: a field whose shape
                                     class has no entry in the tuning table is
                                     first tuned on its own inputs
                                     (pmsz_autotune_*); without the flag the
                                     table is only read */
#define PMSZ_FLAG_HOST_LOOP 64u   /* pmsz_correct_{f32,f64}: run the voxel-list
                                     sweeps from the host, two per round trip
                                     to the device-side stop rule, instead of
                                     as a CUDA graph with a conditional while
                                     node (same kernels, same results; for
                                     profilers and debuggers that cannot
                                     look into conditional graph nodes) */

typedef struct pmsz_opts {
    int32_t q;           /* edit levels; the reference hard-codes q = 5 (pMSz.cu:2630) */
    uint32_t flags;      /* PMSZ_FLAG_* */
    int64_t max_sweeps;  /* cap on detection sweeps; the reference has none */
} pmsz_opts;

/* One record per detection sweep.  fmax / fmin / fdir are the reference's
 * count_f_max / count_f_min / count_f_dir (pMSz.cu:174, 791-895), counted
 * exactly. */
typedef struct pmsz_sweep_record {
    uint64_t fmax, fmin, fdir;
    uint64_t requested;   /* distinct vertices edited in the sweep */
    uint64_t changed;     /* ... whose value changed */
    uint64_t progressed;  /* ... whose value or edit counter changed */
    uint64_t active;      /* voxels the detection pass examined */
    uint64_t bad;         /* NaN / 1e30-sentinel voxels seen (first sweep) */
} pmsz_sweep_record;

typedef struct pmsz_result {
    int64_t sweeps;        /* detection sweeps run, including the final zero one */
    int64_t iteration;     /* the value the reference prints as "iteration is:"
                              (pMSz.cu:2073): sweeps + 1 at one rank */
    uint64_t edits;        /* sum of `requested` over all sweeps */
    pmsz_sweep_record *sweep_log;  /* optional host array, filled with min(sweeps,
                                      sweep_log_cap) records */
    int64_t sweep_log_cap;
    /* With PMSZ_FLAG_TIMING (else 0): device milliseconds of the fused
     * labelling + first detection pass, of all later detection passes, and of
     * all edit passes (sweeps that run inside the device-side sweep loop count
     * whole, edits included, as detection time; in the host-buffer calls,
     * whose first sweeps run behind the copy in, the first-pass figure spans
     * the copy and those sweeps); launches = kernels launched by the call. */
    double ms_first_pass, ms_detect, ms_apply;
    int64_t launches;
    /* Device milliseconds from the first to the last kernel of the loop
     * (always measured): the window of the reference's "comfputational
     * overhead" print, pMSz.cu:2905-2950. */
    double ms_total;
} pmsz_result;

/* Verification counts (replaces the reference's disabled check_consistency
 * block, pMSz.cu:3038-3126, and count_false_cases, pMSz.cu:1852-1870). */
typedef struct pmsz_verify_result {
    uint64_t dir_mismatch;      /* voxels whose steepest asc or desc differs */
    uint64_t ext_mismatch;      /* voxels whose max / min flag differs */
    uint64_t as_mismatch;       /* voxels whose ascending-manifold label differs */
    uint64_t ds_mismatch;       /* voxels whose descending-manifold label differs */
    uint64_t bound_strict;      /* voxels with |f' - f| > eps evaluated in T */
    uint64_t bound_beyond_clamp;/* voxels outside [fl(f - eps), fl(f + eps)]: the
                                   reference's clamp value fl(f - eps) may sit up
                                   to half an ulp beyond eps, so this count is
                                   the one that must be zero */
} pmsz_verify_result;

/*
 * pmsz_correct_{f32,f64}: the correction loop.  Replaces c_loops<T>
 * (pMSz.cu:1872-2074) as called from main at pMSz.cu:2916, at an MPI grid of
 * 1x1x1.  f is the original field, fhat its decompressed copy, corrected in
 * place.  eb is the absolute error bound (argv[2], pMSz.cu:2628);
 * delta = eb / q with the division in double (pMSz.cu:2814).  opts may be
 * NULL (q = 5, no flags, max_sweeps = 10000); res may be NULL.
 * Semantics are snapshot sweeps: every read of a sweep sees the field as it
 * was when the sweep started, and each requested vertex is edited once per
 * sweep with the arithmetic of applyDeltaBuffer_local (pMSz.cu:623-645).
 * Library-owned scratch (direction codes, edit counters, bitmaps) is
 * allocated stream-ordered on `stream` and released before return.
 * Returns PMSZ_ERR_NOT_CONVERGED (fhat holds the last state) if max_sweeps is
 * reached or a sweep requests edits that change nothing (every requested
 * vertex already clamped), where the reference would loop forever.
 */
int pmsz_correct_f32(const float *f, float *fhat, size_t nx, size_t ny, size_t nz,
                     double eb, const pmsz_opts *opts, pmsz_result *res, void *stream);
int pmsz_correct_f64(const double *f, double *fhat, size_t nx, size_t ny, size_t nz,
                     double eb, const pmsz_opts *opts, pmsz_result *res, void *stream);

/*
 * pmsz_correct_naive_{f32,f64}: the naive-MSz strategy, replacing c_loops of
 * naive_MSz.cu (naive_MSz.cu:1887-2220), the reference's second program.  One
 * outer iteration runs extrema-only sweeps (false / missing maxima and minima,
 * no direction rule; naive_MSz.cu:776-826) until one finds none, then one
 * integral-path repair -- AS / DS labels of the current field by pointer
 * jumping, and for every voxel whose label differs from the original's a walk
 * along the agreeing directions to the first divergence, where one vertex is
 * lowered (extract_false_path, naive_MSz.cu:1767-1864) -- then a check that
 * counts false extrema and label mismatches; the loop ends when the check
 * finds none.  The result preserves the extrema and both segmentations (not
 * every steepest direction, which pmsz_correct_* also preserves).  Same
 * arguments, scratch rules and edit arithmetic as pmsz_correct_*.  Records in
 * res->sweep_log: one per extrema sweep {fmax, fmin, 0, requested, changed},
 * one per path repair {0, 0, label mismatches, requested, changed}, one per
 * check {fmax, fmin, voxels with a DS (else AS) label mismatch, 0, 0};
 * res->iteration is the reference's `ite` (2 per outer iteration plus 1 per
 * extrema sweep).  Needs nx*ny*nz < 2^32.  Returns PMSZ_ERR_NOT_CONVERGED at
 * max_sweeps records, when an extrema sweep changes nothing, or when a whole
 * outer iteration changes nothing (the reference would loop forever).
 */
int pmsz_correct_naive_f32(const float *f, float *fhat, size_t nx, size_t ny, size_t nz,
                           double eb, const pmsz_opts *opts, pmsz_result *res, void *stream);
int pmsz_correct_naive_f64(const double *f, double *fhat, size_t nx, size_t ny, size_t nz,
                           double eb, const pmsz_opts *opts, pmsz_result *res, void *stream);

/*
 * pmsz_correct_noalloc: the same correction as pmsz_correct_{f32,f64}, but
 * without allocating any memory -- for callers that cannot call cudaMalloc or
 * a caching allocator while they run, typically because another component
 * already owns the GPU's memory (an in-situ pipeline inside a simulation that
 * reserved HBM up front, a service with a fixed memory budget) or because an
 * allocator call is not acceptable on their path.  It has no counterpart in
 * the reference.  elem_size selects the field type: 4 = float, 8 = double.
 * The caller passes the fields as for pmsz_correct_*; every other buffer is a
 * fixed array inside the library image (PMSZ_NOALLOC_SCRATCH_BYTES, about
 * 5.75 MiB), which every GPU that loads the library holds until the process
 * exits.  Limits, rejected with PMSZ_ERR_ARG and a message: nx*ny*nz <=
 * PMSZ_NOALLOC_MAX_VOXELS (2^21, e.g. 128^3), ceil(nx/32)*ny*nz <=
 * PMSZ_NOALLOC_MAX_WORDS, max_sweeps <= PMSZ_NOALLOC_MAX_SWEEPS (also the
 * default).  Every call looks up the array's device address in the calling
 * thread's current context (cudaGetSymbolAddress, no allocation), so the
 * address stays right after cudaDeviceReset or in another context; the
 * first call in a context also loads the library's device code there, so
 * make it before any stream capture.  All calls on a device share the
 * array and every call clears what must start at zero, so calls that
 * overlap on the GPU (two streams, or two host threads) race: serialise
 * them.  PMSZ_FLAG_TIMING is ignored: ms_first_pass, ms_detect and ms_apply
 * are 0; ms_total is the host clock over the loop, which synchronises the
 * stream after every sweep.
 */
#define PMSZ_NOALLOC_MAX_VOXELS 2097152u
#define PMSZ_NOALLOC_MAX_WORDS 131072u
#define PMSZ_NOALLOC_MAX_SWEEPS 4096u
#define PMSZ_NOALLOC_SCRATCH_BYTES (2u * PMSZ_NOALLOC_MAX_VOXELS + 12u * PMSZ_NOALLOC_MAX_WORDS + 64u * PMSZ_NOALLOC_MAX_SWEEPS)
int pmsz_correct_noalloc(const void *f, void *fhat, size_t elem_size, size_t nx, size_t ny, size_t nz,
                         double eb, const pmsz_opts *opts, pmsz_result *res, void *stream);

/* One field of a batch: device pointers as for pmsz_correct_*, elem_size 4
 * (float) or 8 (double). */
typedef struct pmsz_field {
    const void *f;
    void *fhat;
    size_t nx, ny, nz;
    double eb;
    uint32_t elem_size;
    uint32_t reserved;
} pmsz_field;

/*
 * pmsz_correct_batch: corrects `count` (1..4096) independent fields together --
 * the batched form of the c_loops call (pMSz.cu:1872-2074), which the
 * reference runs one field per program.  One fused first pass covers the tiles
 * of every field, multi-field sweeps follow while the fields' active sets are
 * large, and a single cooperative persistent launch finishes the light tail
 * with a per-field stop decision on the device.  Every field keeps its own
 * scratch, sweep index and stop state, so fields[i].fhat ends bit-identical to
 * what pmsz_correct_* produces for that field alone, and results[i] /
 * statuses[i] (either may be NULL) are what that call would report (timing
 * fields 0).  Fields of both types may be mixed; they run as one batch per
 * type.  Returns PMSZ_OK if every field converged, else the first non-OK
 * status.
 */
int pmsz_correct_batch(const pmsz_field *fields, int count, const pmsz_opts *opts, pmsz_result *results,
                       int *statuses, void *stream);

/*
 * Correction server (continuous batching).  The reference corrects one field
 * per program run; the server accepts jobs from any host thread and runs them
 * on the device current at pmsz_server_create.  A worker thread repeats
 * generations: admit queued jobs in arrival order while the HBM budget (the
 * job's two fields plus its scratch) and the running-job limit allow, run one
 * sweep of every running job in shared multi-field launches (the fused first
 * pass for jobs admitted now), and retire jobs whose correction stopped.  A
 * job's result is bit-identical to pmsz_correct_* on the same field alone.
 * Field pointers are device pointers the caller keeps alive, and whose
 * producing work the caller has completed (e.g. synchronised) before submit;
 * fhat is corrected in place.
 */
typedef struct pmsz_server pmsz_server;

typedef struct pmsz_server_config {
    size_t hbm_budget_bytes;  /* admission budget; 0 = unlimited */
    int32_t max_jobs;         /* running jobs at once; <= 0 selects 256 (max 4096) */
    int32_t q;                /* <= 0 selects 5 */
    int64_t max_sweeps;       /* <= 0 selects 10000 */
} pmsz_server_config;

typedef struct pmsz_job_info {
    int32_t done;             /* 1 once the job finished */
    int32_t status;           /* PMSZ_* of the job's correction */
    int64_t sweeps;
    uint64_t edits;
    double queue_ms;          /* submit -> admission */
    double run_ms;            /* admission -> retirement */
    double latency_ms;        /* submit -> retirement */
} pmsz_job_info;

int pmsz_server_create(const pmsz_server_config *cfg, pmsz_server **out);
int pmsz_server_submit(pmsz_server *srv, const pmsz_field *field, uint64_t *job_id);
/* Waits up to timeout_s seconds (< 0: forever, 0: poll) and fills *info;
 * info->done tells whether the job finished. */
int pmsz_server_wait(pmsz_server *srv, uint64_t job_id, double timeout_s, pmsz_job_info *info);
/* Forgets a finished job. */
int pmsz_server_release(pmsz_server *srv, uint64_t job_id);
/* Finishes every submitted job, then stops the worker and frees the server. */
int pmsz_server_destroy(pmsz_server *srv);

/*
 * pmsz_codes_{f32,f64}: steepest-direction labelling of one field -- the
 * neighbour scan and or_types encoding of iscriticle data_type=1
 * (pMSz.cu:686-783).  codes[i] (device, n bytes): low nibble = stencil rank of
 * the steepest ascent neighbour, high nibble = rank of the steepest descent
 * neighbour (rank 7 = the voxel itself; see pmsz_rank_offset).
 */
int pmsz_codes_f32(const float *v, size_t nx, size_t ny, size_t nz, uint8_t *codes, void *stream);
int pmsz_codes_f64(const double *v, size_t nx, size_t ny, size_t nz, uint8_t *codes, void *stream);

/* (dx, dy, dz) of stencil rank r (0..14); returns PMSZ_ERR_ARG for other r. */
int pmsz_rank_offset(int r, int *dx, int *dy, int *dz);

/*
 * pmsz_labels: ascending / descending manifold labels from direction codes by
 * pointer jumping.  Replaces PathCompression (pMSz.cu:255-271; used in the
 * loop by naive_MSz.cu:1914-1917, 2045-2047).  as_label / ds_label are device
 * arrays of n uint32 flat indices of the maximum / minimum each voxel's
 * steepest path reaches; either may be NULL.  Needs nx*ny*nz < 2^32.
 */
int pmsz_labels(const uint8_t *codes, size_t nx, size_t ny, size_t nz,
                uint32_t *as_label, uint32_t *ds_label, void *stream);

/* pmsz_verify_{f32,f64}: re-verification of a corrected field fp against f. */
int pmsz_verify_f32(const float *f, const float *fp, size_t nx, size_t ny, size_t nz,
                    double eb, pmsz_verify_result *out, void *stream);
int pmsz_verify_f64(const double *f, const double *fp, size_t nx, size_t ny, size_t nz,
                    double eb, pmsz_verify_result *out, void *stream);

/*
 * pmsz_extract_edits_{f32,f64}: edit output.  Replaces extract_edits_kernel +
 * run_extract_edits + compact_edits_dense_to_sparse (pMSz.cu:2090-2226,
 * 227-250).  Over the n voxels in x-fastest order, comparing the corrected
 * field cur with the decompressed field prev:
 *   cur == prev       -> deltas[i] = 0
 *   cur == f - eps    -> deltas[i] = q; f - eps is appended to clamp[] unless 0
 *   otherwise         -> deltas[i] = round((prev - cur) / delta)
 * deltas (n bytes) and clamp (up to n values) are device arrays; *n_clamp and
 * *edit_count (voxels with cur < prev, the reference's "Edit count") are
 * written to host memory.  clamp keeps voxel order, like thrust::copy_if.
 */
int pmsz_extract_edits_f32(const float *prev, const float *cur, const float *f, size_t n,
                           double eb, int q, uint8_t *deltas, float *clamp,
                           uint64_t *n_clamp, uint64_t *edit_count, void *stream);
int pmsz_extract_edits_f64(const double *prev, const double *cur, const double *f, size_t n,
                           double eb, int q, uint8_t *deltas, double *clamp,
                           uint64_t *n_clamp, uint64_t *edit_count, void *stream);

/*
 * pmsz_reconstruct_{f32,f64}: the decoder the reference lacks (validateResult,
 * pMSz.cu:2545-2584, only decompresses); the inverse of pmsz_extract_edits.
 * Over the n voxels, from the decompressed field prev:
 *   deltas[i] == q    -> out[i] = the next value of clamp[] (voxel order)
 *   deltas[i] == k < q -> out[i] = prev[i] lowered k times by delta = (T)(eb/q)
 *                         in T, the correction's own repeated subtraction
 *                         (pMSz.cu:631), so out is bit-identical to the
 *                         corrected field
 * All arrays are device arrays; out may be prev (in place).  PMSZ_ERR_ARG,
 * with nothing written, for a symbol above q or a count of q symbols other
 * than n_clamp (the reference encoder drops clamp values equal to 0, so such
 * a field cannot be rebuilt from its files).
 */
int pmsz_reconstruct_f32(const float *prev, const uint8_t *deltas, const float *clamp,
                         uint64_t n_clamp, size_t n, double eb, int q, float *out,
                         void *stream);
int pmsz_reconstruct_f64(const double *prev, const uint8_t *deltas, const double *clamp,
                         uint64_t n_clamp, size_t n, double eb, int q, double *out,
                         void *stream);

/*
 * Synthetic inputs (not part of the reference's path; its generator is
 * generate_perlin.py).  pmsz_gen_perlin_*: normalised Perlin fBm, bit-identical
 * to the numpy generator in pmsz_anonymous_gb300/fields.py.  perm512: host
 * array of 512 int32; amps / freqs: host arrays of `octaves` doubles.
 * pmsz_standin_*: decompressed stand-ins, kind 0 = "sz3" plateaus,
 * kind 1 = "zfp" bounded noise (same bits as fields.py).
 */
int pmsz_gen_perlin_f32(float *out, size_t nx, size_t ny, size_t nz, const int32_t *perm512,
                        const double *amps, const double *freqs, int octaves, void *stream);
int pmsz_gen_perlin_f64(double *out, size_t nx, size_t ny, size_t nz, const int32_t *perm512,
                        const double *amps, const double *freqs, int octaves, void *stream);
int pmsz_standin_f32(const float *f, float *fhat, size_t n, double eb, int kind,
                     uint64_t seed, void *stream);
int pmsz_standin_f64(const double *f, double *fhat, size_t n, double eb, int kind,
                     uint64_t seed, void *stream);

/*
 * Autotuning.  Two launch parameters are picked per shape class (the ceil-log2
 * of each axis, and the element size for the tile depth) and kept in a
 * process-wide table that every entry point reads:
 *   zchunk      planes per tile column of the fused first pass and the other
 *               tiled passes (tile 32 x 8 x zchunk); candidates 8, 16, 32, 64;
 *               default 32.
 *   jump_rounds pointer-jumping rounds per launch of the label passes
 *               (pmsz_labels, pmsz_verify_*, the naive strategy): each launch
 *               lets every voxel take that many three-hop jumps before the
 *               host reads the convergence flag; candidates 1, 2, 4, 8;
 *               default 1.
 * pmsz_autotune_{f32,f64} times every candidate on the given device field pair
 * (the first pass on f / fhat, then the AS labels of f's codes) on `stream`,
 * records the fastest in the table and returns the measurements.  Results of
 * the correction do not depend on either parameter.
 */
typedef struct pmsz_tune {
    int32_t zchunk;
    int32_t jump_rounds;
    float ms_zchunk[4];  /* first-pass time per candidate 8, 16, 32, 64 (0: not run) */
    float ms_rounds[4];  /* AS-label time per candidate 1, 2, 4, 8 (0: not run) */
} pmsz_tune;

int pmsz_autotune_f32(const float *f, const float *fhat, size_t nx, size_t ny, size_t nz, pmsz_tune *out,
                      void *stream);
int pmsz_autotune_f64(const double *f, const double *fhat, size_t nx, size_t ny, size_t nz, pmsz_tune *out,
                      void *stream);
/* Table entry of a shape class: returns 1 and fills *out if one is recorded,
 * else 0 and the defaults (negative: bad arguments). */
int pmsz_tune_get(size_t nx, size_t ny, size_t nz, size_t elem_size, pmsz_tune *out);
/* The tile depth recorded for a batch's size class (ceil log2 of its total
 * voxels, ceil log2 of its field count, the element size): pmsz_correct_batch
 * with PMSZ_FLAG_AUTOTUNE tunes it over the whole table, since the batch runs
 * one first-pass launch over all its fields.  Returns as pmsz_tune_get. */
int pmsz_tune_batch_get(size_t total_voxels, int count, size_t elem_size, pmsz_tune *out);
/* Records an entry (zchunk in 1..256, jump_rounds in 1..16). */
int pmsz_tune_set(size_t nx, size_t ny, size_t nz, size_t elem_size, const pmsz_tune *t);
/* Text persistence: one line per entry; load merges into the table. */
int pmsz_tune_save(const char *path);
int pmsz_tune_load(const char *path);
void pmsz_tune_clear(void);

/* Human-readable status, and the last error message of the calling thread. */
const char *pmsz_strerror(int status);
const char *pmsz_last_error(void);
int pmsz_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PMSZ_H */
