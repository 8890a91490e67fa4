/*
 * pmsz_oracle.c -- CPU restatement of the pMSz correction hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * implementation in pmsz_anonymous_gb300/csrc.  Only tests/, the smoke()
 * entry point and bench.py's CPU-baseline leg load it; the product path never
 * links or calls it.
 *
 * Semantics.  The reference kernel `iscriticle` (pMSz.cu:649-899) edits the
 * decompressed field in place while other threads of the same launch still
 * read it, so its corrected field depends on warp scheduling.  This oracle
 * fixes one legal interleaving of that kernel: every read of sweep k sees the
 * field as it was at the start of sweep k ("snapshot" or Jacobi sweeps), and
 * the union of the edit requests of the sweep is applied afterwards, each
 * requested vertex once (the reference guards "once per launch" with
 * atomicCAS(&edits[v],0,1), pMSz.cu:795-888).  Everything else is the
 * reference's arithmetic, done in the field's own type T.
 *
 * Indexing.  The reference works on a padded (W+2)(H+2)(D+2) block whose
 * shell holds INVALID_VAL=1e30 (pMSz.cu:215, 346-381) and breaks value ties by
 * the padded flat index (pMSz.cu:610-620).  At an MPI grid of 1x1x1 the
 * padded index and the unpadded index x + W*(y + H*z) order the real voxels
 * identically (both are lexicographic in (z, y, x)), so this file uses the
 * unpadded index and an explicit in-domain test instead of the sentinel.
 *
 * Each public function is generated for T = float and T = double.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Status codes (shared with include/pmsz.h). */
#define PMSZO_OK 0
#define PMSZO_ERR_ARG 1
#define PMSZO_ERR_OOM 2
#define PMSZO_ERR_NOT_CONVERGED 3

/* The 14 stencil offsets in the reference's scan order, pMSz.cu:186-193
 * (`directions_host`): +-x, +-y, +-z, +-(-1,1,0), +-(-1,0,1), +-(0,1,1),
 * +-(-1,1,1). */
static const int PMSZO_DIR[14][3] = {
    {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},
    {0, 0, -1}, {-1, 1, 0}, {1, -1, 0}, {-1, 0, 1}, {1, 0, -1},
    {0, 1, 1},  {0, -1, -1}, {-1, 1, 1}, {1, -1, -1}};

/* Per-sweep record: the three reference counters (count_f_max, count_f_min,
 * count_f_dir; pMSz.cu:174, 791, 815, 861, 876, 887), plus the number of
 * distinct vertices whose edit was requested and the number whose value
 * changed. */
typedef struct {
    uint64_t fmax, fmin, fdir, requested, changed;
} pmszo_sweep_t;

typedef struct {
    int64_t sweeps;          /* detection passes run, incl. the final zero one */
    int64_t edits_applied;   /* sum over sweeps of `requested` */
    int status;
} pmszo_result_t;

int pmszo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void pmszo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---------------------------------------------------------------------- */
/* Steepest ascent / descent of one voxel.                                 */
/* Restates the neighbour scan of iscriticle, pMSz.cu:686-746: `largest`   */
/* and `smallest` start at the voxel itself and are replaced by a          */
/* neighbour that is larger (smaller) under the total order                */
/* (value, index) of islarger_shared / isless_shared, pMSz.cu:610-620.     */
/* A neighbour outside the domain does not exist (pMSz.cu:709).            */
/* ---------------------------------------------------------------------- */
#define PMSZO_DEFINE_STEEPEST(T, SUF)                                           \
    static inline void pmszo_steepest_##SUF(const T *v, int64_t nx,            \
                                            int64_t ny, int64_t nz, int64_t x, \
                                            int64_t y, int64_t z,              \
                                            int64_t *asc, int64_t *desc) {     \
        const int64_t i = x + nx * (y + ny * z);                               \
        const T cv = v[i];                                                     \
        int64_t largest = i, smallest = i;                                     \
        T lv = cv, sv = cv;                                                    \
        for (int d = 0; d < 14; ++d) {                                         \
            const int64_t ax = x + PMSZO_DIR[d][0];                            \
            const int64_t ay = y + PMSZO_DIR[d][1];                            \
            const int64_t az = z + PMSZO_DIR[d][2];                            \
            if (ax < 0 || ax >= nx || ay < 0 || ay >= ny || az < 0 ||          \
                az >= nz)                                                      \
                continue;                                                      \
            const int64_t n = ax + nx * (ay + ny * az);                        \
            const T nv = v[n];                                                 \
            if (nv > lv || (nv == lv && n > largest)) {                        \
                largest = n;                                                   \
                lv = nv;                                                       \
            }                                                                  \
            if (nv < sv || (nv == sv && n < smallest)) {                       \
                smallest = n;                                                  \
                sv = nv;                                                       \
            }                                                                  \
        }                                                                      \
        *asc = largest;                                                        \
        *desc = smallest;                                                      \
    }

PMSZO_DEFINE_STEEPEST(float, f32)
PMSZO_DEFINE_STEEPEST(double, f64)

/* ---------------------------------------------------------------------- */
/* Labelling: steepest ascent / descent neighbour of every voxel.          */
/* pMSz.cu:749-783 stores these as or_types; this keeps the two flat       */
/* indices (asc = or_types "largest", desc = or_types "smallest").         */
/* A voxel is a maximum iff asc[i]==i and a minimum iff desc[i]==i.        */
/* ---------------------------------------------------------------------- */
#define PMSZO_DEFINE_LABEL(T, SUF)                                             \
    int pmszo_label_##SUF(const T *v, int64_t nx, int64_t ny, int64_t nz,      \
                          int64_t *asc, int64_t *desc) {                       \
        if (nx <= 0 || ny <= 0 || nz <= 0) return PMSZO_ERR_ARG;               \
        _Pragma("omp parallel for schedule(static)")                           \
        for (int64_t z = 0; z < nz; ++z)                                       \
            for (int64_t y = 0; y < ny; ++y)                                   \
                for (int64_t x = 0; x < nx; ++x) {                             \
                    const int64_t i = x + nx * (y + ny * z);                   \
                    pmszo_steepest_##SUF(v, nx, ny, nz, x, y, z, &asc[i],      \
                                         &desc[i]);                            \
                }                                                              \
        return PMSZO_OK;                                                       \
    }

PMSZO_DEFINE_LABEL(float, f32)
PMSZO_DEFINE_LABEL(double, f64)

/* ---------------------------------------------------------------------- */
/* The edit primitive, applyDeltaBuffer_local, pMSz.cu:623-645:            */
/*   if |f - (fhat - delta)| <= eps and cnt < q-1: fhat -= delta; cnt++    */
/*   else: cnt = q; fhat = f - eps                                          */
/* computed in T.  Returns 1 if (fhat, cnt) changed.                        */
/* ---------------------------------------------------------------------- */
#define PMSZO_DEFINE_APPLY(T, SUF, FABS)                                       \
    static inline int pmszo_apply_##SUF(const T *f, T *fh, uint8_t *cnt,       \
                                        int64_t v, T eps, T delta, int q,      \
                                        int *value_changed) {                  \
        const T old = fh[v];                                                   \
        const uint8_t oc = cnt[v];                                             \
        const T lowered = old - delta;                                         \
        if (FABS(f[v] - lowered) <= eps && (int)oc < q - 1) {                  \
            fh[v] = lowered;                                                   \
            cnt[v] = (uint8_t)(oc + 1);                                        \
        } else {                                                               \
            cnt[v] = (uint8_t)q;                                               \
            fh[v] = f[v] - eps;                                                \
        }                                                                      \
        *value_changed = memcmp(&old, &fh[v], sizeof(T)) != 0;                 \
        return *value_changed || oc != cnt[v];                                 \
    }

PMSZO_DEFINE_APPLY(float, f32, fabsf)
PMSZO_DEFINE_APPLY(double, f64, fabs)

/* ---------------------------------------------------------------------- */
/* One snapshot detection sweep over all voxels: the rules of iscriticle  */
/* data_type=0, pMSz.cu:786-898.  omax/omin come from the original       */
/* labelling exactly as or_types encodes them (pMSz.cu:749-783): a voxel  */
/* that is both max and min in f is stored as a max (or_types[2i]=-1),    */
/* so it counts as "not an original minimum".                             */
/*   R1 is_max != omax: fmax++; request (omax ? asc : i)                   */
/*   R2 is_min != omin: fmin++; request (omin ? i : odesc)                 */
/*   R3 R1 or R2 fired: fdir++, stop                                       */
/*   R4 asc != oasc:  fdir++; request asc                                  */
/*   R5 desc != odesc: fdir++; request odesc                               */
/* Requests are recorded in req[] (byte per voxel).                        */
/* ---------------------------------------------------------------------- */
#define PMSZO_DEFINE_DETECT(T, SUF, IDX, ISUF)                                 \
    static void pmszo_detect_##SUF##ISUF(const T *fh, int64_t nx, int64_t ny,  \
                                   int64_t nz, const IDX *oasc,                \
                                   const IDX *odesc, uint8_t *req,             \
                                   pmszo_sweep_t *out) {                       \
        uint64_t cmax = 0, cmin = 0, cdir = 0;                                 \
        _Pragma("omp parallel for schedule(static) reduction(+:cmax,cmin,cdir)") \
        for (int64_t z = 0; z < nz; ++z)                                       \
            for (int64_t y = 0; y < ny; ++y)                                   \
                for (int64_t x = 0; x < nx; ++x) {                             \
                    const int64_t i = x + nx * (y + ny * z);                   \
                    int64_t asc, desc;                                         \
                    pmszo_steepest_##SUF(fh, nx, ny, nz, x, y, z, &asc, &desc); \
                    const int is_max = asc == i, is_min = desc == i;           \
                    const int omax = (int64_t)oasc[i] == i;                    \
                    const int omin = !omax && (int64_t)odesc[i] == i;          \
                    const int r1 = is_max != omax, r2 = is_min != omin;        \
                    if (r1) {                                                  \
                        ++cmax;                                                \
                        int64_t t = omax ? asc : i;                            \
                        _Pragma("omp atomic write") req[t] = 1;                \
                    }                                                          \
                    if (r2) {                                                  \
                        ++cmin;                                                \
                        int64_t t = omin ? i : (int64_t)odesc[i];              \
                        _Pragma("omp atomic write") req[t] = 1;                \
                    }                                                          \
                    if (r1 || r2) {                                            \
                        ++cdir;                                                \
                        continue;                                              \
                    }                                                          \
                    if (asc != (int64_t)oasc[i]) {                             \
                        ++cdir;                                                \
                        _Pragma("omp atomic write") req[asc] = 1;              \
                    }                                                          \
                    if (desc != (int64_t)odesc[i]) {                           \
                        ++cdir;                                                \
                        _Pragma("omp atomic write") req[odesc[i]] = 1;         \
                    }                                                          \
                }                                                              \
        out->fmax = cmax;                                                      \
        out->fmin = cmin;                                                      \
        out->fdir = cdir;                                                      \
    }

PMSZO_DEFINE_DETECT(float, f32, int64_t, _i64)
PMSZO_DEFINE_DETECT(double, f64, int64_t, _i64)
PMSZO_DEFINE_DETECT(float, f32, uint32_t, _u32)
PMSZO_DEFINE_DETECT(double, f64, uint32_t, _u32)

/* Labelling into 32-bit indices (fields of fewer than 2^32 voxels: the same
 * values in half the memory, so the oracle reaches 1536^3 on one host). */
#define PMSZO_DEFINE_LABEL32(T, SUF)                                           \
    static void pmszo_label32_##SUF(const T *v, int64_t nx, int64_t ny,        \
                                    int64_t nz, uint32_t *asc, uint32_t *desc) { \
        _Pragma("omp parallel for schedule(static)")                           \
        for (int64_t z = 0; z < nz; ++z)                                       \
            for (int64_t y = 0; y < ny; ++y)                                   \
                for (int64_t x = 0; x < nx; ++x) {                             \
                    const int64_t i = x + nx * (y + ny * z);                   \
                    int64_t a, d;                                              \
                    pmszo_steepest_##SUF(v, nx, ny, nz, x, y, z, &a, &d);      \
                    asc[i] = (uint32_t)a;                                      \
                    desc[i] = (uint32_t)d;                                     \
                }                                                              \
    }

PMSZO_DEFINE_LABEL32(float, f32)
PMSZO_DEFINE_LABEL32(double, f64)

/* ---------------------------------------------------------------------- */
/* The correction loop, c_loops at one rank (pMSz.cu:1872-2074):          */
/*   cnt := 0; label the original field;                                   */
/*   repeat { detect + apply } until a sweep reports fmax=fmin=fdir=0.     */
/* The reference then runs one detect-only pass (pMSz.cu:2022), which at  */
/* one rank sees the same field as the last zero sweep and is omitted.    */
/* The reference loop has no exit for a sweep that requests edits but    */
/* changes nothing (every requested vertex already clamped); this loop    */
/* stops there, and at max_sweeps, with PMSZO_ERR_NOT_CONVERGED.           */
/*   eps   = (T)eb,  delta = (T)(eb / q) with the division in double       */
/*   (pMSz.cu:2814, `delta = bound / (q)`).                                */
/* sweep_log (optional) receives one record per sweep.                     */
/* ---------------------------------------------------------------------- */
#define PMSZO_DEFINE_CORRECT(T, SUF)                                           \
    int pmszo_correct_##SUF(const T *f, T *fh, int64_t nx, int64_t ny,         \
                            int64_t nz, double eb, int q, int64_t max_sweeps,  \
                            uint8_t *cnt_out, pmszo_sweep_t *sweep_log,        \
                            pmszo_result_t *res) {                             \
        if (nx <= 0 || ny <= 0 || nz <= 0 || !(eb > 0) || q < 1 || q > 255 ||  \
            max_sweeps < 1)                                                    \
            return PMSZO_ERR_ARG;                                              \
        const int64_t n = nx * ny * nz;                                        \
        const T eps = (T)eb;                                                   \
        const T delta = (T)(eb / (double)q);                                   \
        const int narrow = n <= (int64_t)UINT32_MAX;                           \
        const size_t isz = narrow ? sizeof(uint32_t) : sizeof(int64_t);        \
        void *oasc = malloc((size_t)n * isz);                                  \
        void *odesc = malloc((size_t)n * isz);                                 \
        uint8_t *req = (uint8_t *)calloc((size_t)n, 1);                        \
        uint8_t *cnt = cnt_out ? cnt_out : (uint8_t *)malloc((size_t)n);       \
        if (!oasc || !odesc || !req || !cnt) {                                 \
            free(oasc); free(odesc); free(req);                                \
            if (!cnt_out) free(cnt);                                           \
            return PMSZO_ERR_OOM;                                              \
        }                                                                      \
        memset(cnt, 0, (size_t)n);                                             \
        if (narrow)                                                            \
            pmszo_label32_##SUF(f, nx, ny, nz, (uint32_t *)oasc, (uint32_t *)odesc); \
        else                                                                   \
            pmszo_label_##SUF(f, nx, ny, nz, (int64_t *)oasc, (int64_t *)odesc); \
        int status = PMSZO_ERR_NOT_CONVERGED;                                  \
        int64_t sweeps = 0, edits = 0;                                         \
        while (sweeps < max_sweeps) {                                          \
            pmszo_sweep_t s;                                                   \
            memset(&s, 0, sizeof(s));                                          \
            if (narrow)                                                        \
                pmszo_detect_##SUF##_u32(fh, nx, ny, nz, (const uint32_t *)oasc,   \
                                         (const uint32_t *)odesc, req, &s);        \
            else                                                               \
                pmszo_detect_##SUF##_i64(fh, nx, ny, nz, (const int64_t *)oasc,    \
                                         (const int64_t *)odesc, req, &s);         \
            ++sweeps;                                                          \
            uint64_t requested = 0, changed = 0, progressed = 0;               \
            _Pragma("omp parallel for schedule(static) reduction(+:requested,changed,progressed)") \
            for (int64_t v = 0; v < n; ++v) {                                  \
                if (!req[v]) continue;                                         \
                req[v] = 0;                                                    \
                ++requested;                                                   \
                int vc = 0;                                                    \
                progressed += (uint64_t)pmszo_apply_##SUF(f, fh, cnt, v, eps,  \
                                                          delta, q, &vc);      \
                changed += (uint64_t)vc;                                       \
            }                                                                  \
            s.requested = requested;                                           \
            s.changed = changed;                                               \
            edits += (int64_t)requested;                                       \
            if (sweep_log) sweep_log[sweeps - 1] = s;                          \
            if (s.fmax == 0 && s.fmin == 0 && s.fdir == 0) {                   \
                status = PMSZO_OK;                                             \
                break;                                                         \
            }                                                                  \
            if (progressed == 0) break; /* stuck: nothing can change */        \
        }                                                                      \
        if (res) {                                                             \
            res->sweeps = sweeps;                                              \
            res->edits_applied = edits;                                        \
            res->status = status;                                              \
        }                                                                      \
        free(oasc); free(odesc); free(req);                                    \
        if (!cnt_out) free(cnt);                                               \
        return status;                                                         \
    }

PMSZO_DEFINE_CORRECT(float, f32)
PMSZO_DEFINE_CORRECT(double, f64)

/* ---------------------------------------------------------------------- */
/* Manifold labels: PathCompression, pMSz.cu:255-271 -- every vertex walks */
/* its direction pointers to the fixpoint (AS root = maximum, DS root =    */
/* minimum).  Applied to the direction arrays as naive_MSz.cu:838-844 and  */
/* 1914-1917 do.                                                            */
/* ---------------------------------------------------------------------- */
int pmszo_path_compress(const int64_t *dir, int64_t *label, int64_t n) {
    if (n < 0) return PMSZO_ERR_ARG;
    _Pragma("omp parallel for schedule(static)")
    for (int64_t i = 0; i < n; ++i) {
        int64_t cur = dir[i];
        int64_t steps = 0;
        while (dir[cur] != cur && steps <= n) {
            cur = dir[cur];
            ++steps;
        }
        label[i] = cur;
    }
    return PMSZO_OK;
}

/* ---------------------------------------------------------------------- */
/* Verification (replaces the disabled check_consistency block,            */
/* pMSz.cu:3038-3126, and count_false_cases, pMSz.cu:1852-1870): counts    */
/*   dir_mismatch   voxels whose asc or desc differs between f and f'      */
/*   ext_mismatch   voxels whose max/min flags differ                      */
/*   as_mismatch / ds_mismatch   voxels whose AS / DS label differs        */
/*   bound_violations  voxels with |f' - f| > eps (computed in T)          */
/* out[5] receives the five counts in that order.                          */
/* ---------------------------------------------------------------------- */
#define PMSZO_DEFINE_VERIFY(T, SUF, FABS)                                      \
    int pmszo_verify_##SUF(const T *f, const T *fp, int64_t nx, int64_t ny,    \
                           int64_t nz, double eb, uint64_t out[5]) {           \
        if (nx <= 0 || ny <= 0 || nz <= 0) return PMSZO_ERR_ARG;               \
        const int64_t n = nx * ny * nz;                                        \
        const T eps = (T)eb;                                                   \
        int64_t *a0 = (int64_t *)malloc((size_t)n * sizeof(int64_t));          \
        int64_t *d0 = (int64_t *)malloc((size_t)n * sizeof(int64_t));          \
        int64_t *a1 = (int64_t *)malloc((size_t)n * sizeof(int64_t));          \
        int64_t *d1 = (int64_t *)malloc((size_t)n * sizeof(int64_t));          \
        int64_t *l0 = (int64_t *)malloc((size_t)n * sizeof(int64_t));          \
        int64_t *l1 = (int64_t *)malloc((size_t)n * sizeof(int64_t));          \
        if (!a0 || !d0 || !a1 || !d1 || !l0 || !l1) {                          \
            free(a0); free(d0); free(a1); free(d1); free(l0); free(l1);        \
            return PMSZO_ERR_OOM;                                              \
        }                                                                      \
        pmszo_label_##SUF(f, nx, ny, nz, a0, d0);                              \
        pmszo_label_##SUF(fp, nx, ny, nz, a1, d1);                             \
        uint64_t dm = 0, em = 0, asm_ = 0, dsm = 0, bv = 0;                    \
        for (int64_t i = 0; i < n; ++i) {                                      \
            dm += (a0[i] != a1[i]) || (d0[i] != d1[i]);                        \
            em += ((a0[i] == i) != (a1[i] == i)) ||                            \
                  ((d0[i] == i) != (d1[i] == i));                              \
            bv += !(FABS(fp[i] - f[i]) <= eps);                                \
        }                                                                      \
        pmszo_path_compress(a0, l0, n);                                        \
        pmszo_path_compress(a1, l1, n);                                        \
        for (int64_t i = 0; i < n; ++i) asm_ += l0[i] != l1[i];                \
        pmszo_path_compress(d0, l0, n);                                        \
        pmszo_path_compress(d1, l1, n);                                        \
        for (int64_t i = 0; i < n; ++i) dsm += l0[i] != l1[i];                 \
        out[0] = dm; out[1] = em; out[2] = asm_; out[3] = dsm; out[4] = bv;    \
        free(a0); free(d0); free(a1); free(d1); free(l0); free(l1);            \
        return PMSZO_OK;                                                       \
    }

PMSZO_DEFINE_VERIFY(float, f32, fabsf)
PMSZO_DEFINE_VERIFY(double, f64, fabs)

/* ---------------------------------------------------------------------- */
/* Edit extraction, extract_edits_kernel, pMSz.cu:2090-2138, over the      */
/* voxels in x-fastest order, comparing the corrected field cur with the  */
/* decompressed field prev:                                                 */
/*   cur == prev            -> delta 0                                      */
/*   cur == f - eps         -> delta q, and f - eps joins the clamp list    */
/*   otherwise              -> delta round((prev - cur) / delta_step)       */
/* The clamp list keeps voxel order and drops exact zeros (the reference   */
/* compacts with thrust::copy_if(v != 0), pMSz.cu:223-247).  edit_count   */
/* counts voxels with cur < prev ("Edit count", pMSz.cu:2114).  The        */
/* reference leaves deltas undefined where cur > prev (only a clamp can    */
/* raise a value); this restatement encodes those like the clamp case.    */
/* ---------------------------------------------------------------------- */
#define PMSZO_DEFINE_EXTRACT(T, SUF, ROUND)                                    \
    int pmszo_extract_edits_##SUF(const T *prev, const T *cur, const T *f,     \
                                  int64_t n, double eb, int q,                 \
                                  uint8_t *deltas, T *clamp,                   \
                                  int64_t *n_clamp, int64_t *edit_count) {     \
        if (n < 0 || q < 1 || q > 255) return PMSZO_ERR_ARG;                   \
        const T eps = (T)eb;                                                   \
        const T delta = (T)(eb / (double)q);                                   \
        int64_t nc = 0, ec = 0;                                                \
        for (int64_t i = 0; i < n; ++i) {                                      \
            const T c = cur[i], p = prev[i];                                   \
            if (c == p) {                                                      \
                deltas[i] = 0;                                                 \
                continue;                                                      \
            }                                                                  \
            ec += c < p;                                                       \
            const T cl = f[i] - eps;                                           \
            if (c != cl) {                                                     \
                deltas[i] = (uint8_t)ROUND((p - c) / delta);                   \
            } else {                                                           \
                deltas[i] = (uint8_t)q;                                        \
                if (cl != 0) clamp[nc++] = cl;                                 \
            }                                                                  \
        }                                                                      \
        *n_clamp = nc;                                                         \
        *edit_count = ec;                                                      \
        return PMSZO_OK;                                                       \
    }

PMSZO_DEFINE_EXTRACT(float, f32, roundf)
PMSZO_DEFINE_EXTRACT(double, f64, round)

/* ---------------------------------------------------------------------- */
/* Reconstruction (the reference has no decoder; validateResult,           */
/* pMSz.cu:2545-2584, only decompresses).  Inverse of extract: delta k<q   */
/* lowers the decompressed value k times by delta_step in T, the loop's    */
/* own repeated subtraction (pMSz.cu:631); delta q takes the next value of */
/* the clamp list.  The reference encoder drops clamp values equal to 0,   */
/* so a field with such a clamp has more q-deltas than list entries; that */
/* case is reported as PMSZO_ERR_ARG instead of shifting the list.         */
/* ---------------------------------------------------------------------- */
#define PMSZO_DEFINE_RECON(T, SUF)                                             \
    int pmszo_reconstruct_##SUF(const T *prev, const uint8_t *deltas,          \
                                const T *clamp, int64_t n_clamp, int64_t n,    \
                                double eb, int q, T *out) {                    \
        const T delta = (T)(eb / (double)q);                                   \
        int64_t c = 0;                                                         \
        for (int64_t i = 0; i < n; ++i) {                                      \
            T v = prev[i];                                                     \
            const int k = deltas[i];                                           \
            if (k == q) {                                                      \
                if (c >= n_clamp) return PMSZO_ERR_ARG;                        \
                v = clamp[c++];                                                \
            } else {                                                           \
                for (int s = 0; s < k; ++s) v = v - delta;                     \
            }                                                                  \
            out[i] = v;                                                        \
        }                                                                      \
        return c == n_clamp ? PMSZO_OK : PMSZO_ERR_ARG;                        \
    }

PMSZO_DEFINE_RECON(float, f32)
PMSZO_DEFINE_RECON(double, f64)

/* ---------------------------------------------------------------------- */
/* 3-bit (generally n-bit) LSB-first packing, pack_nbits pMSz.cu:2328-2348 */
/* with bits_for_max pMSz.cu:2352-2356, and its inverse unpack_nbits       */
/* pMSz.cu:2393-2410.  Returns the packed size, or -1 on a symbol that    */
/* does not fit.                                                            */
/* ---------------------------------------------------------------------- */
unsigned pmszo_bits_for_max(unsigned maxsym) {
    if (maxsym == 0) return 1;
    return (unsigned)ceil(log2((double)maxsym + 1.0));
}

int64_t pmszo_pack_nbits(const uint8_t *sym, int64_t n, unsigned nbits,
                         uint8_t *out) {
    if (nbits == 0 || nbits > 8) return -1;
    uint64_t buf = 0;
    unsigned cnt = 0;
    int64_t o = 0;
    const uint64_t mask = (1ull << nbits) - 1ull;
    for (int64_t i = 0; i < n; ++i) {
        if (sym[i] > mask) return -1;
        buf |= ((uint64_t)sym[i] & mask) << cnt;
        cnt += nbits;
        while (cnt >= 8) {
            out[o++] = (uint8_t)(buf & 0xFF);
            buf >>= 8;
            cnt -= 8;
        }
    }
    if (cnt) out[o++] = (uint8_t)(buf & 0xFF);
    return o;
}

int pmszo_unpack_nbits(const uint8_t *packed, int64_t packed_bytes, int64_t n,
                       unsigned nbits, uint8_t *out) {
    if (nbits == 0 || nbits > 8) return PMSZO_ERR_ARG;
    uint64_t buf = 0;
    unsigned cnt = 0;
    int64_t pos = 0;
    const uint64_t mask = (1ull << nbits) - 1ull;
    for (int64_t i = 0; i < n; ++i) {
        while (cnt < nbits) {
            if (pos >= packed_bytes) return PMSZO_ERR_ARG;
            buf |= (uint64_t)packed[pos++] << cnt;
            cnt += 8;
        }
        out[i] = (uint8_t)(buf & mask);
        buf >>= nbits;
        cnt -= nbits;
    }
    return PMSZO_OK;
}

/* ---------------------------------------------------------------------- */
/* naive-MSz correction: naive_MSz.cu c_loops (1887-2220) with its         */
/* extrema-only iscriticle (645-850) and extract_false_path (1767-1864),   */
/* under snapshot semantics.  One outer iteration:                          */
/*   - extrema sweeps (rules R1/R2 only) while the last count of false or  */
/*     missing extrema is non-zero (initially: at least one sweep);         */
/*   - a path sweep: labels of the current field by path compression; for */
/*     every voxel whose DS (AS) label differs from the original's, walk   */
/*     the steps on which the original and current directions agree to the */
/*     first divergence and lower the original descent neighbour there     */
/*     (resp. the current ascent neighbour); fdir counts each mismatch;    */
/*   - a check: extremum counts and, per voxel, one count if its DS label   */
/*     differs, else one if its AS label differs (fix=1 mode).              */
/* The loop ends when the check is all zero.  Records: extrema sweep        */
/* {fmax,fmin,0,req,chg}, path sweep {0,0,fdir,req,chg}, check              */
/* {fmax,fmin,fdir,0,0}.  Walks follow or_types literally, including its    */
/* encoding of maxima (slot 1 = descent) and minima (slot 0 = -2); a walk   */
/* that would target the -2 marker (the reference would index edits[-2])   */
/* edits nothing.  Walks are bounded by n steps; an outer iteration that   */
/* changes nothing ends the loop with PMSZO_ERR_NOT_CONVERGED.              */
/* ---------------------------------------------------------------------- */
static inline int64_t pmszo_or0(const int64_t *oasc, const int64_t *odesc, int64_t c) {
    if (oasc[c] == c) return -1;          /* original maximum */
    if (odesc[c] == c) return -2;         /* original minimum */
    return odesc[c];
}
static inline int64_t pmszo_or1(const int64_t *oasc, const int64_t *odesc, int64_t c) {
    return oasc[c] == c ? odesc[c] : oasc[c];
}

/* DS walk from i; returns the vertex to lower or -1. */
static int64_t pmszo_walk_ds(const int64_t *oasc, const int64_t *odesc, const int64_t *cdesc, int64_t i, int64_t n) {
    int64_t cur = i;
    for (int64_t steps = 0;; ++steps) {
        const int64_t s0 = pmszo_or0(oasc, odesc, cur);
        if (s0 != cdesc[cur]) break;
        if (cdesc[cur] == cur && s0 == cur) return -1;
        if (s0 == cur) break;
        cur = s0;
        if (steps > n) return -1;
    }
    const int64_t fls = cdesc[cur];
    const int64_t tru = oasc[cur] == cur ? odesc[cur] : pmszo_or0(oasc, odesc, cur);
    return (tru >= 0 && fls != tru) ? tru : -1;
}

/* AS walk from i; returns the vertex to lower or -1. */
static int64_t pmszo_walk_as(const int64_t *oasc, const int64_t *odesc, const int64_t *casc, int64_t i, int64_t n) {
    int64_t cur = i;
    for (int64_t steps = 0;; ++steps) {
        const int64_t s1 = pmszo_or1(oasc, odesc, cur);
        if (s1 != casc[cur]) break;
        if (casc[cur] == cur && s1 == cur) return -1;
        if (s1 == cur) break;
        cur = s1;
        if (steps > n) return -1;
    }
    const int64_t fls = casc[cur], tru = pmszo_or1(oasc, odesc, cur);
    return fls != tru ? fls : -1;
}

#define PMSZO_DEFINE_NAIVE(T, SUF)                                                                   \
    int pmszo_correct_naive_##SUF(const T *f, T *fh, int64_t nx, int64_t ny, int64_t nz, double eb,  \
                                  int q, int64_t max_sweeps, uint8_t *cnt_out, pmszo_sweep_t *log,   \
                                  pmszo_result_t *res) {                                             \
        if (nx <= 0 || ny <= 0 || nz <= 0 || !(eb > 0) || q < 1 || q > 255 || max_sweeps < 1)        \
            return PMSZO_ERR_ARG;                                                                    \
        const int64_t n = nx * ny * nz;                                                              \
        const T eps = (T)eb, delta = (T)(eb / (double)q);                                            \
        int64_t *oa = malloc((size_t)n * 8), *od = malloc((size_t)n * 8), *ca = malloc((size_t)n * 8); \
        int64_t *cd = malloc((size_t)n * 8), *as0 = malloc((size_t)n * 8), *ds0 = malloc((size_t)n * 8); \
        int64_t *as1 = malloc((size_t)n * 8), *ds1 = malloc((size_t)n * 8);                          \
        uint8_t *req = calloc((size_t)n, 1), *cnt = cnt_out ? cnt_out : malloc((size_t)n);           \
        int status = PMSZO_ERR_OOM;                                                                  \
        int64_t nrec = 0, edits = 0;                                                                 \
        if (!oa || !od || !ca || !cd || !as0 || !ds0 || !as1 || !ds1 || !req || !cnt) goto done;     \
        memset(cnt, 0, (size_t)n);                                                                   \
        pmszo_label_##SUF(f, nx, ny, nz, oa, od);                                                    \
        pmszo_path_compress(oa, as0, n);                                                             \
        pmszo_path_compress(od, ds0, n);                                                             \
        status = PMSZO_ERR_NOT_CONVERGED;                                                            \
        uint64_t hmax = 1, hmin = 1;                                                                 \
        for (;;) {                                                                                   \
            uint64_t progressed_outer = 0;                                                           \
            while (hmax || hmin) { /* extrema sweeps */                                             \
                if (nrec >= max_sweeps) goto done;                                                   \
                pmszo_label_##SUF(fh, nx, ny, nz, ca, cd);                                           \
                uint64_t cmax = 0, cmin = 0;                                                         \
                for (int64_t i = 0; i < n; ++i) {                                                    \
                    const int is_max = ca[i] == i, is_min = cd[i] == i;                              \
                    const int omax = oa[i] == i, omin = !omax && od[i] == i;                         \
                    if (is_max != omax) { ++cmax; req[omax ? ca[i] : i] = 1; }                       \
                    if (is_min != omin) { ++cmin; req[omin ? i : od[i]] = 1; }                       \
                }                                                                                    \
                uint64_t rq = 0, ch = 0, pr = 0;                                                     \
                for (int64_t v = 0; v < n; ++v) {                                                    \
                    if (!req[v]) continue;                                                           \
                    req[v] = 0; ++rq; int vc = 0;                                                    \
                    pr += (uint64_t)pmszo_apply_##SUF(f, fh, cnt, v, eps, delta, q, &vc);            \
                    ch += (uint64_t)vc;                                                              \
                }                                                                                    \
                if (log) { pmszo_sweep_t r = {cmax, cmin, 0, rq, ch}; log[nrec] = r; }               \
                ++nrec; edits += (int64_t)rq; progressed_outer += pr;                                \
                hmax = cmax; hmin = cmin;                                                            \
                if ((cmax || cmin) && pr == 0) goto done; /* stuck */                                \
            }                                                                                        \
            /* path sweep */                                                                         \
            if (nrec >= max_sweeps) goto done;                                                       \
            pmszo_label_##SUF(fh, nx, ny, nz, ca, cd);                                               \
            pmszo_path_compress(ca, as1, n);                                                         \
            pmszo_path_compress(cd, ds1, n);                                                         \
            uint64_t fdir = 0;                                                                       \
            for (int64_t i = 0; i < n; ++i) {                                                        \
                if (ds0[i] != ds1[i]) {                                                              \
                    ++fdir;                                                                          \
                    const int64_t t = pmszo_walk_ds(oa, od, cd, i, n);                               \
                    if (t >= 0) req[t] = 1;                                                          \
                }                                                                                    \
                if (as0[i] != as1[i]) {                                                              \
                    ++fdir;                                                                          \
                    const int64_t t = pmszo_walk_as(oa, od, ca, i, n);                               \
                    if (t >= 0) req[t] = 1;                                                          \
                }                                                                                    \
            }                                                                                        \
            uint64_t rq = 0, ch = 0, pr = 0;                                                         \
            for (int64_t v = 0; v < n; ++v) {                                                        \
                if (!req[v]) continue;                                                               \
                req[v] = 0; ++rq; int vc = 0;                                                        \
                pr += (uint64_t)pmszo_apply_##SUF(f, fh, cnt, v, eps, delta, q, &vc);                \
                ch += (uint64_t)vc;                                                                  \
            }                                                                                        \
            if (log) { pmszo_sweep_t r = {0, 0, fdir, rq, ch}; log[nrec] = r; }                      \
            ++nrec; edits += (int64_t)rq; progressed_outer += pr;                                    \
            /* check */                                                                              \
            if (nrec >= max_sweeps) goto done;                                                       \
            pmszo_label_##SUF(fh, nx, ny, nz, ca, cd);                                               \
            pmszo_path_compress(ca, as1, n);                                                         \
            pmszo_path_compress(cd, ds1, n);                                                         \
            uint64_t cmax = 0, cmin = 0, cdir = 0;                                                   \
            for (int64_t i = 0; i < n; ++i) {                                                        \
                const int is_max = ca[i] == i, is_min = cd[i] == i;                                  \
                const int omax = oa[i] == i, omin = !omax && od[i] == i;                             \
                cmax += is_max != omax;                                                              \
                cmin += is_min != omin;                                                              \
                cdir += (ds0[i] != ds1[i]) || (as0[i] != as1[i]);                                    \
            }                                                                                        \
            if (log) { pmszo_sweep_t r = {cmax, cmin, cdir, 0, 0}; log[nrec] = r; }                  \
            ++nrec;                                                                                  \
            if (!cmax && !cmin && !cdir) { status = PMSZO_OK; goto done; }                           \
            if (!progressed_outer) goto done; /* nothing can change any more */                     \
            hmax = cmax; hmin = cmin;                                                                \
        }                                                                                            \
    done:                                                                                            \
        if (res) { res->sweeps = nrec; res->edits_applied = edits; res->status = status; }           \
        free(oa); free(od); free(ca); free(cd); free(as0); free(ds0); free(as1); free(ds1); free(req); \
        if (!cnt_out) free(cnt);                                                                     \
        return status;                                                                               \
    }

PMSZO_DEFINE_NAIVE(float, f32)
PMSZO_DEFINE_NAIVE(double, f64)

/* ---------------------------------------------------------------------- */
/* Synthetic inputs for the CPU legs of the benchmark, so that they need no */
/* GPU and load nothing but this library.  The same bits as the numpy      */
/* generator (pmsz_anonymous_gb300/fields.py) and the CUDA one: improved   */
/* Perlin noise as generate_perlin.py:17-59 writes it (quintic fade, the   */
/* 16-case gradient hash, a 512-entry permutation made by the caller as    */
/* generate_perlin.py:105-108 makes it), summed over octaves with the      */
/* caller's amplitudes and frequencies, then min-max normalised in double  */
/* and cast to T.  Every operation is one IEEE double operation            */
/* (-ffp-contract=off), as numpy evaluates the same expressions.           */
/* ---------------------------------------------------------------------- */
static inline double pmszo_fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }
static inline double pmszo_lerp(double a, double b, double t) { return a + t * (b - a); }
static inline double pmszo_grad(int h, double x, double y, double z) {
    h &= 15;
    const double u = h < 8 ? x : y;
    const double v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
    return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? v : -v);
}
static double pmszo_perlin(double x, double y, double z, const int32_t *p) {
    const double fx = floor(x), fy = floor(y), fz = floor(z);
    const int X = (int)((int64_t)fx & 255), Y = (int)((int64_t)fy & 255), Z = (int)((int64_t)fz & 255);
    x = x - fx;
    y = y - fy;
    z = z - fz;
    const double u = pmszo_fade(x), v = pmszo_fade(y), w = pmszo_fade(z);
    const int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z;
    const int B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
    return pmszo_lerp(
        pmszo_lerp(pmszo_lerp(pmszo_grad(p[AA], x, y, z), pmszo_grad(p[BA], x - 1.0, y, z), u),
                   pmszo_lerp(pmszo_grad(p[AB], x, y - 1.0, z), pmszo_grad(p[BB], x - 1.0, y - 1.0, z), u), v),
        pmszo_lerp(pmszo_lerp(pmszo_grad(p[AA + 1], x, y, z - 1.0), pmszo_grad(p[BA + 1], x - 1.0, y, z - 1.0), u),
                   pmszo_lerp(pmszo_grad(p[AB + 1], x, y - 1.0, z - 1.0),
                              pmszo_grad(p[BB + 1], x - 1.0, y - 1.0, z - 1.0), u), v),
        w);
}
static inline double pmszo_fbm(const int32_t *perm, const double *amps, const double *freqs, int octaves,
                               int64_t x, int64_t y, int64_t z) {
    double total = 0.0;
    for (int o = 0; o < octaves; ++o) {
        const double fr = freqs[o];
        total = total + amps[o] * pmszo_perlin((double)x * fr, (double)y * fr, (double)z * fr, perm);
    }
    return total;
}

/* Two passes (range, then recompute and normalise), so no double copy of  */
/* the field is held: a 1536^3 fp32 field needs only its own 13.5 GB.      */
#define PMSZO_DEFINE_PERLIN(T, SUF)                                                              \
    int pmszo_perlin_##SUF(T *out, int64_t nx, int64_t ny, int64_t nz, const int32_t *perm,      \
                           const double *amps, const double *freqs, int octaves) {               \
        if (nx <= 0 || ny <= 0 || nz <= 0 || octaves < 1 || !out || !perm) return PMSZO_ERR_ARG; \
        for (int i = 0; i < 512; ++i)                                                            \
            if (perm[i] < 0 || perm[i] > 255) return PMSZO_ERR_ARG;                              \
        double mn = INFINITY, mx = -INFINITY;                                                    \
        _Pragma("omp parallel for schedule(static) reduction(min:mn) reduction(max:mx)")         \
        for (int64_t z = 0; z < nz; ++z)                                                         \
            for (int64_t y = 0; y < ny; ++y)                                                     \
                for (int64_t x = 0; x < nx; ++x) {                                               \
                    const double v = pmszo_fbm(perm, amps, freqs, octaves, x, y, z);             \
                    mn = v < mn ? v : mn;                                                        \
                    mx = v > mx ? v : mx;                                                        \
                }                                                                                \
        const double range = mx - mn;                                                            \
        _Pragma("omp parallel for schedule(static)")                                             \
        for (int64_t z = 0; z < nz; ++z)                                                         \
            for (int64_t y = 0; y < ny; ++y)                                                     \
                for (int64_t x = 0; x < nx; ++x)                                                 \
                    out[x + nx * (y + ny * z)] =                                                 \
                        (T)((pmszo_fbm(perm, amps, freqs, octaves, x, y, z) - mn) / range);      \
        return PMSZO_OK;                                                                         \
    }

PMSZO_DEFINE_PERLIN(float, f32)
PMSZO_DEFINE_PERLIN(double, f64)

/* The two labelled compressor stand-ins of fields.py: kind 0, SZ-like      */
/* plateaus fhat = (2 eb) * rint(f / (2 eb)) (rint and numpy's round both   */
/* round half to even); kind 1, ZFP-like noise fhat = f + eb * u with u in  */
/* [-1, 1) from splitmix64 of (index ^ seed << 40).  A voxel with           */
/* |f - fhat| > eps in T falls back to f.                                   */
static inline uint64_t pmszo_splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

#define PMSZO_DEFINE_STANDIN(T, SUF, FABS)                                                       \
    int pmszo_standin_##SUF(const T *f, T *fh, int64_t n, double eb, int kind, uint64_t seed) {  \
        if (n < 0 || !(eb > 0) || (kind != 0 && kind != 1)) return PMSZO_ERR_ARG;               \
        const T eps = (T)eb;                                                                     \
        const double step = 2.0 * eb;                                                            \
        const uint64_t salt = (seed & 0xFFFFFFFFull) << 40;                                      \
        _Pragma("omp parallel for schedule(static)")                                             \
        for (int64_t i = 0; i < n; ++i) {                                                        \
            const T fv = f[i];                                                                   \
            T v;                                                                                 \
            if (kind == 0) {                                                                     \
                v = (T)(step * rint((double)fv / step));                                         \
            } else {                                                                             \
                const uint64_t h = pmszo_splitmix64((uint64_t)i ^ salt);                         \
                const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;    \
                v = (T)((double)fv + eb * u);                                                    \
            }                                                                                    \
            if (!(FABS(fv - v) <= eps)) v = fv;                                                  \
            fh[i] = v;                                                                           \
        }                                                                                        \
        return PMSZO_OK;                                                                         \
    }

PMSZO_DEFINE_STANDIN(float, f32, fabsf)
PMSZO_DEFINE_STANDIN(double, f64, fabs)
