/*
 * pmsz_host.h -- host-side helpers of the GB300-native pMSz path: the edit
 * file encoder / decoder.  Host pointers only.  Buffers returned through
 * `out` / `values` are allocated with malloc and released with pmsz_free.
 */
#ifndef PMSZ_HOST_H
#define PMSZ_HOST_H

#include <stddef.h>
#include <stdint.h>

#include "pmsz.h"

#ifdef __cplusplus
extern "C" {
#endif

/*
 * _deltas.bin payload.  Replaces compress_symbols_0_N (pMSz.cu:2359-2369)
 * with pack_nbits / bits_for_max (pMSz.cu:2328-2356): each delta symbol in
 * 0..q is packed LSB-first in bits_for_max(q) bits (3 bits for q = 5), then
 * zstd level 5 (pMSz.cu:2480).
 */
int pmsz_encode_deltas(const uint8_t *deltas, size_t n, int q, uint8_t **out, size_t *out_len);
/* The same payload from symbols already packed (PMSZ_FLAG_PACKED_DELTAS):
 * zstd level 5 of the `len` packed bytes; identical output. */
int pmsz_encode_packed_deltas(const uint8_t *packed, size_t len, uint8_t **out, size_t *out_len);

/*
 * _edits.bin payload.  Replaces compress_zstd<T> (pMSz.cu:2261-2277, called at
 * pMSz.cu:2473): the clamp values as raw bytes (elem_size 4 or 8), zstd level
 * 3; zero values give an empty payload (*out = NULL, *out_len = 0).
 */
int pmsz_encode_clamps(const void *values, size_t count, size_t elem_size, uint8_t **out, size_t *out_len);

/* Inverses (the reference's decompress_symbols_0_N, pMSz.cu:2413-2426, and
 * decompress_zstd_to_vector, pMSz.cu:2372-2391). */
int pmsz_decode_deltas(const uint8_t *comp, size_t len, size_t n, int q, uint8_t *deltas);
int pmsz_decode_clamps(const uint8_t *comp, size_t len, size_t elem_size, void **values, size_t *count);

void pmsz_free(void *p);

/* Optional outputs of pmsz_correct_host_*. */
typedef struct pmsz_host_outputs {
    uint8_t *deltas;             /* host array of n bytes: edit symbols, or NULL (with
                                    PMSZ_FLAG_PACKED_DELTAS: ceil(n * bits_for_max(q) / 8)
                                    bytes of packed symbols) */
    void *clamp;                 /* host array of n values of the field type, or NULL;
                                    the first n_clamp entries are the clamp list */
    uint64_t n_clamp;            /* out */
    uint64_t edit_count;         /* out: voxels with cur < prev, the reference's "Edit count" */
    pmsz_verify_result *verify;  /* re-verification of the result, or NULL */
} pmsz_host_outputs;

/*
 * pmsz_correct_host_{f32,f64}: the reference main's single-rank pipeline
 * (pMSz.cu:2855-2987: device copies, c_loops, gather_cost_sparse) on HOST
 * arrays.  f and fhat are host arrays of nx*ny*nz values; fhat is replaced by
 * the corrected field.  outs may be NULL.  Device memory is allocated
 * stream-ordered on `stream` (a cudaStream_t, NULL = default stream) and
 * released before return.  Same status codes as pmsz_correct_*.
 */
int pmsz_correct_host_f32(const float *f, float *fhat, size_t nx, size_t ny, size_t nz, double eb,
                          const pmsz_opts *opts, pmsz_result *res, pmsz_host_outputs *outs, void *stream);
int pmsz_correct_host_f64(const double *f, double *fhat, size_t nx, size_t ny, size_t nz, double eb,
                          const pmsz_opts *opts, pmsz_result *res, pmsz_host_outputs *outs, void *stream);

/* ZSTD_versionNumber() of the libzstd the library loaded (byte parity of the
 * edit files holds only for equal zstd versions). */
unsigned pmsz_zstd_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PMSZ_HOST_H */
