/* Declaration-only stand-in for <zstd.h> (see mpi.h in this directory). */
#pragma once
#include <stddef.h>
/* C linkage, as libzstd exports them (oracle/ref_encoder.cu links the real
 * libzstd.so.1; the cubin builds never call them). */
#ifdef __cplusplus
extern "C" {
#endif
size_t ZSTD_compress(void *, size_t, const void *, size_t, int);
size_t ZSTD_compressBound(size_t);
size_t ZSTD_decompress(void *, size_t, const void *, size_t);
unsigned ZSTD_isError(size_t);
const char *ZSTD_getErrorName(size_t);
unsigned ZSTD_versionNumber(void);
#ifdef __cplusplus
}
#endif
