/* Declaration-only stand-in for <zstd.h> (see mpi.h in this directory). */
#pragma once
#include <stddef.h>
size_t ZSTD_compress(void *, size_t, const void *, size_t, int);
size_t ZSTD_compressBound(size_t);
size_t ZSTD_decompress(void *, size_t, const void *, size_t);
unsigned ZSTD_isError(size_t);
const char *ZSTD_getErrorName(size_t);
