/* Declaration-only stand-in for <zfp.h> (see mpi.h in this directory). */
#pragma once
#include <stddef.h>
typedef enum { zfp_type_none = 0, zfp_type_int32, zfp_type_int64, zfp_type_float, zfp_type_double } zfp_type;
typedef struct zfp_field_ zfp_field;
typedef struct zfp_stream_ zfp_stream;
typedef struct bitstream_ bitstream;
zfp_field *zfp_field_3d(void *, zfp_type, size_t, size_t, size_t);
void zfp_field_free(zfp_field *);
zfp_stream *zfp_stream_open(bitstream *);
void zfp_stream_close(zfp_stream *);
double zfp_stream_set_accuracy(zfp_stream *, double);
size_t zfp_stream_maximum_size(const zfp_stream *, const zfp_field *);
void zfp_stream_set_bit_stream(zfp_stream *, bitstream *);
void zfp_stream_rewind(zfp_stream *);
size_t zfp_compress(zfp_stream *, const zfp_field *);
size_t zfp_decompress(zfp_stream *, zfp_field *);
bitstream *stream_open(void *, size_t);
void stream_close(bitstream *);
void stream_rewind(bitstream *);
