/*
 * ref_encoder.cu -- TEST INFRASTRUCTURE ONLY.  Drives the reference's own host
 * encoder of the edit files so that this project's encoder can be pinned to
 * its bytes: the UNMODIFIED reference pMSz.cu is #included (built by
 * oracle/build_ref.py from where it lies; nothing of it is copied), its main
 * renamed, and this file's main calls
 *   compress_symbols_0_N(deltas, q, 5)   pMSz.cu:2359-2369 (pack_nbits, pMSz.cu:2328-2348,
 *                                        then zstd level 5): the _deltas.bin payload, and
 *   compress_zstd<T>(clamps)             pMSz.cu:2261-2277 (zstd level 3): the _edits.bin
 *                                        payload (pMSz.cu:2473, 2478)
 * with the real libzstd.  The MPI, SZ3 and ZFP entry points that the
 * reference's host code names are defined below as single-rank stand-ins;
 * none of them is reached by the two calls above.
 *
 *   ref_encoder deltas <in.u8> <q> <out>
 *   ref_encoder clamps <in.raw> <elem_size 4|8> <out>
 */
#define main pmsz_reference_main
#include "pMSz.cu"
#undef main

#include <chrono>
#include <cstdio>
#include <fstream>
#include <iterator>

// ---- single-rank stand-ins (never called by this driver) ----------------
[[noreturn]] static void not_here(const char *what) {
    std::fprintf(stderr, "ref_encoder: %s is not available in the encoder driver\n", what);
    std::abort();
}
int MPI_Init(int *, char ***) { return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Abort(MPI_Comm, int code) { std::exit(code ? code : 1); }
int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
int MPI_Barrier(MPI_Comm) { return 0; }
double MPI_Wtime(void) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
int MPI_Cart_create(MPI_Comm, int, const int *, const int *, int, MPI_Comm *) { not_here("MPI_Cart_create"); }
int MPI_Cart_coords(MPI_Comm, int, int, int *) { not_here("MPI_Cart_coords"); }
int MPI_Cart_rank(MPI_Comm, const int *, int *) { not_here("MPI_Cart_rank"); }
int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { not_here("MPI_Isend"); }
int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { not_here("MPI_Irecv"); }
int MPI_Waitall(int, MPI_Request *, MPI_Status *) { not_here("MPI_Waitall"); }
int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int, void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
    not_here("MPI_Sendrecv");
}
int MPI_Reduce(const void *, void *, int, MPI_Datatype, MPI_Op, int, MPI_Comm) { not_here("MPI_Reduce"); }
int MPI_Allreduce(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { not_here("MPI_Allreduce"); }
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { not_here("MPI_Bcast"); }
int MPI_Gather(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, int, MPI_Comm) { not_here("MPI_Gather"); }
int MPI_Allgather(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, MPI_Comm) { not_here("MPI_Allgather"); }
int MPI_File_open(MPI_Comm, const char *, int, MPI_Info, MPI_File *) { not_here("MPI_File_open"); }
int MPI_File_close(MPI_File *) { not_here("MPI_File_close"); }
int MPI_File_write_at_all(MPI_File, MPI_Offset, const void *, int, MPI_Datatype, MPI_Status *) {
    not_here("MPI_File_write_at_all");
}
int MPI_File_read_at_all(MPI_File, MPI_Offset, void *, int, MPI_Datatype, MPI_Status *) {
    not_here("MPI_File_read_at_all");
}
int MPI_File_get_size(MPI_File, MPI_Offset *) { not_here("MPI_File_get_size"); }
zfp_field *zfp_field_3d(void *, zfp_type, size_t, size_t, size_t) { not_here("zfp"); }
void zfp_field_free(zfp_field *) { not_here("zfp"); }
zfp_stream *zfp_stream_open(bitstream *) { not_here("zfp"); }
void zfp_stream_close(zfp_stream *) { not_here("zfp"); }
double zfp_stream_set_accuracy(zfp_stream *, double) { not_here("zfp"); }
size_t zfp_stream_maximum_size(const zfp_stream *, const zfp_field *) { not_here("zfp"); }
void zfp_stream_set_bit_stream(zfp_stream *, bitstream *) { not_here("zfp"); }
void zfp_stream_rewind(zfp_stream *) { not_here("zfp"); }
size_t zfp_compress(zfp_stream *, const zfp_field *) { not_here("zfp"); }
size_t zfp_decompress(zfp_stream *, zfp_field *) { not_here("zfp"); }
bitstream *stream_open(void *, size_t) { not_here("zfp"); }
void stream_close(bitstream *) { not_here("zfp"); }
void stream_rewind(bitstream *) { not_here("zfp"); }
SZ3::Config::Config(int, int, int) { not_here("SZ3"); }
template <class T> char *SZ_compress(const SZ3::Config &, const T *, size_t &) { not_here("SZ3"); }
template <class T> void SZ_decompress(const SZ3::Config &, const char *, size_t, T *) { not_here("SZ3"); }
template char *SZ_compress<double>(const SZ3::Config &, const double *, size_t &);
template void SZ_decompress<double>(const SZ3::Config &, const char *, size_t, double *);
template char *SZ_compress<float>(const SZ3::Config &, const float *, size_t &);
template void SZ_decompress<float>(const SZ3::Config &, const char *, size_t, float *);

// ---- driver ---------------------------------------------------------------
static std::vector<uint8_t> read_all(const char *path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) not_here(path);
    return std::vector<uint8_t>(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
}
static void write_all(const char *path, const std::vector<uint8_t> &b) {
    std::ofstream out(path, std::ios::binary);
    out.write(reinterpret_cast<const char *>(b.data()), static_cast<std::streamsize>(b.size()));
}
template <typename T>
static std::vector<uint8_t> clamps_of(const std::vector<uint8_t> &raw) {
    std::vector<T> v(raw.size() / sizeof(T));
    if (!v.empty()) std::memcpy(v.data(), raw.data(), v.size() * sizeof(T));
    return compress_zstd<T>(v);
}
int main(int argc, char **argv) {
    if (argc != 5) {
        std::fprintf(stderr, "usage: ref_encoder deltas <in.u8> <q> <out> | clamps <in.raw> <4|8> <out>\n");
        return 2;
    }
    const std::string mode = argv[1];
    const std::vector<uint8_t> in = read_all(argv[2]);
    const int k = std::atoi(argv[3]);
    if (mode == "deltas") {
        write_all(argv[4], compress_symbols_0_N(in, static_cast<unsigned>(k), 5));
    } else if (mode == "clamps" && (k == 4 || k == 8)) {
        write_all(argv[4], k == 8 ? clamps_of<double>(in) : clamps_of<float>(in));
    } else {
        return 2;
    }
    std::printf("zstd %u\n", ZSTD_versionNumber());
    return 0;
}
