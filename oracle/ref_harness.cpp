// ref_harness.cpp -- runs the REFERENCE's own CUDA kernels at an MPI grid of
// 1x1x1, to pin the oracle (test infrastructure; never part of the product).
//
// oracle/build_ref.py compiles the unmodified pMSz.cu, where it lies, into
// oracle/_ref/pmsz_ref.cubin (device code only, with declaration-only shim
// headers for MPI / SZ3 / ZFP / zstd).  This program loads that cubin with the
// CUDA driver API and restates, in its own code, the host sequence of c_loops
// (pMSz.cu:1872-2074) and run_extract_edits (pMSz.cu:2140-2226) around the
// reference kernels iscriticle<double>, init_counter, init_edits and
// extract_edits_kernel<double>, on the reference's padded layout with the
// INVALID_VAL = 1e30 halo (pMSz.cu:346-381).  fp64 only, like the reference.
//
//   ref_harness <cubin> label   <nx> <ny> <nz> <eb> <f.bin> <fh.bin> <out>
//   ref_harness <cubin> detect  <nx> <ny> <nz> <eb> <f.bin> <fh.bin> <out>
//   ref_harness <cubin> correct <nx> <ny> <nz> <eb> <f.bin> <fh.bin> <out>
//   ref_harness <cubin> extract <nx> <ny> <nz> <eb> <f.bin> <prev.bin> <out> <cur.bin>
//   ref_harness <naive cubin> naive <nx> <ny> <nz> <eb> <f.bin> <fh.bin> <out>
//
// The naive mode loads oracle/_ref/naive_ref.cubin (the unmodified
// naive_MSz.cu, compiled the same way) and restates the host sequence of its
// c_loops (naive_MSz.cu:1887-2220) around its iscriticle<double>,
// PathCompression, extract_false_path<double>, init_counter and init_edits.
//
// Outputs (raw little-endian, padded unless noted): <out>_ortypes.bin (int32,
// 2 per voxel), <out>_dir_as.bin / _dir_ds.bin (int32), <out>_counts.bin
// (3 uint32: count_f_max / min / dir after the last pass), <out>_field.bin
// (double), <out>_ite.bin (int32), <out>_deltas.bin (uint8, core, x fastest),
// <out>_editsout.bin (double, core, before compaction), <out>_hcount.bin,
// <out>_ms.bin (float: device-synchronised ms of the loop, correct / naive).
#include <cuda.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

const char *kIscriticle = "_Z10iscriticleIdEvPiS0_S0_S0_PmPT_S3_S0_PhmmmmS0_mmmmmiS0_iS2_S2_iS2_S2_iiii";
const char *kInitCounter = "_Z12init_countermPh";
const char *kInitEdits = "_Z10init_editsmPi";
const char *kExtract = "_Z20extract_edits_kernelIdEvPKT_S2_S2_PKhPmPhPS0_mmmmmiS0_mPjS0_i";
// naive_MSz.cu's kernels (its iscriticle has no max-only flag: 30 parameters)
const char *kNaiveIscriticle = "_Z10iscriticleIdEvPiS0_S0_S0_PmPT_S3_S0_PhmmmmS0_mmmmmiS0_iS2_S2_iS2_S2_iii";
const char *kPathCompression = "_Z15PathCompressionPimmmmi";
const char *kFalsePath = "_Z18extract_false_pathIdEvPT_S1_PiS2_S2_S2_mmmmS2_S2_S2_S2_PhiS0_S0_iiS2_i";
const double kInvalid = 1e30;

#define CK(x)                                                                      \
    do {                                                                           \
        CUresult r_ = (x);                                                         \
        if (r_ != CUDA_SUCCESS) {                                                  \
            const char *s_ = nullptr;                                              \
            cuGetErrorString(r_, &s_);                                             \
            std::fprintf(stderr, "%s failed: %s\n", #x, s_ ? s_ : "?");            \
            std::exit(3);                                                          \
        }                                                                          \
    } while (0)

std::vector<double> read_core(const char *path, size_t n) {
    std::vector<double> v(n);
    FILE *fp = std::fopen(path, "rb");
    if (!fp || std::fread(v.data(), sizeof(double), n, fp) != n) {
        std::fprintf(stderr, "cannot read %zu doubles from %s\n", n, path);
        std::exit(2);
    }
    std::fclose(fp);
    return v;
}

template <class T>
void write(const std::string &path, const T *p, size_t n) {
    FILE *fp = std::fopen(path.c_str(), "wb");
    if (!fp || std::fwrite(p, sizeof(T), n, fp) != n) {
        std::fprintf(stderr, "cannot write %s\n", path.c_str());
        std::exit(2);
    }
    std::fclose(fp);
}

struct Ref {
    CUmodule mod;
    CUfunction isc, initc, inite, extract, pathc, falsep;
    CUdeviceptr g_max, g_min, g_dir;
    size_t W, H, D, N;  // padded sizes
    unsigned grid;
};

void zero_counters(Ref &r) {
    const unsigned z = 0;
    CK(cuMemcpyHtoD(r.g_max, &z, 4));
    CK(cuMemcpyHtoD(r.g_min, &z, 4));
    CK(cuMemcpyHtoD(r.g_dir, &z, 4));
}

void read_counters(Ref &r, unsigned c[3]) {
    CK(cuMemcpyDtoH(&c[0], r.g_max, 4));
    CK(cuMemcpyDtoH(&c[1], r.g_min, 4));
    CK(cuMemcpyDtoH(&c[2], r.g_dir, 4));
}

// One iscriticle launch with the argument list of c_loops' calls
// (pMSz.cu:1894-1895, 1968-1969, 2022-2023).
void iscriticle(Ref &r, CUdeviceptr dir_as, CUdeviceptr dir_ds, CUdeviceptr input, CUdeviceptr decp, CUdeviceptr edits,
                CUdeviceptr cnt, CUdeviceptr or_types, CUdeviceptr send_flag, int q, double bound, double delta, int ite,
                int data_type, int check_final, size_t nx, size_t ny) {
    CUdeviceptr nullp = 0;
    size_t W = r.W, H = r.H, D = r.D, N = r.N, zero = 0, wt = nx, ht = ny;
    int rank = 0, preserve = 0, maxonly = 0;
    double uth = 0.0, lth = 0.0;
    void *args[] = {&nullp, &nullp, &dir_as, &dir_ds, &nullp, &input, &decp, &edits, &cnt, &W, &H, &D, &N,
                    &or_types, &zero, &zero, &zero, &wt, &ht, &rank, &send_flag, &q, &bound, &delta, &ite, &uth,
                    &lth, &data_type, &preserve, &check_final, &maxonly};
    CK(cuLaunchKernel(r.isc, r.grid, 1, 1, 256, 1, 1, 0, 0, args, nullptr));
    CK(cuCtxSynchronize());
}

// naive_MSz.cu's iscriticle (naive_MSz.cu:645-651): DS_M / AS_M first, and
// data_type, preserveMSS, checkFinal last.
void naive_iscriticle(Ref &r, CUdeviceptr dsm, CUdeviceptr asm_, CUdeviceptr dir_as, CUdeviceptr dir_ds,
                      CUdeviceptr input, CUdeviceptr decp, CUdeviceptr edits, CUdeviceptr cnt, CUdeviceptr or_types,
                      CUdeviceptr send_flag, int q, double bound, double delta, int ite, int data_type,
                      int check_final, size_t nx, size_t ny) {
    CUdeviceptr nullp = 0;
    size_t W = r.W, H = r.H, D = r.D, N = r.N, zero = 0, wt = nx, ht = ny;
    int rank = 0, preserve = 0;
    double uth = 0.0, lth = 0.0;
    void *args[] = {&dsm, &asm_, &dir_as, &dir_ds, &nullp, &input, &decp, &edits, &cnt, &W, &H, &D, &N,
                    &or_types, &zero, &zero, &zero, &wt, &ht, &rank, &send_flag, &q, &bound, &delta, &ite, &uth,
                    &lth, &data_type, &preserve, &check_final};
    CK(cuLaunchKernel(r.isc, r.grid, 1, 1, 256, 1, 1, 0, 0, args, nullptr));
    CK(cuCtxSynchronize());
}

void path_compression(Ref &r, CUdeviceptr label) {
    size_t N = r.N, W = r.W, H = r.H, D = r.D;
    int preserve = 0;  // c_loops passes 0 (naive_MSz.cu:1914-1917, 2045-2047)
    void *args[] = {&label, &N, &W, &H, &D, &preserve};
    CK(cuLaunchKernel(r.pathc, r.grid, 1, 1, 256, 1, 1, 0, 0, args, nullptr));
    CK(cuCtxSynchronize());
}

void false_path(Ref &r, CUdeviceptr decp, CUdeviceptr input, CUdeviceptr dsm0, CUdeviceptr dsm1, CUdeviceptr asm0,
                CUdeviceptr asm1, CUdeviceptr or_types, CUdeviceptr dir_ds, CUdeviceptr dir_as, CUdeviceptr edits,
                CUdeviceptr cnt, int q, double bound, double delta, int ite, CUdeviceptr send_flag, int fix) {
    size_t N = r.N, W = r.W, H = r.H, D = r.D;
    int rank = 0;
    void *args[] = {&decp, &input, &dsm0, &dsm1, &asm0, &asm1, &N, &W, &H, &D, &or_types, &dir_ds, &dir_as,
                    &edits, &cnt, &q, &bound, &delta, &rank, &ite, &send_flag, &fix};
    CK(cuLaunchKernel(r.falsep, r.grid, 1, 1, 256, 1, 1, 0, 0, args, nullptr));
    CK(cuCtxSynchronize());
}

// Device-synchronised wall time of the loop, from the original labelling to
// convergence (the window of the reference's "comfputational overhead" print).
struct Clock {
    CUevent a, b;
    Clock() {
        CK(cuEventCreate(&a, CU_EVENT_DEFAULT));
        CK(cuEventCreate(&b, CU_EVENT_DEFAULT));
    }
    void start() { CK(cuEventRecord(a, 0)); }
    float stop() {
        CK(cuEventRecord(b, 0));
        CK(cuEventSynchronize(b));
        float ms = 0;
        CK(cuEventElapsedTime(&ms, a, b));
        return ms;
    }
};

void init_edits(Ref &r, CUdeviceptr edits) {
    size_t ds = r.N;
    void *a[] = {&ds, &edits};
    CK(cuLaunchKernel(r.inite, r.grid, 1, 1, 256, 1, 1, 0, 0, a, nullptr));
    CK(cuCtxSynchronize());
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 10) {
        std::fprintf(stderr, "usage: ref_harness <cubin> <label|detect|correct|extract|naive> nx ny nz eb f.bin fh.bin out [cur.bin]\n");
        return 2;
    }
    const std::string mode = argv[2];
    const size_t nx = std::strtoull(argv[3], nullptr, 10), ny = std::strtoull(argv[4], nullptr, 10),
                 nz = std::strtoull(argv[5], nullptr, 10);
    const double bound = std::strtod(argv[6], nullptr);
    const std::string out = argv[9];
    const int q = 5;                                   // pMSz.cu:2630
    const double delta = bound / q;                    // pMSz.cu:2814
    const size_t n = nx * ny * nz;

    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    Ref r;
    const bool naive = mode == "naive";
    CK(cuModuleLoad(&r.mod, argv[1]));
    CK(cuModuleGetFunction(&r.isc, r.mod, naive ? kNaiveIscriticle : kIscriticle));
    CK(cuModuleGetFunction(&r.initc, r.mod, kInitCounter));
    CK(cuModuleGetFunction(&r.inite, r.mod, kInitEdits));
    CK(cuModuleGetFunction(&r.extract, r.mod, kExtract));
    if (naive) {
        CK(cuModuleGetFunction(&r.pathc, r.mod, kPathCompression));
        CK(cuModuleGetFunction(&r.falsep, r.mod, kFalsePath));
    }
    size_t gsz;
    CK(cuModuleGetGlobal(&r.g_max, &gsz, r.mod, "count_f_max"));
    CK(cuModuleGetGlobal(&r.g_min, &gsz, r.mod, "count_f_min"));
    CK(cuModuleGetGlobal(&r.g_dir, &gsz, r.mod, "count_f_dir"));
    r.W = nx + 2;
    r.H = ny + 2;
    r.D = nz + 2;
    r.N = r.W * r.H * r.D;
    r.grid = static_cast<unsigned>((r.N + 255) / 256);

    // padded host blocks with the INVALID shell (read_subblock + exchange_ghost_layers at 1 rank)
    auto pad = [&](const std::vector<double> &core) {
        std::vector<double> p(r.N, kInvalid);
        for (size_t z = 0; z < nz; ++z)
            for (size_t y = 0; y < ny; ++y)
                std::memcpy(&p[(z + 1) * r.W * r.H + (y + 1) * r.W + 1], &core[(z * ny + y) * nx], nx * sizeof(double));
        return p;
    };
    const std::vector<double> f = pad(read_core(argv[7], n));
    const std::vector<double> fh = pad(read_core(argv[8], n));

    CUdeviceptr d_in, d_dec, d_copy, d_or, d_as, d_ds, d_edits, d_cnt, d_flag;
    CK(cuMemAlloc(&d_in, r.N * 8));
    CK(cuMemAlloc(&d_dec, r.N * 8));
    CK(cuMemAlloc(&d_copy, r.N * 8));
    CK(cuMemAlloc(&d_or, 2 * r.N * 4));
    CK(cuMemAlloc(&d_as, r.N * 4));
    CK(cuMemAlloc(&d_ds, r.N * 4));
    CK(cuMemAlloc(&d_edits, r.N * 4));
    CK(cuMemAlloc(&d_cnt, r.N));
    CK(cuMemAlloc(&d_flag, 4));
    CK(cuMemsetD32(d_or, 0, 2 * r.N));
    CK(cuMemsetD32(d_as, 0, r.N));
    CK(cuMemsetD32(d_ds, 0, r.N));
    CK(cuMemsetD32(d_edits, 0, r.N));
    CK(cuMemsetD32(d_flag, 0, 1));
    CK(cuMemcpyHtoD(d_in, f.data(), r.N * 8));
    CK(cuMemcpyHtoD(d_dec, fh.data(), r.N * 8));
    CK(cuMemcpyHtoD(d_copy, fh.data(), r.N * 8));

    if (mode == "extract") {
        if (argc < 11) return 2;
        const std::vector<double> cur = pad(read_core(argv[10], n));
        CK(cuMemcpyHtoD(d_dec, cur.data(), r.N * 8));
        CUdeviceptr d_deltas, d_eo, d_count, nullp = 0;
        CK(cuMemAlloc(&d_deltas, n));
        CK(cuMemAlloc(&d_eo, n * 8));
        CK(cuMemAlloc(&d_count, 4));
        CK(cuMemsetD8(d_deltas, 0xEE, n));  // marks entries the kernel leaves unwritten
        CK(cuMemsetD32(d_eo, 0, 2 * n));
        CK(cuMemsetD32(d_count, 0, 1));
        size_t lx = nx, ly = ny, lz = nz, px = r.W, py = r.H, ds = r.N;
        int qq = q, rank = 0;
        double b = bound, dl = delta;
        void *args[] = {&d_dec, &d_copy, &d_in, &d_cnt, &nullp, &d_deltas, &d_eo, &lx, &ly, &lz, &px, &py,
                        &qq, &b, &ds, &d_count, &dl, &rank};
        CK(cuLaunchKernel(r.extract, r.grid, 1, 1, 256, 1, 1, 0, 0, args, nullptr));
        CK(cuCtxSynchronize());
        std::vector<uint8_t> deltas(n);
        std::vector<double> eo(n);
        unsigned hc = 0;
        CK(cuMemcpyDtoH(deltas.data(), d_deltas, n));
        CK(cuMemcpyDtoH(eo.data(), d_eo, n * 8));
        CK(cuMemcpyDtoH(&hc, d_count, 4));
        write(out + "_deltas.bin", deltas.data(), n);
        write(out + "_editsout.bin", eo.data(), n);
        write(out + "_hcount.bin", &hc, 1);
        return 0;
    }

    if (naive) {
        // c_loops of naive_MSz.cu at one rank (naive_MSz.cu:1887-2220); the halo
        // exchange has no neighbour to talk to.  d_as / d_ds hold the current
        // directions, DS_M / AS_M the original labels, dec_* the current ones.
        CUdeviceptr dsm, asm0, dsm1, asm1;
        CK(cuMemAlloc(&dsm, r.N * 4));
        CK(cuMemAlloc(&asm0, r.N * 4));
        CK(cuMemAlloc(&dsm1, r.N * 4));
        CK(cuMemAlloc(&asm1, r.N * 4));
        CK(cuMemsetD32(dsm, 0, r.N));
        CK(cuMemsetD32(asm0, 0, r.N));
        CK(cuMemsetD32(dsm1, 0, r.N));
        CK(cuMemsetD32(asm1, 0, r.N));
        Clock clock;
        clock.start();
        {
            size_t ds = r.N;
            void *args[] = {&ds, &d_cnt};
            CK(cuLaunchKernel(r.initc, r.grid, 1, 1, 256, 1, 1, 0, 0, args, nullptr));
            CK(cuCtxSynchronize());
        }
        int ite = 0;
        naive_iscriticle(r, dsm, asm0, d_as, d_ds, d_in, d_in, d_edits, d_cnt, d_or, d_flag, q, bound, delta, ite, 1, 0,
                         nx, ny);
        path_compression(r, dsm);
        path_compression(r, asm0);
        unsigned c[3] = {0, 0, 0};
        unsigned gmax = 1, gmin = 1, gdir = 0, hmax = 1, hmin = 1;
        int inner = 0, outer = 0;
        std::vector<unsigned> recs;  // per pass: kind, fmax, fmin, fdir (kind 0 extrema, 1 path, 2 check)
        const int cap = 100000;
        while ((gmax > 0 || gmin > 0 || gdir > 0) && ite < cap) {
            ++outer;
            ite += 2;
            while ((hmax > 0 || hmin > 0) && ite < cap) {
                ++ite;
                ++inner;
                init_edits(r, d_edits);
                zero_counters(r);
                naive_iscriticle(r, dsm1, asm1, d_as, d_ds, d_in, d_dec, d_edits, d_cnt, d_or, d_flag, q, bound, delta,
                                 ite, 0, 0, nx, ny);
                read_counters(r, c);
                hmax = c[0];
                hmin = c[1];
                recs.insert(recs.end(), {0u, c[0], c[1], 0u});
            }
            zero_counters(r);
            path_compression(r, dsm1);
            path_compression(r, asm1);
            init_edits(r, d_edits);
            false_path(r, d_dec, d_in, dsm, dsm1, asm0, asm1, d_or, d_ds, d_as, d_edits, d_cnt, q, bound, delta, ite,
                       d_flag, 0);
            read_counters(r, c);
            recs.insert(recs.end(), {1u, 0u, 0u, c[2]});
            naive_iscriticle(r, dsm1, asm1, d_as, d_ds, d_in, d_dec, d_edits, d_cnt, d_or, d_flag, q, bound, delta,
                             ite, 0, 1, nx, ny);
            zero_counters(r);
            naive_iscriticle(r, dsm1, asm1, d_as, d_ds, d_in, d_dec, d_edits, d_cnt, d_or, d_flag, q, bound, delta,
                             ite, 0, 1, nx, ny);
            path_compression(r, dsm1);
            path_compression(r, asm1);
            false_path(r, d_dec, d_in, dsm, dsm1, asm0, asm1, d_or, d_ds, d_as, d_edits, d_cnt, q, bound, delta, ite,
                       d_flag, 1);
            read_counters(r, c);
            recs.insert(recs.end(), {2u, c[0], c[1], c[2]});
            hmax = gmax = c[0];
            hmin = gmin = c[1];
            gdir = c[2];
        }
        const float ms = clock.stop();
        std::vector<double> field(r.N);
        CK(cuMemcpyDtoH(field.data(), d_dec, r.N * 8));
        write(out + "_field.bin", field.data(), r.N);
        write(out + "_ite.bin", &ite, 1);
        write(out + "_ms.bin", &ms, 1);
        const int io[2] = {inner, outer};
        write(out + "_passes.bin", io, 2);
        write(out + "_recs.bin", recs.data(), recs.size());
        return 0;
    }

    // init_counter + original labelling (c_loops, pMSz.cu:1883-1895)
    Clock clock;
    clock.start();
    {
        size_t ds = r.N;
        void *args[] = {&ds, &d_cnt};
        CK(cuLaunchKernel(r.initc, r.grid, 1, 1, 256, 1, 1, 0, 0, args, nullptr));
        CK(cuCtxSynchronize());
    }
    int ite = 0;
    iscriticle(r, d_as, d_ds, d_in, d_in, d_edits, d_cnt, d_or, d_flag, q, bound, delta, ite, 1, 0, nx, ny);
    unsigned c[3] = {0, 0, 0};
    if (mode == "detect") {
        zero_counters(r);
        iscriticle(r, d_as, d_ds, d_in, d_dec, d_edits, d_cnt, d_or, d_flag, q, bound, delta, ite, 0, 1, nx, ny);
        read_counters(r, c);
    } else if (mode == "correct") {
        // the outer / inner loops of c_loops at one rank (pMSz.cu:1943-2071); the
        // halo exchange between them has no neighbour to talk to
        unsigned gmax = 1, gmin = 1, gdir = 0, hmax = 1, hmin = 1, hdir = 1;
        const int cap = 100000;
        while ((gmax > 0 || gmin > 0 || gdir > 0) && ite < cap) {
            ++ite;
            while ((hmax > 0 || hmin > 0 || hdir > 0) && ite < cap) {
                ++ite;
                size_t ds = r.N;
                void *a2[] = {&ds, &d_edits};
                CK(cuLaunchKernel(r.inite, r.grid, 1, 1, 256, 1, 1, 0, 0, a2, nullptr));
                zero_counters(r);
                CK(cuCtxSynchronize());
                iscriticle(r, d_as, d_ds, d_in, d_dec, d_edits, d_cnt, d_or, d_flag, q, bound, delta, ite, 0, 0, nx, ny);
                read_counters(r, c);
                hmax = c[0];
                hmin = c[1];
                hdir = c[2];
            }
            zero_counters(r);
            iscriticle(r, d_as, d_ds, d_in, d_dec, d_edits, d_cnt, d_or, d_flag, q, bound, delta, ite, 0, 1, nx, ny);
            read_counters(r, c);
            gmax = c[0];
            gmin = c[1];
            gdir = c[2];
        }
        const float ms = clock.stop();
        std::vector<double> field(r.N);
        CK(cuMemcpyDtoH(field.data(), d_dec, r.N * 8));
        write(out + "_field.bin", field.data(), r.N);
        write(out + "_ite.bin", &ite, 1);
        write(out + "_ms.bin", &ms, 1);
    } else if (mode != "label") {
        std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
        return 2;
    }
    std::vector<int> ot(2 * r.N), as(r.N), dsd(r.N);
    CK(cuMemcpyDtoH(ot.data(), d_or, 2 * r.N * 4));
    CK(cuMemcpyDtoH(as.data(), d_as, r.N * 4));
    CK(cuMemcpyDtoH(dsd.data(), d_ds, r.N * 4));
    write(out + "_ortypes.bin", ot.data(), 2 * r.N);
    write(out + "_dir_as.bin", as.data(), r.N);
    write(out + "_dir_ds.bin", dsd.data(), r.N);
    write(out + "_counts.bin", c, 3);
    return 0;
}
