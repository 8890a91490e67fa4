// cli.cpp -- `pmsz`, a drop-in for the reference program's command line at an
// MPI grid of 1x1x1 (main, pMSz.cu:2596-3188).
//
//   pmsz <path>,<W>,<H>,<D> <eb> <sz3|zfp> <PX> <PY> <PZ> [options]   (pMSz.cu:2625-2667)
//   pmsz <path> <W> <H> <D> <eb> <sz3|zfp> <PX> <PY> <PZ> [options]    (README.md:68-73)
//   pmsz --reconstruct <decp>,<W>,<H>,<D> <eb> --out FILE [--deltas F] [--edits F]
//
// Reads the raw little-endian field (x fastest, pMSz.cu:274-313), obtains the
// decompressed copy, runs the correction on the GPU, and writes the
// reference's outputs in the working directory: _edits.bin and _deltas.bin
// (pMSz.cu:2516-2523), the per-rank timing file
// Global_performance_with_ite_cuda_<comp>_<name>_rank_0_0.txt (pMSz.cu:2925-2943),
// an appended ./stat_result/Global_base_result_<name>_<comp>_Maxonly_final1_0.txt
// when ./stat_result exists (pMSz.cu:3146-3178), and the same stdout keys.
//
// SZ3 and ZFP are not linked.  The decompressed field comes from --decp FILE
// (raw, same type and size), or else from the labelled stand-in of the named
// compressor (sz3: plateaus, zfp: bounded noise), which is announced on
// stdout.  Errors print a message and return a non-zero status; nothing aborts.
//
// --reconstruct is the decoder the reference lacks (its validateResult,
// pMSz.cu:2545-2584, only decompresses): from the decompressed field and the
// _deltas.bin / _edits.bin of a correction it writes the corrected field,
// bit-identical, through pmsz_reconstruct_*.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "pmsz.h"
#include "pmsz_host.h"

namespace {

struct Args {
    std::string path, comp, decp, out, deltas_file = "_deltas.bin", edits_file = "_edits.bin";
    size_t W = 0, H = 0, D = 0;
    double eb = 0;
    int px = 1, py = 1, pz = 1;
    bool f32 = false, full = false, verify = false, naive = false, recon = false;
    int q = 5;
    long long max_sweeps = 10000;
    double cmp_size = 0;
};

int usage(const char *msg) {
    std::fprintf(stderr,
                 "error: %s\nusage: pmsz <path>,<W>,<H>,<D> <abs_eb> <sz3|zfp> <PX> <PY> <PZ> [options]\n"
                 "       pmsz <path> <W> <H> <D> <abs_eb> <sz3|zfp> <PX> <PY> <PZ> [options]\n"
                 "       pmsz --reconstruct <decp>,<W>,<H>,<D> <abs_eb> --out FILE [--deltas FILE] [--edits FILE]\n"
                 "options: --decp FILE  --dtype f64|f32  --q N  --max-sweeps N  --full-sweeps\n"
                 "         --out FILE   --verify  --cmp-size BYTES\n"
                 "         --naive      the naive-MSz strategy (the reference's naive_MSz program)\n",
                 msg);
    return 2;
}

bool parse_size(const std::string &s, size_t &v) {
    char *end = nullptr;
    const unsigned long long x = std::strtoull(s.c_str(), &end, 10);
    if (!end || *end || s.empty() || x == 0) return false;
    v = static_cast<size_t>(x);
    return true;
}

int parse(int argc, char **argv, Args &a) {
    std::vector<std::string> pos;
    for (int i = 1; i < argc; ++i) {
        std::string s = argv[i];
        auto need = [&](const char *what) -> const char * {
            if (i + 1 >= argc) return nullptr;
            (void)what;
            return argv[++i];
        };
        if (s == "--decp") { const char *v = need("file"); if (!v) return usage("--decp needs a file"); a.decp = v; }
        else if (s == "--out") { const char *v = need("file"); if (!v) return usage("--out needs a file"); a.out = v; }
        else if (s == "--dtype") { const char *v = need("type"); if (!v) return usage("--dtype needs f32|f64");
            if (!std::strcmp(v, "f32")) a.f32 = true; else if (!std::strcmp(v, "f64")) a.f32 = false; else return usage("bad --dtype"); }
        else if (s == "--q") { const char *v = need("q"); if (!v) return usage("--q needs a value"); a.q = std::atoi(v); }
        else if (s == "--max-sweeps") { const char *v = need("n"); if (!v) return usage("--max-sweeps needs a value"); a.max_sweeps = std::atoll(v); }
        else if (s == "--cmp-size") { const char *v = need("n"); if (!v) return usage("--cmp-size needs a value"); a.cmp_size = std::atof(v); }
        else if (s == "--full-sweeps") a.full = true;
        else if (s == "--verify") a.verify = true;
        else if (s == "--naive") a.naive = true;
        else if (s == "--reconstruct") a.recon = true;
        else if (s == "--deltas") { const char *v = need("file"); if (!v) return usage("--deltas needs a file"); a.deltas_file = v; }
        else if (s == "--edits") { const char *v = need("file"); if (!v) return usage("--edits needs a file"); a.edits_file = v; }
        else if (s.size() > 2 && s[0] == '-' && s[1] == '-') return usage(("unknown option " + s).c_str());
        else pos.push_back(s);
    }
    size_t k = 0;
    const size_t npos_args = a.recon ? 2 : 6;  // after path,W,H,D: eb [comp PX PY PZ]
    if (pos.size() == npos_args && pos[0].find(',') != std::string::npos) {
        // comma form: argv[1] = path,W,H,D (pMSz.cu:2655-2667)
        std::istringstream iss(pos[0]);
        std::string part;
        std::vector<std::string> p;
        while (std::getline(iss, part, ',')) p.push_back(part);
        if (p.size() != 4 || !parse_size(p[1], a.W) || !parse_size(p[2], a.H) || !parse_size(p[3], a.D))
            return usage("parsing error for dimensions");
        a.path = p[0];
        k = 1;
    } else if (pos.size() == npos_args + 3) {
        a.path = pos[0];
        if (!parse_size(pos[1], a.W) || !parse_size(pos[2], a.H) || !parse_size(pos[3], a.D))
            return usage("parsing error for dimensions");
        k = 4;
    } else {
        return usage("wrong number of arguments");
    }
    char *end = nullptr;
    a.eb = std::strtod(pos[k].c_str(), &end);
    if (!end || *end || !(a.eb > 0)) return usage("error bound must be a positive number");
    if (a.recon) return a.out.empty() ? usage("--reconstruct needs --out FILE") : 0;
    a.comp = pos[k + 1];
    if (a.comp != "sz3" && a.comp != "zfp") return usage("compressor must be sz3 or zfp");
    a.px = std::atoi(pos[k + 2].c_str());
    a.py = std::atoi(pos[k + 3].c_str());
    a.pz = std::atoi(pos[k + 4].c_str());
    if (a.px != 1 || a.py != 1 || a.pz != 1)
        return usage("this program corrects a field on one GPU per process: PX PY PZ must be 1 1 1");
    return 0;
}

std::string stem(const std::string &p) {  // extractFilename, pMSz.cu:2076-2086
    const size_t s = p.find_last_of("/\\");
    std::string f = s == std::string::npos ? p : p.substr(s + 1);
    const size_t d = f.find_last_of('.');
    return d == std::string::npos ? f : f.substr(0, d);
}

template <typename T>
bool read_raw(const std::string &path, std::vector<T> &v, size_t n) {
    std::ifstream in(path, std::ios::binary | std::ios::ate);
    if (!in) {
        std::fprintf(stderr, "error: cannot open %s\n", path.c_str());
        return false;
    }
    const std::streamsize sz = in.tellg();
    if (sz < static_cast<std::streamsize>(n * sizeof(T))) {
        std::fprintf(stderr, "error: %s holds %lld bytes, expected %zu\n", path.c_str(), (long long)sz, n * sizeof(T));
        return false;
    }
    in.seekg(0);
    v.resize(n);
    in.read(reinterpret_cast<char *>(v.data()), static_cast<std::streamsize>(n * sizeof(T)));
    return static_cast<bool>(in);
}

bool write_file(const std::string &path, const uint8_t *p, size_t n) {
    std::ofstream o(path, std::ios::binary | std::ios::trunc);
    if (!o) return false;
    if (n) o.write(reinterpret_cast<const char *>(p), static_cast<std::streamsize>(n));
    return static_cast<bool>(o);
}

template <typename T>
int run(const Args &a) {
    const size_t n = a.W * a.H * a.D;
    std::cout << std::fixed << std::setprecision(16);
    std::vector<T> f, fh;
    if (!read_raw<T>(a.path, f, n)) return 1;
    const std::string name = stem(a.path);
    const T *pf = f.data();
    T *df = nullptr, *dfh = nullptr;
    if (cudaMalloc(&df, n * sizeof(T)) != cudaSuccess || cudaMalloc(&dfh, n * sizeof(T)) != cudaSuccess) {
        std::fprintf(stderr, "error: device allocation failed\n");
        return 1;
    }
    cudaMemcpy(df, pf, n * sizeof(T), cudaMemcpyHostToDevice);
    if (!a.decp.empty()) {
        if (!read_raw<T>(a.decp, fh, n)) return 1;
        cudaMemcpy(dfh, fh.data(), n * sizeof(T), cudaMemcpyHostToDevice);
    } else {
        std::cout << "decompressed field: " << a.comp << " stand-in (SZ3/ZFP not linked; compressor parity unpinned)"
                  << std::endl;
        const int kind = a.comp == "sz3" ? 0 : 1;
        const int st = sizeof(T) == 4 ? pmsz_standin_f32(reinterpret_cast<const float *>(df), reinterpret_cast<float *>(dfh), n, a.eb, kind, 0, nullptr)
                                      : pmsz_standin_f64(reinterpret_cast<const double *>(df), reinterpret_cast<double *>(dfh), n, a.eb, kind, 0, nullptr);
        if (st) {
            std::fprintf(stderr, "error: stand-in failed: %s\n", pmsz_last_error());
            return 1;
        }
        fh.resize(n);
        cudaMemcpy(fh.data(), dfh, n * sizeof(T), cudaMemcpyDeviceToHost);
    }
    std::cout << "Rank 0 got value = " << a.eb << std::endl;  // pMSz.cu:2803
    std::cout << "decp_" << name << "_" << a.comp << "_" << std::to_string(a.eb) << ".bin" << std::endl;
    cudaFree(df);
    cudaFree(dfh);

    std::vector<T> corrected(fh);
    // delta symbols come back packed (bits_for_max(q) bits each), as the
    // reference's encoder packs them before zstd
    int nbits = 1;
    while ((1 << nbits) < a.q + 1 && nbits < 8) ++nbits;
    std::vector<uint8_t> deltas((n * static_cast<size_t>(nbits) + 7) / 8);
    std::vector<T> clamp(n);
    pmsz_verify_result vr{};
    pmsz_host_outputs outs{};
    outs.deltas = deltas.data();
    outs.clamp = clamp.data();
    outs.verify = a.verify ? &vr : nullptr;
    pmsz_opts opts{a.q, (a.full ? PMSZ_FLAG_FULL_SWEEPS : 0u) | (a.naive ? PMSZ_FLAG_NAIVE : 0u) | PMSZ_FLAG_PACKED_DELTAS,
                   a.max_sweeps};
    pmsz_result res{};
    std::cout << "topology preserving started!" << std::endl;
    const auto t0 = std::chrono::steady_clock::now();
    int st = sizeof(T) == 4
                 ? pmsz_correct_host_f32(reinterpret_cast<const float *>(pf), reinterpret_cast<float *>(corrected.data()), a.W, a.H, a.D, a.eb, &opts, &res, &outs, nullptr)
                 : pmsz_correct_host_f64(reinterpret_cast<const double *>(pf), reinterpret_cast<double *>(corrected.data()), a.W, a.H, a.D, a.eb, &opts, &res, &outs, nullptr);
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st != PMSZ_OK && st != PMSZ_ERR_NOT_CONVERGED) {
        std::fprintf(stderr, "error: correction failed (%s): %s\n", pmsz_strerror(st), pmsz_last_error());
        return 1;
    }
    if (st == PMSZ_ERR_NOT_CONVERGED)
        std::fprintf(stderr, "warning: not converged after %lld sweeps: %s\n", (long long)res.sweeps, pmsz_last_error());
    std::printf("iteration is: %lld\n", (long long)res.iteration);  // pMSz.cu:2073
    std::cout << "comfputational overhead is: " << res.ms_total * 1e-3 << std::endl;  // pMSz.cu:2949
    std::cout << "Edit count: " << outs.edit_count << std::endl;                   // pMSz.cu:2170

    uint8_t *cd = nullptr, *ce = nullptr;
    size_t nd = 0, ne = 0;
    if (pmsz_encode_packed_deltas(deltas.data(), deltas.size(), &cd, &nd) || pmsz_encode_clamps(clamp.data(), outs.n_clamp, sizeof(T), &ce, &ne)) {
        std::fprintf(stderr, "error: edit encoding failed: %s\n", pmsz_last_error());
        return 1;
    }
    if (!write_file("_edits.bin", ce, ne) || !write_file("_deltas.bin", cd, nd)) {
        std::fprintf(stderr, "error: cannot write _edits.bin / _deltas.bin\n");
        return 1;
    }
    std::cout << "compressed deltas: " << nd << ", " << ne << ", 0" << std::endl;
    pmsz_free(cd);
    pmsz_free(ce);
    const double overhead = static_cast<double>(nd + ne);
    if (!a.out.empty() && !write_file(a.out, reinterpret_cast<const uint8_t *>(corrected.data()), n * sizeof(T))) {
        std::fprintf(stderr, "error: cannot write %s\n", a.out.c_str());
        return 1;
    }
    struct stat sb;
    const double orig = ::stat(a.path.c_str(), &sb) == 0 ? static_cast<double>(sb.st_size) : static_cast<double>(n * sizeof(T));
    const double cr = orig / a.cmp_size;  // inf without --cmp-size, as the reference prints (its cmpSize stays 0)
    const double ocr = orig / (a.cmp_size + overhead);
    const double ratio = static_cast<double>(outs.edit_count) / static_cast<double>(n);
    std::cout << "total storage overhead is: " << static_cast<unsigned long long>(overhead) << std::endl;
    std::cout << "original CR is: " << cr << std::endl;
    std::cout << "overall CR is: " << ocr << std::endl;
    std::cout << "overall edit ratio is: " << ratio << " total_edited:" << outs.edit_count << std::endl;
    if (a.verify)
        std::cout << "verify: dir_mismatch " << vr.dir_mismatch << " ext_mismatch " << vr.ext_mismatch << " as_mismatch "
                  << vr.as_mismatch << " ds_mismatch " << vr.ds_mismatch << " bound_strict " << vr.bound_strict
                  << " bound_beyond_clamp " << vr.bound_beyond_clamp << std::endl;

    {   // per-rank timing file, pMSz.cu:2925-2943 (one outer iteration at one rank)
        std::ofstream tf("Global_performance_with_ite_cuda_" + a.comp + "_" + name + "_rank_0_0.txt", std::ios::app);
        if (tf) {
            tf << "iteStep: 0" << std::endl;
            tf << "version 2 iteration: 0: " << res.ms_total * 1e-3 << ", " << res.ms_total * 1e-3 << ", "
               << res.ms_total * 1e-3 << ", " << res.ms_total * 1e-3 << ", " << res.iteration << std::endl;
            tf << "\n" << std::endl;
        }
    }
    {   // stat file, pMSz.cu:3146-3178
        std::ofstream sf("./stat_result/Global_base_result_" + name + "_" + a.comp + "_Maxonly_final1_0.txt", std::ios::app);
        if (!sf) {
            std::cerr << "Unable to open file for writing." << std::endl;
        } else {
            sf << std::to_string(a.eb) << ":" << std::endl;
            sf << "iteration" << ":" << res.iteration << std::endl;
            sf << std::setprecision(10) << "absolute_error: " << a.eb << std::endl;
            sf << std::setprecision(10) << "OCR: " << ocr << std::endl;
            sf << "threshold: " << a.q << std::endl;
            sf << "iteStep: " << 0 << std::endl;
            sf << std::setprecision(10) << "CR: " << cr << std::endl;
            sf << std::setprecision(17) << "edit_ratio: " << ratio << std::endl;
            sf << std::setprecision(17) << "compression_time: " << 0.0 << std::endl;
            sf << std::setprecision(17) << "additional_time: " << res.ms_total * 1e-3 << std::endl;
            sf << std::setprecision(17) << "Edits Time: " << wall << std::endl;
            sf << std::setprecision(17) << "Storage_Overhead: " << static_cast<unsigned long long>(overhead) << std::endl;
            sf << std::setprecision(17) << "Lower Threshold: " << 0.0 << std::endl;
            sf << std::setprecision(17) << "Whole Time: " << wall << std::endl;
            sf << std::setprecision(17) << "Data Time: " << 0.0 << std::endl;
            sf << std::endl << "\n" << std::endl;
            std::cout << "Variables have been appended to output.txt" << std::endl;
        }
    }
    return st == PMSZ_OK ? 0 : 3;
}

bool read_bytes(const std::string &path, std::vector<uint8_t> &v) {
    std::ifstream in(path, std::ios::binary | std::ios::ate);
    if (!in) {
        std::fprintf(stderr, "error: cannot open %s\n", path.c_str());
        return false;
    }
    v.resize(static_cast<size_t>(in.tellg()));
    in.seekg(0);
    in.read(reinterpret_cast<char *>(v.data()), static_cast<std::streamsize>(v.size()));
    return static_cast<bool>(in);
}

// --reconstruct: decompressed field + _deltas.bin + _edits.bin -> corrected field.
template <typename T>
int run_reconstruct(const Args &a) {
    const size_t n = a.W * a.H * a.D;
    std::vector<T> prev;
    std::vector<uint8_t> blob_d, blob_e, deltas(n);
    if (!read_raw<T>(a.path, prev, n) || !read_bytes(a.deltas_file, blob_d) || !read_bytes(a.edits_file, blob_e))
        return 1;
    void *vals = nullptr;
    size_t nc = 0;
    if (pmsz_decode_deltas(blob_d.data(), blob_d.size(), n, a.q, deltas.data()) ||
        pmsz_decode_clamps(blob_e.data(), blob_e.size(), sizeof(T), &vals, &nc)) {
        std::fprintf(stderr, "error: cannot decode the edit files: %s\n", pmsz_last_error());
        return 1;
    }
    T *dprev = nullptr, *dclamp = nullptr;
    uint8_t *dd = nullptr;
    int st = PMSZ_ERR_CUDA;
    if (cudaMalloc(&dprev, n * sizeof(T)) == cudaSuccess && cudaMalloc(&dd, n) == cudaSuccess &&
        cudaMalloc(&dclamp, std::max<size_t>(nc, 1) * sizeof(T)) == cudaSuccess &&
        cudaMemcpy(dprev, prev.data(), n * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess &&
        cudaMemcpy(dd, deltas.data(), n, cudaMemcpyHostToDevice) == cudaSuccess &&
        (nc == 0 || cudaMemcpy(dclamp, vals, nc * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess)) {
        st = sizeof(T) == 4 ? pmsz_reconstruct_f32(reinterpret_cast<const float *>(dprev), dd, reinterpret_cast<const float *>(dclamp), nc, n, a.eb, a.q, reinterpret_cast<float *>(dprev), nullptr)
                            : pmsz_reconstruct_f64(reinterpret_cast<const double *>(dprev), dd, reinterpret_cast<const double *>(dclamp), nc, n, a.eb, a.q, reinterpret_cast<double *>(dprev), nullptr);
        if (st == PMSZ_OK && cudaMemcpy(prev.data(), dprev, n * sizeof(T), cudaMemcpyDeviceToHost) != cudaSuccess)
            st = PMSZ_ERR_CUDA;
    }
    pmsz_free(vals);
    cudaFree(dprev);
    cudaFree(dd);
    cudaFree(dclamp);
    if (st != PMSZ_OK) {
        std::fprintf(stderr, "error: reconstruction failed (%s): %s\n", pmsz_strerror(st), pmsz_last_error());
        return 1;
    }
    if (!write_file(a.out, reinterpret_cast<const uint8_t *>(prev.data()), n * sizeof(T))) {
        std::fprintf(stderr, "error: cannot write %s\n", a.out.c_str());
        return 1;
    }
    std::cout << "reconstructed " << n << " voxels (" << nc << " clamp values) into " << a.out << std::endl;
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    Args a;
    const int rc = parse(argc, argv, a);
    if (rc) return rc;
    if (a.recon) return a.f32 ? run_reconstruct<float>(a) : run_reconstruct<double>(a);
    return a.f32 ? run<float>(a) : run<double>(a);
}
