// gen.cu -- synthetic inputs on the device: Perlin fBm fields and the two
// labelled compressor stand-ins.  Not part of the reference's correction path
// (its generator is generate_perlin.py); these kernels produce the same bits
// as pmsz_anonymous_gb300/fields.py so that large benchmark fields need no
// host-side generation.  Compiled with -fmad=false: every double operation is
// rounded separately, as numpy rounds it.
#include "common.cuh"
#include "internal.h"

#include <algorithm>
#include <cstring>

namespace pmsz {

constexpr int kMaxOctaves = 16;

struct PerlinParams {
    int32_t perm[512];
    double amp[kMaxOctaves];
    double freq[kMaxOctaves];
    int octaves;
};

// Improved Perlin noise, generate_perlin.py:17-59.
__device__ __forceinline__ double fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }
__device__ __forceinline__ double lerp(double a, double b, double t) { return a + t * (b - a); }
__device__ __forceinline__ double grad(int h, double x, double y, double z) {
    h &= 15;
    const double u = h < 8 ? x : y;
    const double v = h < 4 ? y : (h == 12 || h == 14 ? x : z);
    return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? v : -v);
}
__device__ double perlin(double x, double y, double z, const int32_t *p) {
    const double fx = floor(x), fy = floor(y), fz = floor(z);
    const int X = static_cast<int>(static_cast<long long>(fx) & 255);
    const int Y = static_cast<int>(static_cast<long long>(fy) & 255);
    const int Z = static_cast<int>(static_cast<long long>(fz) & 255);
    x = x - fx;
    y = y - fy;
    z = z - fz;
    const double u = fade(x), v = fade(y), w = fade(z);
    const int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z;
    const int B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
    return lerp(lerp(lerp(grad(p[AA], x, y, z), grad(p[BA], x - 1.0, y, z), u),
                     lerp(grad(p[AB], x, y - 1.0, z), grad(p[BB], x - 1.0, y - 1.0, z), u), v),
                lerp(lerp(grad(p[AA + 1], x, y, z - 1.0), grad(p[BA + 1], x - 1.0, y, z - 1.0), u),
                     lerp(grad(p[AB + 1], x, y - 1.0, z - 1.0), grad(p[BB + 1], x - 1.0, y - 1.0, z - 1.0), u), v),
                w);
}

__device__ __forceinline__ double fbm(const PerlinParams &P, const int32_t *perm, int x, int y, int z) {
    double total = 0.0;
    for (int o = 0; o < P.octaves; ++o) {
        const double fr = P.freq[o];
        total = total + P.amp[o] * perlin(static_cast<double>(x) * fr, static_cast<double>(y) * fr,
                                          static_cast<double>(z) * fr, perm);
    }
    return total;
}

// Pass 1: min / max of the raw fBm as order-preserving keys.
__global__ void __launch_bounds__(256) k_fbm_range(const PerlinParams P, Geom g, unsigned long long *mnmx) {
    __shared__ int32_t perm[512];
    for (int i = threadIdx.x; i < 512; i += blockDim.x) perm[i] = P.perm[i];
    __syncthreads();
    unsigned long long mn = ~0ull, mx = 0ull;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < g.n; i += stride) {
        const size_t row = i / g.nx;
        const int x = static_cast<int>(i - row * g.nx), y = static_cast<int>(row % g.ny), z = static_cast<int>(row / g.ny);
        const unsigned long long k = okey(fbm(P, perm, x, y, z));
        mn = k < mn ? k : mn;
        mx = k > mx ? k : mx;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xFFFFFFFFu, mn, o), b = __shfl_xor_sync(0xFFFFFFFFu, mx, o);
        mn = a < mn ? a : mn;
        mx = b > mx ? b : mx;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(mnmx, mn);
        atomicMax(mnmx + 1, mx);
    }
}

__device__ __forceinline__ double from_key(unsigned long long k) {
    const uint64_t b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    return __longlong_as_double(static_cast<long long>(b));
}

// Pass 2: recompute and normalise, (v - mn) / (mx - mn), cast to T.
template <typename T>
__global__ void __launch_bounds__(256) k_fbm_norm(const PerlinParams P, Geom g, const unsigned long long *mnmx, T *out) {
    __shared__ int32_t perm[512];
    for (int i = threadIdx.x; i < 512; i += blockDim.x) perm[i] = P.perm[i];
    __syncthreads();
    const double mn = from_key(mnmx[0]), mx = from_key(mnmx[1]);
    const double range = mx - mn;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < g.n; i += stride) {
        const size_t row = i / g.nx;
        const int x = static_cast<int>(i - row * g.nx), y = static_cast<int>(row % g.ny), z = static_cast<int>(row / g.ny);
        out[i] = static_cast<T>((fbm(P, perm, x, y, z) - mn) / range);
    }
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// kind 0: SZ-like plateaus, fhat = (2 eb) * rint(f / (2 eb)) (numpy rounds
// half to even, as rint does); kind 1: ZFP-like noise f + eb * u.  Any voxel
// with |f - fhat| > eps in T falls back to f.
template <typename T>
__global__ void __launch_bounds__(256) k_standin(const T *__restrict__ f, T *__restrict__ fh, size_t n, double eb,
                                                 int kind, uint64_t seed) {
    const T eps = static_cast<T>(eb);
    const double step = 2.0 * eb;
    const uint64_t salt = (seed & 0xFFFFFFFFull) << 40;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T fv = f[i];
        T v;
        if (kind == 0) {
            v = static_cast<T>(step * rint(static_cast<double>(fv) / step));
        } else {
            const uint64_t h = splitmix64(static_cast<uint64_t>(i) ^ salt);
            const double u = static_cast<double>(h >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
            v = static_cast<T>(static_cast<double>(fv) + eb * u);
        }
        if (!(fabs(fv - v) <= eps)) v = fv;
        fh[i] = v;
    }
}

template <typename T>
int perlin_impl(T *out, size_t nx, size_t ny, size_t nz, const int32_t *perm, const double *amps,
                const double *freqs, int octaves, cudaStream_t s) {
    if (!out || !perm || !amps || !freqs) return set_error(PMSZ_ERR_ARG, "null pointer");
    if (octaves < 1 || octaves > kMaxOctaves) return set_error(PMSZ_ERR_ARG, "octaves must be in 1..16");
    int rc = check_geom(nx, ny, nz);
    if (rc) return rc;
    PerlinParams P;
    std::memcpy(P.perm, perm, sizeof(P.perm));
    for (int o = 0; o < kMaxOctaves; ++o) {
        P.amp[o] = o < octaves ? amps[o] : 0.0;
        P.freq[o] = o < octaves ? freqs[o] : 0.0;
    }
    P.octaves = octaves;
    for (int i = 0; i < 512; ++i)
        if (P.perm[i] < 0 || P.perm[i] > 255) return set_error(PMSZ_ERR_ARG, "permutation entries must be 0..255");
    const Geom g = make_geom(nx, ny, nz);
    Workspace ws(s);
    const size_t o_mm = ws.reserve<unsigned long long>(2);
    if ((rc = ws.commit())) return rc;
    unsigned long long *mm = ws.at<unsigned long long>(o_mm);
    const unsigned long long init[2] = {~0ull, 0ull};
    PMSZ_CUDA(cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, s));
    const unsigned grid = static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>((g.n + 255) / 256, 152 * 8)));
    k_fbm_range<<<grid, 256, 0, s>>>(P, g, mm);
    k_fbm_norm<T><<<grid, 256, 0, s>>>(P, g, mm, out);
    PMSZ_CUDA(cudaGetLastError());
    PMSZ_CUDA(cudaStreamSynchronize(s));  // `init` lives on this stack frame
    return ws.release();
}

template <typename T>
int standin_impl(const T *f, T *fh, size_t n, double eb, int kind, uint64_t seed, cudaStream_t s) {
    if (!f || !fh) return set_error(PMSZ_ERR_ARG, "null pointer");
    if (kind != 0 && kind != 1) return set_error(PMSZ_ERR_ARG, "stand-in kind must be 0 (sz3) or 1 (zfp)");
    if (!(eb > 0.0)) return set_error(PMSZ_ERR_ARG, "error bound must be positive");
    if (n == 0) return PMSZ_OK;
    const unsigned grid = static_cast<unsigned>(std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 152 * 16)));
    k_standin<T><<<grid, 256, 0, s>>>(f, fh, n, eb, kind, seed);
    PMSZ_CUDA(cudaGetLastError());
    return PMSZ_OK;
}

}  // namespace pmsz

using namespace pmsz;

extern "C" int pmsz_gen_perlin_f32(float *out, size_t nx, size_t ny, size_t nz, const int32_t *perm512,
                                   const double *amps, const double *freqs, int octaves, void *stream) {
    return guarded([&] { return perlin_impl<float>(out, nx, ny, nz, perm512, amps, freqs, octaves, as_stream(stream)); });
}
extern "C" int pmsz_gen_perlin_f64(double *out, size_t nx, size_t ny, size_t nz, const int32_t *perm512,
                                   const double *amps, const double *freqs, int octaves, void *stream) {
    return guarded([&] { return perlin_impl<double>(out, nx, ny, nz, perm512, amps, freqs, octaves, as_stream(stream)); });
}
extern "C" int pmsz_standin_f32(const float *f, float *fhat, size_t n, double eb, int kind, uint64_t seed, void *stream) {
    return guarded([&] { return standin_impl<float>(f, fhat, n, eb, kind, seed, as_stream(stream)); });
}
extern "C" int pmsz_standin_f64(const double *f, double *fhat, size_t n, double eb, int kind, uint64_t seed,
                                void *stream) {
    return guarded([&] { return standin_impl<double>(f, fhat, n, eb, kind, seed, as_stream(stream)); });
}
