// common.cuh -- device helpers shared by the pMSz GB300 kernels.
//
// Stencil.  The reference scans the 14 neighbours of the Freudenthal-style
// triangulation in the order of `directions_host` (pMSz.cu:186-193) and breaks
// value ties by flat index (islarger_shared / isless_shared, pMSz.cu:610-620).
// Two valid voxels compare by flat index exactly as their (z, y, x) compare
// lexicographically, and a neighbour at offset (dx,dy,dz) of voxel i has index
// order given by (dz,dy,dx) alone.  So the 15 stencil points (centre included)
// are numbered here by the lexicographic rank of (dz, dy, dx); rank 7 is the
// centre and rank r and rank 14-r are opposite offsets.  Scanning candidates in
// rank order, "replace on >=" gives the reference's argmax and "replace on <"
// its argmin, with no index arithmetic at all.
//
// Keys.  Values are compared as order-preserving unsigned integers: the IEEE
// bit pattern with the sign bit flipped for non-negative values and all bits
// flipped for negative ones, -0.0 first folded onto +0.0.  For every non-NaN
// value, key order and equality are IEEE order and equality; NaN inputs are
// rejected by the first pass.  GB300 executes FP64 at a small fraction of its
// integer rate, so the stencil scan stays in the integer pipes for fp64 too.
//
// Direction codes.  One byte per voxel: low nibble = rank of the steepest
// ascent neighbour, high nibble = rank of the steepest descent neighbour, of
// the ORIGINAL field -- the information of the reference's 8-byte or_types
// entry (pMSz.cu:749-783) in one byte.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace pmsz {

constexpr int kSelf = 7;
constexpr uint32_t kAllValid = 0x7FFFu;

// (dx, dy, dz) of stencil rank r, r = 0..14.
__host__ __device__ constexpr int rank_dx(int r) {
    return r == 1 || r == 3 || r == 5 || r == 8 ? 1
         : r == 6 || r == 9 || r == 11 || r == 13 ? -1 : 0;
}
__host__ __device__ constexpr int rank_dy(int r) {
    return r == 0 || r == 1 || r == 4 || r == 5 ? -1
         : r == 9 || r == 10 || r == 13 || r == 14 ? 1 : 0;
}
__host__ __device__ constexpr int rank_dz(int r) { return r <= 3 ? -1 : r >= 11 ? 1 : 0; }

// Ranks whose neighbour falls off a domain face.
constexpr uint32_t kNegX = (1u << 6) | (1u << 9) | (1u << 11) | (1u << 13);
constexpr uint32_t kPosX = (1u << 1) | (1u << 3) | (1u << 5) | (1u << 8);
constexpr uint32_t kNegY = (1u << 0) | (1u << 1) | (1u << 4) | (1u << 5);
constexpr uint32_t kPosY = (1u << 9) | (1u << 10) | (1u << 13) | (1u << 14);
constexpr uint32_t kNegZ = 0xFu;
constexpr uint32_t kPosZ = 0xFu << 11;

__host__ __device__ __forceinline__ uint32_t valid_mask(int x, int y, int z, int nx, int ny, int nz) {
    uint32_t m = kAllValid;
    if (x == 0) m &= ~kNegX;
    if (x == nx - 1) m &= ~kPosX;
    if (y == 0) m &= ~kNegY;
    if (y == ny - 1) m &= ~kPosY;
    if (z == 0) m &= ~kNegZ;
    if (z == nz - 1) m &= ~kPosZ;
    return m;
}

// Order-preserving keys.
__device__ __forceinline__ uint64_t okey(double v) {
    uint64_t b = static_cast<uint64_t>(__double_as_longlong(v));
    b = (b == 0x8000000000000000ull) ? 0ull : b;
    const uint64_t m = static_cast<uint64_t>(static_cast<int64_t>(b) >> 63);
    return b ^ (m | 0x8000000000000000ull);
}
__device__ __forceinline__ uint32_t okey(float v) {
    uint32_t b = __float_as_uint(v);
    b = (b == 0x80000000u) ? 0u : b;
    const uint32_t m = static_cast<uint32_t>(static_cast<int32_t>(b) >> 31);
    return b ^ (m | 0x80000000u);
}

template <typename T> struct KeyOf;
template <> struct KeyOf<float> { using type = uint32_t; };
template <> struct KeyOf<double> { using type = uint64_t; };

// NaN, or (fp64 only) the reference's halo sentinel 1e30 (pMSz.cu:215), which
// the reference would silently treat as "no voxel" (pMSz.cu:673-679, 709).
__device__ __forceinline__ bool bad_value(double v) {
    const uint64_t b = static_cast<uint64_t>(__double_as_longlong(v));
    return (b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull ||
           b == static_cast<uint64_t>(__double_as_longlong(1e30));
}
__device__ __forceinline__ bool bad_value(float v) {
    return (__float_as_uint(v) & 0x7FFFFFFFu) > 0x7F800000u;
}

// Steepest ascent / descent ranks over the 15 stencil keys (rank order).
template <typename K>
__device__ __forceinline__ void arg_ext(const K (&k)[15], uint32_t valid, int &amax, int &amin) {
    K bmax = 0, bmin = ~K(0);
    amax = kSelf;
    amin = kSelf;
#pragma unroll
    for (int r = 0; r < 15; ++r) {
        if ((valid >> r) & 1u) {
            if (k[r] >= bmax) { bmax = k[r]; amax = r; }
            if (k[r] < bmin) { bmin = k[r]; amin = r; }
        }
    }
}

// Detection rules of iscriticle data_type=0 (pMSz.cu:786-898) on ranks.
//   asc/desc   : steepest ranks on the current field
//   oasc/odesc : steepest ranks of the original field (from the code byte)
// omax / omin follow the or_types encoding (pMSz.cu:749-783): a voxel that is
// both max and min in the original is stored as a max, so it is not an
// "original minimum".  Returns the bit set of requested ranks; adds to the
// three reference counters.
__device__ __forceinline__ uint32_t detect_rules(int asc, int desc, int oasc, int odesc,
                                                 uint32_t &cmax, uint32_t &cmin, uint32_t &cdir) {
    const bool omax = oasc == kSelf;
    const bool omin = !omax && odesc == kSelf;
    const bool is_max = asc == kSelf, is_min = desc == kSelf;
    const bool r1 = is_max != omax, r2 = is_min != omin;
    uint32_t tm = 0;
    if (r1) { ++cmax; tm |= 1u << (omax ? asc : kSelf); }          // pMSz.cu:790-812
    if (r2) { ++cmin; tm |= 1u << (omin ? kSelf : odesc); }        // pMSz.cu:814-836
    if (r1 || r2) { ++cdir; return tm; }                           // pMSz.cu:859-863
    if (asc != oasc) { ++cdir; tm |= 1u << asc; }                  // pMSz.cu:865-879
    if (desc != odesc) { ++cdir; tm |= 1u << odesc; }              // pMSz.cu:881-895
    return tm;
}

// Division by a run-time constant d >= 1 for 32-bit n, as a multiply and a
// shift (Granlund & Montgomery, "Division by invariant integers using
// multiplication", 1994): with s = ceil(log2 d) and
// m = floor(2^32 (2^s - d) / d) + 1, floor(n / d) = (mulhi(n, m) + n) >> s.
struct FastDiv {
    uint32_t d, m, s;
};
inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    uint32_t s = 0;
    while ((uint64_t(1) << s) < d) ++s;
    f.s = s;
    f.m = static_cast<uint32_t>(((uint64_t(1) << 32) * ((uint64_t(1) << s) - d)) / d + 1);
    return f;
}
__host__ __device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
#ifdef __CUDA_ARCH__
    const uint32_t t = __umulhi(n, f.m);
#else
    const uint32_t t = static_cast<uint32_t>((static_cast<uint64_t>(n) * f.m) >> 32);
#endif
    return static_cast<uint32_t>((static_cast<uint64_t>(t) + n) >> f.s);
}

// Blocks of the bitmap-compaction kernels (one contiguous word range each).
constexpr int kCompactBlocks = 152 * 8;

// Field geometry.  Bitmaps hold one bit per voxel with every x-row padded to
// whole 32-bit words: word (wx, y, z) = wx + wpr*(y + ny*z), bit b = x - 32*wx.
struct Geom {
    int nx, ny, nz;
    int wpr;          // words per x-row
    size_t nwords;    // wpr * ny * nz (< 2^32)
    size_t n;         // nx * ny * nz
    FastDiv div_wpr, div_ny, div_nx;  // div_nx: for flat indices below 2^32
    int zc;           // planes per tile column of the tiled passes (tile 32 x 8 x zc)
};

constexpr int kZChunkDefault = 32;  // zc when no tuned value is recorded for the shape

inline Geom make_geom(size_t nx, size_t ny, size_t nz) {
    Geom g;
    g.nx = static_cast<int>(nx);
    g.ny = static_cast<int>(ny);
    g.nz = static_cast<int>(nz);
    g.wpr = static_cast<int>((nx + 31) / 32);
    g.nwords = static_cast<size_t>(g.wpr) * ny * nz;
    g.n = nx * ny * nz;
    g.div_wpr = make_fastdiv(static_cast<uint32_t>(g.wpr));
    g.div_ny = make_fastdiv(static_cast<uint32_t>(ny));
    g.div_nx = make_fastdiv(static_cast<uint32_t>(nx));
    g.zc = kZChunkDefault;
    return g;
}

// (wx, y, z) of bitmap word w.
__host__ __device__ __forceinline__ void word_coords(const Geom &g, size_t w, int &wx, int &y, int &z) {
    const uint32_t w32 = static_cast<uint32_t>(w);
    const uint32_t row = fdiv(w32, g.div_wpr);
    wx = static_cast<int>(w32 - row * static_cast<uint32_t>(g.wpr));
    const uint32_t zz = fdiv(row, g.div_ny);
    y = static_cast<int>(row - zz * static_cast<uint32_t>(g.ny));
    z = static_cast<int>(zz);
}

__host__ __device__ __forceinline__ size_t flat(const Geom &g, int x, int y, int z) {
    return static_cast<size_t>(x) + static_cast<size_t>(g.nx) * (static_cast<size_t>(y) + static_cast<size_t>(g.ny) * z);
}
__host__ __device__ __forceinline__ size_t word_of(const Geom &g, int x, int y, int z) {
    return static_cast<size_t>(x >> 5) + static_cast<size_t>(g.wpr) * (static_cast<size_t>(y) + static_cast<size_t>(g.ny) * z);
}
// Bits of the last word of a row that lie inside the domain.
__host__ __device__ __forceinline__ uint32_t row_tail_mask(const Geom &g, int wx) {
    const int rem = g.nx - 32 * wx;
    return rem >= 32 ? 0xFFFFFFFFu : ((1u << rem) - 1u);
}

// A code byte not yet decided (ranks are 0..14, so no code has a nibble 15).
constexpr uint8_t kCodeUnset = 0xFF;

// Appends v to a global list with one atomic on the list's counter per group
// of lanes that reach the call together (each lane's slot is the group's base
// plus its rank among them).  Used where a full per-block buffer spills:
// lanes spilling one by one would serialise on that counter.
__device__ __forceinline__ void spill_append(uint32_t *__restrict__ list, uint32_t *count, uint32_t v) {
    const uint32_t mask = __activemask();
    uint32_t lane;
    asm("mov.u32 %0, %%laneid;" : "=r"(lane));
    const uint32_t leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, static_cast<uint32_t>(__popc(mask)));
    base = __shfl_sync(mask, base, leader);
    list[base + __popc(mask & ((1u << lane) - 1u))] = v;
}

// Per-sweep device counters (one slot per sweep).  fmax/fmin/fdir are the
// reference's count_f_max / count_f_min / count_f_dir (pMSz.cu:174), counted
// exactly rather than with the reference's racy `+=`.
struct SweepSlot {
    unsigned long long fmax, fmin, fdir;
    unsigned long long requested;   // distinct vertices edited this sweep
    unsigned long long changed;     // of those, vertices whose value changed
    unsigned long long progressed;  // of those, vertices whose value or counter changed
    unsigned long long active;      // voxels examined by the detection pass
    unsigned long long bad;         // NaN / sentinel inputs seen (first pass only)
};

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}
__device__ __forceinline__ uint32_t warp_sum_u32(uint32_t v) {
    return __reduce_add_sync(0xFFFFFFFFu, v);
}

}  // namespace pmsz
