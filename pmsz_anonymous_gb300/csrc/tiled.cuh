// tiled.cuh -- proxy-based sweep kernels, included by correct.cu after its
// shared device helpers.
//
// GB300 executes integer compare / min / max (and FP32 min / max) on one
// 64-lane-per-clock pipe per SM, so a 15-point argmax / argmin on 64-bit keys
// (about five instructions per candidate) is what bounds the sweep, not HBM.
// These kernels compare 32-bit PROXIES instead:
//
//   proxy(v) = high 32 bits of the order-preserving key, low 4 bits cleared
//
// so that `proxy + rank` packs a candidate's stencil rank into the free bits
// and a whole argmax is one min/max instruction per candidate.  Truncation
// can only merge keys, never reorder them (key_a < key_b => proxy_a <=
// proxy_b), so the packed chain is exact whenever the winning proxy is
// unique.  A second chain with the ranks reversed (15 - r) picks the LOWEST
// rank among tied proxies; both chains agree exactly when the winner is
// unique -- the exactness certificate.  Where they disagree (ties in the
// truncated proxy) the voxel takes the exact path on full keys.
//
// Out-of-domain stencil cells hold proxy 0: as `0 + r` they lose every max
// chain (real proxies are >= 16), and the min chains add -16 (or -1) so that
// they wrap to the top of the range and lose every min chain; no per-lane
// boundary branch is needed on the fast path.
#pragma once
#include <cooperative_groups.h>
#include <cuda.h>  // CUtensorMap (the map itself is encoded on the host)

#include "helpers.cuh"

namespace cg = cooperative_groups;

namespace pmsz {

__device__ __forceinline__ uint32_t proxy_of_key(uint64_t k) { return static_cast<uint32_t>(k >> 32) & ~15u; }
__device__ __forceinline__ uint32_t proxy_of_key(uint32_t k) { return k & ~15u; }
template <typename T>
__device__ __forceinline__ uint32_t proxy_of(T v) { return proxy_of_key(okey(v)); }

struct Ext {
    int asc, desc;
    bool exact;
};

// Packed argmax / argmin of 15 proxies in rank order, with certificates.
// General form: out-of-domain candidates carry proxy 0; the min chains add
// -16 (and -1) so those wrap to the top of the range and lose.
// FUSED: each chain step is one fused add-and-max / add-and-min
// (__viaddmax_u32 / __viaddmin_u32: max(a + b, c), min(a + b, c), 32-bit
// wrapping add) -- fewer instructions, for the latency-bound gather kernels;
// the tiled passes, bound by the ALU pipe, keep separate adds and min/max.
template <bool FUSED = false>
__device__ __forceinline__ Ext proxy_ext(const uint32_t (&t)[15]) {
    uint32_t M = t[0], M2 = t[0] + 15u, m = t[0] - 16u, m2 = t[0] - 1u;
#pragma unroll
    for (int r = 1; r < 15; ++r) {
        const uint32_t ra = static_cast<uint32_t>(r), rb = static_cast<uint32_t>(15 - r);
        const uint32_t rc = static_cast<uint32_t>(r) - 16u, rd = 0u - 1u - static_cast<uint32_t>(r);
        if (FUSED) {
            M = __viaddmax_u32(t[r], ra, M);
            M2 = __viaddmax_u32(t[r], rb, M2);
            m = __viaddmin_u32(t[r], rc, m);
            m2 = __viaddmin_u32(t[r], rd, m2);
        } else {
            M = max(M, t[r] + ra);
            M2 = max(M2, t[r] + rb);
            m = min(m, t[r] + rc);
            m2 = min(m2, t[r] + rd);
        }
    }
    Ext e;
    e.asc = static_cast<int>(M & 15u);
    e.desc = static_cast<int>(m & 15u);
    e.exact = e.asc == 15 - static_cast<int>(M2 & 15u) && e.desc == 15 - static_cast<int>(m2 & 15u);
    return e;
}

// Interior form (all 15 candidates inside the domain): the max and min chains
// share the packed values t + r and t + (15 - r), half the adds.
template <bool FUSED = false>
__device__ __forceinline__ Ext proxy_ext_interior(const uint32_t (&t)[15]) {
    uint32_t M = t[0], m = t[0], M2 = t[0] + 15u, m2 = M2;
#pragma unroll
    for (int r = 1; r < 15; ++r) {
        if (FUSED) {
            M = __viaddmax_u32(t[r], static_cast<uint32_t>(r), M);
            m = __viaddmin_u32(t[r], static_cast<uint32_t>(r), m);
            M2 = __viaddmax_u32(t[r], static_cast<uint32_t>(15 - r), M2);
            m2 = __viaddmin_u32(t[r], static_cast<uint32_t>(15 - r), m2);
        } else {
            const uint32_t a = t[r] + static_cast<uint32_t>(r), b = t[r] + static_cast<uint32_t>(15 - r);
            M = max(M, a);
            m = min(m, a);
            M2 = max(M2, b);
            m2 = min(m2, b);
        }
    }
    Ext e;
    e.asc = static_cast<int>(M & 15u);
    e.desc = static_cast<int>(m & 15u);
    e.exact = e.asc == 15 - static_cast<int>(M2 & 15u) && e.desc == 15 - static_cast<int>(m2 & 15u);
    return e;
}

constexpr int kTX = 32, kTY = 8, kHX = kTX + 2, kHY = kTY + 2;
// Planes in the shared-memory ring: 4, one plane computed per barrier; the
// proxy-only tile of the deferring fp32 first pass keeps 8 and computes two
// planes per barrier (fp64 at two planes spills at its 40-register budget and
// measured slower).
template <typename T, bool KEYS>
constexpr int kRingOf = (KEYS || sizeof(T) == 8) ? 4 : 8;
constexpr int kCells = kHX * kHY, kThreads = kTX * kTY;
enum TileMode { kFirst = 0, kDetect = 1, kCodes = 2 };

constexpr uint32_t kFirstXCap = 512;  // deferred voxels buffered per block

// KEYS: full keys beside the proxies for an inline exact path; without them
// (the deferring first pass) a buffer of voxels whose certificate failed.
template <typename T, int NF, bool KEYS>
struct TileSmem;
template <typename T, int NF>
struct TileSmem<T, NF, true> {
    uint32_t p[NF][kRingOf<T, true>][kHY][kHX];                  // proxies
    typename KeyOf<T>::type k[NF][kRingOf<T, true>][kHY][kHX];   // full keys, for the rare exact path
};
template <typename T, int NF>
struct TileSmem<T, NF, false> {
    uint32_t p[NF][kRingOf<T, false>][kHY][kHX];  // proxies
    uint32_t x[kFirstXCap];           // voxels whose certificate failed
    uint32_t xn, xbase;
};

// The tile of a pass: proxies, plus full keys unless the pass defers failed
// certificates.
template <typename T, int MODE, bool DEFER>
using TileOf = TileSmem<T, MODE == kFirst ? 2 : 1, !DEFER>;

__host__ __device__ constexpr int tile_slot_sel(int r) { return rank_dz(r) + 1; }

// ---------------------------------------------------------------------------
// Tiled full-field pass.  Block (32, 8) owns a 32x8 column of the field and
// marches it through g.zc planes; planes (with a one-voxel halo) stream
// through a ring in shared memory (4 slots, one plane computed per barrier;
// 8 slots and two planes per barrier for the proxy-only deferring fp32 pass),
// prefetched ahead of the planes being computed.  Each thread loads the same (at most two) cells of every
// plane, so their coordinates are decoded once per block.
//   kFirst : fa = f, fb = fhat.  Labels f (code byte), writes the proxy array
//            of fhat, and runs the first detection (iscriticle data_type=1
//            fused with the first data_type=0 pass).
//   kDetect: fa = fhat; the original codes come from `codes` (full sweep).
//   kCodes : fa = a field; writes its code byte only (pmsz_codes_*).
// ---------------------------------------------------------------------------
//   DEFER (kFirst only, fields of fewer than 2^32 voxels): a voxel whose
//            certificate fails in either field is not decided here but
//            appended to xlist (k_first_exact decides it on full keys), so no
//            warp runs a one-lane exact path inside the plane loop and no
//            full keys are staged.
//   INT      the block's tile, its halo and the planes zb-1 .. ze lie inside
//            the domain: no bound checks, every voxel has its 15 cells.
template <typename T, int MODE, bool DEFER = false, bool INT = false>
__device__ __forceinline__ void tiled_body(TileOf<T, MODE, DEFER> &sm, const T *__restrict__ fa,
                                           const T *__restrict__ fb, uint8_t *__restrict__ codes,
                                           uint32_t *__restrict__ hp, uint32_t *__restrict__ req,
                                           uint32_t *__restrict__ act_next, SweepSlot *slot, const Geom &g, int bx,
                                           int by, int bz, uint32_t *__restrict__ xlist = nullptr,
                                           uint32_t *xcount = nullptr) {
    static_assert(!DEFER || MODE == kFirst, "only the first pass defers");
    constexpr int NF = MODE == kFirst ? 2 : 1;
    constexpr int kRing = kRingOf<T, !DEFER>;
    constexpr int kPer = kRing / 4;  // planes computed per barrier
    using K = typename KeyOf<T>::type;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTX + tx;
    const int x0 = bx * kTX, y0 = by * kTY;
    const int zb = bz * g.zc, ze = min(g.nz, zb + g.zc);
    const int x = x0 + tx, y = y0 + ty;
    const size_t plane = static_cast<size_t>(g.nx) * g.ny;

    // this thread's load cells (tid and tid + 256 of the 34 x 10 halo plane)
    int cell_s[2];
    size_t cell_g[2];
    bool cell_in[2], cell_own[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int c = tid + j * kThreads;
        const int cy = c / kHX, cx = c - cy * kHX;
        const int gx = x0 - 1 + cx, gy = y0 - 1 + cy;
        cell_s[j] = c;
        cell_in[j] = c < kCells && (INT || (gx >= 0 && gx < g.nx && gy >= 0 && gy < g.ny));
        cell_own[j] = cell_in[j] && cx >= 1 && cx <= kTX && cy >= 1 && cy <= kTY;
        cell_g[j] = cell_in[j] ? static_cast<size_t>(gx) + static_cast<size_t>(gy) * g.nx : 0;
    }
    uint32_t bad = 0;

    // A plane's cells are fetched into registers (fetch_plane) and later
    // converted to proxies and stored in the ring (stash_plane).  fp64 passes
    // fetch the planes they prefetch before their compute and stash them
    // after, so the global loads' latency overlaps the compute (the deferring
    // fp64 pass runs five blocks per SM to hold them without spills: 1.98
    // against 2.08 ms at 512^3); fp32 passes stash at once (measured faster).
    auto fetch_plane = [&](int zz, T (&v)[2][NF]) {
        const bool zin = INT || (zz >= 0 && zz < g.nz);
        const size_t zoff = zin ? static_cast<size_t>(zz) * plane : 0;
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int F = 0; F < NF; ++F)
                v[j][F] = (cell_s[j] < kCells && cell_in[j] && zin) ? (F == 0 ? fa : fb)[zoff + cell_g[j]] : T(0);
    };
    auto stash_plane = [&](int zz, const T (&v)[2][NF]) {
        const int s = zz & (kRing - 1);
        const bool zin = INT || (zz >= 0 && zz < g.nz);
        const bool zown = zz >= zb && zz < ze;
        const size_t zoff = zin ? static_cast<size_t>(zz) * plane : 0;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (cell_s[j] >= kCells) continue;
            const bool in = cell_in[j] && zin;
#pragma unroll
            for (int F = 0; F < NF; ++F) {
                K key = 0;
                uint32_t px = 0;
                if (in) {
                    key = okey(v[j][F]);
                    px = proxy_of_key(key);
                    if (MODE == kFirst && cell_own[j] && zown) {
                        bad |= bad_value(v[j][F]) ? 1u : 0u;
                        if (F == 1) hp[zoff + cell_g[j]] = px;
                    }
                }
                (&sm.p[F][s][0][0])[cell_s[j]] = px;
                if constexpr (!DEFER) (&sm.k[F][s][0][0])[cell_s[j]] = key;
                (void)key;
            }
        }
    };
    auto load_plane = [&](int zz) {
        T v[2][NF];
        fetch_plane(zz, v);
        stash_plane(zz, v);
    };

    auto ext = [&](int F, int z, const int (&slots)[3], bool interior) -> Ext {
        uint32_t t[15];
#pragma unroll
        for (int r = 0; r < 15; ++r) t[r] = sm.p[F][slots[tile_slot_sel(r)]][ty + 1 + rank_dy(r)][tx + 1 + rank_dx(r)];
        Ext e = interior ? proxy_ext_interior(t) : proxy_ext(t);
        if constexpr (!DEFER) {
            if (!e.exact) {  // ties in the truncated proxies: exact keys
                K k[15];
#pragma unroll
                for (int r = 0; r < 15; ++r)
                    k[r] = sm.k[F][slots[tile_slot_sel(r)]][ty + 1 + rank_dy(r)][tx + 1 + rank_dx(r)];
                arg_ext(k, valid_mask(x, y, z, g.nx, g.ny, g.nz), e.asc, e.desc);
                e.exact = true;
            }
        }
        return e;
    };
    if constexpr (DEFER) {
        if (threadIdx.x == 0 && threadIdx.y == 0) sm.xn = 0;  // made visible by the prologue barrier
    }

    // planes zb-1 .. zb+kPer (those up to ze) before the loop; each iteration
    // prefetches the kPer planes after the ones it reads, into ring slots last
    // read kPer iterations earlier (a barrier ends every iteration)
#pragma unroll
    for (int zz = zb - 1; zz <= zb + kPer; ++zz)
        if (zz <= ze) load_plane(zz);
    __syncthreads();
    uint32_t cmax = 0, cmin = 0, cdir = 0, active = 0;
    const bool in = INT || (x < g.nx && y < g.ny);
    const bool xy_interior = INT || (x0 >= 1 && x0 + kTX <= g.nx - 1 && y >= 1 && y <= g.ny - 2);  // warp-uniform
    constexpr bool kOverlap = sizeof(T) == 8;
    for (int z0 = zb; z0 < ze; z0 += kPer) {
        T pend[kPer][2][NF];  // the planes this iteration prefetches, stashed after its compute
#pragma unroll
        for (int p = 1; p <= kPer; ++p) {
            if (z0 + kPer + p > ze) continue;
            if (kOverlap) fetch_plane(z0 + kPer + p, pend[p - 1]);
            else load_plane(z0 + kPer + p);
        }
#pragma unroll 1
        for (int z = z0; z < min(z0 + kPer, ze); ++z) {
            const int slots[3] = {(z + kRing - 1) & (kRing - 1), z & (kRing - 1), (z + 1) & (kRing - 1)};
            const bool interior = INT || (xy_interior && z >= 1 && z <= g.nz - 2);
            uint32_t tm = 0;
            if (in) {
                const size_t i = flat(g, x, y, z);
                if (MODE == kCodes) {
                    const Ext e = ext(0, z, slots, interior);
                    codes[i] = static_cast<uint8_t>(e.asc | (e.desc << 4));
                } else {
                    int oasc, odesc;
                    Ext e;
                    bool decided = true;
                    if constexpr (MODE == kFirst && DEFER && INT) {
                        // Interior voxels of the deferring first pass: the four
                        // chains of f, then of fhat (15 proxies live at a time);
                        // a chain pair certifies its winner when the two ranks
                        // sum to 15, so one test covers all four certificates;
                        // the rules run only where the two codes differ (equal
                        // codes fire no rule unless the voxel is both maximum
                        // and minimum of f, code 0x77).
                        uint32_t M0, m0, N0, n0, M1, m1, N1, n1;
                        {
                            uint32_t ta[15];
#pragma unroll
                            for (int r = 0; r < 15; ++r)
                                ta[r] = sm.p[0][slots[tile_slot_sel(r)]][ty + 1 + rank_dy(r)][tx + 1 + rank_dx(r)];
                            M0 = ta[0]; m0 = ta[0]; N0 = ta[0] + 15u; n0 = N0;
#pragma unroll
                            for (int r = 1; r < 15; ++r) {
                                const uint32_t a = ta[r] + static_cast<uint32_t>(r), b = ta[r] + static_cast<uint32_t>(15 - r);
                                M0 = max(M0, a); m0 = min(m0, a); N0 = max(N0, b); n0 = min(n0, b);
                            }
                        }
                        {
                            uint32_t tb[15];
#pragma unroll
                            for (int r = 0; r < 15; ++r)
                                tb[r] = sm.p[1][slots[tile_slot_sel(r)]][ty + 1 + rank_dy(r)][tx + 1 + rank_dx(r)];
                            M1 = tb[0]; m1 = tb[0]; N1 = tb[0] + 15u; n1 = N1;
#pragma unroll
                            for (int r = 1; r < 15; ++r) {
                                const uint32_t a = tb[r] + static_cast<uint32_t>(r), b = tb[r] + static_cast<uint32_t>(15 - r);
                                M1 = max(M1, a); m1 = min(m1, a); N1 = max(N1, b); n1 = min(n1, b);
                            }
                        }
                        const uint32_t s0 = (M0 + N0) & (m0 + n0);
                        const uint32_t c0 = (M0 & 15u) | ((m0 & 15u) << 4), c1 = (M1 & 15u) | ((m1 & 15u) << 4);
                        decided = false;
                        if ((s0 & (M1 + N1) & (m1 + n1) & 15u) != 15u) {
                            codes[i] = (s0 & 15u) == 15u ? static_cast<uint8_t>(c0) : kCodeUnset;
                            const uint32_t pos = atomicAdd(&sm.xn, 1u);
                            if (pos < kFirstXCap) sm.x[pos] = static_cast<uint32_t>(i);
                            else spill_append(xlist, xcount, static_cast<uint32_t>(i));
                        } else {
                            codes[i] = static_cast<uint8_t>(c0);
                            if (c1 != c0 || c0 == 0x77u) {
                                tm = detect_rules(static_cast<int>(c1 & 15u), static_cast<int>(c1 >> 4),
                                                  static_cast<int>(c0 & 15u), static_cast<int>(c0 >> 4), cmax, cmin,
                                                  cdir);
                                if (tm) request_targets(req, g, x, y, z, tm);
                            }
                        }
                    } else if (MODE == kFirst) {
                        const Ext o = ext(0, z, slots, interior);
                        oasc = o.asc;
                        odesc = o.desc;
                        e = ext(1, z, slots, interior);
                        if (DEFER && !(o.exact && e.exact)) {
                            decided = false;
                            // the original's code when its certificate held (only
                            // fhat's failed, as on plateaus), else the unset mark
                            codes[i] = o.exact ? static_cast<uint8_t>(oasc | (odesc << 4)) : kCodeUnset;
                            if constexpr (DEFER) {
                                const uint32_t pos = atomicAdd(&sm.xn, 1u);
                                if (pos < kFirstXCap) sm.x[pos] = static_cast<uint32_t>(i);
                                else spill_append(xlist, xcount, static_cast<uint32_t>(i));
                            }
                        } else {
                            codes[i] = static_cast<uint8_t>(oasc | (odesc << 4));
                        }
                    } else {
                        const uint8_t c = codes[i];
                        oasc = c & 15;
                        odesc = c >> 4;
                        e = ext(0, z, slots, interior);
                    }
                    if (decided) {
                        tm = detect_rules(e.asc, e.desc, oasc, odesc, cmax, cmin, cdir);
                        if (tm) request_targets(req, g, x, y, z, tm);
                    }
                    ++active;
                }
            }
            if (MODE != kCodes) {
                const uint32_t mism = __ballot_sync(0xFFFFFFFFu, tm != 0);
                if (tx == 0 && (INT || y < g.ny) && mism) act_next[word_of(g, x0, y, z)] = mism;
            }
        }
        // their ring slots were last read kPer iterations ago (not by this one)
#pragma unroll
        for (int p = 1; p <= kPer; ++p)
            if (kOverlap && z0 + kPer + p <= ze) stash_plane(z0 + kPer + p, pend[p - 1]);
        __syncthreads();
    }
    if (MODE != kCodes) {
        const uint32_t v[8] = {cmax, cmin, cdir, 0u, 0u, 0u, active, bad};
        block_flush_slot(slot, v);
    }
    if constexpr (DEFER) {  // sm.xn is final: the plane loop ended with a barrier
        const uint32_t nb = min(sm.xn, kFirstXCap);
        const int tid2 = threadIdx.y * kTX + threadIdx.x;
        if (tid2 == 0) sm.xbase = nb ? atomicAdd(xcount, nb) : 0u;
        __syncthreads();
        for (uint32_t j = tid2; j < nb; j += kThreads) xlist[sm.xbase + j] = sm.x[j];
    }
}

// bz0: index of the first z-chunk the launch covers (a launch may cover a
// z-range of chunks, e.g. the part of the field already copied in).
template <typename T, int MODE, bool DEFER = false>
__global__ void __launch_bounds__(kThreads, MODE == kFirst && DEFER && sizeof(T) == 4 ? 6 : 5) k_tiled(const T *__restrict__ fa, const T *__restrict__ fb,
                                                       uint8_t *__restrict__ codes, uint32_t *__restrict__ hp,
                                                       uint32_t *__restrict__ req, uint32_t *__restrict__ act_next,
                                                       SweepSlot *slot, Geom g, int bz0, uint32_t *xlist = nullptr,
                                                       uint32_t *xcount = nullptr) {
    __shared__ TileOf<T, MODE, DEFER> sm;
    const int bz = bz0 + static_cast<int>(blockIdx.z);
    // a block whose tile, halo included, and planes zb-1 .. ze lie inside the
    // domain runs the check-free body (about three blocks in four at 512^3)
    const int x0 = static_cast<int>(blockIdx.x) * kTX, y0 = static_cast<int>(blockIdx.y) * kTY, zb = bz * g.zc;
    const bool inside = x0 >= 1 && x0 + kTX + 1 <= g.nx && y0 >= 1 && y0 + kTY + 1 <= g.ny && zb >= 1 &&
                        zb + g.zc + 1 <= g.nz;
    if (inside)
        tiled_body<T, MODE, DEFER, true>(sm, fa, fb, codes, hp, req, act_next, slot, g, blockIdx.x, blockIdx.y, bz,
                                         xlist, xcount);
    else
        tiled_body<T, MODE, DEFER, false>(sm, fa, fb, codes, hp, req, act_next, slot, g, blockIdx.x, blockIdx.y, bz,
                                          xlist, xcount);
}

// ---------------------------------------------------------------------------
// TMA-fed first pass.  Every block gets its planes by tensor-map copies: one
// thread issues, per plane, a cp.async.bulk.tensor box of f and one of fhat
// (the tile with its one-voxel halo, widened in x so that the box starts on a
// 16-byte boundary) into a ring of kRawStages shared-memory stages, each
// guarded by an mbarrier that the copy engine completes with the box's byte
// count.  The threads wait for a plane, convert each of its cells to a proxy
// once (the same conversion and NaN / sentinel check as the load path of
// tiled_body), and the stage is refilled with the plane kRawStages ahead after
// the barrier that ends the plane.  No thread computes a global address or
// predicates a load for the tile; the compute is tiled_body's interior
// deferring path, except that each voxel stores its own fhat proxy
// (coalesced) and that the rules of voxels whose codes differ run after the
// last plane (kRuleCap).  Blocks on the domain's faces take the FACE form of
// the body (first_tma_body).
//
// Every mbarrier wait is bounded: a plane that does not arrive within the
// limit sets *err (the host reports PMSZ_ERR_CUDA), and the block still waits,
// again bounded, on every plane it issued before it exits.
// ---------------------------------------------------------------------------
template <typename T> struct RawBox;
template <> struct RawBox<double> { static constexpr int kX = 36, kOff = 1; };  // x0-2 .. x0+33
template <> struct RawBox<float> { static constexpr int kX = 40, kOff = 3; };   // x0-4 .. x0+35
constexpr int kRawStages = 4;
// Voxels of a TMA-fed block whose two codes differ are queued in shared
// memory as (tx | ty << 5 | (z - zb) << 8 | c0 << 16 | c1 << 24) and run
// through the rules by the whole block after its last plane: inline, a warp
// would run the rules whenever one of its 32 voxels needs them.  A full queue
// spills to the deferred list (k_first_exact decides those voxels on keys).
constexpr uint32_t kRuleCap = 1024;
template <typename T>
constexpr int kRawBytes = RawBox<T>::kX * kHY * static_cast<int>(sizeof(T));  // one box of one field
template <typename T>
constexpr int kRawPitch = (kRawBytes<T> + 127) / 128 * 128;  // stages start on 128-byte boundaries

template <typename T>
struct __align__(128) TmaTile {
    // first: the copy engine writes the stages, which must start on 128-byte
    // boundaries (the struct is 128-byte aligned, kRawPitch a multiple of 128)
    alignas(128) unsigned char raw[kRawStages][2][kRawPitch<T>];  // boxes of f and fhat, rows of RawBox<T>::kX
    uint32_t p[2][4][kHY][kHX];                      // proxy ring, as tiled_body's
    uint32_t x[kFirstXCap];                          // voxels whose certificate failed
    uint32_t rq[kRuleCap];                           // voxels whose codes differ, queued for the rules
    unsigned long long mbar[kRawStages];
    uint32_t xn, xbase, rn;
};
static_assert(offsetof(TmaTile<float>, raw) == 0 && offsetof(TmaTile<double>, raw) == 0 &&
                  kRawPitch<float> % 128 == 0 && kRawPitch<double> % 128 == 0,
              "TMA stages must start on 128-byte boundaries");

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

constexpr int kMbarTries = 1 << 22;  // try_wait suspends between tries: a bound of seconds, not a spin count

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
    for (int it = 0; it < kMbarTries; ++it) {
        uint32_t ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(ok) : "r"(addr), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t mbar) {
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                 :: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(mbar) : "memory");
}

// FACE: a block on a domain face (or one whose tile crosses the domain's far
// end).  Planes outside the domain are not copied: their stage's barrier gets
// a plain arrive and their cells proxy 0; cells of a box outside the domain
// in x or y (the copy fills them with zeros) are stored as proxy 0 as well.
// A warp whose row has a voxel on a face runs the general chains (proxy 0
// loses every max chain as 0 + r and every min chain as 0 + r - 16, wrapped);
// threads beyond the domain compute but store nothing.
template <typename T, bool FACE>
__device__ __forceinline__ void first_tma_body(TmaTile<T> &sm, const CUtensorMap *tf, const CUtensorMap *tfh,
                                               uint8_t *__restrict__ codes, uint32_t *__restrict__ hp,
                                               uint32_t *__restrict__ req, uint32_t *__restrict__ act_next,
                                               SweepSlot *slot, const Geom &g, int bx, int by, int bz,
                                               uint32_t *__restrict__ xlist, uint32_t *xcount, uint32_t *err) {
    constexpr int kBX = RawBox<T>::kX, kOff = RawBox<T>::kOff;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTX + tx;
    const int x0 = bx * kTX, y0 = by * kTY, zb = bz * g.zc;
    const int ze = FACE ? min(g.nz, zb + g.zc) : zb + g.zc;  // inside: ze <= nz - 1
    const int x = x0 + tx, y = y0 + ty;
    const bool vin = !FACE || (x < g.nx && y < g.ny);  // this thread's voxels exist
    const size_t plane = static_cast<size_t>(g.nx) * g.ny;
    const int nplanes = ze - zb + 2;  // zb-1 .. ze
    if (tid == 0) {
        for (int s = 0; s < kRawStages; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&sm.mbar[s])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sm.xn = 0;
        sm.rn = 0;
    }
    __syncthreads();
    auto issue = [&](int k) {  // plane zb-1+k into stage k % kRawStages
        const int s = k % kRawStages;
        const uint32_t mb = smem_u32(&sm.mbar[s]);
        if (FACE && (zb - 1 + k < 0 || zb - 1 + k >= g.nz)) {  // nothing to copy: complete the phase
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(mb) : "memory");
            return;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the stage's reads come first
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(mb), "r"(2 * kRawBytes<T>)
                     : "memory");
        tma_load_3d(smem_u32(sm.raw[s][0]), tf, x0 - kOff - 1, y0 - 1, zb - 1 + k, mb);
        tma_load_3d(smem_u32(sm.raw[s][1]), tfh, x0 - kOff - 1, y0 - 1, zb - 1 + k, mb);
    };
    if (tid == 0)
        for (int k = 0; k < kRawStages && k < nplanes; ++k) issue(k);

    // this thread's cells (tid and tid + 256 of the 34 x 10 halo tile)
    int cell_s[2], cell_r[2];
    bool cell_own[2], cell_in[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int c = tid + j * kThreads;
        const int cy = c / kHX, cx = c - cy * kHX;
        const int gx = x0 - 1 + cx, gy = y0 - 1 + cy;
        cell_s[j] = c;
        cell_r[j] = cy * kBX + cx + kOff;
        cell_in[j] = !FACE || (gx >= 0 && gx < g.nx && gy >= 0 && gy < g.ny);
        cell_own[j] = c < kCells && cx >= 1 && cx <= kTX && cy >= 1 && cy <= kTY && cell_in[j];
    }
    uint32_t bad = 0, failed = 0;
    // fp64: only cells whose proxy lies in the ranges of the infinities and
    // NaNs, or equals the proxy of the sentinel 1e30, take the exact test
    const uint32_t sentinel_px = proxy_of(T(1e30));
    auto convert = [&](int k) {  // stage of plane zb-1+k -> its proxy slot
        const int s = k % kRawStages, zz = zb - 1 + k;
        if (!mbar_wait(smem_u32(&sm.mbar[s]), static_cast<uint32_t>((k / kRawStages) & 1))) failed = 1;
        const bool zown = zz >= zb && zz < ze;
        const bool zin = !FACE || (zz >= 0 && zz < g.nz);
        const int ps = zz & 3;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (cell_s[j] >= kCells) continue;
#pragma unroll
            for (int F = 0; F < 2; ++F) {
                const T v = zin ? reinterpret_cast<const T *>(sm.raw[s][F])[cell_r[j]] : T(0);
                const uint32_t px = (!FACE || (zin && cell_in[j])) ? proxy_of(v) : 0u;
                if (cell_own[j] && zown &&
                    (sizeof(T) == 4 || px - 0x00100000u >= 0xFFE00000u || px == sentinel_px))
                    bad |= bad_value(v) ? 1u : 0u;
                (&sm.p[F][ps][0][0])[cell_s[j]] = px;
            }
        }
    };
    convert(0);
    convert(1);
    convert(2);
    __syncthreads();
    if (tid == 0)
        for (int k = kRawStages; k < kRawStages + 3 && k < nplanes; ++k) issue(k);  // stages of planes 0..2
    uint32_t cmax = 0, cmin = 0, cdir = 0;
    size_t i = static_cast<size_t>(x) + static_cast<size_t>(y) * g.nx + static_cast<size_t>(zb) * plane;
    // the four chains of one field (max / min, forward / reverse ranks); GEN:
    // the general form, whose min chains add -16 so that proxy 0 loses
    auto chains = [&](int F, const int (&slots)[3], bool gen, uint32_t &M, uint32_t &m, uint32_t &N, uint32_t &n,
                      uint32_t &self) {
        uint32_t t[15];
#pragma unroll
        for (int r = 0; r < 15; ++r) t[r] = sm.p[F][slots[tile_slot_sel(r)]][ty + 1 + rank_dy(r)][tx + 1 + rank_dx(r)];
        self = t[kSelf];
        if (!FACE || !gen) {
            M = t[0]; m = t[0]; N = t[0] + 15u; n = N;
#pragma unroll
            for (int r = 1; r < 15; ++r) {
                const uint32_t a = t[r] + static_cast<uint32_t>(r), b = t[r] + static_cast<uint32_t>(15 - r);
                M = max(M, a); m = min(m, a); N = max(N, b); n = min(n, b);
            }
        } else {
            M = t[0]; m = t[0] - 16u; N = t[0] + 15u; n = t[0] - 1u;
#pragma unroll
            for (int r = 1; r < 15; ++r) {
                const uint32_t a = t[r] + static_cast<uint32_t>(r), b = t[r] + static_cast<uint32_t>(15 - r);
                M = max(M, a); m = min(m, a - 16u); N = max(N, b); n = min(n, b - 16u);
            }
        }
    };
    for (int z = zb; z < ze; ++z, i += plane) {
        const int slots[3] = {(z + 3) & 3, z & 3, (z + 1) & 3};
        // warp-uniform: every voxel of this warp's row has its 15 cells
        const bool gen = FACE && !(y >= 1 && y + 1 < g.ny && z >= 1 && z + 1 < g.nz && x0 >= 1 && x0 + kTX + 1 <= g.nx);
        bool rule = false;
        uint32_t M0, m0, N0, n0, M1, m1, N1, n1, self0, self1;  // the four chains of f, then of fhat
        chains(0, slots, gen, M0, m0, N0, n0, self0);
        chains(1, slots, gen, M1, m1, N1, n1, self1);
        (void)self0;
        if (vin) hp[i] = self1;  // the proxy array of fhat, one coalesced row per warp
        const uint32_t s0 = (M0 + N0) & (m0 + n0);
        const uint32_t c0 = (M0 & 15u) | ((m0 & 15u) << 4), c1 = (M1 & 15u) | ((m1 & 15u) << 4);
        if (!vin) {
        } else if ((s0 & (M1 + N1) & (m1 + n1) & 15u) != 15u) {
            codes[i] = (s0 & 15u) == 15u ? static_cast<uint8_t>(c0) : kCodeUnset;
            const uint32_t pos = atomicAdd(&sm.xn, 1u);
            if (pos < kFirstXCap) sm.x[pos] = static_cast<uint32_t>(i);
            else spill_append(xlist, xcount, static_cast<uint32_t>(i));
        } else {
            codes[i] = static_cast<uint8_t>(c0);
            rule = c1 != c0 || c0 == 0x77u;
        }
        const uint32_t want = __ballot_sync(0xFFFFFFFFu, rule);
        if (want) {
            uint32_t base = 0;
            if (tx == 0) base = atomicAdd(&sm.rn, static_cast<uint32_t>(__popc(want)));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (rule) {
                const uint32_t pos = base + static_cast<uint32_t>(__popc(want & ((1u << tx) - 1u)));
                if (pos < kRuleCap && g.zc <= 256)
                    sm.rq[pos] = static_cast<uint32_t>(tx) | (static_cast<uint32_t>(ty) << 5) |
                                 (static_cast<uint32_t>(z - zb) << 8) | (c0 << 16) | (c1 << 24);
                else
                    spill_append(xlist, xcount, static_cast<uint32_t>(i));
            }
        }
        const int k = z - zb + 3;  // plane z+2
        if (k < nplanes) convert(k);
        __syncthreads();
        if (tid == 0 && k + kRawStages < nplanes) issue(k + kRawStages);
    }
    // the queued rule voxels (every enqueue precedes the loop's last barrier)
    const uint32_t nr = min(sm.rn, kRuleCap);
    for (uint32_t j = tid; j < nr; j += kThreads) {
        const uint32_t e = sm.rq[j];
        const int ex = x0 + static_cast<int>(e & 31u), ey = y0 + static_cast<int>((e >> 5) & 7u),
                  ez = zb + static_cast<int>((e >> 8) & 0xFFu);
        const uint32_t c0 = (e >> 16) & 0xFFu, c1 = e >> 24;
        const uint32_t tm = detect_rules(static_cast<int>(c1 & 15u), static_cast<int>(c1 >> 4),
                                         static_cast<int>(c0 & 15u), static_cast<int>(c0 >> 4), cmax, cmin, cdir);
        if (tm) {
            request_targets(req, g, ex, ey, ez, tm);
            atomicOr(act_next + word_of(g, x0, ey, ez), 1u << (e & 31u));
        }
    }
    if (failed) atomicOr(err, 1u);
    const uint32_t v[8] = {cmax, cmin, cdir, 0u, 0u, 0u, vin ? static_cast<uint32_t>(ze - zb) : 0u, bad};
    block_flush_slot(slot, v);
    const uint32_t nb = min(sm.xn, kFirstXCap);
    if (tid == 0) sm.xbase = nb ? atomicAdd(xcount, nb) : 0u;
    __syncthreads();
    for (uint32_t j = tid; j < nb; j += kThreads) xlist[sm.xbase + j] = sm.x[j];
}

// The deferring first pass with TMA-fed tiles; tf / tfh map f / fhat as
// (nx, ny, nz) with a box of RawBox<T>::kX x 10 x 1 (the caller falls back to
// k_tiled where no map can be made: rows whose byte length is not a multiple
// of 16, or base pointers off a 16-byte boundary).  f / fh are not read here.
// bz0 as for k_tiled.  Interior blocks run the check-free body, blocks on a
// face the FACE body.  fp32 runs six blocks per SM (40 registers, no spills:
// 3.81 against 3.83 ms at 512^3); fp64 five (at six it spills and is slower).
template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 6 : 5) k_first_tma(const __grid_constant__ CUtensorMap tf,
                                                            const __grid_constant__ CUtensorMap tfh,
                                                            const T *__restrict__ f, const T *__restrict__ fh,
                                                            uint8_t *__restrict__ codes, uint32_t *__restrict__ hp,
                                                            uint32_t *__restrict__ req, uint32_t *__restrict__ act_next,
                                                            SweepSlot *slot, Geom g, int bz0, uint32_t *xlist,
                                                            uint32_t *xcount, uint32_t *err) {
    __shared__ TmaTile<T> sm;
    (void)f;
    (void)fh;
    const int bz = bz0 + static_cast<int>(blockIdx.z);
    const int x0 = static_cast<int>(blockIdx.x) * kTX, y0 = static_cast<int>(blockIdx.y) * kTY, zb = bz * g.zc;
    const bool inside = x0 >= 1 && x0 + kTX + 1 <= g.nx && y0 >= 1 && y0 + kTY + 1 <= g.ny && zb >= 1 &&
                        zb + g.zc + 1 <= g.nz;
    if (inside)
        first_tma_body<T, false>(sm, &tf, &tfh, codes, hp, req, act_next, slot, g, blockIdx.x, blockIdx.y, bz,
                                 xlist, xcount, err);
    else
        first_tma_body<T, true>(sm, &tf, &tfh, codes, hp, req, act_next, slot, g, blockIdx.x, blockIdx.y, bz,
                                xlist, xcount, err);
}

// ---------------------------------------------------------------------------
// Load policies.  Standalone sweep kernels read arrays that no thread of the
// same launch writes through the read-only path (__ldg).  Persistent loop
// kernels (the multi-field loop of batch.cu) write those arrays in one phase
// and read them in the next, across grid-wide barriers, so they read them at
// L2 (__ldcg), never from a possibly stale L1 line.
// ---------------------------------------------------------------------------
struct LdgLoads {
    template <class P>
    static __device__ __forceinline__ P ld(const P *p) { return __ldg(p); }
};
struct CgLoads {
    template <class P>
    static __device__ __forceinline__ P ld(const P *p) { return __ldcg(p); }
};

// ---------------------------------------------------------------------------
// Block-local compaction of a bitmap.  A round covers 2048 consecutive words:
// each of the 256 threads loads 8 of them with two 16-byte loads, and one
// barrier skips the round when all are empty (late sweeps touch a few words of
// a large bitmap, so the scan must move as much per barrier as it can).  In a
// non-empty round the set bits of all 2048 words are ranked by a block scan
// and written to a dense work list in shared memory (entries (word << 5) |
// bit, word local to the round), in passes of at most kListCap entries, and
// all 256 threads share the list: a sparse or clustered bitmap still keeps
// every lane busy, and a sparse round costs a handful of barriers.
// ---------------------------------------------------------------------------
constexpr int kListBlock = 256;
constexpr int kWordsPerThread = 8;
constexpr int kRoundWords = kListBlock * kWordsPerThread;
constexpr uint32_t kListCap = 8192;

struct ListSmem {
    uint32_t list[kListCap];
    uint32_t mask[kRoundWords];   // per-word result bits (mismatch / changed)
    uint32_t warp_tot[kListBlock / 32];
    uint32_t total;
};

// Loads the 8 words of this thread for the round starting at `base` (bitmaps
// are 256-byte aligned and rounds start at multiples of 2048 words, so the
// vector loads are aligned); returns whether any word of the block is set.
template <class L>
__device__ __forceinline__ bool load_round(const uint32_t *__restrict__ bm, size_t base, const Geom &g,
                                           uint32_t (&w8)[kWordsPerThread]) {
    const size_t w0 = base + static_cast<size_t>(threadIdx.x) * kWordsPerThread;
    if (w0 + kWordsPerThread <= g.nwords) {
        const uint4 a = L::ld(reinterpret_cast<const uint4 *>(bm + w0));
        const uint4 b = L::ld(reinterpret_cast<const uint4 *>(bm + w0 + 4));
        w8[0] = a.x; w8[1] = a.y; w8[2] = a.z; w8[3] = a.w;
        w8[4] = b.x; w8[5] = b.y; w8[6] = b.z; w8[7] = b.w;
    } else {
#pragma unroll
        for (int j = 0; j < kWordsPerThread; ++j) w8[j] = w0 + j < g.nwords ? L::ld(bm + w0 + j) : 0u;
    }
    uint32_t any = 0;
#pragma unroll
    for (int j = 0; j < kWordsPerThread; ++j) any |= w8[j];
    return __syncthreads_or(any != 0) != 0;
}

// Calls work(x, y, z, word_local) for every set bit of bitmap `bm` (clearing
// the bitmap); a true result sets the voxel's bit in a per-word result mask,
// and flush(w, mask) is then called once per word with a non-zero mask, by the
// thread that owns the word.  Every thread of the block must call this.
// One round (2048 words from `base`) of for_each_set_bit.
template <class L, class Work, class Flush>
__device__ __forceinline__ void process_round(ListSmem &sm, uint32_t *__restrict__ bm, const Geom &g, size_t base,
                                              Work &work, Flush &flush) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    {
        uint32_t w8[kWordsPerThread];
        if (!load_round<L>(bm, base, g, w8)) return;  // uniform
        const size_t w0 = base + static_cast<size_t>(t) * kWordsPerThread;
        uint32_t c = 0;
#pragma unroll
        for (int j = 0; j < kWordsPerThread; ++j) {
            if (w8[j]) bm[w0 + j] = 0;
            sm.mask[t * kWordsPerThread + j] = 0;
            c += __popc(w8[j]);
        }
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) sm.warp_tot[warp] = inc;
        __syncthreads();
        if (t == 0) {
            uint32_t run = 0;
            for (int k = 0; k < kListBlock / 32; ++k) {
                const uint32_t v = sm.warp_tot[k];
                sm.warp_tot[k] = run;
                run += v;
            }
            sm.total = run;
        }
        __syncthreads();
        const uint32_t first = sm.warp_tot[warp] + inc - c, total = sm.total;
        for (uint32_t lo = 0; lo < total; lo += kListCap) {
            const uint32_t hi = lo + kListCap;
            if (first < hi && first + c > lo) {  // some of my entries fall in this pass
                uint32_t rank = first;
#pragma unroll
                for (int j = 0; j < kWordsPerThread; ++j) {
                    uint32_t bits = w8[j];
                    while (bits) {
                        const int b = __ffs(bits) - 1;
                        bits &= bits - 1;
                        if (rank >= lo && rank < hi)
                            sm.list[rank - lo] = (static_cast<uint32_t>(t * kWordsPerThread + j) << 5) | static_cast<uint32_t>(b);
                        ++rank;
                    }
                }
            }
            __syncthreads();
            const uint32_t n = min(kListCap, total - lo);
            for (uint32_t k = t; k < n; k += kListBlock) {
                const uint32_t e = sm.list[k];
                const uint32_t wl = e >> 5;
                const int b = static_cast<int>(e & 31u);
                int wx, y, z;
                word_coords(g, base + wl, wx, y, z);
                if (work(wx * 32 + b, y, z, wl)) atomicOr(&sm.mask[wl], 1u << b);
            }
            __syncthreads();
        }
#pragma unroll
        for (int j = 0; j < kWordsPerThread; ++j) {
            const uint32_t m = sm.mask[t * kWordsPerThread + j];
            if (w8[j] && m) flush(w0 + j, m);
        }
        __syncthreads();
    }
}

template <class L, class Work, class Flush>
__device__ __forceinline__ void for_each_set_bit(ListSmem &sm, uint32_t *__restrict__ bm, const Geom &g, Work &work,
                                                 Flush &flush) {
    for (size_t base = static_cast<size_t>(blockIdx.x) * kRoundWords; base < g.nwords;
         base += static_cast<size_t>(gridDim.x) * kRoundWords)
        process_round<L>(sm, bm, g, base, work, flush);
}

// ---------------------------------------------------------------------------
// Sparse detection of one voxel of the active set, reading the proxy array of
// fhat (exact keys on a failed certificate), with the reference rules; the
// word's mismatch bits go to act_next through DetectFlush (one writer per
// word).  Counters accumulate in the functor.
// ---------------------------------------------------------------------------
template <class L, typename T>
struct DetectWork {
    const T *fh;
    const uint32_t *hp;
    const uint8_t *codes;
    uint32_t *req;
    Geom g;
    uint32_t cmax = 0, cmin = 0, cdir = 0, active = 0;
    __device__ __forceinline__ bool operator()(int x, int y, int z, uint32_t) {
        const ptrdiff_t sy = g.nx, sz = static_cast<ptrdiff_t>(g.nx) * g.ny;
        const size_t i = flat(g, x, y, z);
        const bool interior = x >= 1 && x <= g.nx - 2 && y >= 1 && y <= g.ny - 2 && z >= 1 && z <= g.nz - 2;
        const uint32_t valid = interior ? kAllValid : valid_mask(x, y, z, g.nx, g.ny, g.nz);
        const uint32_t *c0 = hp + i;
        uint32_t t[15];
#pragma unroll
        for (int r = 0; r < 15; ++r) {
            const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
            t[r] = ((valid >> r) & 1u) ? L::ld(c0 + off) : 0u;
        }
        Ext ex = interior ? proxy_ext_interior<true>(t) : proxy_ext<true>(t);
        if (!ex.exact) {
            typename KeyOf<T>::type kk[15];
#pragma unroll
            for (int r = 0; r < 15; ++r) {
                const ptrdiff_t off = rank_dx(r) + rank_dy(r) * sy + rank_dz(r) * sz;
                kk[r] = ((valid >> r) & 1u) ? okey(L::ld(fh + (static_cast<ptrdiff_t>(i) + off)))
                                            : typename KeyOf<T>::type(0);
            }
            arg_ext(kk, valid, ex.asc, ex.desc);
        }
        const uint8_t c = __ldg(codes + i);
        const uint32_t tm = detect_rules(ex.asc, ex.desc, c & 15, c >> 4, cmax, cmin, cdir);
        ++active;
        if (tm) request_targets(req, g, x, y, z, tm);
        return tm != 0;
    }
    __device__ __forceinline__ void flush_to(SweepSlot *slot) {  // every thread of the block
        const uint32_t v[8] = {cmax, cmin, cdir, 0u, 0u, 0u, active, 0u};
        block_flush_slot(slot, v);
        cmax = cmin = cdir = active = 0;
    }
};

struct DetectFlush {
    uint32_t *act_next;
    __device__ __forceinline__ void operator()(size_t w, uint32_t m) { act_next[w] = m; }
};

template <class L, typename T>
__device__ __forceinline__ void sparse_detect_body(ListSmem &sm, const T *__restrict__ fh, const uint32_t *__restrict__ hp,
                                                   const uint8_t *__restrict__ codes, uint32_t *__restrict__ act_cur,
                                                   uint32_t *__restrict__ act_next, uint32_t *__restrict__ req,
                                                   SweepSlot *slot, const Geom &g) {
    DetectWork<L, T> work{fh, hp, codes, req, g};
    DetectFlush flush{act_next};
    for_each_set_bit<L>(sm, act_cur, g, work, flush);
    work.flush_to(slot);
}

// ---------------------------------------------------------------------------
// Apply with the proxy array: applyDeltaBuffer_local (pMSz.cu:623-645) on
// every requested vertex, in T:
//   if |f - (fhat - delta)| <= eps && cnt < q-1 { fhat -= delta; cnt++ }
//   else { cnt = q; fhat = f - eps }
// the proxy of every changed value refreshed; ApplyFlush marks the closed
// stencil of the changed vertices of a word in act_next (owner thread).
// ---------------------------------------------------------------------------
template <class L, typename T>
struct ApplyWork {
    const T *f;
    T *fh;
    uint8_t *cnt;
    uint32_t *hp;
    Geom g;
    T eps, delta;
    int q;
    uint32_t nreq = 0, nprog = 0;
    __device__ __forceinline__ bool operator()(int x, int y, int z, uint32_t) {
        const size_t v = flat(g, x, y, z);
        const T old = L::ld(fh + v);
        const uint8_t oc = L::ld(cnt + v);
        const T fv = __ldg(f + v);
        const T lowered = old - delta;
        T nv;
        uint8_t nc;
        if (fabs(fv - lowered) <= eps && static_cast<int>(oc) < q - 1) {
            nv = lowered;
            nc = static_cast<uint8_t>(oc + 1);
        } else {
            nc = static_cast<uint8_t>(q);
            nv = fv - eps;
        }
        fh[v] = nv;
        cnt[v] = nc;
        const bool chg = bits_of(old) != bits_of(nv);
        if (chg) hp[v] = proxy_of(nv);
        ++nreq;
        nprog += (chg || nc != oc) ? 1u : 0u;
        return chg;
    }
};

struct ApplyFlush {
    uint32_t *act_next;
    Geom g;
    uint32_t nchg = 0;
    __device__ __forceinline__ void operator()(size_t w, uint32_t m) {
        nchg += __popc(m);
        int wx, y, z;
        word_coords(g, w, wx, y, z);
        mark_stencil(act_next, g, wx, y, z, m);
    }
};

__device__ __forceinline__ void flush_apply_counts(SweepSlot *slot, uint32_t nreq, uint32_t nchg, uint32_t nprog) {
    nreq = warp_sum_u32(nreq);
    nchg = warp_sum_u32(nchg);
    nprog = warp_sum_u32(nprog);
    if ((threadIdx.x & 31) == 0) {
        if (nreq) atomicAdd(&slot->requested, (unsigned long long)nreq);
        if (nchg) atomicAdd(&slot->changed, (unsigned long long)nchg);
        if (nprog) atomicAdd(&slot->progressed, (unsigned long long)nprog);
    }
}

template <class L, typename T>
__device__ __forceinline__ void apply_body(ListSmem &sm, const T *__restrict__ f, T *__restrict__ fh,
                                           uint8_t *__restrict__ cnt, uint32_t *__restrict__ hp,
                                           uint32_t *__restrict__ req, uint32_t *__restrict__ act_next, SweepSlot *slot,
                                           const Geom &g, T eps, T delta, int q) {
    ApplyWork<L, T> work{f, fh, cnt, hp, g, eps, delta, q};
    ApplyFlush flush{act_next, g};
    for_each_set_bit<L>(sm, req, g, work, flush);
    const uint32_t v[8] = {0u, 0u, 0u, work.nreq, flush.nchg, work.nprog, 0u, 0u};
    block_flush_slot(slot, v);
}

template <typename T>
__global__ void __launch_bounds__(kListBlock, 3) k_sparse_px(const T *__restrict__ fh, const uint32_t *__restrict__ hp,
                                                          const uint8_t *__restrict__ codes, uint32_t *__restrict__ act_cur,
                                                          uint32_t *__restrict__ act_next, uint32_t *__restrict__ req,
                                                          SweepSlot *slot, Geom g) {
    __shared__ ListSmem sm;
    sparse_detect_body<LdgLoads>(sm, fh, hp, codes, act_cur, act_next, req, slot, g);
}

template <typename T>
__global__ void __launch_bounds__(kListBlock) k_apply_px(const T *__restrict__ f, T *__restrict__ fh,
                                                         uint8_t *__restrict__ cnt, uint32_t *__restrict__ hp,
                                                         uint32_t *__restrict__ req, uint32_t *__restrict__ act_next,
                                                         SweepSlot *slot, Geom g, T eps, T delta, int q) {
    __shared__ ListSmem sm;
    apply_body<LdgLoads>(sm, f, fh, cnt, hp, req, act_next, slot, g, eps, delta, q);
}

// Stop rule of the correction loop after a sweep (the slot of that sweep):
// converged (no mismatch), stuck (nothing could change), or out of sweeps.
__host__ __device__ __forceinline__ bool sweep_stops(unsigned long long fmax, unsigned long long fmin,
                                                     unsigned long long fdir, unsigned long long progressed,
                                                     int64_t sweeps_done, int64_t max_sweeps) {
    return (fmax == 0 && fmin == 0 && fdir == 0) || progressed == 0 || sweeps_done >= max_sweeps;
}

inline dim3 tiled_grid(const Geom &g) {
    return dim3(static_cast<unsigned>(g.wpr), static_cast<unsigned>((g.ny + kTY - 1) / kTY),
                static_cast<unsigned>((g.nz + g.zc - 1) / g.zc));
}

}  // namespace pmsz
