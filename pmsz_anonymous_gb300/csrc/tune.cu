// tune.cu -- the autotuner: tile depth and pointer-jumping rounds per launch.
//
// Two launch parameters change the speed of the path but never its results:
//   zchunk       planes per tile column of the tiled passes (the fused first
//                pass marches a 32 x 8 column through zchunk planes with a
//                one-plane halo: deeper columns re-read fewer halo planes,
//                shallower ones give small fields more blocks);
//   jump_rounds  three-hop pointer jumps per vertex per launch of the label
//                passes (more rounds, fewer launches and host flag reads).
// A shape class is (ceil log2 nx, ceil log2 ny, ceil log2 nz) and, for the
// tile depth, the element size.  A batch (pmsz_correct_batch) runs its first
// pass as one launch over all its fields, so it has a tile depth of its own,
// tuned on the whole table (batch.cu) and keyed by its size class: ceil log2
// of its voxels, ceil log2 of its field count, and the element size.
// autotune_impl times every candidate on the caller's device fields (first
// pass on f / fhat; AS labels of f's codes) and records the fastest; every
// entry point reads the table (make_geom's default depth and one round per
// launch when a class has no entry).  The table is process-wide behind a
// mutex and persists as text:
//   "pmsz-tune 1" header, then per field entry
//   "<elem> <bx> <by> <bz> <zchunk> <jump_rounds>" and per batch entry
//   "b <elem> <bvoxels> <bfields> <zchunk>".
#include "common.cuh"
#include "internal.h"

#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>

namespace pmsz {

namespace {

constexpr int kZCands[4] = {8, 16, 32, 64};
constexpr int kRoundCands[4] = {1, 2, 4, 8};
constexpr int kDefaultRounds = 1;

int ceil_log2(size_t v) {
    int b = 0;
    while ((static_cast<size_t>(1) << b) < v && b < 63) ++b;
    return b;
}

uint32_t shape_key(size_t nx, size_t ny, size_t nz) {
    return static_cast<uint32_t>(ceil_log2(nx)) | (static_cast<uint32_t>(ceil_log2(ny)) << 6) |
           (static_cast<uint32_t>(ceil_log2(nz)) << 12);
}

struct Table {
    std::mutex mu;
    std::map<uint32_t, int> zc;      // (elem << 18) | shape key -> tile depth
    std::map<uint32_t, int> rounds;  // shape key -> rounds per launch
    std::map<uint32_t, int> batch;   // (elem << 12) | (voxel class << 6) | field class -> tile depth
};

uint32_t batch_key(size_t voxels, int nfields, size_t elem) {
    return (static_cast<uint32_t>(elem) << 12) | (static_cast<uint32_t>(ceil_log2(voxels)) << 6) |
           static_cast<uint32_t>(ceil_log2(static_cast<size_t>(std::max(nfields, 1))));
}

Table &table() {
    static Table t;
    return t;
}

bool valid_elem(size_t e) { return e == 4 || e == 8; }

}  // namespace

int tuned_zchunk(size_t nx, size_t ny, size_t nz, size_t elem) {
    Table &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    auto it = t.zc.find((static_cast<uint32_t>(elem) << 18) | shape_key(nx, ny, nz));
    return it == t.zc.end() ? kZChunkDefault : it->second;
}

int tuned_jump_rounds(size_t nx, size_t ny, size_t nz) {
    Table &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    auto it = t.rounds.find(shape_key(nx, ny, nz));
    return it == t.rounds.end() ? kDefaultRounds : it->second;
}

bool tune_known(size_t nx, size_t ny, size_t nz, size_t elem) {
    Table &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    return t.zc.count((static_cast<uint32_t>(elem) << 18) | shape_key(nx, ny, nz)) != 0;
}

int tuned_batch_zchunk(size_t voxels, int nfields, size_t elem) {
    Table &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    auto it = t.batch.find(batch_key(voxels, nfields, elem));
    return it == t.batch.end() ? kZChunkDefault : it->second;
}

bool batch_tune_known(size_t voxels, int nfields, size_t elem) {
    Table &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    return t.batch.count(batch_key(voxels, nfields, elem)) != 0;
}

void record_batch_zchunk(size_t voxels, int nfields, size_t elem, int zc) {
    Table &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    t.batch[batch_key(voxels, nfields, elem)] = zc;
}

const int *zchunk_candidates(int *count) {
    *count = 4;
    return kZCands;
}

static void record(size_t nx, size_t ny, size_t nz, size_t elem, int zc, int rounds) {
    Table &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    const uint32_t k = shape_key(nx, ny, nz);
    t.zc[(static_cast<uint32_t>(elem) << 18) | k] = zc;
    if (rounds > 0) t.rounds[k] = rounds;
}

template <typename T>
int autotune_impl(const T *f, const T *fh, size_t nx, size_t ny, size_t nz, pmsz_tune *out, cudaStream_t s) {
    if (!f || !fh) return set_error(PMSZ_ERR_ARG, "null field pointer");
    int rc = check_geom(nx, ny, nz);
    if (rc) return rc;
    pmsz_tune r{};
    // tile depths: a depth at or beyond nz is one chunk, like every deeper one
    int zcs[4], mz = 0;
    for (int c : kZCands) {
        zcs[mz++] = c;
        if (static_cast<size_t>(c) >= nz) break;
    }
    const size_t n = nx * ny * nz;
    Workspace ws(s);
    const size_t o_codes = ws.reserve<uint8_t>(n);
    if ((rc = ws.commit())) return rc;
    uint8_t *codes = ws.at<uint8_t>(o_codes);
    float mzs[4] = {0.f, 0.f, 0.f, 0.f};
    if ((rc = time_first_pass<T>(f, fh, nx, ny, nz, codes, zcs, mz, mzs, s))) return rc;
    int best = 0;
    for (int k = 1; k < mz; ++k)
        if (mzs[k] < mzs[best]) best = k;
    r.zchunk = zcs[best];
    for (int k = 0; k < mz; ++k) r.ms_zchunk[k] = mzs[k];
    // rounds per launch (labels exist below 2^32 voxels)
    r.jump_rounds = kDefaultRounds;
    if (n < (static_cast<size_t>(1) << 32)) {
        float mr[4] = {0.f, 0.f, 0.f, 0.f};
        if ((rc = time_jump_rounds(codes, nx, ny, nz, kRoundCands, 4, mr, s))) return rc;
        int br = 0;
        for (int k = 1; k < 4; ++k)
            if (mr[k] < mr[br]) br = k;
        r.jump_rounds = kRoundCands[br];
        for (int k = 0; k < 4; ++k) r.ms_rounds[k] = mr[k];
    }
    record(nx, ny, nz, sizeof(T), r.zchunk, r.jump_rounds);
    if (out) *out = r;
    return ws.release();
}

template int autotune_impl<float>(const float *, const float *, size_t, size_t, size_t, pmsz_tune *, cudaStream_t);
template int autotune_impl<double>(const double *, const double *, size_t, size_t, size_t, pmsz_tune *,
                                   cudaStream_t);

}  // namespace pmsz

using namespace pmsz;

extern "C" int pmsz_autotune_f32(const float *f, const float *fhat, size_t nx, size_t ny, size_t nz, pmsz_tune *out,
                                 void *stream) {
    return guarded([&] { return autotune_impl<float>(f, fhat, nx, ny, nz, out, as_stream(stream)); });
}

extern "C" int pmsz_autotune_f64(const double *f, const double *fhat, size_t nx, size_t ny, size_t nz,
                                 pmsz_tune *out, void *stream) {
    return guarded([&] { return autotune_impl<double>(f, fhat, nx, ny, nz, out, as_stream(stream)); });
}

extern "C" int pmsz_tune_get(size_t nx, size_t ny, size_t nz, size_t elem_size, pmsz_tune *out) {
    if (!out || !valid_elem(elem_size) || nx == 0 || ny == 0 || nz == 0) {
        set_error(PMSZ_ERR_ARG, "bad arguments to pmsz_tune_get");
        return -PMSZ_ERR_ARG;
    }
    *out = pmsz_tune{};
    out->zchunk = tuned_zchunk(nx, ny, nz, elem_size);
    out->jump_rounds = tuned_jump_rounds(nx, ny, nz);
    return tune_known(nx, ny, nz, elem_size) ? 1 : 0;
}

extern "C" int pmsz_tune_set(size_t nx, size_t ny, size_t nz, size_t elem_size, const pmsz_tune *t) {
    if (!t || !valid_elem(elem_size) || nx == 0 || ny == 0 || nz == 0)
        return set_error(PMSZ_ERR_ARG, "bad arguments to pmsz_tune_set");
    if (t->zchunk < 1 || t->zchunk > 256) return set_error(PMSZ_ERR_ARG, "zchunk must be in 1..256");
    if (t->jump_rounds < 1 || t->jump_rounds > 16) return set_error(PMSZ_ERR_ARG, "jump_rounds must be in 1..16");
    record(nx, ny, nz, elem_size, t->zchunk, t->jump_rounds);
    return PMSZ_OK;
}

extern "C" int pmsz_tune_save(const char *path) {
    if (!path) return set_error(PMSZ_ERR_ARG, "null path");
    Table &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    FILE *fp = std::fopen(path, "w");
    if (!fp) return set_error(PMSZ_ERR_IO, std::string("cannot open ") + path);
    std::fprintf(fp, "pmsz-tune 1\n");
    for (const auto &kv : t.zc) {
        const uint32_t k = kv.first & 0x3FFFFu;
        auto r = t.rounds.find(k);
        std::fprintf(fp, "%u %u %u %u %d %d\n", kv.first >> 18, k & 63u, (k >> 6) & 63u, (k >> 12) & 63u, kv.second,
                     r == t.rounds.end() ? kDefaultRounds : r->second);
    }
    for (const auto &kv : t.batch)
        std::fprintf(fp, "b %u %u %u %d\n", kv.first >> 12, (kv.first >> 6) & 63u, kv.first & 63u, kv.second);
    const bool ok = std::fclose(fp) == 0;
    return ok ? PMSZ_OK : set_error(PMSZ_ERR_IO, std::string("write failed: ") + path);
}

extern "C" int pmsz_tune_load(const char *path) {
    if (!path) return set_error(PMSZ_ERR_ARG, "null path");
    FILE *fp = std::fopen(path, "r");
    if (!fp) return set_error(PMSZ_ERR_IO, std::string("cannot open ") + path);
    char line[256];
    int version = 0;
    if (!std::fgets(line, sizeof line, fp) || std::sscanf(line, "pmsz-tune %d", &version) != 1 || version != 1) {
        std::fclose(fp);
        return set_error(PMSZ_ERR_IO, std::string("not a tuning table: ") + path);
    }
    std::map<uint32_t, int> zc, rounds, batch;
    bool ok = true;
    while (ok && std::fgets(line, sizeof line, fp)) {
        unsigned e, a1, a2, a3;
        int z, r;
        char tail;
        if (line[0] == '\n' || line[0] == '\0') continue;
        if (line[0] == 'b') {
            ok = std::sscanf(line, "b %u %u %u %d %c", &e, &a1, &a2, &z, &tail) == 4 && valid_elem(e) && a1 <= 63 &&
                 a2 <= 63 && z >= 1 && z <= 256;
            if (ok) batch[(e << 12) | (a1 << 6) | a2] = z;
        } else {
            ok = std::sscanf(line, "%u %u %u %u %d %d %c", &e, &a1, &a2, &a3, &z, &r, &tail) == 6 && valid_elem(e) &&
                 a1 <= 63 && a2 <= 63 && a3 <= 63 && z >= 1 && z <= 256 && r >= 1 && r <= 16;
            if (ok) {
                const uint32_t k = a1 | (a2 << 6) | (a3 << 12);
                zc[(e << 18) | k] = z;
                rounds[k] = r;
            }
        }
    }
    std::fclose(fp);
    if (!ok) return set_error(PMSZ_ERR_IO, std::string("bad tuning entry in ") + path);
    Table &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    for (const auto &kv : zc) t.zc[kv.first] = kv.second;
    for (const auto &kv : rounds) t.rounds[kv.first] = kv.second;
    for (const auto &kv : batch) t.batch[kv.first] = kv.second;
    return PMSZ_OK;
}

extern "C" int pmsz_tune_batch_get(size_t total_voxels, int count, size_t elem_size, pmsz_tune *out) {
    if (!out || !valid_elem(elem_size) || total_voxels == 0 || count < 1) {
        set_error(PMSZ_ERR_ARG, "bad arguments to pmsz_tune_batch_get");
        return -PMSZ_ERR_ARG;
    }
    *out = pmsz_tune{};
    out->zchunk = tuned_batch_zchunk(total_voxels, count, elem_size);
    out->jump_rounds = kDefaultRounds;
    return batch_tune_known(total_voxels, count, elem_size) ? 1 : 0;
}

extern "C" void pmsz_tune_clear(void) {
    Table &t = table();
    std::lock_guard<std::mutex> lk(t.mu);
    t.zc.clear();
    t.rounds.clear();
    t.batch.clear();
}
