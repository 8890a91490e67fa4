// batch.h -- multi-field correction: the per-field table the multi-field
// kernels read, and the host driver shared by pmsz_correct_batch (batch.cu)
// and the continuous-batching server (server.cpp).
#pragma once
#include "tiled.cuh"
#include "internal.h"

#include <string>
#include <vector>

namespace pmsz {

constexpr int kMaxBatch = 4096;

// One field of a multi-field run, as the kernels see it.
template <typename T>
struct Inst {
    const T *f;
    T *fh;
    uint8_t *codes, *cnt;
    uint32_t *hp, *req, *act0, *act1;
    SweepSlot *slots;   // this field's slot of sweep k is slots[k * stride]
    int64_t stride;
    Geom g;
    T eps, delta;
    int q;
    int64_t max_sweeps;
    int64_t k;          // index of the field's next sweep
    int active;         // runs sweeps
    int first;          // joins now: its fused first pass runs in this generation
    uint32_t tiles_x, tiles_y;
};

template <typename T>
struct FieldSpec {
    const T *f;
    T *fh;
    size_t nx, ny, nz;
    double eb;
};

struct BatchOutcome {
    int status = PMSZ_ERR_NOT_CONVERGED;
    std::string message;
    std::vector<SweepSlot> log;
};

// Scratch of the voxel-list generations of a table of fields (batch_list.cuh).
// State of the device-gated generations of pmsz_correct_batch (k_batch_gate).
struct BatchState {
    long long k;             // sweep index of the next generation
    int go;                  // the next generation runs
    int live;                // fields still running after the last gate
    unsigned long long est;  // their next active sets, estimated (15 * changed + fdir)
};

struct MultiLists {
    uint32_t *wpre = nullptr;   // n + 1 word prefixes (multiples of 4), device
    uint64_t total_words = 0;
    uint32_t *counts = nullptr; // one count per compaction block (kCompactBlocks)
    uint64_t *list = nullptr, *xlist = nullptr;  // capacity: the fields' voxels
    uint32_t *lc = nullptr;     // 4 list lengths
    BatchState *state = nullptr;
};

// Scratch and table of one multi-field run; slot rows are sweep-major
// (row k holds the slot of sweep k of every field).
template <typename T>
struct MultiRun {
    explicit MultiRun(cudaStream_t st) : s(st), ws(st) {}
    ~MultiRun() {
        if (pin) cudaFreeHost(pin);
    }
    MultiRun(const MultiRun &) = delete;
    MultiRun &operator=(const MultiRun &) = delete;
    int setup(const std::vector<FieldSpec<T>> &specs, int64_t max_sweeps, int q, cudaStream_t s);
    // One generation: the fused first pass of fields with `first` set, the
    // detection of every other active field, then the edits of all active
    // fields.  Clears `first` afterwards.
    int generation();
    // The remaining sweeps of all active fields in one cooperative launch.
    int loop(int64_t *iters);
    // The same launch on the device table as it stands when the stream gets
    // there, without waiting: *hiters (pinned) receives the iteration count.
    int enqueue_loop(long long *hiters);
    int read_row(int64_t k, std::vector<SweepSlot> &row);
    // rows k .. k+count-1 in one copy (row j at out[j * n])
    int read_rows(int64_t k, int64_t count, std::vector<SweepSlot> &out);
    // The host table goes up through one of two pinned copies in turn, with
    // no wait: every generation ends in a read_row, which synchronises the
    // stream before the same copy is written again.
    int push_table();
    // Sets every field's tile depth (and the tile prefixes) to zc.
    int set_zchunk(int zc);
    // Times the first-pass launch over the whole table at each candidate
    // depth (scratch re-zeroed afterwards), records the fastest for the
    // batch's size class and sets it.
    int tune_zchunk();

    cudaStream_t s;
    Workspace ws;
    int n = 0;
    int64_t max_sweeps = 0;
    int q = 5;
    std::vector<Inst<T>> host;
    std::vector<uint32_t> tpre, rpre;
    uint32_t total_tiles = 0, total_rounds = 0;
    Inst<T> *dinst = nullptr;
    uint32_t *dtpre = nullptr, *drpre = nullptr;
    long long *diters = nullptr;
    SweepSlot *slots = nullptr;
    MultiLists ml;
    bool lists = false;
    Inst<T> *pin = nullptr;  // 2 * n table entries, pinned
    int pin_next = 0;
    unsigned char *zero_base = nullptr;  // the scratch that starts zeroed (counters, bitmaps, slots)
    size_t zero_total = 0;
    size_t voxels = 0;  // voxel-list generations (all fields together below 2^32 voxels)
};

// One generation over a device table of n fields (see MultiRun::generation),
// and the gather of each field's current-sweep slot into out[0..n).
// ml: the voxel-list scratch, or null for the round-based passes.
template <typename T>
int launch_generation(const Inst<T> *dinst, const uint32_t *dtpre, const uint32_t *drpre, int n,
                      uint32_t total_tiles, uint32_t total_rounds, bool any_first, cudaStream_t s,
                      const MultiLists *ml);

// Word prefixes of a table (each field's bitmap words rounded up to a multiple
// of 4) and their total; false if the list form does not apply (the fields'
// voxels or words reach 2^32).
inline bool list_prefixes(const std::vector<Geom> &geoms, std::vector<uint32_t> &wpre, uint64_t &total_words) {
    wpre.assign(geoms.size() + 1, 0);
    uint64_t words = 0, voxels = 0;
    for (size_t i = 0; i < geoms.size(); ++i) {
        wpre[i] = static_cast<uint32_t>(words);
        words += (geoms[i].nwords + 3) & ~static_cast<size_t>(3);
        voxels += geoms[i].n;
        if (words >= (1ull << 32) || voxels >= (1ull << 32)) return false;
    }
    wpre[geoms.size()] = static_cast<uint32_t>(words);
    total_words = words;
    return true;
}
template <typename T>
int launch_gather(const Inst<T> *dinst, int n, SweepSlot *out, cudaStream_t s);

// Scratch bytes of one field (codes, counters, proxies, three bitmaps) and
// its sweep slots.
inline size_t field_scratch_bytes(const Geom &g, int64_t max_sweeps) {
    auto up = [](size_t b) { return (b + 255) & ~static_cast<size_t>(255); };
    return up(g.n) * 2 + up(4 * g.n) + 3 * up(4 * g.nwords) + up(sizeof(SweepSlot) * static_cast<size_t>(max_sweeps));
}

template <typename T>
int batch_impl(const std::vector<FieldSpec<T>> &specs, const pmsz_opts *opts, std::vector<BatchOutcome> &out,
               cudaStream_t s);

}  // namespace pmsz
