// server.cu -- continuous-batching correction server (pmsz_server_*).
//
// The reference corrects one field per program run.  The server takes
// correction jobs from any host thread and runs them on one GPU with
// continuous batching: a worker thread repeats generations, and in each one
//   1. admits queued jobs in arrival order while the HBM budget (the job's
//      two fields plus its scratch) and the job-slot limit allow,
//   2. runs ONE sweep of every running job in shared launches -- the fused
//      first pass of the jobs admitted now, the detection of the others, the
//      edits of all (the multi-field kernels of batch.cu),
//   3. reads each job's sweep counters, applies the stop rule of the
//      correction loop, and retires finished jobs (scratch freed, waiters
//      woken).
// A job that arrives while others run joins at the next generation, so its
// work overlaps theirs on the device.  Every job keeps its own scratch, sweep
// index and stop state: its corrected field is bit-identical to running it
// alone through pmsz_correct_*.
#include "batch.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

namespace pmsz {

using Clock = std::chrono::steady_clock;

struct Job {
    uint64_t id = 0;
    pmsz_field fd{};
    Geom g{};
    size_t bytes = 0;      // budget charge: fields + scratch
    unsigned char *scratch = nullptr;
    size_t scratch_bytes = 0;
    int64_t k = 0;
    bool first = true, done = false;
    int status = PMSZ_ERR_NOT_CONVERGED;
    std::vector<SweepSlot> log;
    Clock::time_point t_submit, t_start, t_done;
};

template <typename T>
static Inst<T> make_inst(Job &j, int q, int64_t max_sweeps) {
    Inst<T> I{};
    const Geom &g = j.g;
    auto up = [](size_t b) { return (b + 255) & ~static_cast<size_t>(255); };
    unsigned char *p = j.scratch;
    I.cnt = p;
    p += up(g.n);
    I.req = reinterpret_cast<uint32_t *>(p);
    p += up(4 * g.nwords);
    I.act0 = reinterpret_cast<uint32_t *>(p);
    p += up(4 * g.nwords);
    I.act1 = reinterpret_cast<uint32_t *>(p);
    p += up(4 * g.nwords);
    I.slots = reinterpret_cast<SweepSlot *>(p);
    p += up(sizeof(SweepSlot) * static_cast<size_t>(max_sweeps));
    I.codes = p;
    p += up(g.n);
    I.hp = reinterpret_cast<uint32_t *>(p);
    I.f = static_cast<const T *>(j.fd.f);
    I.fh = static_cast<T *>(j.fd.fhat);
    I.stride = 1;
    I.g = g;
    I.eps = static_cast<T>(j.fd.eb);
    I.delta = static_cast<T>(j.fd.eb / static_cast<double>(q));
    I.q = q;
    I.max_sweeps = max_sweeps;
    I.k = j.k;
    I.active = 1;
    I.first = j.first ? 1 : 0;
    I.tiles_x = static_cast<uint32_t>(g.wpr);
    I.tiles_y = static_cast<uint32_t>((g.ny + kTY - 1) / kTY);
    return I;
}

// Zero-initialised part of a job's scratch: counters, bitmaps, slots.
static size_t zero_prefix(const Geom &g, int64_t max_sweeps) {
    auto up = [](size_t b) { return (b + 255) & ~static_cast<size_t>(255); };
    return up(g.n) + 3 * up(4 * g.nwords) + up(sizeof(SweepSlot) * static_cast<size_t>(max_sweeps));
}

class Server {
public:
    explicit Server(const pmsz_server_config &c) : cfg_(c) {
        if (cfg_.max_jobs <= 0 || cfg_.max_jobs > kMaxBatch) cfg_.max_jobs = 256;
        if (cfg_.q <= 0) cfg_.q = 5;
        if (cfg_.max_sweeps <= 0) cfg_.max_sweeps = 10000;
    }
    ~Server() { shutdown(); }

    int start() {
        PMSZ_CUDA(cudaGetDevice(&device_));
        worker_ = std::thread([this] { run(); });
        return PMSZ_OK;
    }

    void shutdown() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (stopping_) return;
            stopping_ = true;
        }
        cv_work_.notify_all();
        if (worker_.joinable()) worker_.join();
    }

    int submit(const pmsz_field &fd, uint64_t *id) {
        int rc = check_geom(fd.nx, fd.ny, fd.nz);
        if (rc) return rc;
        if (!fd.f || !fd.fhat) return set_error(PMSZ_ERR_ARG, "null field pointer");
        if (!(fd.eb > 0.0) || !(fd.eb < 1e300)) return set_error(PMSZ_ERR_ARG, "error bound must be positive and finite");
        if (fd.elem_size != 4 && fd.elem_size != 8) return set_error(PMSZ_ERR_ARG, "elem_size must be 4 or 8");
        auto j = std::make_unique<Job>();
        j->fd = fd;
        j->g = make_geom(fd.nx, fd.ny, fd.nz);
        j->g.zc = tuned_zchunk(fd.nx, fd.ny, fd.nz, fd.elem_size);
        j->scratch_bytes = field_scratch_bytes(j->g, cfg_.max_sweeps);
        // its fields, its scratch, and its share of the group's voxel lists
        j->bytes = j->scratch_bytes + 2 * j->g.n * fd.elem_size + 2 * sizeof(uint64_t) * j->g.n;
        if (cfg_.hbm_budget_bytes && j->bytes > cfg_.hbm_budget_bytes)
            return set_error(PMSZ_ERR_OOM, "job larger than the server's HBM budget");
        j->t_submit = Clock::now();
        std::lock_guard<std::mutex> lk(mu_);
        if (stopping_) return set_error(PMSZ_ERR_ARG, "server is shutting down");
        j->id = ++next_id_;
        *id = j->id;
        pending_.push_back(j.get());
        jobs_[j->id] = std::move(j);
        cv_work_.notify_all();
        return PMSZ_OK;
    }

    int info(uint64_t id, pmsz_job_info *out, double timeout_s) {
        std::unique_lock<std::mutex> lk(mu_);
        auto it = jobs_.find(id);
        if (it == jobs_.end()) return set_error(PMSZ_ERR_ARG, "unknown job id");
        Job *j = it->second.get();
        if (timeout_s != 0.0) {
            auto pred = [&] { return j->done; };
            if (timeout_s < 0) cv_done_.wait(lk, pred);
            else cv_done_.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
        }
        std::memset(out, 0, sizeof(*out));
        out->done = j->done ? 1 : 0;
        if (!j->done) return PMSZ_OK;
        out->status = j->status;
        out->sweeps = static_cast<int64_t>(j->log.size());
        for (const SweepSlot &h : j->log) out->edits += h.requested;
        out->queue_ms = std::chrono::duration<double, std::milli>(j->t_start - j->t_submit).count();
        out->run_ms = std::chrono::duration<double, std::milli>(j->t_done - j->t_start).count();
        out->latency_ms = std::chrono::duration<double, std::milli>(j->t_done - j->t_submit).count();
        return PMSZ_OK;
    }

    int release(uint64_t id) {
        std::lock_guard<std::mutex> lk(mu_);
        auto it = jobs_.find(id);
        if (it == jobs_.end() || !it->second->done) return set_error(PMSZ_ERR_ARG, "job unknown or not finished");
        jobs_.erase(it);
        return PMSZ_OK;
    }

private:
    template <typename T>
    struct Group {
        std::vector<Job *> jobs;
        std::vector<Inst<T>> host;
        Inst<T> *dinst = nullptr;
        uint32_t *dpre = nullptr;
        SweepSlot *dslots = nullptr, *hslots = nullptr;
        int cap = 0;
        MultiLists ml;            // voxel-list scratch of the running set
        uint32_t *dwpre = nullptr;
        size_t list_cap = 0;      // entries of ml.list / ml.xlist
    };

    template <typename T>
    int ensure(Group<T> &G, int n) {
        if (n <= G.cap) return PMSZ_OK;
        if (G.dinst) cudaFree(G.dinst);
        if (G.dpre) cudaFree(G.dpre);
        if (G.dslots) cudaFree(G.dslots);
        if (G.hslots) cudaFreeHost(G.hslots);
        G.cap = std::max(n, 64);
        PMSZ_CUDA(cudaMalloc(&G.dinst, sizeof(Inst<T>) * G.cap));
        PMSZ_CUDA(cudaMalloc(&G.dpre, sizeof(uint32_t) * 2 * (G.cap + 1)));
        PMSZ_CUDA(cudaMalloc(&G.dslots, sizeof(SweepSlot) * G.cap));
        PMSZ_CUDA(cudaMallocHost(&G.hslots, sizeof(SweepSlot) * G.cap));
        if (G.dwpre) cudaFree(G.dwpre);
        PMSZ_CUDA(cudaMalloc(&G.dwpre, sizeof(uint32_t) * (G.cap + 1)));
        return PMSZ_OK;
    }

    // List buffers for `voxels` entries (grown, never shrunk while the server runs).
    template <typename T>
    int ensure_lists(Group<T> &G, size_t voxels) {
        if (!G.ml.counts) {
            PMSZ_CUDA(cudaMalloc(&G.ml.counts, sizeof(uint32_t) * kCompactBlocks));
            PMSZ_CUDA(cudaMalloc(&G.ml.lc, sizeof(uint32_t) * 4));
        }
        if (voxels <= G.list_cap) return PMSZ_OK;
        if (G.ml.list) cudaFree(G.ml.list);
        if (G.ml.xlist) cudaFree(G.ml.xlist);
        G.ml.list = G.ml.xlist = nullptr;
        G.list_cap = 0;
        const size_t cap = std::max<size_t>(voxels, 1 << 20);
        PMSZ_CUDA(cudaMalloc(&G.ml.list, sizeof(uint64_t) * cap));
        PMSZ_CUDA(cudaMalloc(&G.ml.xlist, sizeof(uint64_t) * cap));
        G.list_cap = cap;
        return PMSZ_OK;
    }

    template <typename T>
    void release_group(Group<T> &G) {
        if (G.dinst) cudaFree(G.dinst);
        if (G.dpre) cudaFree(G.dpre);
        if (G.dslots) cudaFree(G.dslots);
        if (G.hslots) cudaFreeHost(G.hslots);
        if (G.dwpre) cudaFree(G.dwpre);
        if (G.ml.counts) cudaFree(G.ml.counts);
        if (G.ml.lc) cudaFree(G.ml.lc);
        if (G.ml.list) cudaFree(G.ml.list);
        if (G.ml.xlist) cudaFree(G.ml.xlist);
        G = Group<T>{};
    }

    // One sweep of every running job of type T.
    template <typename T>
    int step(Group<T> &G) {
        const int n = static_cast<int>(G.jobs.size());
        if (!n) return PMSZ_OK;
        int rc = ensure(G, n);
        if (rc) return rc;
        G.host.resize(n);
        std::vector<uint32_t> pre(2 * (n + 1));
        uint64_t tiles = 0, rounds = 0;
        bool any_first = false;
        for (int i = 0; i < n; ++i) {
            Job &j = *G.jobs[i];
            G.host[i] = make_inst<T>(j, cfg_.q, cfg_.max_sweeps);
            any_first |= j.first;
            pre[i] = static_cast<uint32_t>(tiles);
            pre[n + 1 + i] = static_cast<uint32_t>(rounds);
            tiles += static_cast<uint64_t>(G.host[i].tiles_x) * G.host[i].tiles_y * ((j.g.nz + j.g.zc - 1) / j.g.zc);
            rounds += (j.g.nwords + kRoundWords - 1) / kRoundWords;
        }
        if (tiles >= (1ull << 31) || rounds >= (1ull << 31)) return set_error(PMSZ_ERR_ARG, "running set too large");
        pre[n] = static_cast<uint32_t>(tiles);
        pre[2 * n + 1] = static_cast<uint32_t>(rounds);
        std::vector<Geom> geoms(n);
        size_t voxels = 0;
        for (int i = 0; i < n; ++i) {
            geoms[i] = G.host[i].g;
            voxels += geoms[i].n;
        }
        // Voxel-list generations pay off once the running set's next active
        // sets are large (estimate: 15 * changed + fdir of the last sweep, a
        // sixteenth of a joining field); small groups take the two round-based
        // launches, which cost less than the list form's eight.
        unsigned long long est = 0;
        for (int i = 0; i < n; ++i) {
            const Job &j = *G.jobs[i];
            if (j.first || j.log.empty()) est += j.g.n / 16;
            else est += 15ull * j.log.back().changed + j.log.back().fdir;
        }
        std::vector<uint32_t> wpre;
        const bool lists = est >= std::max<unsigned long long>(1ull << 20, voxels / 32) &&
                           list_prefixes(geoms, wpre, G.ml.total_words);
        if (lists) {
            if ((rc = ensure_lists(G, voxels))) return rc;
            G.ml.wpre = G.dwpre;
            PMSZ_CUDA(cudaMemcpyAsync(G.dwpre, wpre.data(), sizeof(uint32_t) * wpre.size(), cudaMemcpyHostToDevice, s_));
        }
        PMSZ_CUDA(cudaMemcpyAsync(G.dinst, G.host.data(), sizeof(Inst<T>) * n, cudaMemcpyHostToDevice, s_));
        PMSZ_CUDA(cudaMemcpyAsync(G.dpre, pre.data(), sizeof(uint32_t) * pre.size(), cudaMemcpyHostToDevice, s_));
        if ((rc = launch_generation<T>(G.dinst, G.dpre, G.dpre + n + 1, n, static_cast<uint32_t>(tiles),
                                       static_cast<uint32_t>(rounds), any_first, s_, lists ? &G.ml : nullptr)))
            return rc;
        if ((rc = launch_gather<T>(G.dinst, n, G.dslots, s_))) return rc;
        PMSZ_CUDA(cudaMemcpyAsync(G.hslots, G.dslots, sizeof(SweepSlot) * n, cudaMemcpyDeviceToHost, s_));
        PMSZ_CUDA(cudaStreamSynchronize(s_));
        for (int i = 0; i < n; ++i) {
            Job &j = *G.jobs[i];
            const SweepSlot h = G.hslots[i];
            j.log.push_back(h);
            j.first = false;
            if (j.k == 0 && h.bad) {
                j.status = PMSZ_ERR_ARG;
                j.done = true;
            } else if (sweep_stops(h.fmax, h.fmin, h.fdir, h.progressed, j.k + 1, cfg_.max_sweeps)) {
                j.status = (h.fmax == 0 && h.fmin == 0 && h.fdir == 0) ? PMSZ_OK : PMSZ_ERR_NOT_CONVERGED;
                j.done = true;
            } else {
                ++j.k;
            }
        }
        return PMSZ_OK;
    }

    void fail_all(int rc) {
        std::lock_guard<std::mutex> lk(mu_);
        for (Job *j : running_) {
            j->status = rc;
            j->done = true;
            j->t_done = Clock::now();
        }
        running_.clear();
        cv_done_.notify_all();
    }

    void run() {
        cudaSetDevice(device_);
        if (cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking) != cudaSuccess) {
            fail_all(PMSZ_ERR_CUDA);
            return;
        }
        retain_pool_once();
        Group<float> g32;
        Group<double> g64;
        while (true) {
            std::vector<Job *> admitted;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_work_.wait(lk, [&] { return stopping_ || !pending_.empty() || !running_.empty(); });
                if (stopping_ && pending_.empty() && running_.empty()) break;
                while (!pending_.empty() && static_cast<int>(running_.size() + admitted.size()) < cfg_.max_jobs) {
                    Job *j = pending_.front();
                    if (cfg_.hbm_budget_bytes && used_ + j->bytes > cfg_.hbm_budget_bytes) break;  // FIFO admission
                    pending_.pop_front();
                    used_ += j->bytes;
                    admitted.push_back(j);
                }
            }
            for (Job *j : admitted) {
                j->t_start = Clock::now();
                if (cudaMallocAsync(reinterpret_cast<void **>(&j->scratch), j->scratch_bytes, s_) != cudaSuccess ||
                    cudaMemsetAsync(j->scratch, 0, zero_prefix(j->g, cfg_.max_sweeps), s_) != cudaSuccess) {
                    cudaGetLastError();
                    j->status = PMSZ_ERR_OOM;
                    j->done = true;
                }
            }
            {
                std::lock_guard<std::mutex> lk(mu_);
                for (Job *j : admitted) running_.push_back(j);
            }
            g32.jobs.clear();
            g64.jobs.clear();
            for (Job *j : running_)
                if (!j->done) (j->fd.elem_size == 4 ? (std::vector<Job *> &)g32.jobs : g64.jobs).push_back(j);
            int rc = step(g32);
            if (!rc) rc = step(g64);
            if (rc) {
                fail_all(PMSZ_ERR_CUDA);
                continue;
            }
            // retire finished jobs
            std::vector<Job *> keep;
            {
                std::lock_guard<std::mutex> lk(mu_);
                for (Job *j : running_) {
                    if (j->done) {
                        if (j->scratch) cudaFreeAsync(j->scratch, s_);
                        j->scratch = nullptr;
                        used_ -= j->bytes;
                        j->t_done = Clock::now();
                    } else {
                        keep.push_back(j);
                    }
                }
                running_.swap(keep);
            }
            cv_done_.notify_all();
        }
        cudaStreamSynchronize(s_);
        release_group(g32);
        release_group(g64);
        cudaStreamDestroy(s_);
    }

    pmsz_server_config cfg_;
    int device_ = 0;
    cudaStream_t s_ = nullptr;
    std::thread worker_;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<Job *> pending_;
    std::vector<Job *> running_;
    std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs_;
    uint64_t next_id_ = 0;
    size_t used_ = 0;
    bool stopping_ = false;
};

}  // namespace pmsz

using namespace pmsz;

struct pmsz_server {
    std::unique_ptr<Server> impl;
};

extern "C" int pmsz_server_create(const pmsz_server_config *cfg, pmsz_server **out) {
    return guarded([&] {
        if (!cfg || !out) return set_error(PMSZ_ERR_ARG, "null argument");
        auto s = std::make_unique<pmsz_server>();
        s->impl = std::make_unique<Server>(*cfg);
        const int rc = s->impl->start();
        if (rc) return rc;
        *out = s.release();
        return PMSZ_OK;
    });
}

extern "C" int pmsz_server_submit(pmsz_server *srv, const pmsz_field *field, uint64_t *job_id) {
    return guarded([&] {
        if (!srv || !field || !job_id) return set_error(PMSZ_ERR_ARG, "null argument");
        return srv->impl->submit(*field, job_id);
    });
}

extern "C" int pmsz_server_wait(pmsz_server *srv, uint64_t job_id, double timeout_s, pmsz_job_info *info) {
    return guarded([&] {
        if (!srv || !info) return set_error(PMSZ_ERR_ARG, "null argument");
        return srv->impl->info(job_id, info, timeout_s);
    });
}

extern "C" int pmsz_server_release(pmsz_server *srv, uint64_t job_id) {
    return guarded([&] {
        if (!srv) return set_error(PMSZ_ERR_ARG, "null argument");
        return srv->impl->release(job_id);
    });
}

extern "C" int pmsz_server_destroy(pmsz_server *srv) {
    return guarded([&] {
        if (!srv) return PMSZ_OK;
        srv->impl->shutdown();
        delete srv;
        return PMSZ_OK;
    });
}
