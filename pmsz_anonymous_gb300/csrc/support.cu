// support.cu -- error strings, thread-local last-error, scratch allocation.
#include "internal.h"

#include <cstring>
#include <mutex>

namespace pmsz {

static thread_local std::string t_last_error;

int set_error(int status, const std::string &msg) {
    if (status != PMSZ_OK) t_last_error = msg;
    return status;
}

void retain_pool_once() {
    static std::mutex mu;
    static std::vector<int> done;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    std::lock_guard<std::mutex> lk(mu);
    for (int d : done)
        if (d == dev) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    done.push_back(dev);
}

int Workspace::commit() {
    if (total_ == 0) return PMSZ_OK;
    retain_pool_once();
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&base_), total_, s_);
    if (e != cudaSuccess) {
        base_ = nullptr;
        cudaGetLastError();
        return set_error(e == cudaErrorMemoryAllocation ? PMSZ_ERR_OOM : PMSZ_ERR_CUDA,
                         std::string("scratch allocation of ") + std::to_string(total_) +
                             " bytes failed: " + cudaGetErrorString(e));
    }
    return PMSZ_OK;
}

int Workspace::release() {
    if (!base_) return PMSZ_OK;
    cudaError_t e = cudaFreeAsync(base_, s_);
    base_ = nullptr;
    if (e != cudaSuccess) return set_error(PMSZ_ERR_CUDA, std::string("scratch release failed: ") + cudaGetErrorString(e));
    return PMSZ_OK;
}

void *host_pinned(size_t bytes, int slot) {
    struct Block {
        void *p = nullptr;
        size_t n = 0;
    };
    static thread_local Block blocks[2];  // live until process exit
    Block &b = blocks[slot == 1 ? 1 : 0];
    if (b.n < bytes) {
        void *p = nullptr;
        if (cudaMallocHost(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        b.p = p;  // an outgrown block is kept: a pointer to it may still be in use by the caller
        b.n = bytes;
    }
    return b.p;
}

}  // namespace pmsz

extern "C" const char *pmsz_strerror(int status) {
    switch (status) {
        case PMSZ_OK: return "ok";
        case PMSZ_ERR_ARG: return "invalid argument";
        case PMSZ_ERR_OOM: return "out of memory";
        case PMSZ_ERR_NOT_CONVERGED: return "not converged";
        case PMSZ_ERR_CUDA: return "CUDA error";
        case PMSZ_ERR_IO: return "I/O error";
        default: return "unknown status";
    }
}

extern "C" const char *pmsz_last_error(void) { return pmsz::t_last_error.c_str(); }

extern "C" int pmsz_version(void) { return 100; }
