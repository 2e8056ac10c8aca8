// Device-side helpers shared by the sweep engine and the schedule builder:
// CUDA status checks that raise gmr::Error, device buffers, device selection.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "gmr_internal.h"

namespace gmr {

#define GMR_CUDA(call)                                                                                  \
    do {                                                                                                \
        cudaError_t err_ = (call);                                                                      \
        if (err_ != cudaSuccess)                                                                        \
            throw ::gmr::Error(GMR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_));    \
    } while (0)

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void ensure(size_t n) {
        if (n <= bytes) return;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, n ? n : 16);
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw Error(e == cudaErrorMemoryAllocation ? GMR_ERR_OOM : GMR_ERR_CUDA,
                        std::string("cudaMalloc(") + std::to_string(n) + "): " + cudaGetErrorString(e));
        }
        bytes = n;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

template <class T>
inline T* upload(const std::vector<T>& h, DevBuf& b) {
    b.ensure(h.size() * sizeof(T));
    if (!h.empty()) GMR_CUDA(cudaMemcpy(b.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return static_cast<T*>(b.p);
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) GMR_CUDA(cudaSetDevice(dev));
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// Owning typed device array (freed on scope exit).
template <class T>
struct DevArray {
    T* p = nullptr;
    int64_t n = 0;
    DevArray() = default;
    explicit DevArray(int64_t count) { alloc(count); }
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    ~DevArray() {
        if (p) cudaFree(p);
    }
    void alloc(int64_t count) {
        if (p) cudaFree(p);
        p = nullptr;
        n = count;
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, (size_t)(count > 0 ? count : 1) * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            n = 0;
            throw Error(e == cudaErrorMemoryAllocation ? GMR_ERR_OOM : GMR_ERR_CUDA,
                        std::string("cudaMalloc(") + std::to_string(count * (int64_t)sizeof(T)) +
                            "): " + cudaGetErrorString(e));
        }
        p = static_cast<T*>(q);
    }
    void swap(DevArray& o) {
        std::swap(p, o.p);
        std::swap(n, o.n);
    }
};

}  // namespace gmr
