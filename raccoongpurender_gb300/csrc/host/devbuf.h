// devbuf.h — a device allocation owned by a host object, and the CUDA
// error-to-status helpers the C ABI functions share.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "../rgr_internal.h"

namespace rgr {

inline bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}
#define RGR_CUDA(call)                                      \
    do {                                                    \
        if (!::rgr::cuda_ok((call), #call)) return RGR_E_CUDA; \
    } while (0)

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    int alloc(size_t n) {
        if (n <= bytes && p) return RGR_OK;
        release();
        size_t b = std::max<size_t>(n, 256);
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) {
            p = nullptr;
            set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? RGR_E_OOM : RGR_E_CUDA;
        }
        bytes = b;
        return RGR_OK;
    }
    int upload(const void* src, size_t n, cudaStream_t st) {
        int r = alloc(n);
        if (r != RGR_OK) return r;
        if (n) RGR_CUDA(cudaMemcpyAsync(p, src, n, cudaMemcpyHostToDevice, st));
        return RGR_OK;
    }
    template <class T>
    T* as() const {
        return reinterpret_cast<T*>(p);
    }
};

}  // namespace rgr
