// devbuf.cuh -- growable device buffer of the host-side library code.
#pragma once
#include <cstddef>

#include "ct_common.cuh"

namespace ct {

// Device buffer that grows on demand.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t n) {
        if (n <= bytes) return CT_OK;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        CT_CUDA(cudaMalloc(&ptr, n), "cudaMalloc");
        bytes = n;
        return CT_OK;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(ptr); }
};

template <typename T>
inline int upload(DevBuf &b, const T *host, size_t n) {
    int s = b.ensure(sizeof(T) * n);
    if (s) return s;
    CT_CUDA(cudaMemcpy(b.ptr, host, sizeof(T) * n, cudaMemcpyHostToDevice), "upload");
    return CT_OK;
}

}  // namespace ct

