// rbx_devarray.h -- owning device allocation used by the host-side handles.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace rbx {

template <class T> struct DevArray {
    T* p = nullptr;
    size_t n = 0;
    DevArray() = default;
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    ~DevArray() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void swap(DevArray& o) {
        T* tp = p; p = o.p; o.p = tp;
        size_t tn = n; n = o.n; o.n = tn;
    }
    // The allocation is rounded up to a multiple of 256 bytes, so that any element range widened
    // to 16-byte boundaries stays inside it.
    // Device bytes held (the allocation as requested from cudaMalloc).
    size_t bytes() const { return p ? ((n * sizeof(T) + 255) / 256) * 256 : 0; }
    cudaError_t alloc(size_t count) {
        release();
        n = count;
        if (count == 0) return cudaSuccess;
        const size_t bytes = ((count * sizeof(T) + 255) / 256) * 256;
        return cudaMalloc((void**)&p, bytes);
    }
};

}  // namespace rbx
