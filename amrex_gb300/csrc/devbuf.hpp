// Minimal RAII device/pinned buffers.
#pragma once

#include "common.hpp"

namespace mlmg {

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf () = default;
    explicit DevBuf (size_t count) { alloc(count); }
    DevBuf (const DevBuf&) = delete;
    DevBuf& operator= (const DevBuf&) = delete;
    DevBuf (DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf& operator= (DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf () { release(); }
    void alloc (size_t count) {
        release();
        n = count;
        if (count > 0) { MLMG_CUDA_CHECK(cudaMalloc((void**)&p, count * sizeof(T))); }
    }
    void release () {
        if (p) { cudaFree(p); }
        p = nullptr; n = 0;
    }
    void upload (const T* h, size_t count, cudaStream_t s) {
        if (count > n) { alloc(count); }
        if (count > 0) { MLMG_CUDA_CHECK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s)); }
    }
    void upload (const std::vector<T>& v, cudaStream_t s) { upload(v.data(), v.size(), s); }
    void zero (cudaStream_t s) {
        if (n > 0) { MLMG_CUDA_CHECK(cudaMemsetAsync(p, 0, n * sizeof(T), s)); }
    }
};

template <typename T>
struct PinnedBuf {
    T* p = nullptr;
    size_t n = 0;
    PinnedBuf () = default;
    PinnedBuf (const PinnedBuf&) = delete;
    PinnedBuf& operator= (const PinnedBuf&) = delete;
    ~PinnedBuf () { if (p) { cudaFreeHost(p); } }
    void alloc (size_t count) {
        if (p) { cudaFreeHost(p); p = nullptr; }
        n = count;
        if (count > 0) { MLMG_CUDA_CHECK(cudaMallocHost((void**)&p, count * sizeof(T))); }
    }
};

} // namespace mlmg
