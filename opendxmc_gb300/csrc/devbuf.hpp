// devbuf.hpp -- owning device allocation (cudaMalloc / cudaFree), resized on demand.
#pragma once

#include <algorithm>
#include <cstddef>

#include <cuda_runtime.h>

namespace dxmcg {

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n)
    {
        o.p = nullptr;
        o.n = 0;
    }
    ~DevBuf() { reset(); }
    // at least `count` elements; keeps the allocation when it is already that large
    cudaError_t reserve(size_t count)
    {
        if (p && n >= count)
            return cudaSuccess;
        reset();
        const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess)
            n = count;
        else
            p = nullptr;
        return e;
    }
    void reset()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

} // namespace dxmcg
