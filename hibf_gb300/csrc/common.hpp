// common.hpp -- host-side helpers shared by the C-ABI translation units: status codes, the per-thread error
// message, CUDA error mapping and the device row-stride rule.
#pragma once

#include <cstdint>
#include <cstdio>
#include <new>
#include <stdexcept>
#include <string>

#include <cuda_runtime.h>

#include "../../include/hibf_gb300.h"

namespace hibf_gb300
{

void set_last_error(std::string msg);

struct status_error : std::runtime_error
{
    int status;
    status_error(int s, std::string const & m) : std::runtime_error(m), status(s)
    {}
};

[[noreturn]] inline void fail(int status, std::string const & msg)
{
    throw status_error(status, msg);
}

inline void cuda_check(cudaError_t e, char const * what)
{
    if (e == cudaSuccess)
        return;
    (void)cudaGetLastError(); // a non-sticky error (e.g. a failed allocation) must not resurface at a later check
    int st = HIBF_GPU_ERR_CUDA;
    if (e == cudaErrorMemoryAllocation)
        st = HIBF_GPU_ERR_OUT_OF_MEMORY;
    else if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        st = HIBF_GPU_ERR_NO_DEVICE;
    throw status_error(st, std::string(what) + ": " + cudaGetErrorString(e));
}

#define HG_CUDA(call) ::hibf_gb300::cuda_check((call), #call)

// Runs `body`, mapping exceptions to status codes and recording the message for hibf_gpu_last_error().
template <typename F>
int guarded(F && body) noexcept
{
    try
    {
        body();
        return HIBF_GPU_OK;
    }
    catch (status_error const & e)
    {
        set_last_error(e.what());
        return e.status;
    }
    catch (std::bad_alloc const &)
    {
        set_last_error("host allocation failed");
        return HIBF_GPU_ERR_OUT_OF_MEMORY;
    }
    catch (std::exception const & e)
    {
        set_last_error(e.what());
        return HIBF_GPU_ERR_CUDA;
    }
    catch (...)
    {
        set_last_error("unknown error");
        return HIBF_GPU_ERR_CUDA;
    }
}

// Device row stride in 64-bit words: 1, 2, 4 words stay; 3 -> 4; above 4 words round up to a multiple of 4 (32 B),
// so every row covers exactly ceil(bytes / 32) sectors.
inline uint64_t padded_row_words(uint64_t bin_words)
{
    if (bin_words <= 2)
        return bin_words;
    if (bin_words <= 4)
        return 4;
    return (bin_words + 3) / 4 * 4;
}

// Lanes per value for a row of bin_words words: the next power of two, capped at a warp.
inline uint32_t lanes_per_value_log2(uint64_t bin_words)
{
    uint32_t l = 0;
    while ((1ull << l) < bin_words && l < 5)
        ++l;
    return l;
}

inline void require_device()
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
    {
        (void)cudaGetLastError();
        fail(HIBF_GPU_ERR_NO_DEVICE, "no CUDA device available (the library has no CPU fallback)");
    }
}

// RAII device buffer.
struct dbuf
{
    void * p{nullptr};
    size_t bytes{0};
    dbuf() = default;
    dbuf(dbuf const &) = delete;
    dbuf & operator=(dbuf const &) = delete;
    ~dbuf()
    {
        if (p)
            cudaFree(p);
    }
    void ensure(size_t n)
    {
        if (n <= bytes && p)
            return;
        if (p)
            cudaFree(p);
        p = nullptr;
        bytes = 0;
        size_t const want = n < 256 ? 256 : n;
        HG_CUDA(cudaMalloc(&p, want));
        bytes = want;
    }
    template <typename T>
    T * as() const
    {
        return static_cast<T *>(p);
    }
};

// RAII pinned host buffer.
struct hbuf
{
    void * p{nullptr};
    size_t bytes{0};
    hbuf() = default;
    hbuf(hbuf const &) = delete;
    hbuf & operator=(hbuf const &) = delete;
    ~hbuf()
    {
        if (p)
            cudaFreeHost(p);
    }
    void ensure(size_t n)
    {
        if (n <= bytes && p)
            return;
        if (p)
            cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        size_t const want = n < 256 ? 256 : n;
        HG_CUDA(cudaMallocHost(&p, want));
        bytes = want;
    }
    template <typename T>
    T * as() const
    {
        return static_cast<T *>(p);
    }
};

} // namespace hibf_gb300
