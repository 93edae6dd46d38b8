// sketch.cu -- HyperLogLog sketches of user bins on the device: the upstream step of the layout computation
// (compute_sketches, src/sketch/compute_sketches.cpp:27-43), with the same registers as the reference's
// hyperloglog::add (src/sketch/hyperloglog.cpp:55-70), so the host-side layout DP that consumes them is unchanged.
//
// add(v): h = lo ^ hi of the 128-bit product v * 0x9E3779B97F4A7C15 (wyhash's mix); register h >> (64 - bits) takes
// the maximum of its value and countl_zero((h << bits) | (2^bits - 1)) + 1.  The maximum is order-independent, so
// blocks sketch chunks of a user bin in shared memory and merge into the user bin's registers with atomicMax.

#include <algorithm>
#include <vector>

#include "../../include/hibf_gb300_synthetic.h"
#include "common.hpp"

namespace hibf_gb300
{
int sm_count();

namespace
{

constexpr uint64_t kChunk = 1u << 16;   // values per block task
constexpr uint32_t kSmemMaxBits = 14;   // 2^14 32-bit registers = 64 KiB of shared memory

__device__ __forceinline__ void hll_reg(uint64_t v, uint32_t bits, uint32_t & idx, uint32_t & rank)
{
    uint64_t const c = 0x9E3779B97F4A7C15ULL;
    uint64_t const h = (v * c) ^ __umul64hi(v, c);
    uint64_t const mask = (1ull << bits) - 1u;
    idx = static_cast<uint32_t>(h >> (64 - bits));
    rank = static_cast<uint32_t>(__clzll(static_cast<long long>((h << bits) | mask))) + 1u;
}

// One block per chunk task (user bin, first position, count).  d_values == nullptr: the synthetic stream `seed`.
template <bool SMEM>
__global__ void __launch_bounds__(256) k_hll_sketch(uint64_t const * __restrict__ values, uint64_t seed,
                                                    ulonglong4 const * __restrict__ tasks, uint64_t n_tasks,
                                                    uint32_t bits, unsigned int * __restrict__ regs)
{
    extern __shared__ unsigned int s_reg[];
    uint32_t const size = 1u << bits;
    for (uint64_t t = blockIdx.x; t < n_tasks; t += gridDim.x)
    {
        ulonglong4 const task = tasks[t]; // x = user bin, y = first position, z = values
        unsigned int * out = regs + task.x * size;
        if constexpr (SMEM)
        {
            for (uint32_t i = threadIdx.x; i < size; i += blockDim.x)
                s_reg[i] = 0;
            __syncthreads();
        }
        for (uint64_t j = threadIdx.x; j < task.z; j += blockDim.x)
        {
            uint64_t const p = task.y + j;
            uint64_t const v = values ? values[p] : hg_stream_at(seed, p);
            uint32_t idx, rank;
            hll_reg(v, bits, idx, rank);
            if constexpr (SMEM)
                atomicMax(s_reg + idx, rank);
            else
                atomicMax(out + idx, rank);
        }
        if constexpr (SMEM)
        {
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < size; i += blockDim.x)
                if (s_reg[i])
                    atomicMax(out + i, s_reg[i]);
            __syncthreads();
        }
    }
}

__global__ void k_hll_narrow(unsigned int const * __restrict__ regs, uint64_t n, uint8_t * __restrict__ out)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        out[i] = static_cast<uint8_t>(regs[i]);
}

} // namespace
} // namespace hibf_gb300

using namespace hibf_gb300;

extern "C"
{

    int hibf_gpu_hll_sketch_d(uint64_t const * d_values, uint64_t seed, uint64_t const * offsets,
                              uint64_t n_user_bins, uint32_t bits, uint8_t * d_registers, void * stream)
    {
        return guarded(
            [&]
            {
                if (!offsets || (n_user_bins && !d_registers))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (bits < 5 || bits > 16)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "sketch bits must be in [5, 16] on the device");
                require_device();
                if (!n_user_bins)
                    return;
                cudaStream_t const s = static_cast<cudaStream_t>(stream);
                std::vector<ulonglong4> tasks;
                for (uint64_t u = 0; u < n_user_bins; ++u)
                {
                    if (offsets[u + 1] < offsets[u])
                        fail(HIBF_GPU_ERR_INVALID_ARG, "user bin offsets must be non-decreasing");
                    for (uint64_t b = offsets[u]; b < offsets[u + 1]; b += kChunk)
                        tasks.push_back(make_ulonglong4(u, b, std::min<uint64_t>(kChunk, offsets[u + 1] - b), 0));
                }
                uint64_t const size = 1ull << bits;
                uint64_t const n_regs = n_user_bins * size;
                dbuf d_tasks, regs;
                regs.ensure(n_regs * 4);
                HG_CUDA(cudaMemsetAsync(regs.p, 0, n_regs * 4, s));
                if (!tasks.empty())
                {
                    d_tasks.ensure(tasks.size() * sizeof(ulonglong4));
                    HG_CUDA(cudaMemcpyAsync(d_tasks.p, tasks.data(), tasks.size() * sizeof(ulonglong4),
                                            cudaMemcpyHostToDevice, s));
                    unsigned const grid = static_cast<unsigned>(
                        std::min<uint64_t>(tasks.size(), static_cast<uint64_t>(sm_count()) * 8u));
                    if (bits <= kSmemMaxBits)
                    {
                        size_t const smem = size * 4;
                        if (smem > 48 * 1024)
                            HG_CUDA(cudaFuncSetAttribute(k_hll_sketch<true>,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         static_cast<int>(smem)));
                        k_hll_sketch<true><<<grid, 256, smem, s>>>(d_values, seed, d_tasks.as<ulonglong4>(),
                                                                   tasks.size(), bits, regs.as<unsigned int>());
                    }
                    else
                    {
                        k_hll_sketch<false><<<grid, 256, 0, s>>>(d_values, seed, d_tasks.as<ulonglong4>(),
                                                                 tasks.size(), bits, regs.as<unsigned int>());
                    }
                    HG_CUDA(cudaGetLastError());
                }
                unsigned const g2 = static_cast<unsigned>(
                    std::max<uint64_t>(1, std::min<uint64_t>((n_regs + 255) / 256, sm_count() * 16ull)));
                k_hll_narrow<<<g2, 256, 0, s>>>(regs.as<unsigned int>(), n_regs, d_registers);
                HG_CUDA(cudaGetLastError());
                // the staging buffers are freed when this call returns: finish their use first
                HG_CUDA(cudaStreamSynchronize(s));
            });
    }

} // extern "C"
