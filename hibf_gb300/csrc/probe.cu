// probe.cu -- the memory system's random-access ceiling, measured live.
//
// The query kernels read rows of a few bytes at uniformly random addresses of IBFs that are gigabytes large.  A
// copy-bandwidth peak overstates what such reads can reach: every read moves at least one DRAM access unit and
// misses the TLBs once the footprint outgrows their reach.  This probe times independent random 8-byte reads over
// a buffer of a given footprint -- fully random, or confined to windows of `region_bytes` that change every few
// reads -- so the query kernel's rate can be set against the hardware's own random-read rate.

#include <algorithm>

#include "../../include/hibf_gb300_diagnostics.h"
#include "common.hpp"

namespace hibf_gb300
{
int sm_count();

namespace
{

__device__ __forceinline__ uint64_t probe_mix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// Each thread issues `iters` pairs of independent reads; every index is reduced modulo the window, so all reads
// stay inside the buffer.
__global__ void k_probe_gather(uint64_t const * __restrict__ a, uint64_t n_words, uint64_t region_words,
                               uint64_t iters, unsigned long long * sink)
{
    uint64_t const tid = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    uint64_t const warp = tid >> 5;
    uint64_t const nreg = n_words / region_words;
    uint64_t acc = 0;
    for (uint64_t it = 0; it < iters; ++it)
    {
        uint64_t const base = (probe_mix(warp * 1000003ull + it / 16) % nreg) * region_words;
        uint64_t const r0 = probe_mix(tid * 7919ull + it * 2ull);
        uint64_t const r1 = probe_mix(tid * 7919ull + it * 2ull + 1ull);
        acc ^= __ldg(a + base + r0 % region_words);
        acc ^= __ldg(a + base + r1 % region_words);
    }
    if (acc == 0x5a5a5a5a5a5a5a5aull)
        atomicAdd(sink, 1ull);
}

} // namespace
} // namespace hibf_gb300

using namespace hibf_gb300;

extern "C"
{

    int hibf_gpu_probe_random_reads(uint64_t footprint_bytes, uint64_t region_bytes, double * reads_per_s)
    {
        return guarded(
            [&]
            {
                if (!reads_per_s || footprint_bytes < 4096)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                require_device();
                uint64_t const n_words = footprint_bytes / 8;
                uint64_t const region_words = region_bytes ? std::min<uint64_t>(region_bytes / 8, n_words) : n_words;
                if (region_words == 0)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "region too small");
                dbuf buf, sink;
                buf.ensure(n_words * 8);
                sink.ensure(8);
                cudaStream_t s = nullptr;
                HG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
                cudaEvent_t e0 = nullptr, e1 = nullptr;
                try
                {
                    HG_CUDA(cudaMemsetAsync(buf.p, 1, n_words * 8, s));
                    HG_CUDA(cudaEventCreate(&e0));
                    HG_CUDA(cudaEventCreate(&e1));
                    unsigned const grid = static_cast<unsigned>(sm_count()) * 8u, block = 256;
                    uint64_t const iters = 256;
                    k_probe_gather<<<grid, block, 0, s>>>(buf.as<uint64_t>(), n_words, region_words, iters,
                                                          sink.as<unsigned long long>());
                    HG_CUDA(cudaGetLastError());
                    HG_CUDA(cudaEventRecord(e0, s));
                    for (int r = 0; r < 3; ++r)
                        k_probe_gather<<<grid, block, 0, s>>>(buf.as<uint64_t>(), n_words, region_words, iters,
                                                              sink.as<unsigned long long>());
                    HG_CUDA(cudaGetLastError());
                    HG_CUDA(cudaEventRecord(e1, s));
                    HG_CUDA(cudaEventSynchronize(e1));
                    float ms = 0;
                    HG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                    double const reads = 3.0 * grid * block * iters * 2.0;
                    *reads_per_s = reads / (ms / 1e3);
                }
                catch (...)
                {
                    if (e0)
                        cudaEventDestroy(e0);
                    if (e1)
                        cudaEventDestroy(e1);
                    cudaStreamDestroy(s);
                    throw;
                }
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                cudaStreamDestroy(s);
            });
    }

} // extern "C"
