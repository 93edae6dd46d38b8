// synth.cu -- seeded synthetic workloads (include/hibf_gb300_synthetic.h) on the host and on the device.
//
// Benchmark and test support: the same generator functions run in the host entry points and in the device kernel,
// so a workload generated on the GPU equals the one the CPU oracle generates.

#include <algorithm>
#include <cstring>

#include "../../include/hibf_gb300_synthetic.h"
#include "common.hpp"

namespace hibf_gb300
{
int sm_count();

namespace
{

// One thread per query: each query's values come from its own sequential splitmix64 state.
__global__ void k_synth_queries(hg_query_spec spec, uint64_t const * __restrict__ ub_offsets, uint64_t first,
                                uint64_t n, uint64_t const * __restrict__ qoff, uint64_t * __restrict__ out)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        hg_query_values(&spec, ub_offsets, first + i, out + qoff[i]);
}

__global__ void k_synth_ibf_queries(uint64_t seed, uint64_t n_bins, uint64_t vpb, uint64_t first, uint64_t n,
                                    uint64_t * __restrict__ out)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        out[i] = hg_ibf_query_value(seed, n_bins, vpb, first + i);
}

hg_query_spec make_spec(uint64_t seed, int law, uint64_t len_lo, uint64_t len_hi, uint32_t mix_pct,
                        uint32_t noise_pct, uint32_t thr_num, uint32_t thr_den, uint64_t n_user_bins)
{
    if (law != HG_QUERIES_HALF_ONE_BIN && law != HG_QUERIES_MIXED)
        fail(HIBF_GPU_ERR_INVALID_ARG, "unknown query law");
    if (thr_den == 0 || n_user_bins == 0 || len_hi < len_lo)
        fail(HIBF_GPU_ERR_INVALID_ARG, "bad query parameters");
    hg_query_spec s{};
    s.seed = seed;
    s.law = law;
    s.len_lo = len_lo;
    s.len_hi = len_hi;
    s.mix_pct = mix_pct;
    s.noise_pct = noise_pct;
    s.thr_num = thr_num;
    s.thr_den = thr_den;
    s.n_user_bins = n_user_bins;
    return s;
}

} // namespace
} // namespace hibf_gb300

using namespace hibf_gb300;

extern "C"
{

    int hibf_gpu_synth_user_bin_offsets(uint64_t seed, int law, double p0, double p1, uint64_t lo, uint64_t hi,
                                        uint64_t n_user_bins, uint64_t * offsets)
    {
        return guarded(
            [&]
            {
                if (!offsets || lo == 0 || hi < lo)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                offsets[0] = 0;
                for (uint64_t i = 0; i < n_user_bins; ++i)
                    offsets[i + 1] = offsets[i] + hg_user_bin_size(seed, law, p0, p1, lo, hi, i);
            });
    }

    int hibf_gpu_synth_query_offsets(uint64_t seed, int law, uint64_t len_lo, uint64_t len_hi, uint32_t mix_pct,
                                     uint32_t noise_pct, uint32_t thr_num, uint32_t thr_den, uint64_t n_user_bins,
                                     uint64_t first_query, uint64_t n_queries, uint64_t * query_offsets,
                                     uint64_t * thresholds)
    {
        return guarded(
            [&]
            {
                if (!query_offsets)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                hg_query_spec const s =
                    make_spec(seed, law, len_lo, len_hi, mix_pct, noise_pct, thr_num, thr_den, n_user_bins);
                query_offsets[0] = 0;
                for (uint64_t i = 0; i < n_queries; ++i)
                {
                    uint64_t const len = hg_query_length(&s, first_query + i);
                    query_offsets[i + 1] = query_offsets[i] + len;
                    if (thresholds)
                        thresholds[i] = hg_query_threshold(&s, len);
                }
            });
    }

    int hibf_gpu_synth_queries(uint64_t seed, int law, uint64_t len_lo, uint64_t len_hi, uint32_t mix_pct,
                               uint32_t noise_pct, uint32_t thr_num, uint32_t thr_den, uint64_t n_user_bins,
                               uint64_t const * user_bin_offsets, uint64_t first_query, uint64_t n_queries,
                               uint64_t const * query_offsets, uint64_t * values)
    {
        return guarded(
            [&]
            {
                if (!user_bin_offsets || !query_offsets || (n_queries && !values))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                hg_query_spec const s =
                    make_spec(seed, law, len_lo, len_hi, mix_pct, noise_pct, thr_num, thr_den, n_user_bins);
                for (uint64_t i = 0; i < n_queries; ++i)
                    hg_query_values(&s, user_bin_offsets, first_query + i, values + query_offsets[i]);
            });
    }

    int hibf_gpu_synth_queries_d(uint64_t seed, int law, uint64_t len_lo, uint64_t len_hi, uint32_t mix_pct,
                                 uint32_t noise_pct, uint32_t thr_num, uint32_t thr_den, uint64_t n_user_bins,
                                 uint64_t const * d_user_bin_offsets, uint64_t first_query, uint64_t n_queries,
                                 uint64_t const * d_query_offsets, uint64_t * d_values, void * stream)
    {
        return guarded(
            [&]
            {
                if (!d_user_bin_offsets || !d_query_offsets || (n_queries && !d_values))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                hg_query_spec const s =
                    make_spec(seed, law, len_lo, len_hi, mix_pct, noise_pct, thr_num, thr_den, n_user_bins);
                if (!n_queries)
                    return;
                unsigned const block = 128;
                unsigned const grid = static_cast<unsigned>(
                    std::min<uint64_t>((n_queries + block - 1) / block, static_cast<uint64_t>(sm_count()) * 32));
                k_synth_queries<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(s, d_user_bin_offsets,
                                                                                      first_query, n_queries,
                                                                                      d_query_offsets, d_values);
                HG_CUDA(cudaGetLastError());
            });
    }

    int hibf_gpu_synth_ibf_queries(uint64_t seed, uint64_t n_bins, uint64_t values_per_bin, uint64_t first,
                                   uint64_t n, uint64_t * values)
    {
        return guarded(
            [&]
            {
                if ((n && !values) || n_bins == 0 || values_per_bin == 0)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                for (uint64_t i = 0; i < n; ++i)
                    values[i] = hg_ibf_query_value(seed, n_bins, values_per_bin, first + i);
            });
    }

    int hibf_gpu_synth_ibf_queries_d(uint64_t seed, uint64_t n_bins, uint64_t values_per_bin, uint64_t first,
                                     uint64_t n, uint64_t * d_values, void * stream)
    {
        return guarded(
            [&]
            {
                if ((n && !d_values) || n_bins == 0 || values_per_bin == 0)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                if (!n)
                    return;
                unsigned const block = 256;
                unsigned const grid = static_cast<unsigned>(
                    std::min<uint64_t>((n + block - 1) / block, static_cast<uint64_t>(sm_count()) * 16));
                k_synth_ibf_queries<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(seed, n_bins,
                                                                                          values_per_bin, first, n,
                                                                                          d_values);
                HG_CUDA(cudaGetLastError());
            });
    }

} // extern "C"
