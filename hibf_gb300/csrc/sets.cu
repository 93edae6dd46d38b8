// sets.cu -- the build front end's set materialisation on the device.
//
// The reference reads every user bin into a hash set (compute_kmers, src/build/compute_kmers.cpp:23-32) and sizes a
// merged max bin by the distinct count of its subtree's union (src/hierarchical_interleaved_bloom_filter.cpp:39-171,
// the favourite child's kmers).  Here both are sorts on the device:
//   distinct_sets_device  every user bin's distinct values in first-appearance order: a segmented radix sort of
//                         (value, position in the bin) per bin (stable, so equal values keep input order), a flag
//                         on the first of every run, the flagged positions compacted and sorted back into input
//                         order, and the values gathered at them;
//   union_size_device     the distinct count of the union of some user bins' sets: one sort of their
//                         concatenation and a count of run starts.
// Only the order of split user bins' values depends on the reference's hash set (robin_hood iteration order); the
// host replays that from the first-appearance order these produce.
#include <algorithm>
#include <vector>

#include <cub/cub.cuh>

#include "common.hpp"

namespace hibf_gb300
{
int sm_count();

namespace
{

constexpr uint64_t kBatchValues = 1ull << 30; // values per device batch (CUB's segmented sort counts items in int)

// Position p of segment s: its index within the segment, and its segment.
__global__ void k_segment_index(int const * __restrict__ seg_off, uint32_t n_seg, uint32_t * __restrict__ idx,
                                uint32_t * __restrict__ seg)
{
    for (uint32_t s = blockIdx.x; s < n_seg; s += gridDim.x)
    {
        int const b = seg_off[s], e = seg_off[s + 1];
        for (int p = b + static_cast<int>(threadIdx.x); p < e; p += static_cast<int>(blockDim.x))
        {
            idx[p] = static_cast<uint32_t>(p - b);
            seg[p] = s;
        }
    }
}

// After the segmented sort: flag the first of every run of equal values within a segment and record its position
// in the batch (segment start + index in the segment).
__global__ void k_first_of_run(uint64_t const * __restrict__ keys, uint32_t const * __restrict__ idx,
                               uint32_t const * __restrict__ seg, int const * __restrict__ seg_off, uint64_t n,
                               uint64_t * __restrict__ pos, unsigned char * __restrict__ flag)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        uint32_t const s = seg[i];
        bool const first = i == 0 || seg[i - 1] != s || keys[i - 1] != keys[i];
        flag[i] = first ? 1 : 0;
        pos[i] = static_cast<uint64_t>(seg_off[s]) + idx[i];
    }
}

__global__ void k_gather(uint64_t const * __restrict__ values, uint64_t const * __restrict__ pos, uint64_t n,
                         uint64_t * __restrict__ out)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        out[i] = values[pos[i]];
}

// Number of i with i == 0 or keys[i] != keys[i - 1] (keys sorted).
__global__ void k_count_runs(uint64_t const * __restrict__ keys, uint64_t n, unsigned long long * __restrict__ out)
{
    unsigned long long c = 0;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        c += (i == 0 || keys[i - 1] != keys[i]) ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1)
        c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c)
        atomicAdd(out, c);
}

unsigned grid_for(uint64_t n)
{
    return static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, sm_count() * 8ull)));
}

} // namespace

bool device_present()
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    {
        (void)cudaGetLastError();
        return false;
    }
    return true;
}

void distinct_sets_device(uint64_t const * values, std::vector<uint64_t> const & offsets,
                          std::vector<std::vector<uint64_t>> & sets)
{
    uint64_t const nub = offsets.size() - 1;
    sets.assign(nub, {});
    cudaStream_t s = nullptr;
    HG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct stream_guard
    {
        cudaStream_t s;
        ~stream_guard()
        {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    } const guard{s};
    dbuf d_in, d_keys, d_idx_in, d_idx, d_seg, d_off, d_pos, d_flag, d_sel, d_sorted, d_out, d_nsel, d_tmp;
    hbuf h_out;
    for (uint64_t u0 = 0; u0 < nub;)
    {
        // a batch of whole user bins, at most kBatchValues values unless one bin alone is larger
        uint64_t u1 = u0 + 1;
        while (u1 < nub && offsets[u1 + 1] - offsets[u0] <= kBatchValues)
            ++u1;
        uint64_t const base = offsets[u0];
        uint64_t const m = offsets[u1] - base;
        if (m >= (1ull << 31))
            fail(HIBF_GPU_ERR_INVALID_ARG, "a user bin of 2^31 or more values");
        uint32_t const nseg = static_cast<uint32_t>(u1 - u0);
        if (m == 0)
        {
            u0 = u1;
            continue;
        }
        std::vector<int> off(nseg + 1);
        for (uint32_t k = 0; k <= nseg; ++k)
            off[k] = static_cast<int>(offsets[u0 + k] - base);
        d_in.ensure(m * 8);
        d_keys.ensure(m * 8);
        d_idx_in.ensure(m * 4);
        d_idx.ensure(m * 4);
        d_seg.ensure(m * 4);
        d_off.ensure((nseg + 1) * sizeof(int));
        d_pos.ensure(m * 8);
        d_flag.ensure(m);
        d_sel.ensure(m * 8);
        d_sorted.ensure(m * 8);
        d_out.ensure(m * 8);
        d_nsel.ensure(8);
        HG_CUDA(cudaMemcpyAsync(d_in.p, values + base, m * 8, cudaMemcpyHostToDevice, s));
        HG_CUDA(cudaMemcpyAsync(d_off.p, off.data(), (nseg + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
        k_segment_index<<<std::min<uint32_t>(nseg, 65535u), 256, 0, s>>>(d_off.as<int>(), nseg, d_idx_in.as<uint32_t>(),
                                                                       d_seg.as<uint32_t>());
        HG_CUDA(cudaGetLastError());
        int const * begin = d_off.as<int>();
        int const * end = d_off.as<int>() + 1;
        size_t t1 = 0, t2 = 0, t3 = 0;
        HG_CUDA(cub::DeviceSegmentedRadixSort::SortPairs(nullptr, t1, d_in.as<uint64_t>(), d_keys.as<uint64_t>(),
                                                         d_idx_in.as<uint32_t>(), d_idx.as<uint32_t>(),
                                                         static_cast<int>(m), static_cast<int>(nseg), begin, end, 0,
                                                         64, s));
        HG_CUDA(cub::DeviceSelect::Flagged(nullptr, t2, d_pos.as<uint64_t>(), d_flag.as<unsigned char>(),
                                           d_sel.as<uint64_t>(), d_nsel.as<unsigned long long>(), m, s));
        HG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, t3, d_sel.as<uint64_t>(), d_sorted.as<uint64_t>(), m, 0, 64,
                                               s));
        d_tmp.ensure(std::max({t1, t2, t3}));
        HG_CUDA(cub::DeviceSegmentedRadixSort::SortPairs(d_tmp.p, t1, d_in.as<uint64_t>(), d_keys.as<uint64_t>(),
                                                         d_idx_in.as<uint32_t>(), d_idx.as<uint32_t>(),
                                                         static_cast<int>(m), static_cast<int>(nseg), begin, end, 0,
                                                         64, s));
        k_first_of_run<<<grid_for(m), 256, 0, s>>>(d_keys.as<uint64_t>(), d_idx.as<uint32_t>(), d_seg.as<uint32_t>(),
                                                   d_off.as<int>(), m, d_pos.as<uint64_t>(),
                                                   d_flag.as<unsigned char>());
        HG_CUDA(cudaGetLastError());
        HG_CUDA(cub::DeviceSelect::Flagged(d_tmp.p, t2, d_pos.as<uint64_t>(), d_flag.as<unsigned char>(),
                                           d_sel.as<uint64_t>(), d_nsel.as<unsigned long long>(), m, s));
        unsigned long long nsel = 0;
        HG_CUDA(cudaMemcpyAsync(&nsel, d_nsel.p, 8, cudaMemcpyDeviceToHost, s));
        HG_CUDA(cudaStreamSynchronize(s));
        // positions ascending = user bins in order, each in first-appearance order
        HG_CUDA(cub::DeviceRadixSort::SortKeys(d_tmp.p, t3, d_sel.as<uint64_t>(), d_sorted.as<uint64_t>(), nsel, 0, 64,
                                               s));
        k_gather<<<grid_for(nsel), 256, 0, s>>>(d_in.as<uint64_t>(), d_sorted.as<uint64_t>(), nsel,
                                                d_out.as<uint64_t>());
        HG_CUDA(cudaGetLastError());
        std::vector<uint64_t> pos(nsel);
        h_out.ensure(std::max<uint64_t>(nsel, 1) * 8);
        HG_CUDA(cudaMemcpyAsync(h_out.p, d_out.p, nsel * 8, cudaMemcpyDeviceToHost, s));
        HG_CUDA(cudaMemcpyAsync(pos.data(), d_sorted.p, nsel * 8, cudaMemcpyDeviceToHost, s));
        HG_CUDA(cudaStreamSynchronize(s));
        uint64_t const * dist = h_out.as<uint64_t>();
        for (uint32_t k = 0; k < nseg; ++k)
        {
            auto const a = std::lower_bound(pos.begin(), pos.end(), static_cast<uint64_t>(off[k]));
            auto const b = std::lower_bound(pos.begin(), pos.end(), static_cast<uint64_t>(off[k + 1]));
            sets[u0 + k].assign(dist + (a - pos.begin()), dist + (b - pos.begin()));
        }
        u0 = u1;
    }
}

uint64_t union_size_device(std::vector<std::vector<uint64_t>> const & sets, std::vector<uint64_t> const & members)
{
    uint64_t n = 0;
    for (uint64_t u : members)
        n += sets[u].size();
    if (n == 0)
        return 0;
    cudaStream_t s = nullptr;
    HG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct stream_guard
    {
        cudaStream_t s;
        ~stream_guard()
        {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    } const guard{s};
    dbuf d_in, d_sorted, d_tmp, d_count;
    d_in.ensure(n * 8);
    d_sorted.ensure(n * 8);
    d_count.ensure(8);
    uint64_t at = 0;
    for (uint64_t u : members)
    {
        if (!sets[u].empty())
            HG_CUDA(cudaMemcpyAsync(d_in.as<uint64_t>() + at, sets[u].data(), sets[u].size() * 8,
                                    cudaMemcpyHostToDevice, s));
        at += sets[u].size();
    }
    size_t t = 0;
    HG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, t, d_in.as<uint64_t>(), d_sorted.as<uint64_t>(), n, 0, 64, s));
    d_tmp.ensure(t);
    HG_CUDA(cub::DeviceRadixSort::SortKeys(d_tmp.p, t, d_in.as<uint64_t>(), d_sorted.as<uint64_t>(), n, 0, 64, s));
    HG_CUDA(cudaMemsetAsync(d_count.p, 0, 8, s));
    k_count_runs<<<grid_for(n), 256, 0, s>>>(d_sorted.as<uint64_t>(), n, d_count.as<unsigned long long>());
    HG_CUDA(cudaGetLastError());
    unsigned long long c = 0;
    HG_CUDA(cudaMemcpyAsync(&c, d_count.p, 8, cudaMemcpyDeviceToHost, s));
    HG_CUDA(cudaStreamSynchronize(s));
    return c;
}

} // namespace hibf_gb300
