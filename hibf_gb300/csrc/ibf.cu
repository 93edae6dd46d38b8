// ibf.cu -- single-level interleaved Bloom filter on the device: store, emplace/clear/widen kernels, the plain
// (one launch per call) query kernels, and their C-ABI entry points (include/hibf_gb300.h).
//
// Reference interface: seqan::hibf::interleaved_bloom_filter (include/hibf/interleaved_bloom_filter.hpp,
// src/interleaved_bloom_filter.cpp).

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cub/cub.cuh>

#include "../../include/hibf_gb300_synthetic.h"
#include "archive.hpp"
#include "common.hpp"
#include "count.cuh"
#include "device.cuh"

namespace hibf_gb300
{

thread_local std::string g_last_error;

void set_last_error(std::string msg)
{
    g_last_error = std::move(msg);
}

// ---------------------------------------------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------------------------------------------

// emplace (src/interleaved_bloom_filter.cpp:119-140).  One thread per value; atomicOr makes concurrent inserts
// order-independent.  The old words are not needed (an IBF that tracks occupancy inserts through emplace_exact), so
// the atomics return nothing and a warp never waits on them.
__global__ void k_emplace(uint64_t * __restrict__ words, uint64_t bin_size, uint32_t row_words, uint32_t shift,
                          uint32_t h, uint64_t const * __restrict__ values, uint64_t const * __restrict__ bins,
                          uint64_t n, uint64_t bin, uint64_t n_bins, int * bad_bin)
{
    uint64_t const stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        uint64_t const v = values[i];
        uint64_t const b = bins ? bins[i] : bin;
        if (b >= n_bins)
        {
            *bad_bin = 1; // device-supplied bin index out of range: skipped, reported by hibf_gpu_ibf_status
            continue;
        }
        uint64_t const bit = 1ull << (b & 63u);
        uint64_t const wofs = b >> 6;
        for (uint32_t k = 0; k < h; ++k)
        {
            uint64_t const r = hash_row(v, c_hash_seeds[k], shift, bin_size);
            atomicOr(reinterpret_cast<unsigned long long *>(words + r * row_words + wofs),
                     static_cast<unsigned long long>(bit));
        }
    }
}

// emplace of the synthetic single-level workload: value i of the launch is hg_ibf_bin_value of bin
// first_bin + i / vpb, generated in place instead of read (same bits as k_emplace with those values; the atomics
// return nothing).
__global__ void k_synth_emplace(uint64_t * __restrict__ words, uint64_t bin_size, uint32_t row_words, uint32_t shift,
                                uint32_t h, uint64_t seed, uint64_t vpb, uint64_t first_bin, uint64_t n)
{
    uint64_t const stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        uint64_t const b = first_bin + i / vpb;
        uint64_t const v = hg_ibf_bin_value(seed, vpb, b, i % vpb);
        uint64_t const bit = 1ull << (b & 63u);
        uint64_t const wofs = b >> 6;
        for (uint32_t k = 0; k < h; ++k)
        {
            uint64_t const r = hash_row(v, c_hash_seeds[k], shift, bin_size);
            atomicOr(reinterpret_cast<unsigned long long *>(words + r * row_words + wofs),
                     static_cast<unsigned long long>(bit));
        }
    }
}

// ---------------------------------------------------------------------------------------------------------------
// Exact occupancy.  The reference counts a value for its bin when one of its bits was not set yet, inserting one value
// after the other (src/interleaved_bloom_filter.cpp:119-140).  With concurrent atomicOr that depends on timing, so an
// IBF that tracks occupancy inserts in chunks: every (value, hash) position of the chunk becomes a key row * tb + bin,
// a stable sort groups equal positions in insertion order, and a value counts when it is the first of the chunk at a
// position that was unset before the chunk.  Then the bits are set.
// ---------------------------------------------------------------------------------------------------------------
constexpr uint64_t kNoPosition = ~0ull;

template <bool SYNTH>
__global__ void k_occ_keys(uint64_t const * __restrict__ words, uint64_t bin_size, uint32_t row_words, uint32_t shift,
                           uint32_t h, uint64_t const * __restrict__ values, uint64_t const * __restrict__ bins,
                           uint64_t seed, uint64_t vpb, uint64_t first, uint64_t n, uint64_t bin, uint64_t n_bins,
                           uint64_t tb, unsigned long long * __restrict__ keys, unsigned long long * __restrict__ ids,
                           uint8_t * __restrict__ was_set, uint64_t * __restrict__ gen_values)
{
    uint64_t const stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        uint64_t v, b;
        if constexpr (SYNTH)
        {
            b = bin;
            v = hg_ibf_bin_value(seed, vpb, bin, first + i);
            gen_values[i] = v;
        }
        else
        {
            v = values[i];
            b = bins ? bins[i] : bin;
        }
        for (uint32_t k = 0; k < h; ++k)
        {
            uint64_t const idx = i * h + k;
            ids[idx] = idx;
            if (b >= n_bins)
            {
                keys[idx] = kNoPosition;
                was_set[idx] = 1;
                continue;
            }
            uint64_t const r = hash_row(v, c_hash_seeds[k], shift, bin_size);
            keys[idx] = r * tb + b;
            was_set[idx] = static_cast<uint8_t>((words[r * row_words + (b >> 6)] >> (b & 63u)) & 1u);
        }
    }
}

__global__ void k_occ_first(unsigned long long const * __restrict__ keys, unsigned long long const * __restrict__ ids,
                            uint64_t m, uint32_t h, uint8_t const * __restrict__ was_set,
                            unsigned int * __restrict__ newly)
{
    uint64_t const stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < m; j += stride)
    {
        if (keys[j] == kNoPosition || (j > 0 && keys[j] == keys[j - 1]))
            continue;
        uint64_t const idx = ids[j];
        if (!was_set[idx])
            newly[idx / h] = 1u;
    }
}

template <bool SYNTH>
__global__ void k_occ_count(unsigned int const * __restrict__ newly, uint64_t const * __restrict__ bins, uint64_t vpb,
                            uint64_t first, uint64_t n, uint64_t bin, uint64_t n_bins,
                            unsigned long long * __restrict__ occupancy)
{
    uint64_t const stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        uint64_t const b = SYNTH ? bin : (bins ? bins[i] : bin);
        if (newly[i] && b < n_bins)
            atomicAdd(occupancy + b, 1ull);
    }
}

// clear(bin) (src/interleaved_bloom_filter.cpp:142-148): clear one bit of every row.
__global__ void k_clear_bin(uint64_t * __restrict__ words, uint64_t bin_size, uint32_t row_words, uint64_t word,
                            uint64_t keep)
{
    uint64_t const stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t r = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; r < bin_size; r += stride)
        atomicAnd(reinterpret_cast<unsigned long long *>(words + r * row_words + word), keep);
}

// clear(range) (include/hibf/interleaved_bloom_filter.hpp:283-297): per row, clear the listed bins word by word.
__global__ void k_clear_words(uint64_t * __restrict__ words, uint64_t bin_size, uint32_t row_words,
                              uint32_t const * __restrict__ widx, uint64_t const * __restrict__ keep, uint32_t nw)
{
    uint64_t const total = bin_size * nw;
    uint64_t const stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < total; i += stride)
    {
        uint64_t const r = i / nw;
        uint32_t const e = static_cast<uint32_t>(i % nw);
        atomicAnd(reinterpret_cast<unsigned long long *>(words + r * row_words + widx[e]), keep[e]);
    }
}

// increase_bin_number_to (src/interleaved_bloom_filter.cpp:163-202): old row r becomes the first words of new row r.
__global__ void k_widen(uint64_t * __restrict__ dst, uint32_t dst_row_words, uint64_t const * __restrict__ src,
                        uint32_t src_row_words, uint32_t copy_words, uint64_t bin_size)
{
    uint64_t const total = bin_size * dst_row_words;
    uint64_t const stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < total; i += stride)
    {
        uint64_t const r = i / dst_row_words;
        uint32_t const w = static_cast<uint32_t>(i % dst_row_words);
        dst[i] = w < copy_words ? src[r * src_row_words + w] : 0u;
    }
}

// bulk_contains (src/interleaved_bloom_filter.cpp:204-291) for many values: out[v * bin_words + j] = AND of word j
// of the h rows.  LPV lanes per value, one row word per lane per pass (strided when the row is wider than a warp).
template <int LPV>
__global__ void k_bulk_contains(row_params rp, uint64_t const * __restrict__ values, uint64_t n,
                                uint64_t * __restrict__ out)
{
    constexpr int G = 32 / LPV;
    int const lane = threadIdx.x & 31;
    int const g = lane / LPV;
    int const j = lane % LPV;
    uint64_t const warp = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
    uint64_t const nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
    for (uint64_t base = warp * G; base < n; base += nwarps * G)
    {
        uint64_t const i = base + g;
        if (i >= n)
            continue;
        uint64_t const v = values[i];
        uint64_t off[5];
#pragma unroll
        for (int k = 0; k < 5; ++k)
            off[k] = (static_cast<uint32_t>(k) < rp.hash_funs)
                       ? hash_row(v, c_hash_seeds[k], rp.hash_shift, rp.bin_size) * rp.row_words
                       : 0u;
        for (uint32_t w = j; w < rp.bin_words; w += LPV)
        {
            uint64_t x = ~0ull;
#pragma unroll
            for (int k = 0; k < 5; ++k)
                if (static_cast<uint32_t>(k) < rp.hash_funs)
                    x &= __ldg(rp.words + off[k] + w);
            out[i * rp.bin_words + w] = x;
        }
    }
}

// bulk_contains for rows of up to 32 words with H hash functions: the same work mapping as the counting loop
// (count.cuh) -- LPV lanes per row, lanes hash U values each, the H row words of four sub-steps are loaded together
// (4 * H loads per lane in flight) -- and each lane stores its word of the AND.
template <int LPV, int H>
__global__ void __launch_bounds__(256) k_bulk_contains_h(row_params rp, uint64_t const * __restrict__ values,
                                                         uint64_t n, uint64_t * __restrict__ out)
{
    constexpr int G = 32 / LPV;
    constexpr int U = LPV >= 4 ? 1 : 4 / LPV;
    constexpr int STEPS = U * LPV;
    constexpr int BLOCK = 32 * U;
    int const lane = threadIdx.x & 31;
    int const g = lane / LPV;
    int const j = lane % LPV;
    bool const wj = static_cast<uint32_t>(j) < rp.bin_words;
    uint64_t const bw = rp.bin_words;
    uint64_t const * __restrict__ words = rp.words + j;
    uint64_t const warp = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
    uint64_t const nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
    for (uint64_t base = warp * BLOCK; base < n; base += nwarps * BLOCK)
    {
        uint64_t off[U][H];
#pragma unroll
        for (int u = 0; u < U; ++u)
        {
            uint64_t const idx = base + static_cast<uint64_t>(u * 32 + lane);
            uint64_t const v = idx < n ? values[idx] : 0u;
#pragma unroll
            for (int i = 0; i < H; ++i)
                off[u][i] = hash_row(v, c_hash_seeds[i], rp.hash_shift, rp.bin_size) * rp.row_words;
        }
#pragma unroll 1
        for (int s = 0; s < STEPS; s += 4)
        {
            uint64_t w[4][H];
            uint64_t idx[4];
            bool ok[4];
#pragma unroll
            for (int t = 0; t < 4; ++t)
            {
                int const step = s + t;
                int const u = U == 1 ? 0 : step / LPV;
                int const src = (step % LPV) * G + g;
                idx[t] = base + static_cast<uint64_t>(u * 32 + src);
                ok[t] = wj && idx[t] < n;
#pragma unroll
                for (int i = 0; i < H; ++i)
                {
                    uint64_t o = off[u][i];
                    if constexpr (LPV > 1)
                        o = __shfl_sync(kFullMask, o, src);
                    w[t][i] = ok[t] ? ldg_evict_first(words + o) : 0ull;
                }
            }
#pragma unroll
            for (int t = 0; t < 4; ++t)
            {
                uint64_t x = w[t][0];
#pragma unroll
                for (int i = 1; i < H; ++i)
                    x &= w[t][i];
                if (ok[t])
                    out[idx[t] * bw + j] = x;
            }
        }
    }
}

template <int H>
void launch_contains_h(row_params const & rp, uint32_t lpv_log2, uint64_t const * d_values, uint64_t n,
                       uint64_t * d_out, unsigned grid, cudaStream_t s)
{
    switch (lpv_log2)
    {
    case 0:
        k_bulk_contains_h<1, H><<<grid, 256, 0, s>>>(rp, d_values, n, d_out);
        break;
    case 1:
        k_bulk_contains_h<2, H><<<grid, 256, 0, s>>>(rp, d_values, n, d_out);
        break;
    case 2:
        k_bulk_contains_h<4, H><<<grid, 256, 0, s>>>(rp, d_values, n, d_out);
        break;
    case 3:
        k_bulk_contains_h<8, H><<<grid, 256, 0, s>>>(rp, d_values, n, d_out);
        break;
    case 4:
        k_bulk_contains_h<16, H><<<grid, 256, 0, s>>>(rp, d_values, n, d_out);
        break;
    default:
        k_bulk_contains_h<32, H><<<grid, 256, 0, s>>>(rp, d_values, n, d_out);
    }
}

// bulk_count over n values into one counting vector: every warp counts a contiguous chunk into the block's shared
// counters, the block adds them to 64-bit global totals.
// Four blocks per SM (64 registers, some spilled for h >= 3) measured faster than two blocks without spills (1.53 vs
// 2.16 ms for 2^24 values on 1,024 bins, h = 3): more warps keep more row loads in flight.  PRIVATE: every warp
// flushes into counters of its own (no shared-memory atomics), summed by the block at the end; otherwise the block's
// warps share one set of counters.
template <int H, bool PRIVATE>
__global__ void __launch_bounds__(256, 4)
    k_bulk_count(row_params rp, uint32_t lpv_log2, uint64_t const * __restrict__ values, uint64_t n, uint64_t chunk,
                 unsigned long long * __restrict__ totals, uint32_t n_counters)
{
    extern __shared__ uint32_t s_counts[];
    int const nwarps_block = blockDim.x >> 5;
    uint32_t const n_smem = PRIVATE ? n_counters * nwarps_block : n_counters;
    for (uint32_t i = threadIdx.x; i < n_smem; i += blockDim.x)
        s_counts[i] = 0;
    __syncthreads();
    int const lane = threadIdx.x & 31;
    uint32_t * counts = PRIVATE ? s_counts + (threadIdx.x >> 5) * n_counters : s_counts;
    uint64_t const warp = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
    uint64_t const nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
    for (uint64_t start = warp * chunk; start < n; start += nwarps * chunk)
    {
        uint64_t const len = (n - start) < chunk ? (n - start) : chunk;
        if (PRIVATE && rp.bin_words <= 32)
            warp_count_lpv<H, false, true>(rp, lpv_log2, values + start, len, counts, lane);
        else
            warp_count_h<H, true>(rp, lpv_log2, values + start, len, counts, lane);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n_counters; i += blockDim.x)
    {
        uint64_t sum = 0;
        for (int w = 0; w < (PRIVATE ? nwarps_block : 1); ++w)
            sum += s_counts[w * n_counters + i];
        if (sum)
            atomicAdd(totals + i, static_cast<unsigned long long>(sum));
    }
}

// Reduce exact totals modulo the counter width (the reference's counting_vector wraps).
__global__ void k_store_counts(unsigned long long const * __restrict__ totals, uint64_t bins, int width, void * out)
{
    for (uint64_t b = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; b < bins;
         b += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        uint64_t const t = totals[b];
        switch (width)
        {
        case 1:
            static_cast<uint8_t *>(out)[b] = static_cast<uint8_t>(t);
            break;
        case 2:
            static_cast<uint16_t *>(out)[b] = static_cast<uint16_t>(t);
            break;
        case 4:
            static_cast<uint32_t *>(out)[b] = static_cast<uint32_t>(t);
            break;
        default:
            static_cast<uint64_t *>(out)[b] = t;
        }
    }
}

using bulk_count_kernel_t = void (*)(row_params, uint32_t, uint64_t const *, uint64_t, uint64_t,
                                     unsigned long long *, uint32_t);

// Warp-private counters when eight sets fit in 96 KiB of shared memory (up to 3,072 technical bins).
constexpr uint32_t kPrivateCountersMax = 3072;

bulk_count_kernel_t bulk_count_kernel(uint64_t h, bool priv)
{
    switch (h)
    {
    case 1:
        return priv ? k_bulk_count<1, true> : k_bulk_count<1, false>;
    case 2:
        return priv ? k_bulk_count<2, true> : k_bulk_count<2, false>;
    case 3:
        return priv ? k_bulk_count<3, true> : k_bulk_count<3, false>;
    case 4:
        return priv ? k_bulk_count<4, true> : k_bulk_count<4, false>;
    default:
        return priv ? k_bulk_count<5, true> : k_bulk_count<5, false>;
    }
}

int sm_count()
{
    static int n = []
    {
        int dev = 0, c = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) !=
                                                      cudaSuccess)
            return 132;
        return c;
    }();
    return n;
}

inline unsigned grid_for(uint64_t work, unsigned block)
{
    uint64_t const want = (work + block - 1) / block;
    uint64_t const cap = static_cast<uint64_t>(sm_count()) * 16u;
    return static_cast<unsigned>(std::max<uint64_t>(1, std::min(want, cap)));
}

} // namespace hibf_gb300

using namespace hibf_gb300;

// -----------------------------------------------------------------------------------------------------------------
// Object
// -----------------------------------------------------------------------------------------------------------------
struct hibf_gpu_ibf
{
    uint64_t bins{};
    uint64_t bin_size{};
    uint64_t hash_funs{};
    uint64_t bin_words{};
    uint64_t row_words{};
    uint32_t shift{};
    bool track_occupancy{};
    dbuf store;     // bin_size * row_words words
    dbuf occupancy; // technical_bins counters
    dbuf totals;    // technical_bins 64-bit totals (bulk_count scratch)
    dbuf io;        // staging for host-pointer calls
    dbuf io2;
    dbuf flag; // device int: an emplace saw a bin index out of range
    cudaStream_t stream{};
    int status{HIBF_GPU_OK};
    std::mutex mu;

    row_params rp() const
    {
        return row_params{store.as<uint64_t>(), bin_size, static_cast<uint32_t>(row_words),
                          static_cast<uint32_t>(bin_words), shift, static_cast<uint32_t>(hash_funs)};
    }
    uint32_t lpv_log2() const
    {
        return lanes_per_value_log2(bin_words);
    }
    uint64_t technical_bins() const
    {
        return bin_words * 64u;
    }
};

namespace
{

cudaStream_t pick(hibf_gpu_ibf * f, void * s)
{
    return s ? static_cast<cudaStream_t>(s) : f->stream;
}

// Occupancy in insertion order, chunk by chunk, then each chunk's bits; chunks run one after the other, so each sees
// the bits of the chunks before it.  SYNTH: the n values are the generated values of bin `bin` (vpb per bin).
template <bool SYNTH>
void emplace_exact(hibf_gpu_ibf * f, uint64_t const * d_values, uint64_t const * d_bins, uint64_t n, uint64_t bin,
                   uint64_t seed, uint64_t vpb, cudaStream_t s)
{
    constexpr uint64_t kChunk = 1u << 20;
    unsigned const block = 256;
    uint32_t const h = static_cast<uint32_t>(f->hash_funs);
    uint64_t const m_max = std::min(n, kChunk) * h;
    dbuf keys, keys2, ids, ids2, was_set, newly, gen, tmp;
    keys.ensure(m_max * 8);
    keys2.ensure(m_max * 8);
    ids.ensure(m_max * 8);
    ids2.ensure(m_max * 8);
    was_set.ensure(m_max);
    newly.ensure(std::min(n, kChunk) * 4);
    if (SYNTH)
        gen.ensure(std::min(n, kChunk) * 8);
    size_t tmp_bytes = 0;
    HG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.as<unsigned long long>(),
                                            keys2.as<unsigned long long>(), ids.as<unsigned long long>(),
                                            ids2.as<unsigned long long>(), static_cast<int>(m_max), 0, 64, s));
    tmp.ensure(std::max<size_t>(tmp_bytes, 16));
    uint64_t const tb = f->technical_bins();
    for (uint64_t c0 = 0; c0 < n; c0 += kChunk)
    {
        uint64_t const c = std::min(kChunk, n - c0);
        uint64_t const m = c * h;
        uint64_t const * vals = SYNTH ? gen.as<uint64_t>() : d_values + c0;
        uint64_t const * bins = (SYNTH || !d_bins) ? nullptr : d_bins + c0;
        k_occ_keys<SYNTH><<<grid_for(c, block), block, 0, s>>>(
            f->store.as<uint64_t>(), f->bin_size, static_cast<uint32_t>(f->row_words), f->shift, h,
            SYNTH ? nullptr : vals, bins, seed, vpb, c0, c, bin, f->bins, tb, keys.as<unsigned long long>(),
            ids.as<unsigned long long>(), was_set.as<uint8_t>(), SYNTH ? gen.as<uint64_t>() : nullptr);
        HG_CUDA(cudaGetLastError());
        size_t bytes = tmp_bytes;
        HG_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, bytes, keys.as<unsigned long long>(),
                                                keys2.as<unsigned long long>(), ids.as<unsigned long long>(),
                                                ids2.as<unsigned long long>(), static_cast<int>(m), 0, 64, s));
        HG_CUDA(cudaMemsetAsync(newly.p, 0, c * 4, s));
        k_occ_first<<<grid_for(m, block), block, 0, s>>>(keys2.as<unsigned long long>(), ids2.as<unsigned long long>(),
                                                         m, h, was_set.as<uint8_t>(), newly.as<unsigned int>());
        HG_CUDA(cudaGetLastError());
        k_occ_count<SYNTH><<<grid_for(c, block), block, 0, s>>>(newly.as<unsigned int>(), bins, vpb, c0, c, bin,
                                                               f->bins, f->occupancy.as<unsigned long long>());
        HG_CUDA(cudaGetLastError());
        k_emplace<<<grid_for(c, block), block, 0, s>>>(f->store.as<uint64_t>(), f->bin_size,
                                                       static_cast<uint32_t>(f->row_words), f->shift, h, vals,
                                                       SYNTH ? nullptr : bins, c, bin, f->bins, f->flag.as<int>());
        HG_CUDA(cudaGetLastError());
    }
    HG_CUDA(cudaStreamSynchronize(s)); // the scratch buffers are freed on return
}

void launch_emplace(hibf_gpu_ibf * f, uint64_t const * d_values, uint64_t const * d_bins, uint64_t n, uint64_t bin,
                    cudaStream_t s)
{
    if (n == 0)
        return;
    if (f->track_occupancy)
    {
        emplace_exact<false>(f, d_values, d_bins, n, bin, 0, 1, s);
        return;
    }
    unsigned const block = 256;
    k_emplace<<<grid_for(n, block), block, 0, s>>>(f->store.as<uint64_t>(), f->bin_size,
                                                   static_cast<uint32_t>(f->row_words), f->shift,
                                                   static_cast<uint32_t>(f->hash_funs), d_values, d_bins, n, bin,
                                                   f->bins, f->flag.as<int>());
    HG_CUDA(cudaGetLastError());
}

// Per-bin counters bulk_count accumulates for filter f (a multiple of 64, at least its technical bins).
uint64_t count_counters(hibf_gpu_ibf const * f)
{
    return 64u * (f->bin_words <= 32 ? (1u << f->lpv_log2()) : f->bin_words);
}

// bulk_count of n device values into d_out.  `totals` is device scratch for count_counters(f) 64-bit totals; null
// means the filter's own buffer (grown on demand, the only allocation here).
void launch_count(hibf_gpu_ibf * f, uint64_t const * d_values, uint64_t n, int width, void * d_out, cudaStream_t s,
                  unsigned long long * totals = nullptr)
{
    uint64_t const nc = count_counters(f);
    if (!totals)
    {
        f->totals.ensure(nc * sizeof(unsigned long long));
        totals = f->totals.as<unsigned long long>();
    }
    HG_CUDA(cudaMemsetAsync(totals, 0, nc * sizeof(unsigned long long), s));
    if (n)
    {
        unsigned const block = 256;
        // one contiguous chunk per warp of a full wave (4 blocks of 8 warps per SM), at least 512 values: fewer,
        // larger chunks left SMs idle on small calls (128 blocks for 2^21 values with fixed 2,048-value chunks)
        uint64_t const wave = static_cast<uint64_t>(sm_count()) * 4u * 8u;
        uint64_t const chunk = std::max<uint64_t>(512, ((n + wave - 1) / wave + 127) / 128 * 128);
        uint64_t const warps = (n + chunk - 1) / chunk;
        unsigned const grid = static_cast<unsigned>(
            std::max<uint64_t>(1, std::min<uint64_t>((warps + 7) / 8, static_cast<uint64_t>(sm_count()) * 4u)));
        bool const priv = nc <= kPrivateCountersMax;
        size_t const smem = nc * sizeof(uint32_t) * (priv ? block / 32 : 1);
        if (smem > 48 * 1024)
            HG_CUDA(cudaFuncSetAttribute(bulk_count_kernel(f->hash_funs, priv),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
        bulk_count_kernel(f->hash_funs, priv)<<<grid, block, smem, s>>>(f->rp(), f->lpv_log2(), d_values, n, chunk,
                                                                        totals, static_cast<uint32_t>(nc));
        HG_CUDA(cudaGetLastError());
    }
    k_store_counts<<<grid_for(f->bins, 256), 256, 0, s>>>(totals, f->bins, width, d_out);
    HG_CUDA(cudaGetLastError());
}

void launch_contains(hibf_gpu_ibf * f, uint64_t const * d_values, uint64_t n, uint64_t * d_out, cudaStream_t s)
{
    if (n == 0)
        return;
    unsigned const block = 256;
    uint32_t const l = f->lpv_log2();
    row_params const rp = f->rp();
    if (f->bin_words > 32)
    {
        // rows wider than a warp: lanes stride over the words
        k_bulk_contains<32><<<grid_for(n << 5, block), block, 0, s>>>(rp, d_values, n, d_out);
    }
    else
    {
        unsigned const grid = grid_for(n, block);
        switch (f->hash_funs)
        {
        case 1:
            launch_contains_h<1>(rp, l, d_values, n, d_out, grid, s);
            break;
        case 2:
            launch_contains_h<2>(rp, l, d_values, n, d_out, grid, s);
            break;
        case 3:
            launch_contains_h<3>(rp, l, d_values, n, d_out, grid, s);
            break;
        case 4:
            launch_contains_h<4>(rp, l, d_values, n, d_out, grid, s);
            break;
        default:
            launch_contains_h<5>(rp, l, d_values, n, d_out, grid, s);
        }
    }
    HG_CUDA(cudaGetLastError());
}

int width_ok(int width)
{
    return width == 1 || width == 2 || width == 4 || width == 8;
}

// ---------------------------------------------------------------------------------------------------------------
// bulk_count without allocation.  The 64-bit per-bin totals that bulk_count accumulates live in this fixed array
// instead of a cudaMalloc'd buffer.  Every device that loads the library holds it (128 KiB) until the process exits.
// ---------------------------------------------------------------------------------------------------------------
constexpr uint64_t kNoAllocMaxCounters = HIBF_GPU_NOALLOC_MAX_BINS;
static __device__ __align__(256) unsigned long long g_noalloc_totals[kNoAllocMaxCounters];

// Device address of g_noalloc_totals per device.  In host code the array's name is only a host-side stand-in, so
// the address is looked up once per device (cudaGetSymbolAddress, with that device current) and cached.
constexpr int kMaxDevices = 256;
std::mutex g_noalloc_mu;
unsigned long long * g_noalloc_addr[kMaxDevices] = {};

unsigned long long * noalloc_totals()
{
    int dev = 0;
    HG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        fail(HIBF_GPU_ERR_INVALID_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev])
    {
        void * p = nullptr;
        HG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_totals));
        g_noalloc_addr[dev] = static_cast<unsigned long long *>(p);
    }
    return g_noalloc_addr[dev];
}

} // namespace

extern "C"
{

    char const * hibf_gpu_last_error(void)
    {
        return g_last_error.c_str();
    }

    int hibf_gpu_abi_version(void)
    {
        return HIBF_GPU_ABI_VERSION;
    }

    int hibf_gpu_device_count(int * count)
    {
        return guarded(
            [&]
            {
                int n = 0;
                cudaError_t e = cudaGetDeviceCount(&n);
                if (e != cudaSuccess)
                {
                    (void)cudaGetLastError();
                    n = 0;
                }
                if (count)
                    *count = n;
            });
    }

    int hibf_gpu_ibf_create(uint64_t bins, uint64_t bin_size, uint64_t hash_funs, int track_occupancy,
                            hibf_gpu_ibf ** out)
    {
        return guarded(
            [&]
            {
                if (!out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "out is null");
                *out = nullptr;
                if (bins == 0)
                    fail(HIBF_GPU_ERR_LOGIC, "The number of bins must be > 0.");
                if (hash_funs == 0 || hash_funs > 5)
                    fail(HIBF_GPU_ERR_LOGIC, "The number of hash functions must be > 0 and <= 5.");
                if (bin_size == 0)
                    fail(HIBF_GPU_ERR_LOGIC, "The size of a bin must be > 0.");
                require_device();
                auto f = new hibf_gpu_ibf{};
                try
                {
                    f->bins = bins;
                    f->bin_size = bin_size;
                    f->hash_funs = hash_funs;
                    f->bin_words = (bins + 63u) / 64u;
                    f->row_words = padded_row_words(f->bin_words);
                    f->shift = static_cast<uint32_t>(__builtin_clzll(bin_size));
                    f->track_occupancy = track_occupancy != 0;
                    HG_CUDA(cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking));
                    size_t const bytes = bin_size * f->row_words * sizeof(uint64_t);
                    f->store.ensure(bytes);
                    HG_CUDA(cudaMemsetAsync(f->store.p, 0, bytes, f->stream));
                    f->flag.ensure(sizeof(int));
                    HG_CUDA(cudaMemsetAsync(f->flag.p, 0, sizeof(int), f->stream));
                    f->occupancy.ensure(f->technical_bins() * sizeof(uint64_t));
                    HG_CUDA(cudaMemsetAsync(f->occupancy.p, 0, f->technical_bins() * sizeof(uint64_t), f->stream));
                    HG_CUDA(cudaStreamSynchronize(f->stream));
                }
                catch (...)
                {
                    if (f->stream)
                        cudaStreamDestroy(f->stream);
                    delete f;
                    throw;
                }
                *out = f;
            });
    }

    int hibf_gpu_ibf_destroy(hibf_gpu_ibf * f)
    {
        return guarded(
            [&]
            {
                if (!f)
                    return;
                cudaStreamSynchronize(f->stream);
                cudaStreamDestroy(f->stream);
                delete f;
            });
    }

    int hibf_gpu_ibf_info(hibf_gpu_ibf const * f, uint64_t out[5])
    {
        return guarded(
            [&]
            {
                if (!f || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                out[0] = f->bins;
                out[1] = f->bin_size;
                out[2] = f->hash_funs;
                out[3] = f->bin_words * 64u * f->bin_size;
                out[4] = f->row_words * 8u;
            });
    }

    int hibf_gpu_ibf_emplace_d(hibf_gpu_ibf * f, uint64_t const * d_values, uint64_t const * d_bins, uint64_t n,
                               uint64_t bin, void * stream)
    {
        return guarded(
            [&]
            {
                if (!f || (n && !d_values))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (!d_bins && bin >= f->bins)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bin index out of range");
                launch_emplace(f, d_values, d_bins, n, bin, pick(f, stream));
            });
    }

    int hibf_gpu_synth_ibf_emplace(hibf_gpu_ibf * f, uint64_t seed, uint64_t values_per_bin, uint64_t first_bin,
                                   uint64_t n_bins, void * stream)
    {
        return guarded(
            [&]
            {
                if (!f || values_per_bin == 0)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                if (first_bin > f->bins || n_bins > f->bins - first_bin)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bin range out of range");
                if (n_bins && values_per_bin > UINT64_MAX / n_bins)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "too many values");
                uint64_t const n = n_bins * values_per_bin;
                if (!n)
                    return;
                if (f->track_occupancy)
                {
                    for (uint64_t b = first_bin; b < first_bin + n_bins; ++b)
                        emplace_exact<true>(f, nullptr, nullptr, values_per_bin, b, seed, values_per_bin,
                                            pick(f, stream));
                    return;
                }
                unsigned const block = 256;
                k_synth_emplace<<<grid_for(n, block), block, 0, pick(f, stream)>>>(
                    f->store.as<uint64_t>(), f->bin_size, static_cast<uint32_t>(f->row_words), f->shift,
                    static_cast<uint32_t>(f->hash_funs), seed, values_per_bin, first_bin, n);
                HG_CUDA(cudaGetLastError());
            });
    }

    int hibf_gpu_ibf_emplace(hibf_gpu_ibf * f, uint64_t const * values, uint64_t n, uint64_t bin)
    {
        return guarded(
            [&]
            {
                if (!f || (n && !values))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (bin >= f->bins)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bin index out of range");
                std::lock_guard<std::mutex> lk(f->mu);
                f->io.ensure(n * 8);
                HG_CUDA(cudaMemcpyAsync(f->io.p, values, n * 8, cudaMemcpyHostToDevice, f->stream));
                launch_emplace(f, f->io.as<uint64_t>(), nullptr, n, bin, f->stream);
                HG_CUDA(cudaStreamSynchronize(f->stream));
            });
    }

    int hibf_gpu_ibf_emplace_binned(hibf_gpu_ibf * f, uint64_t const * values, uint64_t const * bins, uint64_t n)
    {
        return guarded(
            [&]
            {
                if (!f || (n && (!values || !bins)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                for (uint64_t i = 0; i < n; ++i)
                    if (bins[i] >= f->bins)
                        fail(HIBF_GPU_ERR_INVALID_ARG, "bin index out of range");
                std::lock_guard<std::mutex> lk(f->mu);
                f->io.ensure(n * 8);
                f->io2.ensure(n * 8);
                HG_CUDA(cudaMemcpyAsync(f->io.p, values, n * 8, cudaMemcpyHostToDevice, f->stream));
                HG_CUDA(cudaMemcpyAsync(f->io2.p, bins, n * 8, cudaMemcpyHostToDevice, f->stream));
                launch_emplace(f, f->io.as<uint64_t>(), f->io2.as<uint64_t>(), n, 0, f->stream);
                HG_CUDA(cudaStreamSynchronize(f->stream));
            });
    }

    int hibf_gpu_ibf_clear(hibf_gpu_ibf * f, uint64_t bin)
    {
        return guarded(
            [&]
            {
                if (!f)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (bin >= f->bins)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bin index out of range");
                std::lock_guard<std::mutex> lk(f->mu);
                k_clear_bin<<<grid_for(f->bin_size, 256), 256, 0, f->stream>>>(
                    f->store.as<uint64_t>(), f->bin_size, static_cast<uint32_t>(f->row_words), bin >> 6,
                    ~(1ull << (bin & 63u)));
                HG_CUDA(cudaGetLastError());
                HG_CUDA(cudaMemsetAsync(f->occupancy.as<uint64_t>() + bin, 0, sizeof(uint64_t), f->stream));
                HG_CUDA(cudaStreamSynchronize(f->stream));
            });
    }

    int hibf_gpu_ibf_clear_range(hibf_gpu_ibf * f, uint64_t const * bins, uint64_t n)
    {
        return guarded(
            [&]
            {
                if (!f || (n && !bins))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::vector<uint64_t> masks(f->bin_words, 0);
                for (uint64_t i = 0; i < n; ++i)
                {
                    if (bins[i] >= f->technical_bins())
                        fail(HIBF_GPU_ERR_INVALID_ARG, "bin index out of range");
                    masks[bins[i] >> 6] |= 1ull << (bins[i] & 63u);
                }
                std::vector<uint32_t> widx;
                std::vector<uint64_t> keep;
                for (uint64_t w = 0; w < f->bin_words; ++w)
                    if (masks[w])
                    {
                        widx.push_back(static_cast<uint32_t>(w));
                        keep.push_back(~masks[w]);
                    }
                if (widx.empty())
                    return;
                std::lock_guard<std::mutex> lk(f->mu);
                f->io.ensure(widx.size() * 4);
                f->io2.ensure(keep.size() * 8);
                HG_CUDA(cudaMemcpyAsync(f->io.p, widx.data(), widx.size() * 4, cudaMemcpyHostToDevice, f->stream));
                HG_CUDA(cudaMemcpyAsync(f->io2.p, keep.data(), keep.size() * 8, cudaMemcpyHostToDevice, f->stream));
                uint32_t const nw = static_cast<uint32_t>(widx.size());
                k_clear_words<<<grid_for(f->bin_size * nw, 256), 256, 0, f->stream>>>(
                    f->store.as<uint64_t>(), f->bin_size, static_cast<uint32_t>(f->row_words), f->io.as<uint32_t>(),
                    f->io2.as<uint64_t>(), nw);
                HG_CUDA(cudaGetLastError());
                HG_CUDA(cudaStreamSynchronize(f->stream));
            });
    }

    int hibf_gpu_ibf_try_increase_bin_number_to(hibf_gpu_ibf * f, uint64_t new_bins, int * increased)
    {
        return guarded(
            [&]
            {
                if (!f || !increased)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                uint64_t const nbw = (new_bins + 63u) / 64u;
                *increased = 0;
                if (new_bins < f->bins || nbw > f->bin_words)
                    return;
                f->bins = new_bins;
                *increased = 1;
            });
    }

    int hibf_gpu_ibf_increase_bin_number_to(hibf_gpu_ibf * f, uint64_t new_bins)
    {
        return guarded(
            [&]
            {
                if (!f)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (new_bins < f->bins)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "The number of new bins must be >= the current number of bins.");
                uint64_t const nbw = (new_bins + 63u) / 64u;
                if (nbw <= f->bin_words)
                {
                    f->bins = new_bins;
                    return;
                }
                std::lock_guard<std::mutex> lk(f->mu);
                uint64_t const nrw = padded_row_words(nbw);
                dbuf fresh;
                fresh.ensure(f->bin_size * nrw * 8);
                k_widen<<<grid_for(f->bin_size * nrw, 256), 256, 0, f->stream>>>(
                    fresh.as<uint64_t>(), static_cast<uint32_t>(nrw), f->store.as<uint64_t>(),
                    static_cast<uint32_t>(f->row_words), static_cast<uint32_t>(f->bin_words), f->bin_size);
                HG_CUDA(cudaGetLastError());
                dbuf occ;
                occ.ensure(nbw * 64 * 8);
                HG_CUDA(cudaMemsetAsync(occ.p, 0, nbw * 64 * 8, f->stream));
                HG_CUDA(cudaMemcpyAsync(occ.p, f->occupancy.p, f->technical_bins() * 8, cudaMemcpyDeviceToDevice,
                                        f->stream));
                HG_CUDA(cudaStreamSynchronize(f->stream));
                std::swap(f->store.p, fresh.p);
                std::swap(f->store.bytes, fresh.bytes);
                std::swap(f->occupancy.p, occ.p);
                std::swap(f->occupancy.bytes, occ.bytes);
                f->bins = new_bins;
                f->bin_words = nbw;
                f->row_words = nrw;
            });
    }

    int hibf_gpu_ibf_bulk_contains_d(hibf_gpu_ibf * f, uint64_t const * d_values, uint64_t n, uint64_t * d_out,
                                     void * stream)
    {
        return guarded(
            [&]
            {
                if (!f || (n && (!d_values || !d_out)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                launch_contains(f, d_values, n, d_out, pick(f, stream));
            });
    }

    int hibf_gpu_ibf_bulk_contains(hibf_gpu_ibf * f, uint64_t const * values, uint64_t n, uint64_t * out)
    {
        return guarded(
            [&]
            {
                if (!f || (n && (!values || !out)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (n == 0)
                    return;
                std::lock_guard<std::mutex> lk(f->mu);
                f->io.ensure(n * 8);
                f->io2.ensure(n * f->bin_words * 8);
                HG_CUDA(cudaMemcpyAsync(f->io.p, values, n * 8, cudaMemcpyHostToDevice, f->stream));
                launch_contains(f, f->io.as<uint64_t>(), n, f->io2.as<uint64_t>(), f->stream);
                HG_CUDA(cudaMemcpyAsync(out, f->io2.p, n * f->bin_words * 8, cudaMemcpyDeviceToHost, f->stream));
                HG_CUDA(cudaStreamSynchronize(f->stream));
            });
    }

    int hibf_gpu_ibf_bulk_count_d(hibf_gpu_ibf * f, uint64_t const * d_values, uint64_t n, int width, void * d_out,
                                  void * stream)
    {
        return guarded(
            [&]
            {
                if (!f || (n && !d_values) || !d_out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (!width_ok(width))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "width must be 1, 2, 4 or 8");
                launch_count(f, d_values, n, width, d_out, pick(f, stream));
            });
    }

    int hibf_gpu_ibf_bulk_count(hibf_gpu_ibf * f, uint64_t const * values, uint64_t n, int width, void * out)
    {
        return guarded(
            [&]
            {
                if (!f || (n && !values) || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (!width_ok(width))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "width must be 1, 2, 4 or 8");
                std::lock_guard<std::mutex> lk(f->mu);
                f->io.ensure(n * 8);
                f->io2.ensure(f->bins * 8);
                if (n)
                    HG_CUDA(cudaMemcpyAsync(f->io.p, values, n * 8, cudaMemcpyHostToDevice, f->stream));
                launch_count(f, f->io.as<uint64_t>(), n, width, f->io2.p, f->stream);
                HG_CUDA(cudaMemcpyAsync(out, f->io2.p, f->bins * width, cudaMemcpyDeviceToHost, f->stream));
                HG_CUDA(cudaStreamSynchronize(f->stream));
            });
    }

    int hibf_gpu_ibf_membership_for(hibf_gpu_ibf * f, uint64_t const * values, uint64_t n, uint16_t threshold,
                                    uint64_t * out_ids, uint64_t * n_out)
    {
        return guarded(
            [&]
            {
                if (!f || (n && !values) || !out_ids || !n_out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::vector<uint16_t> counts(f->bins);
                int const st = hibf_gpu_ibf_bulk_count(f, values, n, 2, counts.data());
                if (st != HIBF_GPU_OK)
                    fail(st, g_last_error);
                uint64_t m = 0;
                for (uint64_t b = 0; b < f->bins; ++b)
                    if (counts[b] >= threshold)
                        out_ids[m++] = b;
                *n_out = m;
            });
    }

    int hibf_gpu_ibf_save(hibf_gpu_ibf * f, char const * path)
    {
        return guarded(
            [&]
            {
                if (!f || !path)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::lock_guard<std::mutex> lk(f->mu);
                HG_CUDA(cudaStreamSynchronize(f->stream));
                file_writer w(path);
                write_ibf_header(w, f->bins, f->bin_size, f->hash_funs);
                write_rows(w, f->store.as<uint64_t>(), f->bin_size, f->bin_words, f->row_words, f->stream);
                uint64_t const tb = f->technical_bins();
                std::vector<uint64_t> occ(tb, 0);
                if (f->track_occupancy)
                {
                    HG_CUDA(cudaMemcpyAsync(occ.data(), f->occupancy.p, tb * 8, cudaMemcpyDeviceToHost, f->stream));
                    HG_CUDA(cudaStreamSynchronize(f->stream));
                }
                w.u64s(occ);
                w.u8(f->track_occupancy ? 1 : 0);
                w.close();
            });
    }

    int hibf_gpu_ibf_load(char const * path, hibf_gpu_ibf ** out)
    {
        return guarded(
            [&]
            {
                if (!path || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *out = nullptr;
                file_reader r(path);
                ibf_header const h = read_ibf_header(r);
                long const words_at = r.tell();
                r.skip(h.bin_size * h.bin_words * 8);
                std::vector<uint64_t> const occ = r.u64s(h.technical_bins);
                uint8_t const track = r.u8();
                if (occ.size() != h.technical_bins || track > 1 || !r.at_end())
                    fail(HIBF_GPU_ERR_INVALID_ARG, "archive: malformed interleaved_bloom_filter");
                hibf_gpu_ibf * f = nullptr;
                int const st = hibf_gpu_ibf_create(h.bins, h.bin_size, h.hash_funs, track, &f);
                if (st != HIBF_GPU_OK)
                    fail(st, g_last_error);
                try
                {
                    r.seek(words_at);
                    read_rows(r, f->store.as<uint64_t>(), f->bin_size, f->bin_words, f->row_words, f->stream);
                    HG_CUDA(cudaMemcpyAsync(f->occupancy.p, occ.data(), occ.size() * 8, cudaMemcpyHostToDevice,
                                            f->stream));
                    HG_CUDA(cudaStreamSynchronize(f->stream));
                }
                catch (...)
                {
                    hibf_gpu_ibf_destroy(f);
                    throw;
                }
                *out = f;
            });
    }

    int hibf_gpu_ibf_upload_words(hibf_gpu_ibf * f, uint64_t const * words, uint64_t n_words)
    {
        return guarded(
            [&]
            {
                if (!f || !words)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (n_words != f->bin_words * f->bin_size)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "word count does not match the filter");
                std::lock_guard<std::mutex> lk(f->mu);
                HG_CUDA(cudaMemcpy2DAsync(f->store.p, f->row_words * 8, words, f->bin_words * 8, f->bin_words * 8,
                                          f->bin_size, cudaMemcpyHostToDevice, f->stream));
                HG_CUDA(cudaStreamSynchronize(f->stream));
            });
    }

    int hibf_gpu_ibf_download_words(hibf_gpu_ibf * f, uint64_t * words, uint64_t n_words)
    {
        return guarded(
            [&]
            {
                if (!f || !words)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (n_words != f->bin_words * f->bin_size)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "word count does not match the filter");
                std::lock_guard<std::mutex> lk(f->mu);
                HG_CUDA(cudaMemcpy2DAsync(words, f->bin_words * 8, f->store.p, f->row_words * 8, f->bin_words * 8,
                                          f->bin_size, cudaMemcpyDeviceToHost, f->stream));
                HG_CUDA(cudaStreamSynchronize(f->stream));
            });
    }

    int hibf_gpu_ibf_download_occupancy(hibf_gpu_ibf * f, uint64_t * out, uint64_t n)
    {
        return guarded(
            [&]
            {
                if (!f || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (n != f->technical_bins())
                    fail(HIBF_GPU_ERR_INVALID_ARG, "occupancy has technical_bins entries");
                std::lock_guard<std::mutex> lk(f->mu);
                HG_CUDA(cudaMemcpyAsync(out, f->occupancy.p, n * 8, cudaMemcpyDeviceToHost, f->stream));
                HG_CUDA(cudaStreamSynchronize(f->stream));
            });
    }

    int hibf_gpu_ibf_track_occupancy(hibf_gpu_ibf const * f, int * out)
    {
        return guarded(
            [&]
            {
                if (!f || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *out = f->track_occupancy ? 1 : 0;
            });
    }

    int hibf_gpu_ibf_status(hibf_gpu_ibf * f)
    {
        if (!f)
            return HIBF_GPU_ERR_INVALID_ARG;
        cudaError_t const e = cudaStreamSynchronize(f->stream);
        if (e != cudaSuccess)
        {
            set_last_error(cudaGetErrorString(e));
            return HIBF_GPU_ERR_CUDA;
        }
        int bad = 0;
        if (cudaMemcpy(&bad, f->flag.p, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && bad)
        {
            cudaMemset(f->flag.p, 0, sizeof(int));
            set_last_error("an emplace received a bin index out of range; those values were skipped");
            return HIBF_GPU_ERR_INVALID_ARG;
        }
        return f->status;
    }

    // Same result as hibf_gpu_ibf_bulk_count_d, for callers that cannot allocate device memory.  The counting
    // scratch is the static array above, passed to the same launch as bulk_count_d: this call makes no cudaMalloc,
    // cudaFree or other allocating call.  The first call on a device looks up the array's device address and keeps it
    // for the process (issue it before any stream capture; a device reset after it is not supported); calls that
    // overlap on the GPU share the array and race; the totals are cleared at the start of every call.
    int hibf_gpu_ibf_bulk_count_noalloc_d(hibf_gpu_ibf * f, uint64_t const * d_values, uint64_t n, int width,
                                          void * d_out, void * stream)
    {
        return guarded(
            [&]
            {
                if (!f || (n && !d_values) || !d_out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (!width_ok(width))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "width must be 1, 2, 4 or 8");
                if (count_counters(f) > kNoAllocMaxCounters)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "hibf_gpu_ibf_bulk_count_noalloc_d supports at most " +
                                                       std::to_string(kNoAllocMaxCounters) +
                                                       " bins; use hibf_gpu_ibf_bulk_count_d");
                launch_count(f, d_values, n, width, d_out, pick(f, stream), noalloc_totals());
            });
    }

} // extern "C"
