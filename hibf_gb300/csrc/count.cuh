// count.cuh -- the per-warp counting loop shared by IBF bulk_count and the HIBF query kernels.
//
// For every value: hash it h times, fetch the h rows, AND them, add the resulting bit vector to per-bin counters
// (include/hibf/interleaved_bloom_filter.hpp:652-665 + counting_vector::operator+=, counting_vector.hpp:171-175).
//
// Work mapping.  A row of bin_words 64-bit words is read by LPV = next_pow2(bin_words) lanes (capped at 32), lane
// j of a group reading word j, so a row is one coalesced access of ceil(bytes/32) sectors.  Each lane first hashes
// a different value (32 values per warp per pass), then the groups take turns on those values, receiving the row
// offsets by shuffle.  Each lane accumulates its word's 64 bins in K bit-sliced planes (planes_add4) and flushes
// them through a warp transpose into 32-bit counters in shared memory before they can overflow (2^K - 1 masks).
// Counts are exact; the caller reduces them modulo the counter width, which equals the reference's wraparound.
#pragma once

#include "device.cuh"

namespace hibf_gb300
{

struct row_params
{
    uint64_t const * words;
    uint64_t bin_size;
    uint32_t row_words;
    uint32_t bin_words;
    uint32_t hash_shift;
    uint32_t hash_funs;
};

// `added` (warp-uniform) masks went into the planes since the last flush, so planes k with 2^k > added are zero and
// are not transposed.  Lane j of an LPV-lane group holds word W * j (+ the caller's offset of `out`) of its rows.
template <int LPV, int K, bool ATOMIC, int W = 1>
__device__ __forceinline__ void planes_flush_to(uint64_t (&P)[K], uint32_t * out, int lane, int added)
{
    int const kmax = 32 - __clz(added);
    uint32_t lo[K], hi[K];
#pragma unroll
    for (int k = 0; k < K; ++k)
    {
        if (k < kmax)
        {
            lo[k] = warp_transpose32(static_cast<uint32_t>(P[k]), lane);
            hi[k] = warp_transpose32(static_cast<uint32_t>(P[k] >> 32), lane);
        }
        else
        {
            lo[k] = 0;
            hi[k] = 0;
        }
        P[k] = 0;
    }
#pragma unroll
    for (int j = 0; j < LPV; ++j)
    {
        uint32_t gm = 0;
#pragma unroll
        for (int g = 0; g < 32 / LPV; ++g)
            gm |= 1u << (g * LPV + j);
        uint32_t cl = 0, ch = 0;
#pragma unroll
        for (int k = 0; k < K; ++k)
        {
            cl += static_cast<uint32_t>(__popc(lo[k] & gm)) << k;
            ch += static_cast<uint32_t>(__popc(hi[k] & gm)) << k;
        }
        if constexpr (ATOMIC)
        {
            if (cl)
                atomicAdd(out + 64 * W * j + lane, cl);
            if (ch)
                atomicAdd(out + 64 * W * j + 32 + lane, ch);
        }
        else
        {
            out[64 * W * j + lane] += cl;
            out[64 * W * j + 32 + lane] += ch;
        }
    }
}

// A row word loaded with L2 evict-first priority: for a single-level IBF every row read is random and not read again
// soon, and the hint measured 4% faster counting there.  (The HIBF kernels keep the default: their small lower-level
// IBFs hit in L2, and evict-first made them slower.)
__device__ __forceinline__ uint64_t ldg_evict_first(uint64_t const * p)
{
    uint64_t pol, w;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm("ld.global.nc.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(w) : "l"(p), "l"(pol));
    return w;
}

template <int W, bool EF = false>
__device__ __forceinline__ void load_row_words(uint64_t const * p, uint64_t (&w)[W])
{
    if constexpr (W == 1)
    {
        w[0] = EF ? ldg_evict_first(p) : __ldg(p);
    }
    else
    {
        ulonglong2 const x = __ldg(reinterpret_cast<ulonglong2 const *>(p));
        w[0] = x.x;
        w[1] = x.y;
    }
}

// Values are read with ld.global.cg (cached in L2 only): a streamed host batch's values are written by the copy
// engine while the kernel runs, and a task reads them only after their chunk's arrival counter (query.cuh), so the
// loads must not come from a non-coherent cache.  Each task reads its values once, so L1 gives them nothing.
//
// One warp counts vals[0, n) into counts[0, 64 * LPV * W) with H hash functions.  ATOMIC: counters shared with other
// warps.  A row is read by LPV lanes, each loading W consecutive words (W = 2: one 16-byte load; the row stride
// must then be even).  Each lane hashes U values per pass and keeps their H row offsets; the row words of
// GS = 4 * UM masks per lane are loaded together, so GS * H * W loads per lane are in flight.  K planes count up to
// 2^K - 1 masks between flushes.
//
// stage (optional): every value read is also stored at stage[i], so that later reads of the same values (the lower
// levels of an in-place host batch) come from device memory instead of the host link.
template <int LPV, int H, int K, bool ATOMIC, int UM = 1, int W = 1, bool EF = false>
__device__ __forceinline__ void warp_count(row_params const & rp, uint64_t const * __restrict__ vals, uint64_t n,
                                           uint32_t * counts, int lane, uint64_t * __restrict__ stage = nullptr)
{
    constexpr int G = 32 / LPV;
    constexpr int U = UM * (LPV >= 4 ? 1 : 4 / LPV);
    constexpr int STEPS = U * LPV;
    constexpr int GS = 4 * UM;
    constexpr int BLOCK = 32 * U;
    static_assert(STEPS % GS == 0, "masks are consumed in groups of GS");
    static_assert((1 << K) - 1 >= 2 * GS, "the planes must hold at least two groups between flushes");
    int const g = lane / LPV;
    int const j = lane % LPV;
    bool const wj = static_cast<uint32_t>(j * W) < rp.bin_words;
    uint64_t const * __restrict__ words = rp.words + j * W;

    uint64_t P[W][K];
#pragma unroll
    for (int e = 0; e < W; ++e)
#pragma unroll
        for (int k = 0; k < K; ++k)
            P[e][k] = 0;
    int acc = 0;

    for (uint64_t base = 0; base < n; base += BLOCK)
    {
        uint64_t off[U][H];
#pragma unroll
        for (int u = 0; u < U; ++u)
        {
            uint64_t const idx = base + static_cast<uint64_t>(u * 32 + lane);
            uint64_t const v = idx < n ? __ldcg(vals + idx) : 0u;
            if (stage && idx < n)
                stage[idx] = v;
#pragma unroll
            for (int i = 0; i < H; ++i)
                off[u][i] = hash_row(v, c_hash_seeds[i], rp.hash_shift, rp.bin_size) * rp.row_words;
        }
        // one group: GS masks per lane (GS sub-steps of LPV-lane groups), their H * W loads issued together
        auto group = [&](int s)
        {
            uint64_t w[GS][H][W];
            bool ok[GS];
#pragma unroll
            for (int t = 0; t < GS; ++t)
            {
                int const step = s + t;
                int const u = U == 1 ? 0 : step / LPV;
                int const src = (step % LPV) * G + g;
                ok[t] = wj && (base + static_cast<uint64_t>(u * 32 + src) < n);
#pragma unroll
                for (int i = 0; i < H; ++i)
                {
                    uint64_t o = off[u][i];
                    if constexpr (LPV > 1)
                        o = __shfl_sync(kFullMask, o, src);
                    if (ok[t])
                        load_row_words<W, EF>(words + o, w[t][i]);
                    else
#pragma unroll
                        for (int e = 0; e < W; ++e)
                            w[t][i][e] = 0ull;
                }
            }
#pragma unroll
            for (int t0 = 0; t0 < GS; t0 += 4)
            {
#pragma unroll
                for (int e = 0; e < W; ++e)
                {
                    uint64_t m[4];
#pragma unroll
                    for (int t = 0; t < 4; ++t)
                    {
                        uint64_t x = w[t0 + t][0][e];
#pragma unroll
                        for (int i = 1; i < H; ++i)
                            x &= w[t0 + t][i][e];
                        m[t] = x;
                    }
                    planes_add4<K>(P[e], m[0], m[1], m[2], m[3]);
                }
                acc += 4;
                if (acc > (1 << K) - 1 - 4)
                {
#pragma unroll
                    for (int e = 0; e < W; ++e)
                        planes_flush_to<LPV, K, ATOMIC, W>(P[e], counts + 64 * e, lane, acc);
                    acc = 0;
                }
            }
        };
        if constexpr (STEPS <= GS)
        {
            group(0);
        }
        else
        {
#pragma unroll 1
            for (int s = 0; s < STEPS; s += GS)
                group(s);
        }
    }
    if (acc)
    {
#pragma unroll
        for (int e = 0; e < W; ++e)
            planes_flush_to<LPV, K, ATOMIC, W>(P[e], counts + 64 * e, lane, acc);
    }
}

// Rows wider than a warp (bin_words > 32): lanes stride over the words, set bits are added one by one.
__device__ __forceinline__ void warp_count_wide(row_params const & rp, uint64_t const * __restrict__ vals, uint64_t n,
                                                uint32_t * counts, int lane, uint64_t * __restrict__ stage = nullptr)
{
    for (uint64_t i = 0; i < n; ++i)
    {
        uint64_t const v = __ldcg(vals + i);
        if (stage && lane == 0)
            stage[i] = v;
        uint64_t off[5];
#pragma unroll
        for (int k = 0; k < 5; ++k)
            off[k] = (static_cast<uint32_t>(k) < rp.hash_funs)
                       ? hash_row(v, c_hash_seeds[k], rp.hash_shift, rp.bin_size) * rp.row_words
                       : 0u;
        for (uint32_t wi = lane; wi < rp.bin_words; wi += 32)
        {
            uint64_t x = ~0ull;
#pragma unroll
            for (int k = 0; k < 5; ++k)
                if (static_cast<uint32_t>(k) < rp.hash_funs)
                    x &= __ldg(rp.words + off[k] + wi);
            while (x)
            {
                int const b = __ffsll(static_cast<long long>(x)) - 1;
                x &= x - 1;
                atomicAdd(counts + 64 * wi + b, 1u);
            }
        }
    }
}

template <int H, bool ATOMIC, bool EF = false>
__device__ __forceinline__ void warp_count_lpv(row_params const & rp, uint32_t lpv_log2, uint64_t const * vals,
                                               uint64_t n, uint32_t * counts, int lane, uint64_t * stage = nullptr)
{
    switch (lpv_log2)
    {
    case 0:
        warp_count<1, H, 7, ATOMIC, 1, 1, EF>(rp, vals, n, counts, lane, stage);
        break;
    case 1:
        warp_count<2, H, 7, ATOMIC, 1, 1, EF>(rp, vals, n, counts, lane, stage);
        break;
    case 2:
        warp_count<4, H, 7, ATOMIC, 1, 1, EF>(rp, vals, n, counts, lane, stage);
        break;
    case 3:
        warp_count<8, H, 7, ATOMIC, 1, 1, EF>(rp, vals, n, counts, lane, stage);
        break;
    case 4:
        warp_count<16, H, 7, ATOMIC, 1, 1, EF>(rp, vals, n, counts, lane, stage);
        break;
    default:
        warp_count<32, H, 7, ATOMIC, 1, 1, EF>(rp, vals, n, counts, lane, stage);
    }
}

// Dispatch on lanes-per-value for a compile-time hash function count (rows wider than a warp use the generic loop).
template <int H, bool ATOMIC>
__device__ __forceinline__ void warp_count_h(row_params const & rp, uint32_t lpv_log2, uint64_t const * vals,
                                             uint64_t n, uint32_t * counts, int lane, uint64_t * stage = nullptr)
{
    if (rp.bin_words > 32)
        warp_count_wide(rp, vals, n, counts, lane, stage);
    else
        warp_count_lpv<H, ATOMIC>(rp, lpv_log2, vals, n, counts, lane, stage);
}

// Dispatch on the node's hash function count and lanes-per-value (log2).  K = 7 planes: flush every 124 masks per
// lane.
template <bool ATOMIC>
__device__ __forceinline__ void warp_count_any(row_params const & rp, uint32_t lpv_log2, uint64_t const * vals,
                                               uint64_t n, uint32_t * counts, int lane)
{
    if (rp.bin_words > 32)
    {
        warp_count_wide(rp, vals, n, counts, lane);
        return;
    }
    switch (rp.hash_funs)
    {
    case 1:
        warp_count_lpv<1, ATOMIC>(rp, lpv_log2, vals, n, counts, lane);
        break;
    case 2:
        warp_count_lpv<2, ATOMIC>(rp, lpv_log2, vals, n, counts, lane);
        break;
    case 3:
        warp_count_lpv<3, ATOMIC>(rp, lpv_log2, vals, n, counts, lane);
        break;
    case 4:
        warp_count_lpv<4, ATOMIC>(rp, lpv_log2, vals, n, counts, lane);
        break;
    default:
        warp_count_lpv<5, ATOMIC>(rp, lpv_log2, vals, n, counts, lane);
    }
}

} // namespace hibf_gb300
