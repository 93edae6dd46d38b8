// device.cuh -- device-side building blocks shared by the IBF and HIBF kernels.
//
// Layout of one IBF in HBM (the "bit store"):
//   bin_size rows; row r holds technical_bins bits (technical_bins = 64 * bin_words), LSB-first in 64-bit words,
//   starting at word r * row_words.  row_words >= bin_words pads a row so that it never straddles a 32-byte sector:
//   rows of 8/16/32 bytes stay as they are, 24 bytes become 32, longer rows are rounded up to a multiple of 32 bytes.
//   Bin b of row r is bit (b % 64) of word r * row_words + b / 64 -- the reference's bit_vector layout
//   (include/hibf/interleaved_bloom_filter.hpp:146; src/interleaved_bloom_filter.cpp:48-52) with a padded stride.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace hibf_gb300
{

constexpr unsigned kFullMask = 0xFFFFFFFFu;

// The multiplicative hashing seeds of include/hibf/interleaved_bloom_filter.hpp:172-176.  A filter's bit positions
// are defined by them, so bit-exact parity requires the same five constants.
__constant__ uint64_t c_hash_seeds[5] = {13572355802537770549ULL,
                                         13043817825332782213ULL,
                                         10650232656628343401ULL,
                                         16499269484942379435ULL,
                                         4893150838803335377ULL};

// Row selected by hash function `i` (hash_and_fit, include/hibf/interleaved_bloom_filter.hpp:185-195, divided by
// technical_bins): multiply by the seed, fold the high bits down by hash_shift = countl_zero(bin_size), multiply by
// 2^64 / golden ratio, then fastrange into [0, bin_size) with the high half of a 64x64-bit product.
__device__ __forceinline__ uint64_t hash_row(uint64_t v, uint64_t seed, uint32_t shift, uint64_t bin_size)
{
    uint64_t h = v * seed;
    h ^= h >> shift;
    h *= 11400714819323198485ULL;
    return __umul64hi(h, bin_size);
}

__device__ __forceinline__ uint64_t ldg_nc(uint64_t const * p)
{
    uint64_t r;
    asm volatile("ld.global.nc.L1::no_allocate.u64 %0, [%1];" : "=l"(r) : "l"(p));
    return r;
}

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------------------------------------------
// Bit-sliced ("vertical") counters.  P[k] holds bit k of 64 independent counters, one per bin of a 64-bit row word.
// Adding four 0/1 masks costs a carry-save tree (full adder + three half adders) plus a ripple through the planes:
// about a dozen LOP3 per 32-bit half, instead of 64 per-bin adds.
// ---------------------------------------------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void planes_add4(uint64_t (&P)[K], uint64_t a, uint64_t b, uint64_t c, uint64_t d)
{
    uint64_t const u = a ^ b;
    uint64_t const s1 = u ^ c;
    uint64_t const c1 = (a & b) | (u & c); // weight 2
    uint64_t const w1 = s1 ^ d;
    uint64_t const c2 = s1 & d; // weight 2
    uint64_t const w2 = c1 ^ c2;
    uint64_t const w4 = c1 & c2;
    // plane 0 += w1
    uint64_t carry = P[0] & w1;
    P[0] ^= w1;
    // plane 1 += w2 + carry
    uint64_t t = P[1] ^ w2;
    uint64_t carry2 = (P[1] & w2) | (t & carry);
    P[1] = t ^ carry;
    // plane 2 += w4 + carry2
    t = P[2] ^ w4;
    carry = (P[2] & w4) | (t & carry2);
    P[2] = t ^ carry2;
#pragma unroll
    for (int k = 3; k < K; ++k)
    {
        uint64_t const n = P[k] & carry;
        P[k] ^= carry;
        carry = n;
    }
}

// 32x32 bit transpose across a warp: on entry lane r holds row r (bit c = A[r][c]); on exit lane c holds column c
// (bit r = A[r][c]).  Five butterfly exchanges of shrinking blocks.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, int lane)
{
    uint32_t constexpr masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int i = 0; i < 5; ++i)
    {
        int const s = 16 >> i;
        uint32_t const m = masks[i];
        uint32_t const y = __shfl_xor_sync(kFullMask, x, s);
        x = (lane & s) ? ((x & ~m) | ((y & ~m) >> s)) : ((x & m) | ((y & m) << s));
    }
    return x;
}

} // namespace hibf_gb300
