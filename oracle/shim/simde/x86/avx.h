// Portable stand-in for the two simde 0.8.2 AVX operations the reference's HyperLogLog uses.
// Lane semantics follow Intel's documentation: set_ps lists lanes from highest (e7) to lowest (e0);
// add_ps is a lane-wise IEEE single-precision add, so sums are bit-identical to the native instruction.
#pragma once
#include <cstdint>
struct alignas(32) simde__m256
{
    float f[8];
};
struct alignas(32) simde__m256i
{
    std::uint8_t u8[32];
};
inline simde__m256 simde_mm256_set1_ps(float a)
{
    simde__m256 r;
    for (int i = 0; i < 8; ++i)
        r.f[i] = a;
    return r;
}
inline simde__m256 simde_mm256_set_ps(float e7, float e6, float e5, float e4, float e3, float e2, float e1, float e0)
{
    simde__m256 r;
    r.f[0] = e0;
    r.f[1] = e1;
    r.f[2] = e2;
    r.f[3] = e3;
    r.f[4] = e4;
    r.f[5] = e5;
    r.f[6] = e6;
    r.f[7] = e7;
    return r;
}
inline simde__m256 simde_mm256_add_ps(simde__m256 a, simde__m256 b)
{
    simde__m256 r;
    for (int i = 0; i < 8; ++i)
        r.f[i] = a.f[i] + b.f[i];
    return r;
}
