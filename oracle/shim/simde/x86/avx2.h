// Portable stand-in: lane-wise unsigned byte maximum (Intel's _mm256_max_epu8 semantics).
#pragma once
#include <simde/x86/avx.h>
inline simde__m256i simde_mm256_max_epu8(simde__m256i a, simde__m256i b)
{
    simde__m256i r;
    for (int i = 0; i < 32; ++i)
        r.u8[i] = a.u8[i] > b.u8[i] ? a.u8[i] : b.u8[i];
    return r;
}
