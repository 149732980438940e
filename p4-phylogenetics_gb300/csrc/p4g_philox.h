// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011): ten rounds of
// two 32x32->64 multiplies with the published multipliers and Weyl key
// increments.  The n-th uniform of a stream is a pure function of (seed, n),
// so every thread of a simulation can draw the number the sequential loop
// would have drawn at that point without a shared state.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define P4G_HD __host__ __device__ __forceinline__
#else
#define P4G_HD inline
#endif

namespace p4g {

P4G_HD void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c[0] = hi1 ^ c[1] ^ k0;
        c[1] = lo1;
        c[2] = hi0 ^ c[3] ^ k1;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// The n-th uniform of stream `seed`, in [0, 1) with 32-bit resolution (the
// first output word of block n, times 2^-32).
P4G_HD double philoxUniform(uint64_t seed, uint64_t n)
{
    uint32_t c[4] = {(uint32_t)n, (uint32_t)(n >> 32), 0u, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return (double)c[0] * 0x1p-32;
}

}  // namespace p4g
