// gbmp_philox.h -- Philox4x32-10 counter-based generator (Salmon, Moraes, Dror,
// Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11), written from the
// published round function.  Usable from host and device so that the CPU oracle
// reproduces every sample.
#pragma once

#if defined(__CUDACC__)
#define GBMP_HD __host__ __device__ __forceinline__
#else
#define GBMP_HD static inline
#endif

namespace gbmp {

GBMP_HD unsigned mulhi32(unsigned a, unsigned b) {
    return (unsigned)(((unsigned long long)a * (unsigned long long)b) >> 32);
}

// ctr: 4 x 32-bit counter, key: 2 x 32-bit key; 10 rounds.
GBMP_HD void philox4x32_10(unsigned ctr[4], unsigned key0, unsigned key1) {
    const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const unsigned W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    unsigned k0 = key0, k1 = key1;
    for (int r = 0; r < 10; ++r) {
        const unsigned hi0 = mulhi32(M0, ctr[0]), lo0 = M0 * ctr[0];
        const unsigned hi1 = mulhi32(M1, ctr[2]), lo1 = M1 * ctr[2];
        const unsigned c0 = hi1 ^ ctr[1] ^ k0;
        const unsigned c2 = hi0 ^ ctr[3] ^ k1;
        ctr[0] = c0; ctr[1] = lo1; ctr[2] = c2; ctr[3] = lo0;
        k0 += W0; k1 += W1;
    }
}

// Uniform float in [0, 1) for (seed, counter, lane): 24 high bits of word 0.
GBMP_HD float philox_uniform(unsigned long long seed, unsigned long long counter, unsigned lane) {
    unsigned c[4] = {(unsigned)counter, (unsigned)(counter >> 32), lane, 0u};
    philox4x32_10(c, (unsigned)seed, (unsigned)(seed >> 32));
    return (float)(c[0] >> 8) * (1.0f / 16777216.0f);
}

}  // namespace gbmp
