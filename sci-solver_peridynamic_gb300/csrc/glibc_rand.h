// glibc_rand.h -- glibc-compatible rand() stream (host).
#pragma once

#include <cstdint>

namespace pdgb {

// ---- glibc-compatible rand() ----------------------------------------------------
// glibc's rand() is random_r() with the default TYPE_3 state: an additive
// lagged-Fibonacci generator r[i] = r[i-3] + r[i-31] (mod 2^32) seeded by the
// Park-Miller LCG r[i] = 16807 r[i-1] mod (2^31 - 1) (i = 1..30), with
// r[31..33] = r[0..2], outputs r[34..343] discarded and each later output
// shifted right by one bit.  Restated so that s0 sampling (srand(1973),
// src/core/simulator.cu:852) does not touch the caller's C-library state.
struct GlibcRand {
    uint32_t h[64];   // ring buffer of the last words
    long long i;
    explicit GlibcRand(int32_t seed)
    {
        if (seed == 0) seed = 1;
        int32_t s[31];
        s[0] = seed;
        for (int k = 1; k < 31; ++k) {
            const int32_t hi = s[k - 1] / 127773;
            const int32_t lo = s[k - 1] % 127773;
            int32_t word = 16807 * lo - 2836 * hi;
            if (word < 0) word += 2147483647;
            s[k] = word;
        }
        for (int k = 0; k < 31; ++k) h[k] = (uint32_t)s[k];
        for (int k = 31; k < 34; ++k) h[k] = (uint32_t)s[k - 31];
        i = 34;
        for (int k = 34; k < 344; ++k) step();
    }
    uint32_t at(long long k) const { return h[k & 63]; }
    uint32_t step()
    {
        const uint32_t v = at(i - 31) + at(i - 3);
        h[i & 63] = v;
        ++i;
        return v;
    }
    int next() { return (int)(step() >> 1); }   // rand(), RAND_MAX = 2^31 - 1
};


}  // namespace pdgb
