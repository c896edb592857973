// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC 2011): the counter-based
// generator behind every device-side variate of glass_gb300.  Checked against
// the published Random123 known-answer vectors by the oracle tests.
#pragma once

#include <stdint.h>

namespace glg_rng {

struct U4 {
    uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                            uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return {c0, c1, c2, c3};
}


// Uniform in (0, 1) from two 32-bit words: (K + 1/2) 2^-53 with the 53-bit
// integer K = (a >> 5) 2^26 + (b >> 6), exact in FP64.
__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6) + 0.5) * 1.1102230246251565e-16;
}

}  // namespace glg_rng
