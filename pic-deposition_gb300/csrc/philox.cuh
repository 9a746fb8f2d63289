// Counter-based random numbers for the device-side particle generators.
#pragma once

#include <cstdint>

namespace picgb {

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): counter-based, so particle i of run r always draws the
// same numbers.
struct U4 {
    uint32_t v[4];
};
__device__ __forceinline__ U4 philox(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t h0 = __umulhi(0xD2511F53u, c.v[0]), l0 = 0xD2511F53u * c.v[0];
        const uint32_t h1 = __umulhi(0xCD9E8D57u, c.v[2]), l1 = 0xCD9E8D57u * c.v[2];
        U4 n;
        n.v[0] = h1 ^ c.v[1] ^ k0;
        n.v[1] = l1;
        n.v[2] = h0 ^ c.v[3] ^ k1;
        n.v[3] = l0;
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}
// a double in (0, 1] from two random 32-bit words (53 random bits)
__device__ __forceinline__ double unit_open0(uint32_t a, uint32_t b) {
    const uint64_t m = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
    return ((double)(m & ((1ull << 53) - 1)) + 1.0) * (1.0 / 9007199254740992.0);
}

}  // namespace picgb
