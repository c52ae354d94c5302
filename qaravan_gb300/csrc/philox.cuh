// Philox4x32-10 counter-based random numbers (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), restated from the
// paper: ten rounds of the bijection on a 128-bit counter under a 64-bit key;
// 53-bit uniforms in [0, 1) from the first two output words. Streams in use:
// trajectories (event, trajectory, stream, 0); shot sampling (shot lo, shot
// hi, 0, 1).
#pragma once

#include <stdint.h>

namespace qgb {

struct Philox {
    __host__ __device__ static inline void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
        const uint64_t p = uint64_t(a) * uint64_t(b);
        hi = uint32_t(p >> 32);
        lo = uint32_t(p);
    }
    // ten rounds of the Philox4x32 bijection
    __host__ __device__ static inline void gen(uint32_t c[4], uint32_t k0, uint32_t k1) {
        for (int r = 0; r < 10; ++r) {
            uint32_t hi0, lo0, hi1, lo1;
            mulhilo(0xD2511F53u, c[0], hi0, lo0);
            mulhilo(0xCD9E8D57u, c[2], hi1, lo1);
            const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
            c[0] = n0;
            c[1] = lo1;
            c[2] = n2;
            c[3] = lo0;
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
    }
    // uniform in [0, 1) with 53 random bits from counter (c0, c1, c2, c3)
    __host__ __device__ static inline double uniform4(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                      uint32_t k0, uint32_t k1) {
        uint32_t c[4] = {c0, c1, c2, c3};
        gen(c, k0, k1);
        const uint64_t bits = (uint64_t(c[0]) << 21) ^ uint64_t(c[1] >> 11);
        return double(bits & ((uint64_t(1) << 53) - 1)) * (1.0 / 9007199254740992.0);
    }
    // the trajectory stream: counter (event, trajectory, stream, 0)
    __host__ __device__ static inline double uniform(uint32_t event, uint32_t traj, uint32_t stream, uint32_t k0,
                                                     uint32_t k1) {
        return uniform4(event, traj, stream, 0u, k0, k1);
    }
};

}  // namespace qgb
