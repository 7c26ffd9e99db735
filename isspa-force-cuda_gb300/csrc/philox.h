// philox.h -- counter-based Philox4x32-10 generator (Salmon, Moraes, Dror,
// Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11), host and
// device.  Replaces the reference's per-thread curand XORWOW states
// (init_rand.cu:10-16, isspa_force_cuda.cu:90-105, leapfrog_cuda.cu:44-55):
// every random number is a pure function of (seed, step, window, index), so
// any MC point or thermostat draw can be regenerated without stored state.
//
// Stream layout (ctr = {index, sub, step, window << 8 | stream}):
//   stream 0: MC point of index p, sub = rejection attempt
//   stream 1: thermostat of atom i, sub 0 = collision test, sub 1 = normals
//   stream 2: initial Maxwell-Boltzmann velocities (host)
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define ISSPA_HD __host__ __device__ __forceinline__
#else
#define ISSPA_HD inline
#endif

namespace isspa {

struct u32x4 {
    uint32_t x, y, z, w;
};

ISSPA_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
#if defined(__CUDA_ARCH__)
    lo = a * b;
    hi = __umulhi(a, b);
#else
    uint64_t p = (uint64_t)a * b;
    lo = (uint32_t)p;
    hi = (uint32_t)(p >> 32);
#endif
}

ISSPA_HD u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c.x, hi0, lo0);
        mulhilo32(0xCD9E8D57u, c.z, hi1, lo1);
        c = u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    }
    return c;
}

// uniform in [0, 1): 24 random bits, exact in float
ISSPA_HD float u01(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-08f; }
// uniform in (0, 1]
ISSPA_HD float u01_open0(uint32_t x) { return ((float)(x >> 8) + 1.0f) * 5.9604644775390625e-08f; }

}  // namespace isspa
