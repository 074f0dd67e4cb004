// Counter-based Gaussian noise for the Langevin kick and the initial conditions.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper.
// Stream convention (part of the library's contract; a seed reproduces the
// same fields on any device and in any batching):
//   counter = { site, step_lo, step_hi, (stream << 24) | (mu << 8) | j }
//   key     = { seed_lo, seed_hi }
// One Philox block gives the Box-Muller pair for colour components
// a = 2j (cosine branch) and a = 2j + 1 (sine branch) of E^a_mu(site).
// In the reference the Langevin noise is a serial GSL loop over z,y,x,mu,a
// (DYNAMICS/LangevinDynamics.cpp:260-286); here each thread draws its own
// components in registers, with no noise array in memory.
#pragma once

#include "tcym_math.cuh"

namespace tcym {

enum : uint32_t { STREAM_NOISE = 0u, STREAM_EFIELD = 1u, STREAM_LINKS = 2u };

TCYM_HD void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
        uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
        uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// Box-Muller pair (z0 for a = 2j, z1 for a = 2j + 1) in precision T.
template <class T>
TCYM_HD void normal_pair(uint64_t seed, uint32_t stream, uint64_t step, uint32_t site, uint32_t mu, uint32_t j, T *z0,
                         T *z1) {
    uint32_t c[4] = {site, (uint32_t)step, (uint32_t)(step >> 32), (stream << 24) | (mu << 8) | j};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const T two_m32 = T(2.3283064365386963e-10);
    T u1 = (T(c[0]) + T(1)) * two_m32;  // (0, 1]
    T u2 = T(c[1]) * two_m32;           // [0, 1)
    T r = Real<T>::sqrt_(T(-2) * Real<T>::log_(u1));
    T s, co;
    Real<T>::sincospi_(T(2) * u2, &s, &co);
    *z0 = r * co;
    *z1 = r * s;
}

// All NA standard normals of E_mu(site) for one step.
template <class T, int NA>
TCYM_HD void normals(uint64_t seed, uint32_t stream, uint64_t step, uint32_t site, uint32_t mu, T *z) {
#pragma unroll
    for (int j = 0; j < (NA + 1) / 2; ++j) {
        T a, b;
        normal_pair<T>(seed, stream, step, site, mu, (uint32_t)j, &a, &b);
        z[2 * j] = a;
        if (2 * j + 1 < NA) z[2 * j + 1] = b;
    }
}

}  // namespace tcym
