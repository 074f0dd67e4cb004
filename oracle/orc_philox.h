/*
 * ORACLE (test infrastructure only): counter-based Gaussian stream shared by
 * the CPU restatement (tcym_oracle.c) and by the RNG shim that replaces GSL
 * when the reference's own sources are compiled (ref_wrap.cpp).
 *
 * Philox4x32-10 is written from its publication (J. Salmon, M. Moraes,
 * R. Dror, D. Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11):
 * ten rounds of two 32x32->64 multiplies with a Weyl key schedule.
 *
 * Stream convention (identical in the CUDA product, csrc/tcym_rng.cuh):
 *   counter = { site, step_lo, step_hi, (stream << 24) | (mu << 8) | j }
 *   key     = { seed_lo, seed_hi }
 * One Philox block gives two Box-Muller normals, for colour components
 * a = 2j (cosine branch) and a = 2j + 1 (sine branch) of E^a_mu(site).
 * The reference draws its Langevin noise in the order z,y,x,mu,a
 * (DYNAMICS/LangevinDynamics.cpp:265-280), which is exactly the linear
 * index a + NA*(mu + 3*site) of ElectricFields (LATTICE/ElectricFields.cpp:36-41),
 * so a sequential shim reproduces (site, mu, a) from the call count.
 */
#ifndef ORC_PHILOX_H
#define ORC_PHILOX_H

#include <math.h>
#include <stdint.h>

#define ORC_STREAM_NOISE 0u   /* Langevin kick xi^a_mu(x, step) */
#define ORC_STREAM_EFIELD 1u  /* Gaussian initial electric field */
#define ORC_STREAM_LINKS 2u   /* algebra angles of random initial links */

static inline void orc_mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

static inline void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        orc_mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
        orc_mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Standard normal for colour component a of E_mu(site) in the given stream and step. */
static inline double orc_normal(uint64_t seed, uint32_t stream, uint64_t step, uint32_t site, uint32_t mu, uint32_t a) {
    uint32_t ctr[4] = {site, (uint32_t)step, (uint32_t)(step >> 32), (stream << 24) | (mu << 8) | (a >> 1)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t x[4];
    orc_philox4x32_10(ctr, key, x);
    const double two_m32 = 2.3283064365386963e-10; /* 2^-32 */
    double u1 = ((double)x[0] + 1.0) * two_m32;     /* (0, 1] */
    double u2 = (double)x[1] * two_m32;             /* [0, 1) */
    double r = sqrt(-2.0 * log(u1));
    double th = 6.283185307179586476925286766559 * u2;
    return (a & 1u) ? r * sin(th) : r * cos(th);
}

#endif
