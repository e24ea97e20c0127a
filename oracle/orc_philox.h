/*
 * Oracle copy of the counter-based normal generator that feeds every initial
 * condition (test infrastructure only: nothing in the product includes this).
 *
 * Philox-4x32-10 follows J. Salmon, M. Moraes, R. Dror, D. Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3", SC'11 (multipliers 0xD2511F53 and
 * 0xCD9E8D57, Weyl key increments 0x9E3779B9 / 0xBB67AE85, ten rounds).
 * The normal transform is Box-Muller (G. Box, M. Muller, Ann. Math. Stat.
 * 29 (1958) 610) on two 53-bit uniforms.
 *
 * The reference draws four arrays of `length` Gaussian deviates in sequence
 * from one MKL VSL_BRNG_SFMT19937 stream (src/common/init.cpp:40,49-52).
 * MKL is not available, so the deviate for array a (0..3) at lattice offset m
 * is defined here as orc_normal(seed, a, m); the GPU initialiser computes the
 * same function of (seed, a, m), which makes the draw order-independent.
 */
#ifndef ORC_PHILOX_H
#define ORC_PHILOX_H

#include <stdint.h>
#include <math.h>

static inline void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Gaussian deviate number m of array a (a = 0..3) for a given seed. */
static inline double orc_normal(uint64_t seed, int a, int64_t m) {
    uint32_t ctr[4] = { (uint32_t)((uint64_t)m & 0xffffffffu), (uint32_t)((uint64_t)m >> 32),
                        (uint32_t)(a >> 1), 0x41585331u };
    uint32_t key[2] = { (uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32) };
    uint32_t x[4];
    orc_philox4x32_10(ctr, key, x);
    uint64_t b1 = ((uint64_t)x[0] << 21) ^ (uint64_t)(x[1] >> 11);   /* 53 bits */
    uint64_t b2 = ((uint64_t)x[2] << 21) ^ (uint64_t)(x[3] >> 11);
    b1 &= ((uint64_t)1 << 53) - 1;
    b2 &= ((uint64_t)1 << 53) - 1;
    const double two_m53 = 1.1102230246251565404e-16; /* 2^-53 */
    double u1 = (double)(b1 + 1) * two_m53;           /* (0, 1] */
    double u2 = (double)b2 * two_m53;                 /* [0, 1) */
    double r = sqrt(-2.0 * log(u1));
    double ang = 6.283185307179586232 * u2;
    return (a & 1) ? r * sin(ang) : r * cos(ang);
}

#endif
