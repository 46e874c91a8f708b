/*
 * tabledigest.h -- digest of every contingency table of a scan (TEST
 * INFRASTRUCTURE ONLY; shared by oracle.c and ref_driver.cpp).
 *
 * digest = sum over the combinations c (mod 2^64) of term(c), where
 *   v    = c[0] n^(k-1) + c[1] n^(k-2) + ... + c[k-1]   (uint64, wrapping)
 *   h    = mix(v + 0x9E3779B97F4A7C15)
 *   h    = mix(h ^ (cases[x] << 32 | ctrls[x]))          for every cell x in
 *                                                         reference cell order
 *   term = h
 * and mix is the output function of SplitMix64 (Steele, Lea and Flood,
 * "Fast splittable pseudorandom number generators", OOPSLA 2014).  The sum
 * does not depend on the order in which combinations are visited, and a
 * table that differs in any cell, or sits at another combination, changes it.
 * The CUDA library computes the same digest from its kernels' own tables.
 */
#ifndef FIU_TABLEDIGEST_H
#define FIU_TABLEDIGEST_H
#include <stdint.h>

static inline uint64_t td_mix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline uint64_t td_term(const int *c, int k, uint64_t n, const uint32_t *cases, const uint32_t *ctrls,
                               int cells)
{
    uint64_t v = 0;
    for (int t = 0; t < k; ++t) v = v * n + (uint64_t)c[t];
    uint64_t h = td_mix(v + 0x9E3779B97F4A7C15ull);
    for (int x = 0; x < cells; ++x) h = td_mix(h ^ (((uint64_t)cases[x] << 32) | ctrls[x]));
    return h;
}
#endif
