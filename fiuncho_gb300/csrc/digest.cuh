// Digest of a scan's contingency tables (fiu_scan_digest): the sum over the
// combinations (mod 2^64) of a hash of the combination and its 3^k x 2 cells,
//     v = c[0] n^(k-1) + ... + c[k-1],  h = mix(v + 0x9E3779B97F4A7C15),
//     h = mix(h ^ (cases[x] << 32 | controls[x]))  for each cell x in the
//     reference's cell order (first SNP most significant),
// with mix the SplitMix64 output function (Steele, Lea and Flood, OOPSLA
// 2014).  The sum does not depend on the order of evaluation, so every
// kernel's digest of a whole scan can be compared with the same number taken
// from the reference's own GenotypeTable::combine_and_popcnt tables
// (src/base/gt_popcnt.cpp:4-35) over every combination.
#pragma once

#include "common.cuh"

namespace fiu {

constexpr int kDigestSlots = 256;  // partial sums, summed on the host (spreads the atomics)

__host__ __device__ __forceinline__ unsigned long long dg_mix(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ unsigned long long dg_begin(const int* c, int k, int n) {
    unsigned long long v = 0;
    for (int t = 0; t < k; ++t) v = v * (unsigned long long)n + (unsigned long long)c[t];
    return dg_mix(v + 0x9E3779B97F4A7C15ull);
}

__host__ __device__ __forceinline__ unsigned long long dg_cell(unsigned long long h, uint32_t a, uint32_t b) {
    return dg_mix(h ^ (((unsigned long long)a << 32) | b));
}

// Adds each lane's term (0 for a lane without a combination) into one of the
// partial sums; every lane of the warp calls it.
__device__ __forceinline__ void dg_warp_add(unsigned long long* slots, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(slots + ((blockIdx.x * 32u + (threadIdx.x >> 5)) & (kDigestSlots - 1)), v);
}

// Term of a table held as cases at o[0..cells) and controls at o[cells..2 cells).
__device__ __forceinline__ unsigned long long dg_table(const int* c, int k, int n, const uint32_t* o, int cells) {
    unsigned long long h = dg_begin(c, k, n);
    for (int x = 0; x < cells; ++x) h = dg_cell(h, o[x], o[cells + x]);
    return h;
}

}  // namespace fiu
