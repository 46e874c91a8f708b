// Per-prefix body of the reduced-work (one-hot) counting kernels and their
// helpers, shared by elided.cu (single scan) and batch.cu (round kernel).
// Semantics: see elided.cu.
#pragma once

#include "digest.cuh"
#include "internal.h"

namespace fiu {

constexpr int kEThreads = 256;

__device__ __forceinline__ void csa(uint32_t& h, uint32_t& l, uint32_t a, uint32_t b, uint32_t c) {
    const uint32_t u = a ^ b;
    h = (a & b) | (u & c);
    l = u ^ c;
}

// Carry-save counter of one cell: value = 16*tot + 8*pc(eights) + 4*pc(fours) + 2*pc(twos) + pc(ones) + extra.
struct HSCounter {
    uint32_t ones, twos, fours, eights, tot;
    __device__ __forceinline__ void zero() { ones = twos = fours = eights = tot = 0; }
    __device__ __forceinline__ uint32_t value() const {
        return 16u * tot + 8u * __popc(eights) + 4u * __popc(fours) + 2u * __popc(twos) + __popc(ones);
    }
    // adds the 16 32-bit words (p[k] & q[k]) for k < 8 (64-bit words)
    __device__ __forceinline__ void add8(const uint64_t* p, const uint64_t* q) {
#define D(k) ((uint32_t)((p[(k) >> 1] & q[(k) >> 1]) >> (((k) & 1) * 32)))
        uint32_t twosA, twosB, foursA, foursB, eightsA, eightsB, sixteens;
        csa(twosA, ones, ones, D(0), D(1));
        csa(twosB, ones, ones, D(2), D(3));
        csa(foursA, twos, twos, twosA, twosB);
        csa(twosA, ones, ones, D(4), D(5));
        csa(twosB, ones, ones, D(6), D(7));
        csa(foursB, twos, twos, twosA, twosB);
        csa(eightsA, fours, fours, foursA, foursB);
        csa(twosA, ones, ones, D(8), D(9));
        csa(twosB, ones, ones, D(10), D(11));
        csa(foursA, twos, twos, twosA, twosB);
        csa(twosA, ones, ones, D(12), D(13));
        csa(twosB, ones, ones, D(14), D(15));
        csa(foursB, twos, twos, twosA, twosB);
        csa(eightsB, fours, fours, foursA, foursB);
        csa(sixteens, eights, eights, eightsA, eightsB);
        tot += __popc(sixteens);
#undef D
    }
};

__device__ __forceinline__ long long pair_index(int i, int j, int n) {
    return (long long)i * (2ll * n - i - 1) / 2 + (j - i - 1);
}

// Pair cores packed as 8 uint16 in one 16-byte word: [class][x][y].
__device__ __forceinline__ uint32_t pcore(const uint4& v, int cls, int x, int y) {
    const int k = cls * 4 + x * 2 + y;
    const uint32_t w = (&v.x)[k >> 1];
    return (k & 1) ? (w >> 16) : (w & 0xffffu);
}

// Full order-3 table of one class from its 8 core cells core[(x*2+y)*2+z]
// (genotypes 0/1), the pair cores of (i,j), (i,l), (j,l), the single cores of
// i, j, l and the class size: t[(x*3+y)*3+z] for x, y, z in {0,1,2}.
__device__ __forceinline__ void expand3(const uint32_t* core, const uint4& pij, const uint4& pil, const uint4& pjl,
                                        uint32_t si0, uint32_t si1, uint32_t sj0, uint32_t sj1, uint32_t sl0,
                                        uint32_t sl1, uint32_t n, int cls, uint32_t* t) {
    const uint32_t si[2] = {si0, si1}, sj[2] = {sj0, sj1};
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
#pragma unroll
            for (int z = 0; z < 2; ++z) t[(x * 3 + y) * 3 + z] = core[(x * 2 + y) * 2 + z];
            t[(x * 3 + y) * 3 + 2] = pcore(pij, cls, x, y);
        }
#pragma unroll
    for (int x = 0; x < 2; ++x) {
#pragma unroll
        for (int z = 0; z < 2; ++z) t[(x * 3 + 2) * 3 + z] = pcore(pil, cls, x, z);
        t[(x * 3 + 2) * 3 + 2] = si[x];
    }
#pragma unroll
    for (int y = 0; y < 2; ++y) {
#pragma unroll
        for (int z = 0; z < 2; ++z) t[(2 * 3 + y) * 3 + z] = pcore(pjl, cls, y, z);
        t[(2 * 3 + y) * 3 + 2] = sj[y];
    }
    t[24] = sl0;
    t[25] = sl1;
    t[26] = n;
#pragma unroll
    for (int xy = 0; xy < 9; ++xy) t[xy * 3 + 2] -= t[xy * 3 + 0] + t[xy * 3 + 1];
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int z = 0; z < 3; ++z) t[(x * 3 + 2) * 3 + z] -= t[(x * 3 + 0) * 3 + z] + t[(x * 3 + 1) * 3 + z];
#pragma unroll
    for (int yz = 0; yz < 9; ++yz) t[18 + yz] -= t[yz] + t[9 + yz];
}

// ---------------------------------------------------------------------------
// The reduced-work counting kernel.  Same scheduling as count_full: CTA per
// owned prefix (grid-stride over ordinals), one last SNP l per thread; the
// 2^(K-1) prefix core rows of both classes are staged whole in shared memory.
// One prefix (owned ordinal m) of count_elided; synchronises the block.
// `sp` holds 2^(K-1) * (cw + tw) words.
// Processed by the TP threads of group `grp` (TP = l-tile width); synchronises that group only.
template <int K, bool HS, int TP>
__device__ __forceinline__ void elided_prefix(const ScanWork& w, long long m, const CandSink& sink, uint32_t* dump,
                                              const uint32_t* __restrict__ single, const uint4* __restrict__ pairs,
                                              uint64_t* sp, int grp) {
    constexpr int P = K - 1;
    constexpr int PR = 1 << P;   // prefix core rows
    constexpr int CC = PR * 2;   // counted cells per class
    constexpr int CELLS = K == 2 ? 9 : 27;
    const DevData& d = w.d;
    const int S = d.snps, WT = d.cw + d.tw;
    const size_t per_snp = 3 * (size_t)WT;
    const int lane = threadIdx.x & 31;
    const int gt = threadIdx.x % TP;
    const uint32_t ncls[2] = {(uint32_t)d.n_cases, (uint32_t)d.n_ctrls};
    {
        int c[K];
        unrank((long long)w.dist_offset + m * (long long)w.dist_step, w.dist_n, P, c);
        const int last = c[P - 1];
        if (last + 1 >= S) return;  // uniform across the CTA
        if (sink.evaluated && gt == 0) atomicAdd(sink.evaluated, (unsigned long long)(S - 1 - last));
        group_sync<TP>(grp);
        for (int e = gt; e < PR * WT; e += TP) {
            const int r = e / WT, ww = e - r * WT;
            const bool cls = ww >= d.cw;
            const int W = cls ? d.tw : d.cw, wd = cls ? ww - d.cw : ww;
            uint64_t v = ~0ull;
#pragma unroll
            for (int t = 0; t < P; ++t) {
                const int x = (r >> (P - 1 - t)) & 1;
                v &= __ldg(d.ref + (size_t)c[t] * per_snp + (cls ? 3 * (size_t)d.cw : 0) + (size_t)x * W + wd);
            }
            sp[e] = v;
        }
        group_sync<TP>(grp);
        // prefix-only marginals
        uint32_t si[2][2], sj[2][2];
        uint4 pij = make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int cls = 0; cls < 2; ++cls)
#pragma unroll
            for (int x = 0; x < 2; ++x) {
                si[cls][x] = __ldg(single + c[0] * 4 + cls * 2 + x);
                sj[cls][x] = K == 3 ? __ldg(single + c[P - 1] * 4 + cls * 2 + x) : 0;
            }
        if (K == 3) pij = __ldg(pairs + pair_index(c[0], c[1], S));

        for (int l0 = last + 1; l0 < S; l0 += TP) {
            const int l = l0 + gt;
            const bool valid = l < S;
            long long key = w.base_key;
            unsigned long long dg = 0;
            uint32_t cnt[2][CC];
            if (valid) {
#pragma unroll
                for (int cls = 0; cls < 2; ++cls) {
                    const int W = cls ? d.tw : d.cw;
                    const uint64_t* L = d.tr + (size_t)(cls ? 3 * d.cw : 0) * S + l;
                    const uint64_t* pr = sp + (cls ? d.cw : 0);
                    int wq = 0;
                    if (HS) {
                        HSCounter hc[CC];
#pragma unroll
                        for (int q = 0; q < CC; ++q) hc[q].zero();
                        for (; wq + 8 <= W; wq += 8) {
#pragma unroll
                            for (int z = 0; z < 2; ++z) {
                                uint64_t lz[8];
#pragma unroll
                                for (int k = 0; k < 8; ++k) lz[k] = __ldg(L + (size_t)(z * W + wq + k) * S);
#pragma unroll
                                for (int r = 0; r < PR; ++r) hc[r * 2 + z].add8(pr + r * WT + wq, lz);
                            }
                        }
#pragma unroll
                        for (int q = 0; q < CC; ++q) cnt[cls][q] = hc[q].value();
                    } else {
#pragma unroll
                        for (int q = 0; q < CC; ++q) cnt[cls][q] = 0;
                    }
                    for (; wq < W; ++wq) {
                        const uint64_t l0v = __ldg(L + (size_t)wq * S), l1v = __ldg(L + (size_t)(W + wq) * S);
#pragma unroll
                        for (int r = 0; r < PR; ++r) {
                            const uint64_t p = pr[r * WT + wq];
                            cnt[cls][r * 2 + 0] += __popcll(p & l0v);
                            cnt[cls][r * 2 + 1] += __popcll(p & l1v);
                        }
                    }
                }
                // expand to the full table per class and fold into the key
                uint32_t full[2][CELLS];
                uint4 pil = make_uint4(0, 0, 0, 0), pjl = make_uint4(0, 0, 0, 0);
                if (K == 3) {
                    pil = __ldg(pairs + pair_index(c[0], l, S));
                    pjl = __ldg(pairs + pair_index(c[1], l, S));
                }
#pragma unroll
                for (int cls = 0; cls < 2; ++cls) {
                    const uint32_t sl0 = __ldg(single + l * 4 + cls * 2), sl1 = __ldg(single + l * 4 + cls * 2 + 1);
                    uint32_t* t = full[cls];
                    if (K == 2) {
                        // t[x*3 + z]; index 2 holds "*" before the transform
#pragma unroll
                        for (int x = 0; x < 2; ++x) {
#pragma unroll
                            for (int z = 0; z < 2; ++z) t[x * 3 + z] = cnt[cls][x * 2 + z];
                            t[x * 3 + 2] = si[cls][x];
                        }
                        t[6] = sl0;
                        t[7] = sl1;
                        t[8] = ncls[cls];
#pragma unroll
                        for (int x = 0; x < 3; ++x) t[x * 3 + 2] -= t[x * 3 + 0] + t[x * 3 + 1];
#pragma unroll
                        for (int z = 0; z < 3; ++z) t[6 + z] -= t[z] + t[3 + z];
                    } else {
                        // t[(x*3 + y)*3 + z]
#pragma unroll
                        for (int x = 0; x < 2; ++x)
#pragma unroll
                            for (int y = 0; y < 2; ++y) {
#pragma unroll
                                for (int z = 0; z < 2; ++z) t[(x * 3 + y) * 3 + z] = cnt[cls][(x * 2 + y) * 2 + z];
                                t[(x * 3 + y) * 3 + 2] = pcore(pij, cls, x, y);
                            }
#pragma unroll
                        for (int x = 0; x < 2; ++x) {
#pragma unroll
                            for (int z = 0; z < 2; ++z) t[(x * 3 + 2) * 3 + z] = pcore(pil, cls, x, z);
                            t[(x * 3 + 2) * 3 + 2] = si[cls][x];
                        }
#pragma unroll
                        for (int y = 0; y < 2; ++y) {
#pragma unroll
                            for (int z = 0; z < 2; ++z) t[(2 * 3 + y) * 3 + z] = pcore(pjl, cls, y, z);
                            t[(2 * 3 + y) * 3 + 2] = sj[cls][y];
                        }
                        t[(2 * 3 + 2) * 3 + 0] = sl0;
                        t[(2 * 3 + 2) * 3 + 1] = sl1;
                        t[26] = ncls[cls];
#pragma unroll
                        for (int xy = 0; xy < 9; ++xy) t[xy * 3 + 2] -= t[xy * 3 + 0] + t[xy * 3 + 1];
#pragma unroll
                        for (int x = 0; x < 3; ++x)
#pragma unroll
                            for (int z = 0; z < 3; ++z) t[(x * 3 + 2) * 3 + z] -= t[(x * 3 + 0) * 3 + z] + t[(x * 3 + 1) * 3 + z];
#pragma unroll
                        for (int yz = 0; yz < 9; ++yz) t[18 + yz] -= t[yz] + t[9 + yz];
                    }
                }
#pragma unroll
                for (int q = 0; q < CELLS; ++q) {
                    // derived cells of consistent one-hot data never exceed the class
                    // size; the clamp keeps any inconsistency inside the table
                    const uint32_t a = min(full[0][q], ncls[0]), b = min(full[1][q], ncls[1]);
                    key += __ldg(d.ftab + a) + __ldg(d.ftab + b) - __ldg(d.ftab + a + b);
                }
                if (dump) {
                    uint32_t* o = dump + ((size_t)m * S + l) * 2 * CELLS;
#pragma unroll
                    for (int q = 0; q < CELLS; ++q) {
                        o[q] = full[0][q];
                        o[CELLS + q] = full[1][q];
                    }
                }
                if (sink.digest) {
                    c[P] = l;
                    dg = dg_begin(c, K, S);
#pragma unroll
                    for (int q = 0; q < CELLS; ++q) dg = dg_cell(dg, full[0][q], full[1][q]);
                }
            }
            if (sink.digest) dg_warp_add(sink.digest, dg);
            const bool pass = valid && key >= sink.thr;
            const unsigned mask = __ballot_sync(0xffffffffu, pass);
            if (mask) {
                const int leader = __ffs(mask) - 1;
                unsigned base = 0;
                if (lane == leader) base = atomicAdd(sink.count, (unsigned)__popc(mask));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (pass) {
                    const unsigned idx = base + __popc(mask & ((1u << lane) - 1u));
                    if (idx < sink.cap) {
                        c[P] = l;
                        sink.buf[idx] = Cand{key, pack_code(c, K, w.bits)};
                    } else {
                        atomicOr(sink.overflow, 1u);
                    }
                }
            }
        }
    }
}

}  // namespace fiu
