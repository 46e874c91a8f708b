// Per-prefix body of the order-4 reduced-work counting kernel, shared by
// elided4.cu (single scan) and batch.cu (round kernel).
//
// For one-hot data a combination (i, j, k, l) is counted on its 16 core cells
// per class -- genotypes x, y, z, w in {0, 1} -- from the 8 prefix rows
// (x, y, z) of (i, j, k), staged in shared memory, and the last SNP's rows 0
// and 1; the other 65 cells follow exactly (the genotype-2 slice of an axis is
// the marginal minus its 0 and 1 slices).  Slice w in {0, 1} of the 81-cell
// table is an order-3 derivation whose pair-like marginals are the cores of
// the triples (i,j,l), (i,k,l), (j,k,l) at w, whose single-like marginals are
// the cores of the pairs (i,l), (j,l), (k,l) at w and whose size is l's core
// w; slice w = 2 is the full table of the prefix triple (i, j, k) minus slices
// 0 and 1.  The MI key is accumulated in three streaming passes over the 81
// cells -- cases, controls, totals -- (the derivation is linear, so the totals
// table is the derivation of the summed cores) with at most two slices live
// in registers.  The tables are identical to combine_and_popcnt's
// (src/base/gt_popcnt.cpp:4-35) for one-hot data.
#pragma once

#include "elided_prefix.cuh"

namespace fiu {

// Lexicographic rank of the triple i < j < k among the triples of n SNPs:
// C(n,3) - C(n-i,3) triples start below i, then the pair (j, k) among the
// n-i-1 SNPs after i.
__host__ __device__ __forceinline__ long long triple_index(int i, int j, int k, int n) {
    auto c3 = [](long long m) { return m < 3 ? 0ll : m * (m - 1) * (m - 2) / 6; };
    const long long m = n - i - 1, a = j - i - 1, b = k - i - 1;
    return c3(n) - c3(n - i) + a * (2 * m - a - 1) / 2 + (b - a - 1);
}

// Shared-memory words of one group: 8 prefix rows of cw + tw words, then the
// prefix triple's packed star table (27 uint32: cases | controls << 16).
__host__ __device__ inline size_t elided4_words(int cw, int tw) { return 8 * (size_t)(cw + tw) + 14; }

// The star table of three SNPs holds at (a, b, c), a, b, c in {0, 1, 2}
// ((a*3+b)*3+c; 2 = any genotype), the core count of the SNPs not at "any".
// Subtracting the 0 and 1 slices from the "any" slice, axis by axis, turns it
// in place into the contingency table t[(x*3+y)*3+z].
__device__ __forceinline__ void star_to_table(uint32_t* t) {
#pragma unroll
    for (int xy = 0; xy < 9; ++xy) t[xy * 3 + 2] -= t[xy * 3 + 0] + t[xy * 3 + 1];
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int z = 0; z < 3; ++z) t[(x * 3 + 2) * 3 + z] -= t[(x * 3 + 0) * 3 + z] + t[(x * 3 + 1) * 3 + z];
#pragma unroll
    for (int yz = 0; yz < 9; ++yz) t[18 + yz] -= t[yz] + t[9 + yz];
}

// Cell (x, y, z) of one class's triple word (8 uint16: [x][y][z]).
__device__ __forceinline__ uint32_t tcell(const uint4& v, int x, int y, int z) {
    const int q = x * 4 + y * 2 + z;
    const uint32_t wv = (&v.x)[q >> 1];
    return (q & 1) ? (wv >> 16) : (wv & 0xffffu);
}

// Value of pass PC (0 cases, 1 controls, 2 both classes summed) from a
// per-class pair of values.
// Sum of 27 floats, pairwise (every term takes part in at most 5 roundings).
__device__ __forceinline__ float e4_sum27(const float* f) {
    float a[14];
#pragma unroll
    for (int q = 0; q < 13; ++q) a[q] = f[2 * q] + f[2 * q + 1];
    a[13] = f[26];
    float b[7];
#pragma unroll
    for (int q = 0; q < 7; ++q) b[q] = a[2 * q] + a[2 * q + 1];
    const float c0 = b[0] + b[1], c1 = b[2] + b[3], c2 = b[4] + b[5], c3 = b[6];
    return (c0 + c1) + (c2 + c3);
}

template <int PC>
__device__ __forceinline__ uint32_t by_pass(uint32_t a, uint32_t b) {
    return PC == 0 ? a : PC == 1 ? b : a + b;
}

// Locations of the sub-combination cores of one combination (i, j, k, l).
// Each pass loads what it reads itself, after a compiler memory barrier, so
// that the loads of a pass are not hoisted above the previous one (fewer
// registers held across the passes; the reloads hit L1).
struct E4Src {
    const uint4* tij;  // triple (i,j,l): two words, cases then controls
    const uint4* tik;  // triple (i,k,l)
    const uint4* tjk;  // triple (j,k,l)
    const uint4* pil;  // pairs (i,l), (j,l), (k,l): [class][x][y] uint16
    const uint4* pjl;
    const uint4* pkl;
    const uint4* sl;   // single l: [class][x]
};

// Sub-combination cores of one combination as read by one pass PC: the triple
// words of the pass's class (ta: cases, or controls for PC 1; tb: controls for
// PC 2, else zero) of (i,j,l), (i,k,l), (j,k,l), and the pair / single words.
struct E4Words {
    uint4 ta[3], tb[3];
    uint4 pil, pjl, pkl, sl;
};

template <int PC>
__device__ __forceinline__ E4Words e4_load(const E4Src& src) {
    asm volatile("" ::: "memory");
    E4Words wd;
    const uint4* tp[3] = {src.tij, src.tik, src.tjk};
#pragma unroll
    for (int u = 0; u < 3; ++u) {
        wd.ta[u] = __ldg(tp[u] + (PC == 1 ? 1 : 0));
        wd.tb[u] = PC == 2 ? __ldg(tp[u] + 1) : make_uint4(0, 0, 0, 0);
    }
    wd.pil = __ldg(src.pil);
    wd.pjl = __ldg(src.pjl);
    wd.pkl = __ldg(src.pkl);
    wd.sl = __ldg(src.sl);
    return wd;
}

// One pass over the 81 cells: the slices l = 0, 1, 2, each an order-3
// derivation from its star table (slice 2's is the prefix's star table,
// pstar(q), minus slices 0 and 1: the derivation is linear); use(sw, t)
// receives each slice's 27 cells t[(x*3+y)*3+z] (cell index
// ((x*3+y)*3+z)*3 + sw).  The counted cores arrive packed:
// cp[cls][r] = core (r, w=0) | core (r, w=1) << 16.
template <int PC, class PStar, class Use>
__device__ __forceinline__ void e4_slices_w(const uint32_t (&cp)[2][8], const E4Words& wd, const PStar& pstar,
                                            Use&& use) {
    auto tri = [&](int u, int x, int y, int z) {
        return PC == 2 ? tcell(wd.ta[u], x, y, z) + tcell(wd.tb[u], x, y, z) : tcell(wd.ta[u], x, y, z);
    };
    auto pr = [&](const uint4& v, int x, int y) { return by_pass<PC>(pcore(v, 0, x, y), pcore(v, 1, x, y)); };
    auto star = [&](int w, int q) -> uint32_t {
        const int a = q / 9, b = (q / 3) % 3, z = q % 3;
        if (a < 2 && b < 2 && z < 2) {
            const int r = (a * 2 + b) * 2 + z;
            return by_pass<PC>(w ? cp[0][r] >> 16 : cp[0][r] & 0xffffu, w ? cp[1][r] >> 16 : cp[1][r] & 0xffffu);
        }
        if (a < 2 && b < 2) return tri(0, a, b, w);
        if (a < 2 && z < 2) return tri(1, a, z, w);
        if (b < 2 && z < 2) return tri(2, b, z, w);
        if (a < 2) return pr(wd.pil, a, w);
        if (b < 2) return pr(wd.pjl, b, w);
        if (z < 2) return pr(wd.pkl, z, w);
        return by_pass<PC>(w ? wd.sl.y : wd.sl.x, w ? wd.sl.w : wd.sl.z);
    };
#pragma unroll
    for (int sw = 0; sw < 3; ++sw) {
        uint32_t t[27];
#pragma unroll
        for (int q = 0; q < 27; ++q) t[q] = sw < 2 ? star(sw, q) : pstar(q) - star(0, q) - star(1, q);
        star_to_table(t);
        use(sw, t);
    }
}

// Both classes in one derivation, packed: a cell's case count in the low and
// its control count in the high 16 bits of one word.  Every count lies below
// 2^16 (classes of at most 65 535 samples) and every intermediate count of a
// consistent one-hot data set is non-negative, so the packed subtractions never
// borrow across the halves.
__device__ __forceinline__ uint32_t pk16(uint32_t c, uint32_t t, int hi) {
    return __byte_perm(c, t, hi ? 0x7632 : 0x5410);  // (c half, t half) -> c | t << 16
}

// Sub-combination cores of one combination (i, j, k, l) for both classes: the
// case (tc) and control (tt) words of the triples (i,j,l), (i,k,l), (j,k,l),
// and the pair / single words (both classes in each).
struct E4Both {
    uint4 tc[3], tt[3];
    uint4 pil, pjl, pkl, sl;
};

// The three slices, packed; use(sw, t) receives slice sw's 27 cells
// t[(x*3+y)*3+z]; ps(q) is the prefix's packed star table.
template <class PS, class Use>
__device__ __forceinline__ void e4_slices_packed(const uint32_t (&cp)[2][8], const E4Both& wd, const PS& ps,
                                                 Use&& use) {
    auto star = [&](int w, int q) -> uint32_t {
        const int a = q / 9, b = (q / 3) % 3, z = q % 3;
        if (a < 2 && b < 2 && z < 2) {
            const int r = (a * 2 + b) * 2 + z;
            return pk16(cp[0][r], cp[1][r], w);
        }
        auto tri = [&](int u, int x, int y) {
            const int c = x * 4 + y * 2 + w;
            return pk16((&wd.tc[u].x)[c >> 1], (&wd.tt[u].x)[c >> 1], c & 1);
        };
        auto pr = [&](const uint4& v, int x) { return pk16((&v.x)[x], (&v.x)[2 + x], w); };
        if (a < 2 && b < 2) return tri(0, a, b);
        if (a < 2 && z < 2) return tri(1, a, z);
        if (b < 2 && z < 2) return tri(2, b, z);
        if (a < 2) return pr(wd.pil, a);
        if (b < 2) return pr(wd.pjl, b);
        if (z < 2) return pr(wd.pkl, z);
        return __byte_perm(w ? wd.sl.y : wd.sl.x, w ? wd.sl.w : wd.sl.z, 0x5410);
    };
#pragma unroll
    for (int sw = 0; sw < 3; ++sw) {
        uint32_t t[27];
#pragma unroll
        for (int q = 0; q < 27; ++q) t[q] = sw < 2 ? star(sw, q) : ps(q) - star(0, q) - star(1, q);
        star_to_table(t);
        use(sw, t);
    }
}

// One slice's contribution to the key estimate, cell by cell, in units of
// 2^-16 bits: the pairwise single-precision sum over its 27 packed cells of
// g = a lg2 a + b lg2 b - (a+b) lg2 (a+b) (a cases, b controls; each g lies in
// [-(a+b), 0]), rounded to 2^-16.  Each 16-bit half becomes the float 2^23 + c
// by a byte permutation, minus 2^23.
__device__ __forceinline__ long long e4_slice_estimate_packed(const uint32_t* t) {
    const float tiny = 9.5367431640625e-07f;  // 2^-20: c*lg2(c + tiny) = 0 at c = 0
    float g[27];
#pragma unroll
    for (int q = 0; q < 27; ++q) {
        const float a = __uint_as_float(__byte_perm(t[q], 0x4B000000u, 0x7610)) - 8388608.0f;
        const float b = __uint_as_float(__byte_perm(t[q], 0x4B000000u, 0x7632)) - 8388608.0f;
        const float sab = a + b;
        float la, lb, ls;
        asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(la) : "f"(a + tiny));
        asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(lb) : "f"(b + tiny));
        asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(ls) : "f"(sab + tiny));
        g[q] = fmaf(a, la, fmaf(b, lb, -sab * ls));
    }
    return __float2ll_rn(e4_sum27(g) * 65536.0f);
}

// The same with the words loaded from their locations (the loads of a pass are
// not hoisted above the previous pass: fewer registers held across passes).
template <int PC, class PStar, class Use>
__device__ __forceinline__ void e4_slices(const uint32_t (&cp)[2][8], const E4Src& src, const PStar& pstar,
                                          Use&& use) {
    const E4Words wd = e4_load<PC>(src);
    e4_slices_w<PC>(cp, wd, pstar, use);
}

// One pass of the exact key: the sum of T[cell] over the pass's 81 cells;
// writes the cells to o[PC * 81 + ((x*3+y)*3+z)*3 + w] if o (cases, controls).
template <int PC, class PStar>
__device__ __forceinline__ long long e4_pass(const uint32_t (&cp)[2][8], const E4Src& src, const PStar& pstar,
                                             const long long* __restrict__ ftab, uint32_t nc, uint32_t* o) {
    long long part = 0;
    e4_slices<PC>(cp, src, pstar, [&](int sw, const uint32_t* t) {
        // derived cells of consistent one-hot data never exceed the class
        // size; the clamp keeps any inconsistency inside the table
#pragma unroll
        for (int q = 0; q < 27; ++q) part += __ldg(ftab + min(t[q], nc));
        if (PC < 2 && o) {
#pragma unroll
            for (int q = 0; q < 27; ++q) o[PC * 81 + q * 3 + sw] = t[q];
        }
    });
    return part;
}

// Locations of the sub-combination cores of a prefix triple (i, j, k).
struct E4Prefix {
    const uint4* tijk;             // triple (i,j,k): cases word, controls word
    const uint4 *pij, *pik, *pjk;  // pairs
    const uint4 *si, *sj, *sk;     // singles
};

// Star table of the prefix triple for pass PC, entry q; nc = the pass's class size.
template <int PC>
struct E4PrefixStar {
    uint4 ta, tb, pij, pik, pjk, si, sj, sk;
    uint32_t nc;
    __device__ __forceinline__ E4PrefixStar(const E4Prefix& pre, uint32_t n) : nc(n) {
        asm volatile("" ::: "memory");
        ta = __ldg(pre.tijk + (PC == 1 ? 1 : 0));
        tb = PC == 2 ? __ldg(pre.tijk + 1) : make_uint4(0, 0, 0, 0);
        pij = __ldg(pre.pij);
        pik = __ldg(pre.pik);
        pjk = __ldg(pre.pjk);
        si = __ldg(pre.si);
        sj = __ldg(pre.sj);
        sk = __ldg(pre.sk);
    }
    __device__ __forceinline__ uint32_t pr(const uint4& v, int x, int y) const {
        return by_pass<PC>(pcore(v, 0, x, y), pcore(v, 1, x, y));
    }
    __device__ __forceinline__ uint32_t sg(const uint4& v, int x) const {
        return by_pass<PC>(x ? v.y : v.x, x ? v.w : v.z);
    }
    __device__ __forceinline__ uint32_t operator()(int q) const {
        const int a = q / 9, b = (q / 3) % 3, z = q % 3;
        if (a < 2 && b < 2 && z < 2) return PC == 2 ? tcell(ta, a, b, z) + tcell(tb, a, b, z) : tcell(ta, a, b, z);
        if (a < 2 && b < 2) return pr(pij, a, b);
        if (a < 2 && z < 2) return pr(pik, a, z);
        if (b < 2 && z < 2) return pr(pjk, b, z);
        if (a < 2) return sg(si, a);
        if (b < 2) return sg(sj, b);
        if (z < 2) return sg(sk, z);
        return nc;
    }
};

// Packed star table of the prefix triple (i, j, k) (both classes), entry q,
// from the prefix's cores: triple (cases tc, controls tt), pairs (i,j), (i,k),
// (j,k), singles i, j, k; nn = n_cases | n_ctrls << 16.
struct E4PrefixStarPacked {
    uint4 tc, tt, pij, pik, pjk, si, sj, sk;
    uint32_t nn;
    __device__ __forceinline__ uint32_t operator()(int q) const {
        const int a = q / 9, b = (q / 3) % 3, z = q % 3;
        auto pr = [](const uint4& v, int x, int y) { return pk16((&v.x)[x], (&v.x)[2 + x], y); };
        auto sg = [](const uint4& v, int x) { return __byte_perm(x ? v.y : v.x, x ? v.w : v.z, 0x5410); };
        if (a < 2 && b < 2 && z < 2) {
            const int c = a * 4 + b * 2 + z;
            return pk16((&tc.x)[c >> 1], (&tt.x)[c >> 1], c & 1);
        }
        if (a < 2 && b < 2) return pr(pij, a, b);
        if (a < 2 && z < 2) return pr(pik, a, z);
        if (b < 2 && z < 2) return pr(pjk, b, z);
        if (a < 2) return sg(si, a);
        if (b < 2) return sg(sj, b);
        if (z < 2) return sg(sk, z);
        return nn;
    }
};

// Both classes' words of one combination, loaded from their locations.
__device__ __forceinline__ E4Both e4_load_both(const E4Src& src) {
    E4Both wd;
    const uint4* tp[3] = {src.tij, src.tik, src.tjk};
#pragma unroll
    for (int u = 0; u < 3; ++u) {
        wd.tc[u] = __ldg(tp[u]);
        wd.tt[u] = __ldg(tp[u] + 1);
    }
    wd.pil = __ldg(src.pil);
    wd.pjl = __ldg(src.pjl);
    wd.pkl = __ldg(src.pkl);
    wd.sl = __ldg(src.sl);
    return wd;
}

// The packed star table of a prefix triple from its cores' locations.
__device__ __forceinline__ E4PrefixStarPacked e4_prefix_packed(const E4Prefix& pre, uint32_t n0, uint32_t n1) {
    E4PrefixStarPacked ps;
    ps.tc = __ldg(pre.tijk);
    ps.tt = __ldg(pre.tijk + 1);
    ps.pij = __ldg(pre.pij);
    ps.pik = __ldg(pre.pik);
    ps.pjk = __ldg(pre.pjk);
    ps.si = __ldg(pre.si);
    ps.sj = __ldg(pre.sj);
    ps.sk = __ldg(pre.sk);
    ps.nn = n0 | n1 << 16;
    return ps;
}

// The exact key of one combination (minus the base) from one packed
// derivation of both classes: the sum over the 81 cells of
// T[a] + T[b] - T[a + b] (a cases, b controls; each clamped to its class
// size, so that an inconsistent input stays inside the table).  Equal to the
// three passes e4_pass<0> + e4_pass<1> - e4_pass<2> on consistent one-hot
// data; writes the tables to o (cases at o[q*3+sw], controls at
// o[81+q*3+sw]) if o.
template <class PS>
__device__ __forceinline__ long long e4_exact_packed(const uint32_t (&cp)[2][8], const E4Both& wd, const PS& ps,
                                                     const long long* __restrict__ ftab, uint32_t n0, uint32_t n1,
                                                     uint32_t* o) {
    long long part = 0;
    e4_slices_packed(cp, wd, ps, [&](int sw, const uint32_t* t) {
#pragma unroll
        for (int q = 0; q < 27; ++q) {
            const uint32_t a = min(t[q] & 0xffffu, n0), b = min(t[q] >> 16, n1);
            part += __ldg(ftab + a) + __ldg(ftab + b) - __ldg(ftab + a + b);
        }
        if (o) {
#pragma unroll
            for (int q = 0; q < 27; ++q) {
                o[q * 3 + sw] = t[q] & 0xffffu;
                o[81 + q * 3 + sw] = t[q] >> 16;
            }
        }
    });
    return part;
}

// Exact pass with the prefix star table computed from the prefix's cores.
template <int PC>
__device__ __forceinline__ long long e4p_pass(const uint32_t (&cp)[2][8], const E4Src& src, const E4Prefix& pre,
                                              const long long* __restrict__ ftab, uint32_t nc, uint32_t* o) {
    const E4PrefixStar<PC> ps(pre, nc);
    return e4_pass<PC>(cp, src, ps, ftab, nc, o);
}

// One prefix (owned ordinal m): the TP threads of group grp, one last SNP per
// thread; sp holds elided4_words(cw, tw) words.  Synchronises the group only.
template <bool HS, int TP>
__device__ __forceinline__ void elided4_prefix(const ScanWork& w, long long m, const CandSink& sink, uint32_t* dump,
                                               const uint32_t* __restrict__ single, const uint4* __restrict__ pairs,
                                               const uint4* __restrict__ triples, uint64_t* sp, int grp) {
    const DevData& d = w.d;
    const int S = d.snps, WT = d.cw + d.tw;
    const size_t per_snp = 3 * (size_t)WT;
    const int lane = threadIdx.x & 31;
    const int gt = threadIdx.x % TP;
    const uint4* single4 = reinterpret_cast<const uint4*>(single);
    uint32_t* ptab = reinterpret_cast<uint32_t*>(sp + 8 * (size_t)WT);
    int c[4];
    unrank((long long)w.dist_offset + m * (long long)w.dist_step, w.dist_n, 3, c);
    const int last = c[2];
    if (last + 1 >= S) return;  // uniform across the group
    if (sink.evaluated && gt == 0) atomicAdd(sink.evaluated, (unsigned long long)(S - 1 - last));
    group_sync<TP>(grp);
    for (int e = gt; e < 8 * WT; e += TP) {
        const int r = e / WT, ww = e - r * WT;
        const bool cls = ww >= d.cw;
        const int W = cls ? d.tw : d.cw, wd = cls ? ww - d.cw : ww;
        const size_t off = (cls ? 3 * (size_t)d.cw : 0) + (size_t)wd;
        sp[e] = __ldg(d.ref + (size_t)c[0] * per_snp + off + (size_t)(r >> 2) * W) &
                __ldg(d.ref + (size_t)c[1] * per_snp + off + (size_t)((r >> 1) & 1) * W) &
                __ldg(d.ref + (size_t)c[2] * per_snp + off + (size_t)(r & 1) * W);
    }
    if (gt == 0) {  // packed star table of the prefix triple
        E4Prefix pre;
        pre.tijk = triples + 2 * triple_index(c[0], c[1], c[2], S);
        pre.pij = pairs + pair_index(c[0], c[1], S);
        pre.pik = pairs + pair_index(c[0], c[2], S);
        pre.pjk = pairs + pair_index(c[1], c[2], S);
        pre.si = single4 + c[0];
        pre.sj = single4 + c[1];
        pre.sk = single4 + c[2];
        const E4PrefixStarPacked st = e4_prefix_packed(pre, d.n_cases, d.n_ctrls);
#pragma unroll
        for (int q = 0; q < 27; ++q) ptab[q] = st(q);
    }
    group_sync<TP>(grp);

    for (int l0 = last + 1; l0 < S; l0 += TP) {
        const int l = l0 + gt;
        const bool valid = l < S;
        long long key = w.base_key;
        unsigned long long dg = 0;
        if (valid) {
            uint32_t cnt[2][16];
#pragma unroll
            for (int cls = 0; cls < 2; ++cls) {
                const int W = cls ? d.tw : d.cw;
                const uint64_t* L = d.tr + (size_t)(cls ? 3 * d.cw : 0) * S + l;
                const uint64_t* pr = sp + (cls ? d.cw : 0);
                int wq = 0;
                if (HS) {
                    HSCounter hc[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) hc[q].zero();
                    for (; wq + 8 <= W; wq += 8) {
#pragma unroll
                        for (int z = 0; z < 2; ++z) {
                            uint64_t lz[8];
#pragma unroll
                            for (int k = 0; k < 8; ++k) lz[k] = __ldg(L + (size_t)(z * W + wq + k) * S);
#pragma unroll
                            for (int r = 0; r < 8; ++r) hc[r * 2 + z].add8(pr + r * WT + wq, lz);
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 16; ++q) cnt[cls][q] = hc[q].value();
                } else {
#pragma unroll
                    for (int q = 0; q < 16; ++q) cnt[cls][q] = 0;
                }
                for (; wq < W; ++wq) {
                    const uint64_t l0v = __ldg(L + (size_t)wq * S), l1v = __ldg(L + (size_t)(W + wq) * S);
#pragma unroll
                    for (int r = 0; r < 8; ++r) {
                        const uint64_t p = pr[r * WT + wq];
                        cnt[cls][r * 2 + 0] += __popcll(p & l0v);
                        cnt[cls][r * 2 + 1] += __popcll(p & l1v);
                    }
                }
            }
            uint32_t cp[2][8];  // cores <= class size <= 65535
#pragma unroll
            for (int cls = 0; cls < 2; ++cls)
#pragma unroll
                for (int r = 0; r < 8; ++r) cp[cls][r] = cnt[cls][r * 2] | (cnt[cls][r * 2 + 1] << 16);
            E4Src src;
            src.tij = triples + 2 * triple_index(c[0], c[1], l, S);
            src.tik = triples + 2 * triple_index(c[0], c[2], l, S);
            src.tjk = triples + 2 * triple_index(c[1], c[2], l, S);
            src.pil = pairs + pair_index(c[0], l, S);
            src.pjl = pairs + pair_index(c[1], l, S);
            src.pkl = pairs + pair_index(c[2], l, S);
            src.sl = single4 + l;
            uint32_t* o = dump ? dump + ((size_t)m * S + l) * 2 * 81 : nullptr;
            const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
            if (sink.digest && gtid < sink.dscratch_threads) o = sink.dscratch + (size_t)gtid * 2 * 81;
            // key = base + sum over the 81 cells of T[case] + T[control] - T[total]
            key += e4_exact_packed(cp, e4_load_both(src), [&](int q) { return ptab[q]; }, d.ftab, d.n_cases,
                                   d.n_ctrls, o);
            if (sink.digest && o) {
                c[3] = l;
                dg = dg_table(c, 4, S, o, 81);
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
                    c[3] = l;
                    sink.buf[idx] = Cand{key, pack_code(c, 4, w.bits)};
                } else {
                    atomicOr(sink.overflow, 1u);
                }
            }
        }
    }
}

}  // namespace fiu
