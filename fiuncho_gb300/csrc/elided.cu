// Reduced-work counting kernels for one-hot data (orders 2 and 3).
//
// When every SNP's three genotype rows partition the samples of each class
// (checked on upload, the reference's own invariant tests/dataset.cpp:25-44),
// a contingency table is determined by its "core" cells -- genotypes 0 and 1
// only, 2^k of the 3^k cells -- together with the cores of every
// sub-combination.  Writing * for "any genotype", the table over
// {0, 1, *}^k holds at each pattern the core count of the SNPs not at *; the
// genotype-2 slice of an axis is then exactly
//     t[.., 2, ..] = t[.., *, ..] - t[.., 0, ..] - t[.., 1, ..],
// applied axis by axis.  So the kernels count 2^k cells per class (8 instead
// of 27 at order 3) and read the sub-combination cores from precomputed
// tables: single-SNP cores (2 per class) and, for order 3, pair cores
// (4 per class, all pairs, uint16).  The resulting tables are identical to
// combine_and_popcnt's (src/base/gt_popcnt.cpp:4-35) for one-hot data.
//
// Two accumulation schemes:
//   POPC  -- acc += popc(p & l) per 64-bit word (XU pipe, 16 lanes/clk/SM);
//   HS    -- Harley-Seal carry-save adders: per 16 32-bit words, 15 full adders
//            (2 LOP3 each, ALU pipe) and one POPC of the weight-16 word.
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

// ---------------------------------------------------------------------------
// Cores of single SNPs: single[s*4 + cls*2 + x] = popcount of row x of class cls.
__global__ void single_cores_kernel(DevData d, uint32_t* __restrict__ single) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const size_t per_snp = 3 * (size_t)(d.cw + d.tw);
    for (int q = warp; q < d.snps * 4; q += nwarps) {
        const int s = q >> 2, cls = (q >> 1) & 1, x = q & 1;
        const int W = cls ? d.tw : d.cw;
        const uint64_t* row = d.ref + s * per_snp + (cls ? 3 * (size_t)d.cw : 0) + (size_t)x * W;
        uint32_t acc = 0;
        for (int w = lane; w < W; w += 32) acc += __popcll(row[w]);
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) single[q] = acc;
    }
}

// Cores of all pairs i < j (4 cells per class as uint16).  CTA per first SNP i
// (grid-stride), threads over j; i's two core rows staged in shared memory.
__global__ void __launch_bounds__(kEThreads) pair_cores_kernel(DevData d, uint4* __restrict__ pairs) {
    extern __shared__ uint64_t srow[];  // [2][cw + tw]
    const int WT = d.cw + d.tw, S = d.snps;
    const size_t per_snp = 3 * (size_t)WT;
    for (int i = blockIdx.x; i < S - 1; i += gridDim.x) {
        __syncthreads();
        for (int e = threadIdx.x; e < 2 * WT; e += kEThreads) {
            const int x = e / WT, ww = e - x * WT;
            const bool cls = ww >= d.cw;
            const int W = cls ? d.tw : d.cw, w = cls ? ww - d.cw : ww;
            srow[e] = d.ref[i * per_snp + (cls ? 3 * (size_t)d.cw : 0) + (size_t)x * W + w];
        }
        __syncthreads();
        for (int j = i + 1 + threadIdx.x; j < S; j += kEThreads) {
            uint32_t c[2][4];
#pragma unroll
            for (int cls = 0; cls < 2; ++cls) {
                const int W = cls ? d.tw : d.cw;
                const uint64_t* L = d.tr + (size_t)(cls ? 3 * d.cw : 0) * S + j;
                const uint64_t* p0 = srow + (cls ? d.cw : 0);
                const uint64_t* p1 = p0 + WT;
                uint32_t a00 = 0, a01 = 0, a10 = 0, a11 = 0;
                for (int w = 0; w < W; ++w) {
                    const uint64_t l0 = __ldg(L + (size_t)w * S), l1 = __ldg(L + (size_t)(W + w) * S);
                    a00 += __popcll(p0[w] & l0);
                    a01 += __popcll(p0[w] & l1);
                    a10 += __popcll(p1[w] & l0);
                    a11 += __popcll(p1[w] & l1);
                }
                c[cls][0] = a00;
                c[cls][1] = a01;
                c[cls][2] = a10;
                c[cls][3] = a11;
            }
            uint4 v;
            v.x = c[0][0] | (c[0][1] << 16);
            v.y = c[0][2] | (c[0][3] << 16);
            v.z = c[1][0] | (c[1][1] << 16);
            v.w = c[1][2] | (c[1][3] << 16);
            pairs[pair_index(i, j, S)] = v;
        }
    }
}

cudaError_t build_cores(const DevData& d, uint32_t* single, uint4* pairs, int sms, cudaStream_t s) {
    single_cores_kernel<<<sms * 4, 256, 0, s>>>(d, single);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !pairs) return e;
    const size_t smem = 2 * (size_t)(d.cw + d.tw) * sizeof(uint64_t);
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    e = cudaFuncSetAttribute(pair_cores_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int grid = d.snps - 1 < sms * 8 ? (d.snps - 1 > 0 ? d.snps - 1 : 1) : sms * 8;
    pair_cores_kernel<<<grid, kEThreads, smem, s>>>(d, pairs);
    count_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The reduced-work counting kernel.  Same scheduling as count_full: CTA per
// owned prefix (grid-stride over ordinals), one last SNP l per thread; the
// 2^(K-1) prefix core rows of both classes are staged whole in shared memory.
template <int K, bool HS>
__global__ void __launch_bounds__(kEThreads) count_elided(ScanWork w, long long m0, long long m1, CandSink sink,
                                                         uint32_t* dump, const uint32_t* __restrict__ single,
                                                         const uint4* __restrict__ pairs) {
    constexpr int P = K - 1;
    constexpr int PR = 1 << P;   // prefix core rows
    constexpr int CC = PR * 2;   // counted cells per class
    constexpr int CELLS = K == 2 ? 9 : 27;
    extern __shared__ uint64_t sp[];  // [PR][cw + tw]
    const DevData d = w.d;
    const int S = d.snps, WT = d.cw + d.tw;
    const size_t per_snp = 3 * (size_t)WT;
    const int lane = threadIdx.x & 31;
    const uint32_t ncls[2] = {(uint32_t)d.n_cases, (uint32_t)d.n_ctrls};

    for (long long m = m0 + blockIdx.x; m < m1; m += gridDim.x) {
        int c[K];
        unrank((long long)w.dist_offset + m * (long long)w.dist_step, w.dist_n, P, c);
        const int last = c[P - 1];
        if (last + 1 >= S) continue;  // uniform across the CTA
        if (sink.evaluated && threadIdx.x == 0) atomicAdd(sink.evaluated, (unsigned long long)(S - 1 - last));
        __syncthreads();
        for (int e = threadIdx.x; e < PR * WT; e += kEThreads) {
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
        __syncthreads();
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

        for (int l0 = last + 1; l0 < S; l0 += kEThreads) {
            const int l = l0 + threadIdx.x;
            const bool valid = l < S;
            long long key = w.base_key;
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
                    const uint32_t a = full[0][q], b = full[1][q];
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
            }
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

size_t elided_smem(int order, int cw, int tw) { return (size_t)(1 << (order - 1)) * (cw + tw) * sizeof(uint64_t); }

template <int K, bool HS>
static cudaError_t launch_el(const ScanWork& w, long long m0, long long m1, const CandSink& sink, uint32_t* dump,
                             const uint32_t* single, const uint4* pairs, cudaStream_t s, int sms) {
    const size_t smem = elided_smem(K, w.d.cw, w.d.tw);
    static int per_sm = 0;
    static size_t per_sm_smem = 0;
    if (!per_sm || per_sm_smem != smem) {
        cudaError_t e = cudaFuncSetAttribute(count_elided<K, HS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, count_elided<K, HS>, kEThreads, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        per_sm_smem = smem;
    }
    const long long items = m1 - m0;
    if (items <= 0) return cudaSuccess;
    const long long grid = items < (long long)sms * per_sm ? items : (long long)sms * per_sm;
    count_elided<K, HS><<<(unsigned)grid, kEThreads, smem, s>>>(w, m0, m1, sink, dump, single, pairs);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_elided(bool hs, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                          uint32_t* dump, const uint32_t* single, const uint4* pairs, cudaStream_t s, int sms) {
    if (w.order == 2) return hs ? launch_el<2, true>(w, m0, m1, sink, dump, single, pairs, s, sms)
                                : launch_el<2, false>(w, m0, m1, sink, dump, single, pairs, s, sms);
    if (w.order == 3) return hs ? launch_el<3, true>(w, m0, m1, sink, dump, single, pairs, s, sms)
                                : launch_el<3, false>(w, m0, m1, sink, dump, single, pairs, s, sms);
    return cudaErrorInvalidValue;
}

}  // namespace fiu
