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
#include "elided_prefix.cuh"

namespace fiu {

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
    static LaunchCache cache;
    int per_sm = 1;
    e = blocks_per_sm(cache, pair_cores_kernel, kEThreads, smem, per_sm);
    if (e != cudaSuccess) return e;
    const int grid = d.snps - 1 < sms * 8 ? (d.snps - 1 > 0 ? d.snps - 1 : 1) : sms * 8;
    pair_cores_kernel<<<grid, kEThreads, smem, s>>>(d, pairs);
    count_launch();
    return cudaGetLastError();
}

template <int K, bool HS, int TP>
__global__ void __launch_bounds__(kEThreads) count_elided(ScanWork w, long long m0, long long m1, CandSink sink,
                                                         uint32_t* dump, const uint32_t* __restrict__ single,
                                                         const uint4* __restrict__ pairs) {
    extern __shared__ uint64_t sp[];  // (kEThreads / TP) groups x 2^(K-1) x (cw + tw)
    constexpr int G = kEThreads / TP;
    const int grp = threadIdx.x / TP;
    const size_t words = (size_t)(1 << (K - 1)) * (w.d.cw + w.d.tw);
    for (long long m = m0 + (long long)blockIdx.x * G + grp; m < m1; m += (long long)gridDim.x * G)
        elided_prefix<K, HS, TP>(w, m, sink, dump, single, pairs, sp + grp * words, grp);
}

size_t elided_smem(int order, int cw, int tw) { return (size_t)(1 << (order - 1)) * (cw + tw) * sizeof(uint64_t); }

template <int K, bool HS, int TP>
static cudaError_t launch_el(const ScanWork& w, long long m0, long long m1, const CandSink& sink, uint32_t* dump,
                             const uint32_t* single, const uint4* pairs, cudaStream_t s, int sms) {
    constexpr int G = kEThreads / TP;
    const size_t smem = G * elided_smem(K, w.d.cw, w.d.tw);
    if (smem > kMaxGroupSmem) return cudaErrorInvalidConfiguration;
    static LaunchCache cache;
    int per_sm = 1;
    const cudaError_t e = blocks_per_sm(cache, count_elided<K, HS, TP>, kEThreads, smem, per_sm);
    if (e != cudaSuccess) return e;
    const long long ctas = (m1 - m0 + G - 1) / G;
    if (ctas <= 0) return cudaSuccess;
    const long long grid = ctas < (long long)sms * per_sm ? ctas : (long long)sms * per_sm;
    count_elided<K, HS, TP><<<(unsigned)grid, kEThreads, smem, s>>>(w, m0, m1, sink, dump, single, pairs);
    count_launch();
    return cudaGetLastError();
}

template <int K, bool HS>
static cudaError_t launch_el_tp(int tp, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                                uint32_t* dump, const uint32_t* single, const uint4* pairs, cudaStream_t s, int sms) {
    switch (tp) {
        case 32: return launch_el<K, HS, 32>(w, m0, m1, sink, dump, single, pairs, s, sms);
        case 64: return launch_el<K, HS, 64>(w, m0, m1, sink, dump, single, pairs, s, sms);
        case 128: return launch_el<K, HS, 128>(w, m0, m1, sink, dump, single, pairs, s, sms);
        default: return launch_el<K, HS, 256>(w, m0, m1, sink, dump, single, pairs, s, sms);
    }
}

cudaError_t launch_elided(bool hs, int tp, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                          uint32_t* dump, const uint32_t* single, const uint4* pairs, cudaStream_t s, int sms) {
    if (w.order == 2) return hs ? launch_el_tp<2, true>(tp, w, m0, m1, sink, dump, single, pairs, s, sms)
                                : launch_el_tp<2, false>(tp, w, m0, m1, sink, dump, single, pairs, s, sms);
    if (w.order == 3) return hs ? launch_el_tp<3, true>(tp, w, m0, m1, sink, dump, single, pairs, s, sms)
                                : launch_el_tp<3, false>(tp, w, m0, m1, sink, dump, single, pairs, s, sms);
    return cudaErrorInvalidValue;
}

}  // namespace fiu
