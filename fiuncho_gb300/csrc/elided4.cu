// Reduced-work counting kernel for one-hot data at order 4 (16 of the 81
// cells counted per class; derivation in elided4_prefix.cuh) and the triple
// cores it reads.
#include "elided4_prefix.cuh"

#include <algorithm>

namespace fiu {

// Cores of all triples i < j < k (8 cells per class as uint16, two 16-byte
// words).  CTA per pair (i, j) (grid-stride over pair ranks), its four AND
// rows (x, y) staged in shared memory, threads over k.
__global__ void __launch_bounds__(kEThreads) triple_cores_kernel(DevData d, uint4* __restrict__ triples) {
    extern __shared__ uint64_t srow[];  // [4][cw + tw]
    const int WT = d.cw + d.tw, S = d.snps;
    const size_t per_snp = 3 * (size_t)WT;
    const long long npairs = (long long)S * (S - 1) / 2;
    for (long long p = blockIdx.x; p < npairs; p += gridDim.x) {
        // unrank the pair: the first element i is the largest with rank(i, i+1) <= p
        int lo = 0, hi = S - 2;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((long long)mid * (2ll * S - mid - 1) / 2 <= p) lo = mid;
            else hi = mid - 1;
        }
        const int i = lo, j = i + 1 + (int)(p - (long long)i * (2ll * S - i - 1) / 2);
        if (j >= S - 1) continue;  // no k after j (uniform across the CTA)
        __syncthreads();
        for (int e = threadIdx.x; e < 4 * WT; e += kEThreads) {
            const int r = e / WT, ww = e - r * WT;
            const bool cls = ww >= d.cw;
            const int W = cls ? d.tw : d.cw, w = cls ? ww - d.cw : ww;
            const size_t off = (cls ? 3 * (size_t)d.cw : 0) + (size_t)w;
            srow[e] = d.ref[i * per_snp + off + (size_t)(r >> 1) * W] & d.ref[j * per_snp + off + (size_t)(r & 1) * W];
        }
        __syncthreads();
        for (int k = j + 1 + threadIdx.x; k < S; k += kEThreads) {
            uint32_t c[2][8];
#pragma unroll
            for (int cls = 0; cls < 2; ++cls) {
                const int W = cls ? d.tw : d.cw;
                const uint64_t* L = d.tr + (size_t)(cls ? 3 * d.cw : 0) * S + k;
                const uint64_t* pr = srow + (cls ? d.cw : 0);
#pragma unroll
                for (int q = 0; q < 8; ++q) c[cls][q] = 0;
                for (int w = 0; w < W; ++w) {
                    const uint64_t l0 = __ldg(L + (size_t)w * S), l1 = __ldg(L + (size_t)(W + w) * S);
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        const uint64_t pv = pr[r * WT + w];
                        c[cls][r * 2 + 0] += __popcll(pv & l0);
                        c[cls][r * 2 + 1] += __popcll(pv & l1);
                    }
                }
            }
            const long long t = triple_index(i, j, k, S);
            triples[2 * t] = make_uint4(c[0][0] | (c[0][1] << 16), c[0][2] | (c[0][3] << 16),
                                        c[0][4] | (c[0][5] << 16), c[0][6] | (c[0][7] << 16));
            triples[2 * t + 1] = make_uint4(c[1][0] | (c[1][1] << 16), c[1][2] | (c[1][3] << 16),
                                            c[1][4] | (c[1][5] << 16), c[1][6] | (c[1][7] << 16));
        }
    }
}

size_t triples_bytes(int snps) { return (size_t)binom(snps, 3) * 2 * sizeof(uint4); }

cudaError_t build_triples(const DevData& d, uint4* triples, int sms, cudaStream_t s) {
    const size_t smem = 4 * (size_t)(d.cw + d.tw) * sizeof(uint64_t);
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(triple_cores_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long npairs = (long long)d.snps * (d.snps - 1) / 2;
    const int grid = (int)std::min<long long>(std::max<long long>(npairs, 1), (long long)sms * 8);
    triple_cores_kernel<<<grid, kEThreads, smem, s>>>(d, triples);
    count_launch();
    return cudaGetLastError();
}

size_t elided4_smem(int cw, int tw) { return elided4_words(cw, tw) * sizeof(uint64_t); }

template <bool HS, int TP>
__global__ void __launch_bounds__(kEThreads, 2) count_elided4(ScanWork w, long long m0, long long m1, CandSink sink,
                                                          uint32_t* dump, const uint32_t* __restrict__ single,
                                                          const uint4* __restrict__ pairs,
                                                          const uint4* __restrict__ triples) {
    extern __shared__ uint64_t sp[];  // (kEThreads / TP) groups x elided4_words
    constexpr int G = kEThreads / TP;
    const int grp = threadIdx.x / TP;
    const size_t words = elided4_words(w.d.cw, w.d.tw);
    for (long long m = m0 + (long long)blockIdx.x * G + grp; m < m1; m += (long long)gridDim.x * G)
        elided4_prefix<HS, TP>(w, m, sink, dump, single, pairs, triples, sp + grp * words, grp);
}

template <bool HS, int TP>
static cudaError_t launch_e4(const ScanWork& w, long long m0, long long m1, const CandSink& sink, uint32_t* dump,
                             const uint32_t* single, const uint4* pairs, const uint4* triples, cudaStream_t s,
                             int sms) {
    constexpr int G = kEThreads / TP;
    const size_t smem = G * elided4_smem(w.d.cw, w.d.tw);
    if (smem > kMaxGroupSmem) return cudaErrorInvalidConfiguration;
    static int per_sm = 0;
    static size_t per_sm_smem = 0;
    if (!per_sm || per_sm_smem != smem) {
        cudaError_t e =
            cudaFuncSetAttribute(count_elided4<HS, TP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, count_elided4<HS, TP>, kEThreads, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        per_sm_smem = smem;
    }
    const long long ctas = (m1 - m0 + G - 1) / G;
    if (ctas <= 0) return cudaSuccess;
    const long long grid = ctas < (long long)sms * per_sm ? ctas : (long long)sms * per_sm;
    count_elided4<HS, TP><<<(unsigned)grid, kEThreads, smem, s>>>(w, m0, m1, sink, dump, single, pairs, triples);
    count_launch();
    return cudaGetLastError();
}

template <bool HS>
static cudaError_t launch_e4_tp(int tp, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                                uint32_t* dump, const uint32_t* single, const uint4* pairs, const uint4* triples,
                                cudaStream_t s, int sms) {
    switch (tp) {
        case 32: return launch_e4<HS, 32>(w, m0, m1, sink, dump, single, pairs, triples, s, sms);
        case 64: return launch_e4<HS, 64>(w, m0, m1, sink, dump, single, pairs, triples, s, sms);
        case 128: return launch_e4<HS, 128>(w, m0, m1, sink, dump, single, pairs, triples, s, sms);
        default: return launch_e4<HS, 256>(w, m0, m1, sink, dump, single, pairs, triples, s, sms);
    }
}

cudaError_t launch_elided4(bool hs, int tp, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                           uint32_t* dump, const uint32_t* single, const uint4* pairs, const uint4* triples,
                           cudaStream_t s, int sms) {
    if (w.order != 4 || !single || !pairs || !triples) return cudaErrorInvalidValue;
    return hs ? launch_e4_tp<true>(tp, w, m0, m1, sink, dump, single, pairs, triples, s, sms)
              : launch_e4_tp<false>(tp, w, m0, m1, sink, dump, single, pairs, triples, s, sms);
}

}  // namespace fiu
