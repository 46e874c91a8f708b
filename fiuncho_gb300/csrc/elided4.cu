// Reduced-work counting kernel for one-hot data at order 4 (16 of the 81
// cells counted per class; derivation in elided4_prefix.cuh) and the triple
// cores it reads.
#include "elided4_prefix.cuh"

#include <algorithm>
#include <vector>

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
    static LaunchCache cache;
    int per_sm = 1;
    const cudaError_t e = blocks_per_sm(cache, triple_cores_kernel, kEThreads, smem, per_sm);
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
    static LaunchCache cache;
    int per_sm = 1;
    const cudaError_t e = blocks_per_sm(cache, count_elided4<HS, TP>, kEThreads, smem, per_sm);
    if (e != cudaSuccess) return e;
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

// ---------------------------------------------------------------------------
// Pair-major schedule for a whole-data-set order-4 scan.  A work item is a
// pair (i, j) and a run of kE4PItem consecutive pairs (k, l), j < k < l, in
// lexicographic order; one warp processes it in tiles of 32 lanes, one (k, l)
// per lane, so lanes stay busy across k (a per-prefix tile leaves the lanes
// past the prefix's last SNP idle).  The warp stages the four AND rows (x, y)
// of (i, j) in shared memory, interleaved per word; each lane ANDs them with
// its own k and l rows (one three-input AND per 32-bit half) and counts the
// same 16 core cells per class.  Items of the pairs (i, j) with second element
// j start at begin[j]: j pairs, ceil(C(S-1-j, 2) / kE4PItem) items each.
constexpr int kE4PTiles = 8;
constexpr int kE4PItem = 32 * kE4PTiles;

static long long e4p_items_per_pair(int snps, int j) {
    const long long m = snps - 1 - j;
    return m < 2 ? 0 : (m * (m - 1) / 2 + kE4PItem - 1) / kE4PItem;
}

std::vector<long long> e4p_item_begin(int snps) {
    std::vector<long long> b((size_t)snps + 1, 0);
    for (int j = 0; j < snps; ++j) b[j + 1] = b[j] + (long long)j * e4p_items_per_pair(snps, j);
    return b;
}

size_t e4p_smem(int cw, int tw) { return (size_t)(kEThreads / 32) * 4 * (cw + tw) * sizeof(uint64_t); }

// DIGEST: the digest mode of fiu_scan_digest, compiled separately (the search's
// instantiation carries none of its code).
template <bool DIGEST>
__global__ void __launch_bounds__(kEThreads, 2)
    count_elided4p(ScanWork w, const long long* __restrict__ begin, long long g0, long long g1, CandSink sink,
                   uint32_t* dump, const uint32_t* __restrict__ single, const uint4* __restrict__ pairs,
                   const uint4* __restrict__ triples) {
    extern __shared__ uint64_t sm[];  // per warp: [cw + tw words][4 rows (x, y)]
    const DevData& d = w.d;
    const int S = d.snps, WT = d.cw + d.tw;
    const size_t per_snp = 3 * (size_t)WT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int WPB = kEThreads / 32;
    uint64_t* rows = sm + (size_t)warp * 4 * WT;
    const uint4* single4 = reinterpret_cast<const uint4*>(single);
    for (long long g = g0 + (long long)blockIdx.x * WPB + warp; g < g1; g += (long long)gridDim.x * WPB) {
        // item -> (j, i, run): j is the largest with begin[j] <= g
        int lo = 0, hi = S - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(begin + mid) <= g) lo = mid;
            else hi = mid - 1;
        }
        const int j = lo;
        const long long mm = S - 1 - j, npairs = mm * (mm - 1) / 2;
        const long long per = (npairs + kE4PItem - 1) / kE4PItem;
        const long long rel = g - __ldg(begin + j);
        const int i = (int)(rel / per);
        const long long t0 = (rel - (long long)i * per) * kE4PItem;
        __syncwarp();
        for (int e = lane; e < 4 * WT; e += 32) {
            const int ww = e >> 2, r = e & 3;
            const bool cls = ww >= d.cw;
            const int W = cls ? d.tw : d.cw, wd = cls ? ww - d.cw : ww;
            const size_t off = (cls ? 3 * (size_t)d.cw : 0) + (size_t)wd;
            rows[e] = __ldg(d.ref + (size_t)i * per_snp + off + (size_t)(r >> 1) * W) &
                      __ldg(d.ref + (size_t)j * per_snp + off + (size_t)(r & 1) * W);
        }
        __syncwarp();
        E4Prefix pre;
        pre.pij = pairs + pair_index(i, j, S);
        pre.si = single4 + i;
        pre.sj = single4 + j;
#pragma unroll 1
        for (int tile = 0; tile < kE4PTiles; ++tile) {
            const long long t = t0 + tile * 32 + lane;
            const bool valid = t < npairs;
            if (!__any_sync(0xffffffffu, valid)) break;
            // (k, l) = (j + 1 + a, j + 1 + b), (a, b) the pair of rank t among mm SNPs
            int a = 0;
            if (valid) {
                const double B = 2.0 * (double)mm - 1.0;
                a = (int)((B - sqrt(B * B - 8.0 * (double)t)) * 0.5);
                a = max(0, min(a, (int)mm - 2));
                while (a > 0 && (long long)a * (2 * mm - a - 1) / 2 > t) --a;
                while (a + 1 <= mm - 2 && (long long)(a + 1) * (2 * mm - a - 2) / 2 <= t) ++a;
            }
            const int b = valid ? (int)(t - (long long)a * (2 * mm - a - 1) / 2) + a + 1 : 1;
            const int k = j + 1 + a, l = j + 1 + b;
            long long key = w.base_key;
            unsigned long long dg = 0;
            if (valid) {
                uint32_t cnt[2][16];
#pragma unroll
                for (int cls = 0; cls < 2; ++cls) {
                    const int W = cls ? d.tw : d.cw;
                    const uint64_t* K = d.tr + (size_t)(cls ? 3 * d.cw : 0) * S + k;
                    const uint64_t* L = d.tr + (size_t)(cls ? 3 * d.cw : 0) * S + l;
                    const uint4* R = reinterpret_cast<const uint4*>(rows + (cls ? 4 * (size_t)d.cw : 0));
#pragma unroll
                    for (int q = 0; q < 16; ++q) cnt[cls][q] = 0;
                    for (int wq = 0; wq < W; ++wq) {
                        const uint64_t k0 = __ldg(K + (size_t)wq * S), k1 = __ldg(K + (size_t)(W + wq) * S);
                        const uint64_t l0 = __ldg(L + (size_t)wq * S), l1 = __ldg(L + (size_t)(W + wq) * S);
                        const uint4 r01 = R[2 * wq], r23 = R[2 * wq + 1];
                        const uint64_t pr[4] = {((uint64_t)r01.y << 32) | r01.x, ((uint64_t)r01.w << 32) | r01.z,
                                                ((uint64_t)r23.y << 32) | r23.x, ((uint64_t)r23.w << 32) | r23.z};
#pragma unroll
                        for (int xy = 0; xy < 4; ++xy) {
                            cnt[cls][(xy * 2 + 0) * 2 + 0] += __popcll(pr[xy] & k0 & l0);
                            cnt[cls][(xy * 2 + 0) * 2 + 1] += __popcll(pr[xy] & k0 & l1);
                            cnt[cls][(xy * 2 + 1) * 2 + 0] += __popcll(pr[xy] & k1 & l0);
                            cnt[cls][(xy * 2 + 1) * 2 + 1] += __popcll(pr[xy] & k1 & l1);
                        }
                    }
                }
                uint32_t cp[2][8];  // cores <= class size <= 65535
#pragma unroll
                for (int cls = 0; cls < 2; ++cls)
#pragma unroll
                    for (int r = 0; r < 8; ++r) cp[cls][r] = cnt[cls][r * 2] | (cnt[cls][r * 2 + 1] << 16);
                E4Src src;
                src.tij = triples + 2 * triple_index(i, j, l, S);
                src.tik = triples + 2 * triple_index(i, k, l, S);
                src.tjk = triples + 2 * triple_index(j, k, l, S);
                src.pil = pairs + pair_index(i, l, S);
                src.pjl = pairs + pair_index(j, l, S);
                src.pkl = pairs + pair_index(k, l, S);
                src.sl = single4 + l;
                pre.tijk = triples + 2 * triple_index(i, j, k, S);
                pre.pik = pairs + pair_index(i, k, S);
                pre.pjk = pairs + pair_index(j, k, S);
                pre.sk = single4 + k;
                uint32_t* o = dump ? dump + ((size_t)triple_index(i, j, k, S) * S + l) * 2 * 81 : nullptr;
                const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
                if (DIGEST && gtid < sink.dscratch_threads) o = sink.dscratch + (size_t)gtid * 2 * 81;
                key += e4_exact_packed(cp, e4_load_both(src), e4_prefix_packed(pre, d.n_cases, d.n_ctrls), d.ftab,
                                       d.n_cases, d.n_ctrls, o);
                if (DIGEST && o) {
                    const int cmb[4] = {i, j, k, l};
                    dg = dg_table(cmb, 4, S, o, 81);
                }
            }
            if (DIGEST) dg_warp_add(sink.digest, dg);
            if (sink.evaluated) {
                const unsigned vm = __ballot_sync(0xffffffffu, valid);
                if (lane == 0) atomicAdd(sink.evaluated, (unsigned long long)__popc(vm));
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
                        const int c[4] = {i, j, k, l};
                        sink.buf[idx] = Cand{key, pack_code(c, 4, w.bits)};
                    } else {
                        atomicOr(sink.overflow, 1u);
                    }
                }
            }
        }
    }
}

cudaError_t launch_elided4p(const ScanWork& w, const long long* begin, long long g0, long long g1,
                            const CandSink& sink, uint32_t* dump, const uint32_t* single, const uint4* pairs,
                            const uint4* triples, cudaStream_t s, int sms) {
    if (w.order != 4 || !begin || !single || !pairs || !triples) return cudaErrorInvalidValue;
    const size_t smem = e4p_smem(w.d.cw, w.d.tw);
    if (smem > kMaxGroupSmem) return cudaErrorInvalidConfiguration;
    static LaunchCache cache[2];
    const bool dg = sink.digest != nullptr;
    auto fn = dg ? count_elided4p<true> : count_elided4p<false>;
    int per_sm = 1;
    const cudaError_t e = blocks_per_sm(cache[dg ? 1 : 0], fn, kEThreads, smem, per_sm);
    if (e != cudaSuccess) return e;
    constexpr int WPB = kEThreads / 32;
    const long long ctas = (g1 - g0 + WPB - 1) / WPB;
    if (ctas <= 0) return cudaSuccess;
    const long long grid = ctas < (long long)sms * per_sm ? ctas : (long long)sms * per_sm;
    fn<<<(unsigned)grid, kEThreads, smem, s>>>(w, begin, g0, g1, sink, dump, single, pairs, triples);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_elided4(bool hs, int tp, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                           uint32_t* dump, const uint32_t* single, const uint4* pairs, const uint4* triples,
                           cudaStream_t s, int sms) {
    if (w.order != 4 || !single || !pairs || !triples) return cudaErrorInvalidValue;
    return hs ? launch_e4_tp<true>(tp, w, m0, m1, sink, dump, single, pairs, triples, s, sms)
              : launch_e4_tp<false>(tp, w, m0, m1, sink, dump, single, pairs, triples, s, sms);
}

}  // namespace fiu
