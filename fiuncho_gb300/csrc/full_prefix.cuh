// Per-prefix body of the generic full-table counting kernel (shared by the
// single-scan kernel in count.cu and the multi-scan round kernel in batch.cu).
// Semantics: see count.cu.
#pragma once

#include "digest.cuh"
#include "internal.h"

namespace fiu {

__host__ __device__ constexpr int pow3(int k) { return k == 0 ? 1 : 3 * pow3(k - 1); }

constexpr int kThreads = 256;   // one last SNP per thread, 256 per l-block
constexpr int kWordChunk = 64;  // prefix words staged per pass

// Shared-memory words one group of the full-table kernel stages.
__host__ __device__ constexpr int full_group_words(int order) {
    return (pow3(order - 1) < 9 ? pow3(order - 1) : 9) * kWordChunk;
}

// ---------------------------------------------------------------------------
// Kernel 0: full 3^K table for any data.  One CTA iterates owned prefixes
// (grid-stride over prefix ordinals [m0, m1)); per prefix it stages the
// 3^(K-1) prefix rows of a word chunk in shared memory (the combine step) and
// every thread accumulates the cells of its own last SNP l, reading the
// last-SNP rows from the SNP-fastest transposed copy (coalesced 256 B per warp).
// Prefix rows are processed in groups of up to 9 so that the accumulators
// (2 classes x 27) stay in registers for every order.
// One prefix (owned ordinal m) of count_full, processed by the TP threads of
// group `grp` (TP = last SNPs per pass, the l-tile width); the function
// synchronises that group only.  `sp` holds RG * kWordChunk words.
template <int K, int TP>
__device__ __forceinline__ void full_prefix(const ScanWork& w, long long m, const CandSink& sink, uint32_t* dump,
                                            uint64_t* sp, int grp) {
    constexpr int P = K - 1;
    constexpr int ROWS = pow3(P);
    constexpr int RG = ROWS < 9 ? ROWS : 9;
    constexpr int NG = ROWS / RG;
    constexpr int CELLS = ROWS * 3;
    const DevData& d = w.d;
    const int S = d.snps;
    const size_t per_snp = 3 * (size_t)(d.cw + d.tw);
    const int lane = threadIdx.x & 31;
    const int gt = threadIdx.x % TP;
    {
        int c[K];
        unrank((long long)w.dist_offset + m * (long long)w.dist_step, w.dist_n, P, c);
        const int last = c[P - 1];
        if (sink.evaluated && gt == 0 && last + 1 < S)
            atomicAdd(sink.evaluated, (unsigned long long)(S - 1 - last));
        for (int l0 = last + 1; l0 < S; l0 += TP) {
            const int l = l0 + gt;
            const bool valid = l < S;
            long long key = w.base_key;
            for (int g = 0; g < NG; ++g) {
                uint32_t acc[2][RG * 3];
#pragma unroll
                for (int q = 0; q < RG * 3; ++q) acc[0][q] = acc[1][q] = 0;
#pragma unroll
                for (int cls = 0; cls < 2; ++cls) {
                    const int W = cls ? d.tw : d.cw;
                    const int roff = cls ? 3 * d.cw : 0;
                    for (int w0 = 0; w0 < W; w0 += kWordChunk) {
                        const int wn = min(kWordChunk, W - w0);
                        group_sync<TP>(grp);
                        for (int e = gt; e < RG * wn; e += TP) {
                            const int rr = e / wn, ww = e - rr * wn;
                            int rem = g * RG + rr;
                            uint64_t v = ~0ull;
#pragma unroll
                            for (int t = P - 1; t >= 0; --t) {
                                const int x = rem % 3;
                                rem /= 3;
                                v &= __ldg(d.ref + (size_t)c[t] * per_snp + roff + (size_t)x * W + w0 + ww);
                            }
                            sp[rr * kWordChunk + ww] = v;
                        }
                        group_sync<TP>(grp);
                        if (valid) {
                            const uint64_t* col = d.tr + (size_t)(roff + w0) * S + l;
                            for (int ww = 0; ww < wn; ++ww) {
                                const uint64_t L0 = __ldg(col + (size_t)ww * S);
                                const uint64_t L1 = __ldg(col + (size_t)(ww + W) * S);
                                const uint64_t L2 = __ldg(col + (size_t)(ww + 2 * W) * S);
#pragma unroll
                                for (int rr = 0; rr < RG; ++rr) {
                                    const uint64_t p = sp[rr * kWordChunk + ww];
                                    acc[cls][rr * 3 + 0] += __popcll(p & L0);
                                    acc[cls][rr * 3 + 1] += __popcll(p & L1);
                                    acc[cls][rr * 3 + 2] += __popcll(p & L2);
                                }
                            }
                        }
                    }
                }
                if (valid) {
#pragma unroll
                    for (int q = 0; q < RG * 3; ++q) {
                        const uint32_t a = acc[0][q], b = acc[1][q];
                        key += __ldg(d.ftab + a) + __ldg(d.ftab + b) - __ldg(d.ftab + a + b);
                    }
                    // the digest mode of orders <= 4 assembles the table in the thread's scratch row
                    uint32_t* o = dump ? dump + ((size_t)m * S + l) * 2 * CELLS : nullptr;
                    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
                    if (K <= 4 && sink.digest && gtid < sink.dscratch_threads)
                        o = sink.dscratch + (size_t)gtid * 2 * CELLS;
                    if (o) {
                        o += g * RG * 3;
#pragma unroll
                        for (int q = 0; q < RG * 3; ++q) {
                            o[q] = acc[0][q];
                            o[CELLS + q] = acc[1][q];
                        }
                    }
                }
            }
            if (K <= 4 && sink.digest) {
                unsigned long long dg = 0;
                const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
                if (valid && gtid < sink.dscratch_threads) {
                    c[P] = l;
                    dg = dg_table(c, K, S, sink.dscratch + (size_t)gtid * 2 * CELLS, CELLS);
                }
                dg_warp_add(sink.digest, dg);
            }
            // Top-N filter: warp-aggregated append of candidates >= threshold.
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
