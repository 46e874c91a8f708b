// Contingency-table kernels of the search hot path with the fused mutual
// information epilogue and the top-N candidate filter.
//
// Reference semantics reproduced here (paths in the Fiuncho source tree):
//   prefix table  = chained GenotypeTable::combine      src/base/gt_combine.cpp:3-27
//   cell counts   = GenotypeTable::combine_and_popcnt   src/base/gt_popcnt.cpp:4-35
//   the scan      = ThreadedSearch hot loop             include/fiuncho/ThreadedSearch.h:157-180
//   MI            = MutualInformation<float>::compute   src/base/mi_compute.cpp:16-41
// Cell index of a combination (c_0 < ... < c_{k-1}) with genotypes (x_0..x_{k-1})
// is sum_t x_t * 3^(k-1-t), as the chained combine lays it out.
//
// MI is evaluated exactly in integer fixed point: with T[c] = round(c ln c 2^32),
//   N*MI*2^32 = T[N] - T[n_cases] - T[n_ctrls] + sum_cells (T[a] + T[b] - T[a+b])
// where a, b are the case / control counts of a cell (the identity
// MI = ln N + (S_xy - S_x - S_y)/N holds for any table, so this equals the
// reference's H(X) + H(Y) - H(X,Y) without the cancellation of its FP32 sums).
#include "internal.h"

namespace fiu {

__host__ __device__ constexpr int pow3(int k) { return k == 0 ? 1 : 3 * pow3(k - 1); }

constexpr int kThreads = 256;   // one last SNP per thread, 256 per l-block
constexpr int kWordChunk = 64;  // prefix words staged per pass

// ---------------------------------------------------------------------------
// Kernel 0: full 3^K table for any data.  One CTA iterates owned prefixes
// (grid-stride over prefix ordinals [m0, m1)); per prefix it stages the
// 3^(K-1) prefix rows of a word chunk in shared memory (the combine step) and
// every thread accumulates the cells of its own last SNP l, reading the
// last-SNP rows from the SNP-fastest transposed copy (coalesced 256 B per warp).
// Prefix rows are processed in groups of up to 9 so that the accumulators
// (2 classes x 27) stay in registers for every order.
template <int K>
__global__ void __launch_bounds__(kThreads) count_full(ScanWork w, long long m0, long long m1, CandSink sink,
                                                       uint32_t* dump) {
    constexpr int P = K - 1;
    constexpr int ROWS = pow3(P);
    constexpr int RG = ROWS < 9 ? ROWS : 9;
    constexpr int NG = ROWS / RG;
    constexpr int CELLS = ROWS * 3;
    __shared__ uint64_t sp[RG * kWordChunk];
    const DevData d = w.d;
    const int S = d.snps;
    const size_t per_snp = 3 * (size_t)(d.cw + d.tw);
    const int lane = threadIdx.x & 31;

    for (long long m = m0 + blockIdx.x; m < m1; m += gridDim.x) {
        int c[K];
        unrank((long long)w.dist_offset + m * (long long)w.dist_step, w.dist_n, P, c);
        const int last = c[P - 1];
        if (sink.evaluated && threadIdx.x == 0 && last + 1 < S)
            atomicAdd(sink.evaluated, (unsigned long long)(S - 1 - last));
        for (int l0 = last + 1; l0 < S; l0 += kThreads) {
            const int l = l0 + threadIdx.x;
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
                        __syncthreads();
                        for (int e = threadIdx.x; e < RG * wn; e += kThreads) {
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
                        __syncthreads();
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
                    if (dump) {
                        uint32_t* o = dump + ((size_t)m * S + l) * 2 * CELLS + g * RG * 3;
#pragma unroll
                        for (int q = 0; q < RG * 3; ++q) {
                            o[q] = acc[0][q];
                            o[CELLS + q] = acc[1][q];
                        }
                    }
                }
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

template <int K>
static cudaError_t launch_full(const ScanWork& w, long long m0, long long m1, const CandSink& sink, uint32_t* dump,
                               cudaStream_t s, int sms) {
    static int per_sm = 0;
    if (!per_sm) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, count_full<K>, kThreads, 0);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    const long long items = m1 - m0;
    if (items <= 0) return cudaSuccess;
    const long long grid = items < (long long)sms * per_sm ? items : (long long)sms * per_sm;
    count_full<K><<<(unsigned)grid, kThreads, 0, s>>>(w, m0, m1, sink, dump);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_count(int kernel, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                         uint32_t* dump, cudaStream_t s, int sms) {
    if (kernel != 0) return cudaErrorInvalidValue;
    switch (w.order) {
        case 2: return launch_full<2>(w, m0, m1, sink, dump, s, sms);
        case 3: return launch_full<3>(w, m0, m1, sink, dump, s, sms);
        case 4: return launch_full<4>(w, m0, m1, sink, dump, s, sms);
        case 5: return launch_full<5>(w, m0, m1, sink, dump, s, sms);
        case 6: return launch_full<6>(w, m0, m1, sink, dump, s, sms);
        case 7: return launch_full<7>(w, m0, m1, sink, dump, s, sms);
        case 8: return launch_full<8>(w, m0, m1, sink, dump, s, sms);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace fiu
