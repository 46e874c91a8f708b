// Device pieces of the top-N reduction shared by topn.cu and batch.cu:
// the total order of candidates, a one-CTA bitonic sort, and the FP64
// re-scoring of a combination from its recomputed full table.
#pragma once

#include "internal.h"

namespace fiu {

constexpr unsigned kSortCap = 8192;  // largest set sorted inside one CTA
constexpr int kSortThreads = 1024;

struct CandBetter {
    __device__ bool operator()(const Cand& a, const Cand& b) const {
        return a.key > b.key || (a.key == b.key && a.code < b.code);
    }
};

struct Scored {
    double v;
    unsigned long long code;
    long long key;
};

struct ScoredBetter {
    __device__ bool operator()(const Scored& a, const Scored& b) const {
        return a.v > b.v || (a.v == b.v && a.code < b.code);
    }
};

// Best-first bitonic sort of s[0..p) (p a power of two) by the whole block.
template <typename T, typename Better>
__device__ __forceinline__ void block_bitonic(T* s, unsigned p) {
    Better better;
    for (unsigned k = 2; k <= p; k <<= 1) {
        for (unsigned j = k >> 1; j > 0; j >>= 1) {
            for (unsigned i = threadIdx.x; i < p; i += blockDim.x) {
                const unsigned ixj = i ^ j;
                if (ixj > i) {
                    const T a = s[i], b = s[ixj];
                    const bool first_half = (i & k) == 0;
                    if (first_half ? better(b, a) : better(a, b)) {
                        s[i] = b;
                        s[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Sorts n <= kSortCap elements best-first in one CTA (bitonic network in
// shared memory, padded to a power of two with `worst`).
template <typename T, typename Better>
__global__ void __launch_bounds__(kSortThreads) sort_block(T* data, unsigned n, T worst) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* s = reinterpret_cast<T*>(smem_raw);
    unsigned p = 1;
    while (p < n) p <<= 1;
    for (unsigned i = threadIdx.x; i < p; i += blockDim.x) s[i] = i < n ? data[i] : worst;
    __syncthreads();
    block_bitonic<T, Better>(s, p);
    for (unsigned i = threadIdx.x; i < n; i += blockDim.x) data[i] = s[i];
}

// ---- tables of given combinations and FP64 MI --------------------------------
// One warp per combination: for every cell (x_0..x_{K-1}) the lanes stride the
// words of the AND of the K rows, then reduce.  FP64 MI follows the definition
// H(X) + H(Y) - H(X,Y) with p = count / N, cells in index order.
__device__ inline void combo_tables(const DevData& d, int K, const int* c, int lane, uint32_t* cases_out,
                             uint32_t* ctrls_out, double* mi) {
    const size_t per_snp = 3 * (size_t)(d.cw + d.tw);
    int cells = 1;
    for (int t = 0; t < K; ++t) cells *= 3;
    const double N = (double)d.n_cases + (double)d.n_ctrls;
    double h_y = 0.0, h_x = 0.0, h_xy = 0.0;
    if (d.n_cases) h_y -= (d.n_cases / N) * log(d.n_cases / N);
    if (d.n_ctrls) h_y -= (d.n_ctrls / N) * log(d.n_ctrls / N);
    for (int cell = 0; cell < cells; ++cell) {
        uint32_t cnt[2];
        for (int cls = 0; cls < 2; ++cls) {
            const int W = cls ? d.tw : d.cw;
            const size_t roff = cls ? 3 * (size_t)d.cw : 0;
            uint32_t acc = 0;
            for (int w = lane; w < W; w += 32) {
                uint64_t v = ~0ull;
                int rem = cell;
                for (int t = K - 1; t >= 0; --t) {
                    const int x = rem % 3;
                    rem /= 3;
                    v &= __ldg(d.ref + (size_t)c[t] * per_snp + roff + (size_t)x * W + w);
                }
                acc += __popcll(v);
            }
            for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            cnt[cls] = acc;
        }
        if (cases_out && lane == 0) {
            cases_out[cell] = cnt[0];
            ctrls_out[cell] = cnt[1];
        }
        const double pc = cnt[0] / N, pt = cnt[1] / N, pa = pc + pt;
        if (cnt[0]) h_xy -= pc * log(pc);
        if (cnt[1]) h_xy -= pt * log(pt);
        if (cnt[0] + cnt[1]) h_x -= pa * log(pa);
    }
    if (mi) *mi = h_x + h_y - h_xy;
}

}  // namespace fiu
