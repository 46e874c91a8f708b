// Top-N reduction, FP64 re-scoring and table evaluation of given combinations.
//
// Reference: MaxArray<Result<int,float>>::add (include/fiuncho/utils/MaxArray.h:31-46)
// per thread, then the merge + std::sort(rbegin, rend) + truncate of
// ThreadedSearch::run (include/fiuncho/ThreadedSearch.h:241-245).  Here the
// order is total -- value descending, then combination ascending -- so results
// do not depend on how the work was split.
#include "topn_dev.cuh"

namespace fiu {

template <typename T, typename Better>
static cudaError_t sort_small(T* data, unsigned n, T worst, cudaStream_t st) {
    if (n <= 1) return cudaSuccess;
    if (n > kSortCap) return cudaErrorInvalidValue;
    unsigned p = 1;
    while (p < n) p <<= 1;
    const size_t bytes = (size_t)p * sizeof(T);
    // set once, by whichever host thread comes first (thread-safe static initialisation)
    static const cudaError_t attr = cudaFuncSetAttribute(
        sort_block<T, Better>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kSortCap * sizeof(T)));
    if (attr != cudaSuccess) return attr;
    sort_block<T, Better><<<1, kSortThreads, bytes, st>>>(data, n, worst);
    count_launch();
    return cudaGetLastError();
}

// ---- radix split for sets larger than one CTA can sort ----------------------
// Composite 128-bit rank V = (key ^ 2^63, ~code): larger V is better.
__device__ __forceinline__ unsigned digit_of(const Cand& c, int pass) {
    const unsigned long long hi = (unsigned long long)c.key ^ 0x8000000000000000ull, lo = ~c.code;
    return pass < 8 ? (unsigned)((hi >> (56 - 8 * pass)) & 255u) : (unsigned)((lo >> (56 - 8 * (pass - 8))) & 255u);
}

__global__ void hist_kernel(const Cand* __restrict__ in, unsigned M, int pass, unsigned* __restrict__ hist) {
    __shared__ unsigned h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x)
        atomicAdd(&h[digit_of(in[i], pass)], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// state: [0] need (in/out), [1] chosen digit, [2] entries above the digit, [3] unused
__global__ void pick_kernel(unsigned* hist, unsigned* state) {
    if (threadIdx.x == 0) {
        const unsigned need = state[0];
        unsigned cum = 0;
        int d = 255;
        for (; d > 0; --d) {
            if (cum + hist[d] >= need) break;
            cum += hist[d];
        }
        state[1] = (unsigned)d;
        state[2] = cum;
        state[0] = need - cum;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
}

__global__ void split_kernel(const Cand* __restrict__ in, unsigned M, int pass, const unsigned* __restrict__ state,
                             Cand* __restrict__ sure, unsigned* sure_count, Cand* __restrict__ work,
                             unsigned* work_count) {
    const unsigned dstar = state[1];
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        const Cand c = in[i];
        const unsigned d = digit_of(c, pass);
        if (d > dstar) sure[atomicAdd(sure_count, 1u)] = c;
        else if (d == dstar) work[atomicAdd(work_count, 1u)] = c;
    }
}

__global__ void append_kernel(Cand* dst, const unsigned* dst_count, const Cand* src, unsigned n) {
    const unsigned base = *dst_count;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[base + i] = src[i];
}

cudaError_t select_top(Cand* buf, unsigned M, unsigned keep, Cand* tmp, unsigned* scratch, cudaStream_t s) {
    const Cand worst{(long long)0x8000000000000000ull, ~0ull};
    if (keep == 0 || M == 0) return cudaSuccess;
    if (M <= kSortCap) return sort_small<Cand, CandBetter>(buf, M, worst, s);
    if (keep > kSortCap) return cudaErrorInvalidValue;
    // scratch layout: [0..255] hist, [256..259] state, [260] sure count, [261] work count
    unsigned* hist = scratch;
    unsigned* state = scratch + 256;
    unsigned* sure_count = scratch + 260;
    unsigned* work_count = scratch + 261;
    // The entries known to be kept (fewer than keep <= kSortCap) collect in the
    // first kSortCap slots of tmp; the undecided working set ping-pongs between
    // buf and tmp + kSortCap (so tmp holds kSortCap + M entries).
    Cand* sure = tmp;
    Cand* bufs[2] = {buf, tmp + kSortCap};
    cudaError_t e;
    if ((e = cudaMemsetAsync(scratch, 0, 262 * sizeof(unsigned), s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(state, &keep, sizeof(unsigned), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
    unsigned cur = 0, m = M;
    for (int pass = 0; pass < 16 && m > kSortCap; ++pass) {
        const int grid = (int)((m + 255) / 256 < 1024 ? (m + 255) / 256 : 1024);
        hist_kernel<<<grid, 256, 0, s>>>(bufs[cur], m, pass, hist);
        pick_kernel<<<1, 256, 0, s>>>(hist, state);
        if ((e = cudaMemsetAsync(work_count, 0, sizeof(unsigned), s)) != cudaSuccess) return e;
        split_kernel<<<grid, 256, 0, s>>>(bufs[cur], m, pass, state, sure, sure_count, bufs[cur ^ 1], work_count);
        count_launch(3);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(&m, work_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        cur ^= 1;
    }
    if (m > kSortCap) return cudaErrorInvalidValue;
    // best `need` of the working set join the sure set
    unsigned st[4];
    if ((e = sort_small<Cand, CandBetter>(bufs[cur], m, worst, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(st, state, sizeof(st), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    unsigned nsure = 0;
    if ((e = cudaMemcpyAsync(&nsure, sure_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    const unsigned need = st[0] < m ? st[0] : m;
    if (need) {
        append_kernel<<<(need + 255) / 256, 256, 0, s>>>(sure, sure_count, bufs[cur], need);
        count_launch();
    }
    const unsigned total = nsure + need;
    if ((e = sort_small<Cand, CandBetter>(sure, total, worst, s)) != cudaSuccess) return e;
    return cudaMemcpyAsync(buf, sure, (size_t)(total < keep ? total : keep) * sizeof(Cand), cudaMemcpyDeviceToDevice,
                           s);
}

__global__ void rescore_kernel(DevData d, int K, int bits, const Cand* __restrict__ cands, unsigned n,
                               Scored* __restrict__ out) {
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    int c[kMaxOrder];
    unpack_code(cands[warp].code, K, bits, c);
    double mi = 0.0;
    combo_tables(d, K, c, lane, nullptr, nullptr, &mi);
    if (lane == 0) out[warp] = Scored{mi, cands[warp].code, cands[warp].key};
}

__global__ void unscore_kernel(const Scored* __restrict__ in, unsigned n, Cand* __restrict__ cands,
                               double* __restrict__ mi64) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        cands[i] = Cand{in[i].key, in[i].code};
        mi64[i] = in[i].v;
    }
}

cudaError_t rescore_sort(const DevData& d, int order, int bits, Cand* cands, unsigned n, double* mi64,
                         cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (n > kSortCap) return cudaErrorInvalidValue;
    // Scored scratch lives in the mi64 buffer's companion: allocate transiently.
    Scored* sc = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&sc, (size_t)n * sizeof(Scored), s);
    if (e != cudaSuccess) return e;
    rescore_kernel<<<(n * 32 + 255) / 256, 256, 0, s>>>(d, order, bits, cands, n, sc);
    count_launch();
    if ((e = cudaGetLastError()) == cudaSuccess)
        e = sort_small<Scored, ScoredBetter>(sc, n, Scored{-1.0e300, ~0ull, 0}, s);
    if (e == cudaSuccess) {
        unscore_kernel<<<(n + 255) / 256, 256, 0, s>>>(sc, n, cands, mi64);
        count_launch();
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaFreeAsync(sc, s);
    return e != cudaSuccess ? e : e2;
}

__global__ void tables_kernel(DevData d, int K, const int* __restrict__ combos, size_t count,
                              uint32_t* __restrict__ cases_out, uint32_t* __restrict__ ctrls_out,
                              double* __restrict__ mi64) {
    const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= count) return;
    int cells = 1;
    for (int t = 0; t < K; ++t) cells *= 3;
    int c[kMaxOrder];
    for (int t = 0; t < K; ++t) c[t] = combos[warp * K + t];
    double mi = 0.0;
    combo_tables(d, K, c, lane, cases_out + warp * cells, ctrls_out + warp * cells, &mi);
    if (mi64 && lane == 0) mi64[warp] = mi;
}

cudaError_t launch_tables(const DevData& d, int order, const int* combos, size_t count, uint32_t* cases_out,
                          uint32_t* ctrls_out, double* mi64, cudaStream_t s) {
    if (count == 0) return cudaSuccess;
    const size_t blocks = (count * 32 + 255) / 256;
    tables_kernel<<<(unsigned)blocks, 256, 0, s>>>(d, order, combos, count, cases_out, ctrls_out, mi64);
    count_launch();
    return cudaGetLastError();
}

// MutualInformation::compute over given tables.  mode 0: fixed point (the
// search epilogue), terms beyond the table are evaluated in FP64; mode 1: FP64.
__device__ __forceinline__ long long fix_term(const long long* ftab, long long ftab_max, unsigned long long c) {
    if ((long long)c <= ftab_max) return ftab[c];
    const double v = (double)c * log((double)c) * 4294967296.0;
    return (long long)llrint(v);
}

__global__ void mi_kernel(const uint32_t* __restrict__ cases, const uint32_t* __restrict__ ctrls, size_t cells,
                          size_t count, int n_cases, int n_ctrls, const long long* __restrict__ ftab,
                          long long ftab_max, int mode, float* __restrict__ out, double* __restrict__ out64) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    const uint32_t* a = cases + q * cells;
    const uint32_t* b = ctrls + q * cells;
    const long long Nn = (long long)n_cases + n_ctrls;
    double mi;
    if (mode == 0) {
        long long key = fix_term(ftab, ftab_max, Nn) - fix_term(ftab, ftab_max, n_cases) -
                        fix_term(ftab, ftab_max, n_ctrls);
        for (size_t i = 0; i < cells; ++i)
            key += fix_term(ftab, ftab_max, a[i]) + fix_term(ftab, ftab_max, b[i]) -
                   fix_term(ftab, ftab_max, (unsigned long long)a[i] + b[i]);
        mi = (double)key / ((double)Nn * 4294967296.0);
    } else {
        const double N = (double)Nn;
        double h_y = 0.0, h_x = 0.0, h_xy = 0.0;
        if (n_cases) h_y -= (n_cases / N) * log(n_cases / N);
        if (n_ctrls) h_y -= (n_ctrls / N) * log(n_ctrls / N);
        for (size_t i = 0; i < cells; ++i) {
            const double pc = a[i] / N, pt = b[i] / N, pa = pc + pt;
            if (a[i]) h_xy -= pc * log(pc);
            if (b[i]) h_xy -= pt * log(pt);
            if ((unsigned long long)a[i] + b[i]) h_x -= pa * log(pa);
        }
        mi = h_x + h_y - h_xy;
    }
    out[q] = (float)mi;
    if (out64) out64[q] = mi;
}

cudaError_t launch_mi(const uint32_t* cases, const uint32_t* ctrls, size_t cells, size_t count, int n_cases,
                      int n_ctrls, const long long* ftab, long long ftab_max, int mode, float* out, double* out64,
                      cudaStream_t s) {
    if (count == 0) return cudaSuccess;
    mi_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(cases, ctrls, cells, count, n_cases, n_ctrls, ftab,
                                                              ftab_max, mode, out, out64);
    count_launch();
    return cudaGetLastError();
}

}  // namespace fiu
