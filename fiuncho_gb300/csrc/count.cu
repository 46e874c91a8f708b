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
#include "full_prefix.cuh"

namespace fiu {

template <int K, int TP>
__global__ void __launch_bounds__(kThreads) count_full(ScanWork w, long long m0, long long m1, CandSink sink,
                                                       uint32_t* dump) {
    extern __shared__ uint64_t sp[];  // (kThreads / TP) groups x full_group_words(K)
    constexpr int G = kThreads / TP;
    const int grp = threadIdx.x / TP;
    for (long long m = m0 + (long long)blockIdx.x * G + grp; m < m1; m += (long long)gridDim.x * G)
        full_prefix<K, TP>(w, m, sink, dump, sp + grp * full_group_words(K), grp);
}

template <int K, int TP>
static cudaError_t launch_full(const ScanWork& w, long long m0, long long m1, const CandSink& sink, uint32_t* dump,
                               cudaStream_t s, int sms) {
    constexpr int G = kThreads / TP;
    const size_t smem = (size_t)G * full_group_words(K) * sizeof(uint64_t);
    static LaunchCache cache;
    int per_sm = 1;
    const cudaError_t e = blocks_per_sm(cache, count_full<K, TP>, kThreads, smem, per_sm);
    if (e != cudaSuccess) return e;
    const long long ctas = (m1 - m0 + G - 1) / G;
    if (ctas <= 0) return cudaSuccess;
    const long long grid = ctas < (long long)sms * per_sm ? ctas : (long long)sms * per_sm;
    count_full<K, TP><<<(unsigned)grid, kThreads, smem, s>>>(w, m0, m1, sink, dump);
    count_launch();
    return cudaGetLastError();
}

template <int K>
static cudaError_t launch_full_tp(int tp, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                                  uint32_t* dump, cudaStream_t s, int sms) {
    switch (tp) {
        case 32: return launch_full<K, 32>(w, m0, m1, sink, dump, s, sms);
        case 64: return launch_full<K, 64>(w, m0, m1, sink, dump, s, sms);
        case 128: return launch_full<K, 128>(w, m0, m1, sink, dump, s, sms);
        default: return launch_full<K, 256>(w, m0, m1, sink, dump, s, sms);
    }
}

cudaError_t launch_count(int tp, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                         uint32_t* dump, cudaStream_t s, int sms) {
    switch (w.order) {
        case 2: return launch_full_tp<2>(tp, w, m0, m1, sink, dump, s, sms);
        case 3: return launch_full_tp<3>(tp, w, m0, m1, sink, dump, s, sms);
        case 4: return launch_full_tp<4>(tp, w, m0, m1, sink, dump, s, sms);
        case 5: return launch_full_tp<5>(tp, w, m0, m1, sink, dump, s, sms);
        case 6: return launch_full<6, 256>(w, m0, m1, sink, dump, s, sms);
        case 7: return launch_full<7, 256>(w, m0, m1, sink, dump, s, sms);
        case 8: return launch_full<8, 256>(w, m0, m1, sink, dump, s, sms);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace fiu
