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

template <int K>
__global__ void __launch_bounds__(kThreads) count_full(ScanWork w, long long m0, long long m1, CandSink sink,
                                                       uint32_t* dump) {
    constexpr int ROWS = pow3(K - 1);
    __shared__ uint64_t sp[(ROWS < 9 ? ROWS : 9) * kWordChunk];
    for (long long m = m0 + blockIdx.x; m < m1; m += gridDim.x) full_prefix<K>(w, m, sink, dump, sp);
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
