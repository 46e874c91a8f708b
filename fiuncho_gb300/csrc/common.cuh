// Shared device/host definitions of the GB300 epistasis-search library.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fiu {

constexpr int kMaxOrder = 8;
// counting-kernel ids (same values as FIU_KERNEL_* in fiuncho_gpu.h)
constexpr int FIU_KERNEL_FULL_ID = 1;
constexpr int FIU_KERNEL_ELIDED_POPC_ID = 2;
constexpr int FIU_KERNEL_ELIDED_HS_ID = 3;
constexpr int FIU_KERNEL_TENSOR_ID = 4;
constexpr int kFixShift = 32;  // fixed-point scale of the c*ln(c) table: 2^32

// Candidate of the running top-N: `key` is the fixed-point N*MI*2^32 (larger
// is better), `code` the combination packed most-significant-first with
// `bits` bits per SNP index (so numeric order == lexicographic order).
struct Cand {
    long long key;
    unsigned long long code;
};

// Device view of one scan's genotype data.
//   ref : reference layout, per SNP [3 case rows x cw][3 control rows x tw]
//   tr  : the same matrix transposed, row r of the reference block stored as
//         tr[r * snps + snp] (SNP fastest), r = g*cw + w for cases and
//         3*cw + g*tw + w for controls.  Used for coalesced last-SNP loads.
struct DevData {
    const uint64_t* ref;
    const uint64_t* tr;
    const long long* ftab;  // round(c*ln(c)*2^32), c in [0, 64*(cw+tw)]
    int snps;
    int cw, tw;
    int n_cases, n_ctrls;
};

// Work of one scan: Distribution(n, order-1, step, offset) prefixes
// (include/fiuncho/Distribution.h:24-203); prefix ordinal m has lexicographic
// rank offset + m*step.
struct ScanWork {
    DevData d;
    int order;
    int dist_n, dist_step, dist_offset;
    int bits;              // bits per index in Cand::code
    long long n_prefixes;  // prefixes owned
    long long base_key;    // fixed-point T[N] - T[n_cases] - T[n_ctrls]
};

// Saturating binomial coefficient C(n, k), n < 2^31.
__host__ __device__ inline unsigned long long binom(long long n, int k) {
    if (k < 0 || n < k) return 0;
    if (k > n - k) k = (int)(n - k);
    unsigned long long r = 1;
    for (int i = 1; i <= k; ++i) {
        unsigned __int128 t = (unsigned __int128)r * (unsigned long long)(n - k + i);
        t /= (unsigned)i;
        if (t >> 63) return 1ull << 63;
        r = (unsigned long long)t;
    }
    return r;
}

// Lexicographic unranking of a k-combination of {0..n-1} (rank < C(n,k)).
// The count of combinations whose first element is below x is
// C(n,k) - C(n-x,k) (hockey-stick identity), so each position is found by
// binary search.
__host__ __device__ inline void unrank(long long rank, int n, int k, int* c) {
    int lo_start = 0;
    unsigned long long r = (unsigned long long)rank;
    for (int t = 0; t < k; ++t) {
        const int m = n - lo_start;     // elements still available
        const int kk = k - t;           // elements still to choose
        const unsigned long long total = binom(m, kk);
        // largest x in [0, m-kk] with total - C(m-x, kk) <= r
        int lo = 0, hi = m - kk;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (total - binom(m - mid, kk) <= r) lo = mid; else hi = mid - 1;
        }
        r -= total - binom(m - lo, kk);
        c[t] = lo_start + lo;
        lo_start = c[t] + 1;
    }
}

__host__ __device__ inline unsigned long long pack_code(const int* c, int k, int bits) {
    unsigned long long v = 0;
    for (int t = 0; t < k; ++t) v = (v << bits) | (unsigned long long)c[t];
    return v;
}

__host__ __device__ inline void unpack_code(unsigned long long v, int k, int bits, int* c) {
    const unsigned long long mask = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
    for (int t = k - 1; t >= 0; --t) {
        c[t] = (int)(v & mask);
        v >>= bits;
    }
}

}  // namespace fiu
