// Multi-scan kernels: many scans of different sizes, orders and sample counts
// progress together in rounds.  A round is one persistent launch over the
// union of every active scan's next chunk of prefixes: work items are
// (scan, prefix ordinal) pairs that the CTAs' groups pull from a device work
// queue (one 64-bit cursor per launch, advanced with atomicAdd), locate by
// binary search over the round's entries and unrank on the device.  A group
// takes its next item when it finishes the last, so scans whose prefixes cost
// more (more samples, more last SNPs) never leave a statically assigned tail.
// Each round is followed by one CTA per scan that
// selects its best candidates and raises its admission threshold on the
// device -- so no host round trip is needed between rounds and a whole batch
// can be captured as one CUDA graph.  The final pass re-scores every scan's
// kept candidates in FP64 and writes its top-N.
//
// Reference semantics per scan are those of the single-scan path
// (ThreadedSearch::run, include/fiuncho/ThreadedSearch.h:207-246; MaxArray,
// include/fiuncho/utils/MaxArray.h:31-46), with the same total order.
#include "elided4_prefix.cuh"
#include "full_prefix.cuh"
#include "topn_dev.cuh"

namespace fiu {

constexpr int kRoundThreads = 256;
static_assert(kRoundThreads == kThreads && kRoundThreads == kEThreads, "one block shape for all prefix bodies");

// Round kernels are specialised per family and per l-tile width TP so that
// each keeps the registers of its own prefix bodies: family 0 = reduced-work
// kernels (orders 2-3, Harley-Seal counting), family 1 = full-table kernel
// (orders 2-4; higher orders take the single-scan path), family 2 = the
// order-4 reduced-work kernel (POPC counting).  A CTA holds
// 256 / TP groups, each working on its own prefix.
template <int FAMILY, int TP>
__device__ __forceinline__ void run_prefix(const ScanDesc& sd, long long m, const CandSink& sink, uint64_t* sm,
                                           int grp) {
    if (FAMILY == 0) {
        if (sd.w.order == 2) elided_prefix<2, true, TP>(sd.w, m, sink, nullptr, sd.single, sd.pairs, sm, grp);
        else elided_prefix<3, true, TP>(sd.w, m, sink, nullptr, sd.single, sd.pairs, sm, grp);
    } else if (FAMILY == 2) {
        elided4_prefix<false, TP>(sd.w, m, sink, nullptr, sd.single, sd.pairs, sd.triples, sm, grp);
    } else {
        switch (sd.w.order) {
            case 2: full_prefix<2, TP>(sd.w, m, sink, nullptr, sm, grp); break;
            case 3: full_prefix<3, TP>(sd.w, m, sink, nullptr, sm, grp); break;
            case 4: full_prefix<4, TP>(sd.w, m, sink, nullptr, sm, grp); break;
            default: break;
        }
    }
}

// Shared-memory words of one group for a scan.
__host__ __device__ inline size_t group_words(const ScanDesc& sd) {
    if (sd.kind == FIU_KERNEL_FULL_ID) return (size_t)full_group_words(sd.w.order);
    if (sd.w.order == 4) return elided4_words(sd.w.d.cw, sd.w.d.tw);
    return (size_t)(1 << (sd.w.order - 1)) * (sd.w.d.cw + sd.w.d.tw);
}

size_t round_smem(const ScanDesc& sd) { return (size_t)(kRoundThreads / sd.tp) * group_words(sd) * sizeof(uint64_t); }

// The groups of one CTA may work on prefixes of different scans at once, so
// every group owns a fixed slice of `stride` words (the launch's shared memory
// divided by the groups), never a slice sized by its current scan.
template <int FAMILY, int TP>
__global__ void __launch_bounds__(kRoundThreads, 2) round_kernel(const ScanDesc* __restrict__ scans,
                                                                 ScanState* states,
                                                                 const RoundEntry* __restrict__ ents, int n_ents,
                                                                 long long total, size_t stride,
                                                                 unsigned long long* queue) {
    extern __shared__ uint64_t sm[];
    constexpr int G = kRoundThreads / TP;
    __shared__ long long claim[2][G];  // double-buffered: one group barrier per claim
    const int grp = threadIdx.x / TP;
    for (int it = 0;; ++it) {
        long long g;
        if (TP == 32) {
            unsigned long long c = 0;
            if ((threadIdx.x & 31) == 0) c = atomicAdd(queue, 1ull);
            g = (long long)__shfl_sync(0xffffffffu, c, 0);
        } else {
            if (threadIdx.x % TP == 0) claim[it & 1][grp] = (long long)atomicAdd(queue, 1ull);
            group_sync<TP>(grp);
            g = claim[it & 1][grp];
        }
        if (g >= total) break;
        int lo = 0, hi = n_ents - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (ents[mid].begin <= g) lo = mid;
            else hi = mid - 1;
        }
        const RoundEntry e = ents[lo];
        const ScanDesc& sd = scans[e.scan];
        ScanState* st = states + e.scan;
        const CandSink sink{sd.cand, &st->count, &st->overflow, sd.cap,
                            *reinterpret_cast<volatile long long*>(&st->thr), &st->evaluated};
        run_prefix<FAMILY, TP>(sd, e.m0 + (g - e.begin), sink, sm + grp * stride, grp);
    }
}

static size_t g_round_attr[3][4] = {};
static int g_round_per_sm[3][4] = {};
static bool g_select_attr = false, g_finish_attr = false;
static std::mutex g_round_mu;  // the tables above are shared by every host thread

__global__ void select_scans_kernel(const ScanDesc* __restrict__ scans, ScanState* states, int final_pass);
__global__ void finish_scans_kernel(const ScanDesc* __restrict__ scans, ScanState* states);

static int tp_index(int tp) { return tp == 32 ? 0 : tp == 64 ? 1 : tp == 128 ? 2 : 3; }

static const void* round_fn(int family, int ti) {
    static const void* fns[3][4] = {
        {(const void*)round_kernel<0, 32>, (const void*)round_kernel<0, 64>, (const void*)round_kernel<0, 128>,
         (const void*)round_kernel<0, 256>},
        {(const void*)round_kernel<1, 32>, (const void*)round_kernel<1, 64>, (const void*)round_kernel<1, 128>,
         (const void*)round_kernel<1, 256>},
        {(const void*)round_kernel<2, 32>, (const void*)round_kernel<2, 64>, (const void*)round_kernel<2, 128>,
         (const void*)round_kernel<2, 256>}};
    return fns[family][ti];
}

// Sets the dynamic shared-memory limits of the multi-scan kernels (never
// inside a stream capture) and caches the round kernels' occupancy.
cudaError_t prepare_round_kernels(size_t smem) {
    std::lock_guard<std::mutex> g(g_round_mu);
    cudaError_t e = cudaSuccess;
    for (int f = 0; f < 3; ++f)
        for (int t = 0; t < 4; ++t) {
            if (smem > g_round_attr[f][t] || !g_round_per_sm[f][t]) {
                const size_t want = smem > g_round_attr[f][t] ? smem : g_round_attr[f][t];
                const void* fn = round_fn(f, t);
                e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want);
                if (e != cudaSuccess) return e;
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_round_per_sm[f][t], fn, kRoundThreads, want);
                if (e != cudaSuccess) return e;
                if (g_round_per_sm[f][t] < 1) g_round_per_sm[f][t] = 1;
                g_round_attr[f][t] = want;
            }
        }
    if (!g_select_attr) {
        e = cudaFuncSetAttribute(select_scans_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(kSortCap * sizeof(Cand)));
        if (e != cudaSuccess) return e;
        g_select_attr = true;
    }
    if (!g_finish_attr) {
        e = cudaFuncSetAttribute(finish_scans_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(kSortCap * sizeof(ScoredRec)));
        if (e != cudaSuccess) return e;
        g_finish_attr = true;
    }
    return e;
}

template <int FAMILY, int TP>
static void launch_round_t(unsigned grid, size_t smem, const ScanDesc* scans, ScanState* states,
                           const RoundEntry* ents, int n_ents, long long total, unsigned long long* queue,
                           cudaStream_t s) {
    const size_t stride = smem / sizeof(uint64_t) / (kRoundThreads / TP);
    round_kernel<FAMILY, TP><<<grid, kRoundThreads, smem, s>>>(scans, states, ents, n_ents, total, stride, queue);
}

cudaError_t launch_round(int family, int tp, const ScanDesc* scans, ScanState* states, const RoundEntry* ents,
                         int n_ents, long long total, size_t smem, int sms, unsigned long long* queue,
                         cudaStream_t s) {
    if (total <= 0 || n_ents <= 0) return cudaSuccess;
    if (!queue) return cudaErrorInvalidValue;
    const int ti = tp_index(tp);
    if (family < 0 || family > 2) return cudaErrorInvalidValue;
    size_t sm = 0;
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> g(g_round_mu);
        sm = g_round_attr[family][ti];
        per_sm = g_round_per_sm[family][ti];
    }
    if (smem > sm || !per_sm) return cudaErrorInvalidConfiguration;  // prepare_round_kernels first
    const long long G = kRoundThreads / tp;
    const long long ctas = (total + G - 1) / G, cap = (long long)sms * per_sm;
    const unsigned grid = (unsigned)(ctas < cap ? ctas : cap);
    if (family == 2) {
        switch (ti) {
            case 0: launch_round_t<2, 32>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
            case 1: launch_round_t<2, 64>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
            case 2: launch_round_t<2, 128>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
            default: launch_round_t<2, 256>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
        }
    } else if (family == 0) {
        switch (ti) {
            case 0: launch_round_t<0, 32>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
            case 1: launch_round_t<0, 64>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
            case 2: launch_round_t<0, 128>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
            default: launch_round_t<0, 256>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
        }
    } else {
        switch (ti) {
            case 0: launch_round_t<1, 32>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
            case 1: launch_round_t<1, 64>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
            case 2: launch_round_t<1, 128>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
            default: launch_round_t<1, 256>(grid, sm, scans, states, ents, n_ents, total, queue, s); break;
        }
    }
    count_launch();
    return cudaGetLastError();
}

// One CTA per scan: keeps the best `keep` candidates (streaming tournament over
// kSortCap-entry windows in shared memory), sets the scan's threshold to the
// keep-th best key once `keep` are held.  final_pass also sorts a set that
// never exceeded `keep`.
__global__ void __launch_bounds__(kSortThreads) select_scans_kernel(const ScanDesc* __restrict__ scans,
                                                                    ScanState* states, int final_pass) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cand* sb = reinterpret_cast<Cand*>(smem_raw);
    const ScanDesc& sd = scans[blockIdx.x];
    ScanState* st = states + blockIdx.x;
    unsigned M = st->count;
    if (M > sd.cap) M = sd.cap;
    const unsigned keep = sd.keep;
    if (M <= keep && !final_pass) {
        if (threadIdx.x == 0) st->have = M;
        return;
    }
    const Cand worst{(long long)0x8000000000000000ull, ~0ull};
    unsigned kept = 0, pos = 0;
    do {
        const unsigned room = kSortCap - kept;
        const unsigned take = M - pos < room ? M - pos : room;
        unsigned p = 1;
        while (p < kept + take) p <<= 1;
        for (unsigned i = threadIdx.x; i < p - kept; i += blockDim.x) sb[kept + i] = i < take ? sd.cand[pos + i] : worst;
        __syncthreads();
        block_bitonic<Cand, CandBetter>(sb, p);
        pos += take;
        kept = kept + take < keep ? kept + take : keep;
        __syncthreads();
    } while (pos < M);
    for (unsigned i = threadIdx.x; i < kept; i += blockDim.x) sd.cand[i] = sb[i];
    if (threadIdx.x == 0) {
        st->have = kept;
        st->count = kept;
        if (kept == keep && M > keep) st->thr = sb[keep - 1].key;
    }
}

cudaError_t launch_select_scans(const ScanDesc* scans, ScanState* states, int n_scans, int final_pass,
                                cudaStream_t s) {
    if (n_scans <= 0) return cudaSuccess;
    if (!g_select_attr) return cudaErrorInvalidConfiguration;
    select_scans_kernel<<<n_scans, kSortThreads, kSortCap * sizeof(Cand), s>>>(scans, states, final_pass);
    count_launch();
    return cudaGetLastError();
}

// FP64 re-score: one warp per kept candidate slot of every scan.
__global__ void rescore_scans_kernel(const ScanDesc* __restrict__ scans, const ScanState* __restrict__ states,
                                     const unsigned* __restrict__ slot_begin, int n_scans, unsigned total_slots) {
    const unsigned q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= total_slots) return;
    int lo = 0, hi = n_scans - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (slot_begin[mid] <= q) lo = mid;
        else hi = mid - 1;
    }
    const ScanDesc& sd = scans[lo];
    const unsigned i = q - slot_begin[lo];
    if (i >= states[lo].have) return;
    const Cand c = sd.cand[i];
    int comb[kMaxOrder];
    unpack_code(c.code, sd.w.order, sd.w.bits, comb);
    double mi = 0.0;
    combo_tables(sd.w.d, sd.w.order, comb, lane, nullptr, nullptr, &mi);
    if (lane == 0) sd.scored[i] = ScoredRec{mi, c.code, c.key};
}

struct RecBetter {
    __device__ bool operator()(const ScoredRec& a, const ScoredRec& b) const {
        return a.v > b.v || (a.v == b.v && a.code < b.code);
    }
};

// One CTA per scan: sort the re-scored set (MI desc, combination asc) and write the top-N.
__global__ void __launch_bounds__(kSortThreads) finish_scans_kernel(const ScanDesc* __restrict__ scans,
                                                                    ScanState* states) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ScoredRec* sb = reinterpret_cast<ScoredRec*>(smem_raw);
    const ScanDesc& sd = scans[blockIdx.x];
    ScanState* st = states + blockIdx.x;
    const unsigned n = st->have;
    unsigned p = 1;
    while (p < n) p <<= 1;
    for (unsigned i = threadIdx.x; i < p; i += blockDim.x)
        sb[i] = i < n ? sd.scored[i] : ScoredRec{-1.0e300, ~0ull, 0};
    __syncthreads();
    block_bitonic<ScoredRec, RecBetter>(sb, p);
    const unsigned nout = n < sd.outputs ? n : sd.outputs;
    const int k = sd.w.order;
    for (unsigned i = threadIdx.x; i < nout; i += blockDim.x) {
        int comb[kMaxOrder];
        unpack_code(sb[i].code, k, sd.w.bits, comb);
        for (int t = 0; t < k; ++t) sd.out_comb[(size_t)i * k + t] = comb[t];
        sd.out_val[i] = (float)sb[i].v;
        sd.out_val64[i] = sb[i].v;
    }
    if (threadIdx.x == 0) st->n_out = nout;
}

cudaError_t launch_finish_scans(const ScanDesc* scans, ScanState* states, const unsigned* slot_begin, int n_scans,
                                unsigned total_slots, cudaStream_t s) {
    if (n_scans <= 0) return cudaSuccess;
    if (!g_finish_attr) return cudaErrorInvalidConfiguration;
    if (total_slots) {
        rescore_scans_kernel<<<(unsigned)(((size_t)total_slots * 32 + 255) / 256), 256, 0, s>>>(
            scans, states, slot_begin, n_scans, total_slots);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    finish_scans_kernel<<<n_scans, kSortThreads, kSortCap * sizeof(ScoredRec), s>>>(scans, states);
    count_launch();
    return cudaGetLastError();
}

}  // namespace fiu
