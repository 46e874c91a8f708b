// C ABI of the library (include/fiuncho_gpu.h): contexts, resident data sets,
// the search driver and the kernel-level entries.
#include <algorithm>
#include <chrono>
#include <map>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/fiuncho_gpu.h"
#include "ctx.h"
#include "digest.cuh"

namespace fiu {
thread_local unsigned long long* g_launch_counter = nullptr;
}

using namespace fiu;

namespace fiu {

// Message of the last failure of a call made without a context (this thread).
static thread_local std::string g_free_err;

int fail(fiu_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    else g_free_err = msg;
    return code;
}

int cuda_fail(fiu_ctx* ctx, cudaError_t e, const char* what) {
    const int code = e == cudaErrorMemoryAllocation ? FIU_ERR_NOMEM : FIU_ERR_CUDA;
    return fail(ctx, code, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
static int grow(fiu_ctx* ctx, T*& p, size_t& cap, size_t need) {
    if (need <= cap) return FIU_OK;
    const size_t n = std::max(need, cap * 2);
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc((void**)&p, n * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "device scratch allocation");
    cap = n;
    return FIU_OK;
}

int grow_bytes(fiu_ctx* ctx, char*& p, size_t& cap, size_t need) { return grow(ctx, p, cap, need); }

int grow_host(fiu_ctx* ctx, size_t need) {
    if (need <= ctx->host_arena_cap) return FIU_OK;
    if (ctx->host_arena) cudaFreeHost(ctx->host_arena);
    ctx->host_arena = nullptr;
    ctx->host_arena_cap = 0;
    const size_t n = std::max(need, (size_t)1 << 20);
    cudaError_t e = cudaMallocHost((void**)&ctx->host_arena, n);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pinned host allocation");
    ctx->host_arena_cap = n;
    return FIU_OK;
}

static int bits_for(long long n) {
    int b = 1;
    while ((1ll << b) < n) ++b;
    return b;
}

// Validates (order, distribution, outputs) against a data set and fills the work description.
int make_work(fiu_ctx* ctx, const fiu_resident* res, unsigned order, const fiu_distribution* dist,
              unsigned outputs, ScanWork& w) {
    if (!res) return fail(ctx, FIU_ERR_INVALID, "null data set");
    if (order < 2 || order > FIU_MAX_ORDER)
        return fail(ctx, order < 2 ? FIU_ERR_INVALID : FIU_ERR_UNSUPPORTED, "order must be in [2, 8]");
    if (outputs > FIU_MAX_OUTPUTS) return fail(ctx, FIU_ERR_UNSUPPORTED, "outputs above FIU_MAX_OUTPUTS");
    fiu_distribution dd{res->d.snps, (int)order - 1, 1, 0};
    if (dist) dd = *dist;
    if (dd.k != (int)order - 1) return fail(ctx, FIU_ERR_INVALID, "distribution.k must be order - 1");
    if (dd.step < 1 || dd.offset < 0 || dd.n < 0 || dd.n > res->d.snps)
        return fail(ctx, FIU_ERR_INVALID, "distribution needs step >= 1, offset >= 0, 0 <= n <= snps");
    const int bits = bits_for(res->d.snps);
    if ((long long)bits * order > 64)
        return fail(ctx, FIU_ERR_UNSUPPORTED, "order x index bits exceeds 64 (too many SNPs for this order)");
    for (int j = 0; j <= dd.k; ++j)
        if (binom(dd.n, j) >= (1ull << 62)) return fail(ctx, FIU_ERR_UNSUPPORTED, "combination count overflow");
    const unsigned long long total = binom(dd.n, dd.k);
    w.d = res->d;
    w.order = (int)order;
    w.dist_n = dd.n;
    w.dist_step = dd.step;
    w.dist_offset = dd.offset;
    w.bits = bits;
    w.n_prefixes = (unsigned long long)dd.offset < total ? (long long)((total - 1 - dd.offset) / dd.step + 1) : 0;
    const long long N = (long long)res->d.n_cases + res->d.n_ctrls;
    auto T = [](long long c) -> long long {
        return c < 2 ? 0 : (long long)llround((double)c * std::log((double)c) * 4294967296.0);
    };
    w.base_key = T(N) - T(res->d.n_cases) - T(res->d.n_ctrls);
    return FIU_OK;
}

// Triple cores of the order-4 reduced-work kernel are kept up to this size
// (C(n,3) x 32 bytes: about 1 150 SNPs); larger data sets use the full kernel.
constexpr size_t kMaxTriplesBytes = 8ull << 30;

// Chooses the counting kernel of a request and makes sure its tables exist.
int choose_kernel(fiu_ctx* ctx, const fiu_resident* res_c, unsigned order, int requested, int& kernel) {
    fiu_resident* res = const_cast<fiu_resident*>(res_c);
    const bool classes_ok = res->one_hot && res->d.n_cases <= 65535 && res->d.n_ctrls <= 65535;
    const bool elided_ok =
        classes_ok && (((order == 2 || order == 3) && elided_smem(order, res->d.cw, res->d.tw) <= 160 * 1024) ||
                       (order == 4 && res->d.snps >= 4 && elided4_smem(res->d.cw, res->d.tw) <= 160 * 1024 &&
                        triples_bytes(res->d.snps) <= kMaxTriplesBytes));
    // measured: Harley-Seal counting wins at orders 2-3, plain POPC at order 4
    // (its 16 Harley-Seal counters do not fit two CTAs per SM)
    kernel = requested ? requested
                       : (elided_ok ? (order == 4 ? FIU_KERNEL_ELIDED_POPC : FIU_KERNEL_ELIDED_HS) : FIU_KERNEL_FULL);
    if (kernel < FIU_KERNEL_FULL || kernel > FIU_KERNEL_TENSOR) return fail(ctx, FIU_ERR_INVALID, "unknown kernel id");
    if (kernel == FIU_KERNEL_TENSOR && (order < 2 || order > 4))
        return fail(ctx, FIU_ERR_UNSUPPORTED, "the tensor-core kernels serve orders 2, 3 and 4");
    if (kernel == FIU_KERNEL_FULL) return FIU_OK;
    if (!elided_ok)
        return fail(ctx, FIU_ERR_UNSUPPORTED,
                    "elided kernels need one-hot data, order 2, 3 or 4 (at most 1 150 SNPs), classes <= 65535");
    const bool need_pairs = order >= 3 && !res->pairs, need_triples = order == 4 && !res->triples;
    if (!res->single || need_pairs || need_triples) {
        const long long np = (long long)res->d.snps * (res->d.snps - 1) / 2;
        cudaError_t e = cudaSuccess;
        if (!res->single) e = cudaMalloc((void**)&res->single, (size_t)res->d.snps * 4 * sizeof(uint32_t));
        if (e == cudaSuccess && need_pairs && np > 0) e = cudaMalloc((void**)&res->pairs, (size_t)np * sizeof(uint4));
        if (e == cudaSuccess) e = build_cores(res->d, res->single, need_pairs ? res->pairs : nullptr, ctx->sms, ctx->stream);
        if (e == cudaSuccess && need_triples) e = cudaMalloc((void**)&res->triples, triples_bytes(res->d.snps));
        if (e == cudaSuccess && need_triples) e = build_triples(res->d, res->triples, ctx->sms, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "core tables");
    }
    return FIU_OK;
}

cudaError_t launch_kernel(int kernel, int tp, const fiu_resident* res, const ScanWork& w, long long m0, long long m1,
                          const CandSink& sink, uint32_t* dump, cudaStream_t s, int sms) {
    if (kernel == FIU_KERNEL_FULL) return launch_count(tp, w, m0, m1, sink, dump, s, sms);
    if (w.order == 4)
        return launch_elided4(kernel == FIU_KERNEL_ELIDED_HS, tp, w, m0, m1, sink, dump, res->single, res->pairs,
                              res->triples, s, sms);
    return launch_elided(kernel == FIU_KERNEL_ELIDED_HS, tp, w, m0, m1, sink, dump, res->single, res->pairs, s, sms);
}

static size_t group_smem(int kernel, const ScanWork& w) {
    if (kernel == FIU_KERNEL_FULL) {
        int rows = 1;
        for (int t = 0; t < w.order - 1; ++t) rows *= 3;
        return (size_t)(rows < 9 ? rows : 9) * 64 * sizeof(uint64_t);
    }
    return w.order == 4 ? elided4_smem(w.d.cw, w.d.tw) : elided_smem(w.order, w.d.cw, w.d.tw);
}

static bool tile_ok(int kernel, int tp, const ScanWork& w) {
    if (kernel == FIU_KERNEL_FULL && w.order > 5 && tp != 256) return false;
    return (size_t)(256 / tp) * group_smem(kernel, w) <= kMaxGroupSmem;
}

// Heuristic tile: the smallest width that still covers a prefix's typical
// run of last SNPs, (n - k + 1) / k on average.
static int heuristic_tp(int kernel, const ScanWork& w) {
    const double L = (double)(w.d.snps - w.order + 1) / w.order;
    int tp = L >= 384 ? 256 : L >= 160 ? 128 : L >= 64 ? 64 : 32;
    while (tp < 256 && !tile_ok(kernel, tp, w)) tp *= 2;
    return tp;
}

static bool whole_data_set(const fiu_resident* res, const ScanWork& w) {
    return w.dist_step == 1 && w.dist_offset == 0 && w.dist_n == res->d.snps;
}

// A whole-data-set order-4 scan on the reduced-work POPC kernel runs pair-major
// (work items of (k, l) runs per pair (i, j), see elided4.cu).
bool e4_pair_major(int kernel, const fiu_resident* res, const ScanWork& w) {
    return kernel == FIU_KERNEL_ELIDED_POPC && w.order == 4 && whole_data_set(res, w);
}

// Work-item table of the pair-major order-4 schedule, built once per data set.
static int ensure_e4_items(fiu_ctx* ctx, const fiu_resident* res_c) {
    fiu_resident* res = const_cast<fiu_resident*>(res_c);
    if (res->e4_begin) return FIU_OK;
    const std::vector<long long> b = e4p_item_begin(res->d.snps);
    long long* d = nullptr;
    CK(cudaMalloc((void**)&d, b.size() * sizeof(long long)), "work-item table");
    cudaError_t e = cudaMemcpy(d, b.data(), b.size() * sizeof(long long), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(ctx, e, "work-item table");
    }
    res->e4_begin = d;
    res->e4_items = b.back();
    return FIU_OK;
}

static bool tensor_ok(const fiu_resident* res, const ScanWork& w) {
    const bool data_ok = res->one_hot && res->d.n_cases >= 1 && res->d.n_ctrls >= 1 && res->d.n_cases <= 65535 &&
                         res->d.n_ctrls <= 65535 && res->d.snps < (1 << 21);
    // a Distribution layer of the whole data set: order 2 (the owned SNPs of one residue), order 3 (the
    // owned j of each i: list mode), order 4 (the owned k of each pair)
    if (data_ok && !whole_data_set(res, w) && w.dist_n == res->d.snps &&
        (w.order == 2 || w.order == 3 ||
         (w.order == 4 && res->d.snps >= 4 && triples_bytes(res->d.snps) <= kMaxTriplesBytes)))
        return true;
    const bool base = data_ok && whole_data_set(res, w);
    if (w.order == 2 || w.order == 3) return base;
    // order 4: triple cores within their limit
    return base && w.order == 4 && res->d.snps >= 4 && triples_bytes(res->d.snps) <= kMaxTriplesBytes;
}

// Below this many samples an order-4 scan is faster on the CUDA-core
// pair-major kernel: the tensor kernel's per-combination epilogue then
// outweighs the counting it saves (measured at 150 SNPs, pair-major vs
// tensor: 1 060 samples 7.1 vs 6.2 ms, 1 800 samples 8.9 vs 6.3 ms, 4 000
// samples 14.8 vs 7.0 ms, 14 900 samples 44.8 vs 16.9 ms; the pair-major
// time falls with the samples, the tensor kernel's hardly below 6 ms).
// Forcing FIU_KERNEL_TENSOR still uses it.
constexpr int kT4MinSamples = 1024;

int choose_tile(fiu_ctx* ctx, const fiu_resident* res, const ScanWork& w, int requested_kernel, int& kernel, int& tp,
                bool allow_tensor) {
    const bool auto_tensor = allow_tensor && tensor_ok(res, w) &&
                             (w.order != 4 || res->d.n_cases + res->d.n_ctrls >= kT4MinSamples);
    if (requested_kernel == FIU_KERNEL_TENSOR || (requested_kernel == FIU_KERNEL_AUTO && auto_tensor)) {
        if (!allow_tensor || !tensor_ok(res, w))
            return fail(ctx, FIU_ERR_UNSUPPORTED,
                        "the tensor-core kernels need one-hot data, order 2, 3 or 4 and the whole data set on one "
                        "worker");
        int rc = choose_kernel(ctx, res, (unsigned)w.order, FIU_KERNEL_ELIDED_HS, kernel);  // builds the core tables
        if (rc) return rc;
        fiu_resident* r = const_cast<fiu_resident*>(res);
        if (!r->t3) {
            auto* plan = new (std::nothrow) T3Plan;
            if (!plan) return fail(ctx, FIU_ERR_NOMEM, "tensor plan");
            cudaError_t e = tensor3_prepare(r->d, *plan, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) {
                tensor3_release(*plan);
                delete plan;
                return cuda_fail(ctx, e, "tensor operand planes");
            }
            r->t3 = plan;
        }
        if (!whole_data_set(res, w)) {
            cudaError_t e = tensor3_layer(*r->t3, w, ctx->stream);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "tensor work items of a distribution layer");
        } else {
            cudaError_t e = tensor3_order_items(*r->t3, r->d, w.order);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "tensor work items");
        }
        kernel = FIU_KERNEL_TENSOR;
        // GEMM width N: order 3 uses 256 with one accumulator for both classes, 192 with one per class
        tp = (w.order != 3 || r->t3->pack) ? 256 : 192;
        return FIU_OK;
    }
    int rc = choose_kernel(ctx, res, (unsigned)w.order, requested_kernel, kernel);
    if (rc) return rc;
    if (e4_pair_major(kernel, res, w)) {  // one warp per work item: no l-tile to choose
        tp = 32;
        return ensure_e4_items(ctx, res);
    }
    tp = heuristic_tp(kernel, w);
    const double work = (double)binom(w.dist_n, w.order) / std::max(1, w.dist_step) * (w.d.n_cases + w.d.n_ctrls);
    if (!ctx->autotune || work < 2e11 || w.n_prefixes < 64) return FIU_OK;
    auto lg = [](double x) { int b = 0; while (x >= 2) { x /= 2; ++b; } return b; };
    const bool family_elided = kernel != FIU_KERNEL_FULL;
    const unsigned long long key = ((unsigned long long)w.order << 56) | ((unsigned long long)family_elided << 48) |
                                   ((unsigned long long)(requested_kernel & 0xff) << 40) |
                                   ((unsigned long long)lg(w.d.cw + w.d.tw) << 20) | (unsigned long long)lg(w.d.snps);
    auto it = ctx->tuned.find(key);
    if (it != ctx->tuned.end()) {
        kernel = it->second.first;
        tp = it->second.second;
        return FIU_OK;
    }
    // candidates: l-tile widths x (for one-hot data, unless a kernel was forced) both counting schemes
    std::vector<std::pair<int, int>> cand;
    std::vector<int> kernels{kernel};
    if (family_elided && requested_kernel == FIU_KERNEL_AUTO) kernels = {FIU_KERNEL_ELIDED_HS, FIU_KERNEL_ELIDED_POPC};
    for (int k : kernels)
        for (int t : {32, 64, 128, 256})
            if (tile_ok(k, t, w)) cand.push_back({k, t});
    // uniform sample of the prefixes: every stride-th owned prefix
    ScanWork sw = w;
    const long long want = (long long)ctx->sms * 16;
    const long long stride = std::max<long long>(1, w.n_prefixes / want);
    sw.dist_step = w.dist_step * (int)std::min<long long>(stride, 1 << 20);
    sw.n_prefixes = (w.n_prefixes - 1) / stride + 1;
    const CandSink none{ctx->cand, ctx->ctl + 8, ctx->ctl + 9, 0, (long long)0x7fffffffffffffffll, nullptr};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0), "tuning events");
    CK(cudaEventCreate(&e1), "tuning events");
    float best = 1e30f;
    for (auto& c : cand) {
        float ms = 0;
        cudaError_t e = launch_kernel(c.first, c.second, res, sw, 0, sw.n_prefixes, none, nullptr, ctx->stream, ctx->sms);
        if (e == cudaSuccess) e = cudaEventRecord(e0, ctx->stream);
        if (e == cudaSuccess)
            e = launch_kernel(c.first, c.second, res, sw, 0, sw.n_prefixes, none, nullptr, ctx->stream, ctx->sms);
        if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return cuda_fail(ctx, e, "autotuning");
        }
        if (ms < best) {
            best = ms;
            kernel = c.first;
            tp = c.second;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->tuned[key] = {kernel, tp};
    return FIU_OK;
}

// The search on a resident data set (ThreadedSearch::run semantics).
int search_impl(fiu_ctx* ctx, const fiu_resident* res, unsigned order, const fiu_distribution* dist,
                unsigned outputs, int32_t* out_comb, float* out_vals, double* out_vals64, unsigned* out_count,
                int kernel, unsigned shard, unsigned n_shards) {
    if (!ctx) return FIU_ERR_INVALID;
    Scope scope(ctx);
    if (!out_count || (outputs && (!out_comb || !out_vals)))
        return fail(ctx, FIU_ERR_INVALID, "null output pointer");
    if (n_shards == 0 || shard >= n_shards) return fail(ctx, FIU_ERR_INVALID, "shard out of range");
    *out_count = 0;
    ScanWork w;
    int rc = make_work(ctx, res, order, dist, outputs, w);
    if (rc) return rc;
    if (outputs == 0 || w.n_prefixes == 0) return FIU_OK;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    int tp = 256;
    if ((rc = choose_tile(ctx, res, w, kernel ? kernel : ctx->kernel, kernel, tp, true))) return rc;
    ctx->last_kernel = kernel;
    ctx->last_tp = tp;
    const bool tensor = kernel == FIU_KERNEL_TENSOR;
    const bool pair_major = e4_pair_major(kernel, res, w);
    const long long units = tensor ? tensor_units(*res->t3, w) : pair_major ? res->e4_items : w.n_prefixes;
    int* t_status = (int*)(ctx->ctl + 16);
    if (tensor) CK(cudaMemsetAsync(t_status, 0, sizeof(int), ctx->stream), "status reset");
    const unsigned keep = outputs + std::max(32u, outputs / 8);
    const size_t cap = std::max<size_t>({65536, (size_t)16 * keep, (size_t)res->d.snps + keep});
    if ((rc = grow(ctx, ctx->cand, ctx->cand_cap, cap)) ||
        (rc = grow(ctx, ctx->tmp, ctx->tmp_cap, cap + 8192)) ||
        (rc = grow(ctx, ctx->mi64, ctx->mi64_cap, (size_t)keep)))
        return rc;
    cudaStream_t s = ctx->stream;
    unsigned* count = ctx->ctl;
    unsigned* overflow = ctx->ctl + 1;
    unsigned* scratch = ctx->ctl + 4;
    long long thr = (long long)0x8000000000000000ull;
    unsigned have = 0;
    const double per_prefix = (double)binom(w.dist_n, order) / std::max<double>(1.0, (double)binom(w.dist_n, order - 1));
    const double per_unit = tensor       ? tensor_item_combos(*res->t3, w)
                            : pair_major ? (double)binom(w.dist_n, 4) / std::max(1ll, res->e4_items)
                                         : per_prefix;
    // Chunk schedule.  While fewer than `keep` candidates are held every
    // combination is one; afterwards the threshold is the keep-th best key of
    // the `seen` combinations so far, and about keep / seen of the next
    // chunk's combinations pass it.  Chunks are sized for a quarter of the
    // candidate buffer under that estimate (a chunk that overflows all the
    // same is re-run in smaller pieces), so a scan takes a few launches and
    // the same launches on every run.  On a context whose searches can be
    // cancelled a chunk also stays under about a quarter second (measured per
    // unit on the previous chunk), so that a cancellation takes effect soon.
    long long chunk = std::max<long long>(1, (long long)(keep / std::max(1.0, per_unit)));
    double seen = 0, sec_per_unit = 0;
    long long m = units / n_shards * shard + std::min<long long>(shard, units % n_shards);
    const long long m_end = m + units / n_shards + (shard < units % n_shards ? 1 : 0);
    while (m < m_end) {
        if (ctx->cancel.load(std::memory_order_relaxed)) return fail(ctx, FIU_ERR_CANCELLED, "search cancelled");
        const long long m1 = std::min(m_end, m + chunk);
        const auto t_chunk = std::chrono::steady_clock::now();
        ctx->pinned[0] = have;
        ctx->pinned[1] = 0;
        CK(cudaMemcpyAsync(count, ctx->pinned, 2 * sizeof(unsigned), cudaMemcpyHostToDevice, s), "reset counters");
        CandSink sink{ctx->cand, count, overflow, (unsigned)cap, thr, ctx->timing ? ctx->evaluated : nullptr};
        if (ctx->timing) CK(cudaEventRecord(ctx->ev0, s), "event");
        if (tensor)
            CK(launch_tensor3(w, *res->t3, m, m1, sink, nullptr, res->single, res->pairs, res->triples, t_status, s,
                              ctx->sms),
               "tensor kernel launch");
        else if (pair_major)
            CK(launch_elided4p(w, res->e4_begin, m, m1, sink, nullptr, res->single, res->pairs, res->triples, s,
                               ctx->sms),
               "count kernel launch");
        else
            CK(launch_kernel(kernel, tp, res, w, m, m1, sink, nullptr, s, ctx->sms), "count kernel launch");
        if (ctx->timing) CK(cudaEventRecord(ctx->ev1, s), "event");
        CK(cudaMemcpyAsync(ctx->pinned, count, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read counters");
        CK(cudaStreamSynchronize(s), "count kernel");
        sec_per_unit = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_chunk).count() /
                       (double)(m1 - m);
        if (ctx->timing) {
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "event time");
            ctx->count_ms += ms;
            ctx->count_launches += 1;
        }
        const unsigned M = std::min<unsigned>(ctx->pinned[0], (unsigned)cap);
        if (ctx->pinned[1]) {  // overflow: drop this chunk's candidates and retry smaller
            if (m1 - m == 1) return fail(ctx, FIU_ERR_UNSUPPORTED, "candidate buffer overflow on one prefix");
            chunk = std::max<long long>(1, (m1 - m) / 4);
            continue;
        }
        seen += (double)(m1 - m) * per_unit;
        if (M > keep) {
            CK(select_top(ctx->cand, M, keep, ctx->tmp, scratch, s), "top-N selection");
            Cand last;
            CK(cudaMemcpyAsync(&last, ctx->cand + keep - 1, sizeof(Cand), cudaMemcpyDeviceToHost, s), "threshold");
            CK(cudaStreamSynchronize(s), "top-N selection");
            thr = last.key;
            have = keep;
        } else {
            have = M;
        }
        m = m1;
        const double next = have < keep ? (double)(cap - have) / (4.0 * std::max(1.0, per_unit))
                                        : (double)cap / 4.0 * seen / ((double)keep * std::max(1.0, per_unit));
        const double time_cap = ctx->cancellable ? 0.25 / std::max(sec_per_unit, 1e-12) : 4.0e18;
        chunk = (long long)std::max(1.0, std::min({next, time_cap, 4.0e18}));
    }
    if (tensor) {
        int st = 0;
        CK(cudaMemcpyAsync(&st, t_status, sizeof(int), cudaMemcpyDeviceToHost, s), "status");
        CK(cudaStreamSynchronize(s), "status");
        if (st) return fail(ctx, FIU_ERR_TIMEOUT, "tensor kernel: a tensor-memory wait ran past its limit");
    }
    // Final order of the kept set, then FP64 re-score of every kept candidate.
    CK(select_top(ctx->cand, have, keep, ctx->tmp, scratch, s), "top-N selection");
    const unsigned n = std::min(have, keep);
    CK(rescore_sort(w.d, (int)order, w.bits, ctx->cand, n, ctx->mi64, s), "FP64 rescore");
    const unsigned nout = std::min(n, outputs);
    std::vector<Cand> hc(nout);
    std::vector<double> hv(nout);
    CK(cudaMemcpyAsync(hc.data(), ctx->cand, nout * sizeof(Cand), cudaMemcpyDeviceToHost, s), "results");
    CK(cudaMemcpyAsync(hv.data(), ctx->mi64, nout * sizeof(double), cudaMemcpyDeviceToHost, s), "results");
    CK(cudaStreamSynchronize(s), "results");
    for (unsigned i = 0; i < nout; ++i) {
        int c[kMaxOrder];
        unpack_code(hc[i].code, (int)order, w.bits, c);
        for (unsigned t = 0; t < order; ++t) out_comb[(size_t)i * order + t] = c[t];
        out_vals[i] = (float)hv[i];
        if (out_vals64) out_vals64[i] = hv[i];
    }
    *out_count = nout;
    return FIU_OK;
}

int check_sizes(fiu_ctx* ctx, uint64_t snps, uint64_t cases, uint64_t ctrls, uint64_t cw, uint64_t tw) {
    if (snps < 1 || snps > 0x7fffffffull || cw > 0x7fffffffull / 8 || tw > 0x7fffffffull / 8)
        return fail(ctx, FIU_ERR_INVALID, "data set sizes out of range");
    if (cases > 64 * cw || ctrls > 64 * tw) return fail(ctx, FIU_ERR_INVALID, "more samples than the row words hold");
    if (cases + ctrls == 0) return fail(ctx, FIU_ERR_INVALID, "empty data set");
    if (cw + tw == 0) return fail(ctx, FIU_ERR_INVALID, "rows without words");
    return FIU_OK;
}

// A resident data set with its reference-layout buffer allocated (not filled).
int new_resident(fiu_ctx* ctx, uint64_t snps, uint64_t cases, uint64_t ctrls, uint64_t cw, uint64_t tw,
                 fiu_resident** out) {
    auto* r = new (std::nothrow) fiu_resident;
    if (!r) return fail(ctx, FIU_ERR_NOMEM, "host allocation");
    r->device = ctx->device;
    r->d = DevData{nullptr, nullptr, nullptr, (int)snps, (int)cw, (int)tw, (int)cases, (int)ctrls};
    const size_t words = (size_t)snps * 3 * (size_t)(cw + tw);
    cudaError_t e = cudaMalloc((void**)&r->ref, words * 8);
    if (e != cudaSuccess) {
        delete r;
        return cuda_fail(ctx, e, "data set upload");
    }
    *out = r;
    return FIU_OK;
}

// Once r->ref holds the reference layout on the device (queued on the
// context's stream): the transposed copy, the c ln c table and the one-hot
// check.  Frees r on failure.
int finish_resident(fiu_ctx* ctx, fiu_resident* r) {
    const int snps = r->d.snps, cw = r->d.cw, tw = r->d.tw;
    const size_t rows = 3 * (size_t)(cw + tw);
    const size_t words = (size_t)snps * rows;
    const long long tmax = 64ll * (cw + tw);
    std::vector<long long> ftab;
    try {
        ftab.resize(tmax + 1);
    } catch (const std::exception&) {
        fiu_dataset_free(ctx, r);
        return fail(ctx, FIU_ERR_NOMEM, "host c ln c table");
    }
    for (long long c = 0; c <= tmax; ++c)
        ftab[c] = c < 2 ? 0 : (long long)llround((double)c * std::log((double)c) * 4294967296.0);
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaMalloc((void**)&r->tr, words * 8);
    if (e == cudaSuccess) e = cudaMalloc((void**)&r->ftab, ftab.size() * 8);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r->ftab, ftab.data(), ftab.size() * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_transpose(r->ref, r->tr, snps, (int)rows, s);
    int* bad = (int*)(ctx->ctl + 300);
    if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), s);
    if (e == cudaSuccess) e = launch_onehot_check(r->ref, snps, cw, tw, r->d.n_cases, r->d.n_ctrls, bad, s);
    int hb = 1;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        fiu_dataset_free(ctx, r);
        return cuda_fail(ctx, e, "data set upload");
    }
    r->one_hot = hb == 0;
    r->ftab_max = tmax;
    r->d = DevData{r->ref, r->tr, r->ftab, snps, cw, tw, r->d.n_cases, r->d.n_ctrls};
    return FIU_OK;
}

}  // namespace fiu

extern "C" {

int fiu_create(int device, fiu_ctx** out) {
    if (!out) return FIU_ERR_INVALID;
    *out = nullptr;
    auto* ctx = new (std::nothrow) fiu_ctx;
    if (!ctx) return FIU_ERR_NOMEM;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n) {
        delete ctx;
        return e != cudaSuccess ? FIU_ERR_CUDA : FIU_ERR_INVALID;
    }
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc((void**)&ctx->ctl, 512 * sizeof(unsigned)) != cudaSuccess ||
        cudaMallocHost((void**)&ctx->pinned, 16 * sizeof(unsigned)) != cudaSuccess) {
        fiu_destroy(ctx);
        return FIU_ERR_CUDA;
    }
    *out = ctx;
    return FIU_OK;
}

void fiu_destroy(fiu_ctx* ctx) {
    if (!ctx) return;
    for (fiu_ctx*& l : ctx->lanes) {
        fiu_destroy(l);
        l = nullptr;
    }
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->cand);
    cudaFree(ctx->tmp);
    cudaFree(ctx->ctl);
    cudaFree(ctx->mi64);
    cudaFree(ctx->evaluated);
    cudaFree(ctx->arena);
    if (ctx->host_arena) cudaFreeHost(ctx->host_arena);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* fiu_last_error(const fiu_ctx* ctx) {
    if (ctx) return ctx->err.c_str();
    return g_free_err.empty() ? "null context" : g_free_err.c_str();
}

uint64_t fiu_launch_count(const fiu_ctx* ctx) { return ctx ? ctx->launches : 0; }

int fiu_set_autotune(fiu_ctx* ctx, int enable) {
    if (!ctx) return FIU_ERR_INVALID;
    ctx->autotune = enable != 0;
    return FIU_OK;
}

int fiu_last_tile(const fiu_ctx* ctx, int* kernel, int* tp) {
    if (!ctx) return FIU_ERR_INVALID;
    if (kernel) *kernel = ctx->last_kernel;
    if (tp) *tp = ctx->last_tp;
    return FIU_OK;
}

int fiu_set_kernel(fiu_ctx* ctx, int kernel) {
    if (!ctx) return FIU_ERR_INVALID;
    if (kernel < FIU_KERNEL_AUTO || kernel > FIU_KERNEL_TENSOR) return fail(ctx, FIU_ERR_INVALID, "unknown kernel id");
    ctx->kernel = kernel;
    return FIU_OK;
}

void* fiu_stream(const fiu_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int fiu_set_kernel_timing(fiu_ctx* ctx, int enable) {
    if (!ctx) return FIU_ERR_INVALID;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (enable && !ctx->ev0) {
        CK(cudaEventCreate(&ctx->ev0), "event");
        CK(cudaEventCreate(&ctx->ev1), "event");
        CK(cudaMalloc((void**)&ctx->evaluated, sizeof(unsigned long long)), "counter");
    }
    if (enable) CK(cudaMemsetAsync(ctx->evaluated, 0, sizeof(unsigned long long), ctx->stream), "counter");
    CK(cudaStreamSynchronize(ctx->stream), "counter");
    ctx->timing = enable != 0;
    ctx->count_ms = 0;
    ctx->count_launches = 0;
    return FIU_OK;
}

int fiu_kernel_timing(const fiu_ctx* ctx_c, double* count_ms, uint64_t* count_launches, uint64_t* combinations) {
    fiu_ctx* ctx = const_cast<fiu_ctx*>(ctx_c);
    if (!ctx) return FIU_ERR_INVALID;
    if (count_ms) *count_ms = ctx->count_ms;
    if (count_launches) *count_launches = ctx->count_launches;
    if (combinations) {
        unsigned long long v = 0;
        if (ctx->evaluated) {
            CK(cudaSetDevice(ctx->device), "cudaSetDevice");
            CK(cudaMemcpyAsync(&v, ctx->evaluated, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream), "counter");
            CK(cudaStreamSynchronize(ctx->stream), "counter");
        }
        *combinations = v;
    }
    return FIU_OK;
}

int fiu_probe_popc_rate(fiu_ctx* ctx, double* rate) {
    if (!ctx || !rate) return FIU_ERR_INVALID;
    Scope scope(ctx);
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(probe_popc_rate(ctx->sms, ctx->stream, rate), "popc probe");
    return FIU_OK;
}

int fiu_probe_lg2_error(fiu_ctx* ctx, unsigned max_c, double* max_abs_err) {
    if (!ctx || !max_abs_err) return FIU_ERR_INVALID;
    Scope scope(ctx);
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(probe_lg2_error(max_c, max_abs_err, ctx->stream), "lg2 probe");
    return FIU_OK;
}

int fiu_probe_wait_limit(fiu_ctx* ctx, unsigned limit_us, int arrive, int* completed, double* elapsed_ms) {
    if (!ctx || !completed || !elapsed_ms || limit_us > 1000000) return FIU_ERR_INVALID;
    Scope scope(ctx);
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(probe_wait_limit(limit_us, arrive, completed, elapsed_ms, ctx->stream), "wait probe");
    return FIU_OK;
}

int fiu_dataset_upload(fiu_ctx* ctx, const fiu_dataset* h, fiu_resident** out) {
    if (!ctx || !out) return FIU_ERR_INVALID;
    Scope scope(ctx);
    *out = nullptr;
    if (!h || !h->data) return fail(ctx, FIU_ERR_INVALID, "null data set");
    int rc = check_sizes(ctx, h->snps, h->cases, h->ctrls, h->cases_words, h->ctrls_words);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t words = (size_t)h->snps * 3 * (size_t)(h->cases_words + h->ctrls_words);
    fiu_resident* r = nullptr;
    if ((rc = new_resident(ctx, h->snps, h->cases, h->ctrls, h->cases_words, h->ctrls_words, &r))) return rc;
    cudaError_t e = cudaMemcpyAsync(r->ref, h->data, words * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        fiu_dataset_free(ctx, r);
        return cuda_fail(ctx, e, "data set upload");
    }
    if ((rc = finish_resident(ctx, r))) return rc;
    *out = r;
    return FIU_OK;
}

void fiu_dataset_free(fiu_ctx* ctx, fiu_resident* r) {
    if (!r) return;
    if (ctx) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    cudaFree(r->ref);
    cudaFree(r->tr);
    cudaFree(r->ftab);
    cudaFree(r->single);
    cudaFree(r->pairs);
    cudaFree(r->triples);
    cudaFree(r->e4_begin);
    if (r->t3) {
        tensor3_release(*r->t3);
        delete r->t3;
    }
    delete r;
}

int fiu_dataset_is_one_hot(const fiu_resident* r) { return r ? r->one_hot : 0; }

int fiu_search(fiu_ctx* ctx, const fiu_dataset* dataset, unsigned order, const fiu_distribution* distribution,
               unsigned outputs, int32_t* out_combinations, float* out_vals, unsigned* out_count) {
    fiu_resident* r = nullptr;
    int rc = fiu_dataset_upload(ctx, dataset, &r);
    if (rc) return rc;
    rc = search_impl(ctx, r, order, distribution, outputs, out_combinations, out_vals, nullptr, out_count, 0);
    fiu_dataset_free(ctx, r);
    return rc;
}

int fiu_search_resident(fiu_ctx* ctx, const fiu_resident* res, unsigned order, const fiu_distribution* distribution,
                        unsigned outputs, int32_t* out_combinations, float* out_vals, unsigned* out_count) {
    return search_impl(ctx, res, order, distribution, outputs, out_combinations, out_vals, nullptr, out_count, 0);
}

int fiu_search_resident64(fiu_ctx* ctx, const fiu_resident* res, unsigned order,
                          const fiu_distribution* distribution, unsigned outputs, int32_t* out_combinations,
                          float* out_vals, double* out_vals64, unsigned* out_count) {
    return search_impl(ctx, res, order, distribution, outputs, out_combinations, out_vals, out_vals64, out_count, 0);
}

int fiu_search_shard(fiu_ctx* ctx, const fiu_dataset* dataset, unsigned order, unsigned shard, unsigned n_shards,
                     unsigned outputs, int32_t* out_combinations, float* out_vals, unsigned* out_count) {
    if (!ctx || !dataset) return FIU_ERR_INVALID;
    fiu_resident* r = nullptr;
    int rc = fiu_dataset_upload(ctx, dataset, &r);
    if (rc) return rc;
    const fiu_distribution whole{(int)dataset->snps, (int)order - 1, 1, 0};
    rc = search_impl(ctx, r, order, &whole, outputs, out_combinations, out_vals, nullptr, out_count, 0, shard,
                     n_shards);
    fiu_dataset_free(ctx, r);
    return rc;
}

int fiu_search_shard_resident64(fiu_ctx* ctx, const fiu_resident* res, unsigned order, unsigned shard,
                                unsigned n_shards, unsigned outputs, int32_t* out_combinations, float* out_vals,
                                double* out_vals64, unsigned* out_count) {
    if (!ctx || !res) return FIU_ERR_INVALID;
    const fiu_distribution whole{(int)res->d.snps, (int)order - 1, 1, 0};
    return search_impl(ctx, res, order, &whole, outputs, out_combinations, out_vals, out_vals64, out_count, 0, shard,
                       n_shards);
}

int fiu_combine(fiu_ctx* ctx, const uint64_t* t1, unsigned size1, const uint64_t* t2, uint64_t cases_words,
                uint64_t ctrls_words, uint64_t* out) {
    if (!ctx) return FIU_ERR_INVALID;
    Scope scope(ctx);
    if (!t1 || !t2 || !out || size1 == 0 || cases_words + ctrls_words == 0 || cases_words > (1u << 28) ||
        ctrls_words > (1u << 28) || size1 > (1u << 20))
        return fail(ctx, FIU_ERR_INVALID, "invalid combine arguments");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t n1 = (size_t)size1 * (cases_words + ctrls_words), n2 = 3 * (cases_words + ctrls_words),
                 no = 3 * n1;
    uint64_t *d1 = nullptr, *d2 = nullptr, *dout = nullptr;
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaMallocAsync((void**)&d1, n1 * 8, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&d2, n2 * 8, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dout, no * 8, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d1, t1, n1 * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d2, t2, n2 * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_combine(d1, (int)size1, d2, (int)cases_words, (int)ctrls_words, dout, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, no * 8, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d1, s);
    cudaFreeAsync(d2, s);
    cudaFreeAsync(dout, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "combine");
    return FIU_OK;
}

int fiu_combine_and_popcnt(fiu_ctx* ctx, const uint64_t* t1, unsigned size1, const uint64_t* t2,
                           uint64_t cases_words, uint64_t ctrls_words, uint32_t* cases_out, uint32_t* ctrls_out,
                           unsigned ct_size) {
    if (!ctx) return FIU_ERR_INVALID;
    Scope scope(ctx);
    if (!t1 || !t2 || !cases_out || !ctrls_out || size1 == 0 || ct_size < 3 * size1 ||
        cases_words + ctrls_words == 0 || cases_words > (1u << 28) || ctrls_words > (1u << 28) || size1 > (1u << 20))
        return fail(ctx, FIU_ERR_INVALID, "invalid combine_and_popcnt arguments");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t n1 = (size_t)size1 * (cases_words + ctrls_words), n2 = 3 * (cases_words + ctrls_words);
    uint64_t *d1 = nullptr, *d2 = nullptr;
    uint32_t* dout = nullptr;
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaMallocAsync((void**)&d1, n1 * 8, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&d2, n2 * 8, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dout, 2 * (size_t)ct_size * 4, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d1, t1, n1 * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d2, t2, n2 * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = launch_combine_popcnt(d1, (int)size1, d2, (int)cases_words, (int)ctrls_words, dout, dout + ct_size,
                                  (int)ct_size, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cases_out, dout, (size_t)ct_size * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctrls_out, dout + ct_size, (size_t)ct_size * 4, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d1, s);
    cudaFreeAsync(d2, s);
    cudaFreeAsync(dout, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "combine_and_popcnt");
    return FIU_OK;
}

int fiu_mi_compute(fiu_ctx* ctx, const uint32_t* cases, const uint32_t* ctrls, size_t cells, size_t count,
                   unsigned n_cases, unsigned n_ctrls, int mode, float* out, double* out64) {
    if (!ctx) return FIU_ERR_INVALID;
    Scope scope(ctx);
    const long long tmax = (long long)n_cases + n_ctrls;  // no unsigned wrap
    if (!cases || !ctrls || !out || cells == 0 || (mode != 0 && mode != 1) || tmax == 0)
        return fail(ctx, FIU_ERR_INVALID, "invalid mi_compute arguments");
    if (tmax > 0x7fffffffll) return fail(ctx, FIU_ERR_UNSUPPORTED, "n_cases + n_ctrls above 2^31 - 1");
    if (count == 0) return FIU_OK;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    std::vector<long long> ftab;
    try {
        ftab.resize((size_t)tmax + 1);
    } catch (const std::exception&) {
        return fail(ctx, FIU_ERR_NOMEM, "host c ln c table");
    }
    for (long long c = 0; c <= tmax; ++c)
        ftab[c] = c < 2 ? 0 : (long long)llround((double)c * std::log((double)c) * 4294967296.0);
    uint32_t *da = nullptr, *db = nullptr;
    long long* dt = nullptr;
    float* dout = nullptr;
    double* d64 = nullptr;
    cudaStream_t s = ctx->stream;
    const size_t n = cells * count;
    cudaError_t e = cudaMallocAsync((void**)&da, n * 4, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&db, n * 4, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dt, ftab.size() * 8, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dout, count * 4, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&d64, count * 8, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(da, cases, n * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(db, ctrls, n * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, ftab.data(), ftab.size() * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = launch_mi(da, db, cells, count, (int)n_cases, (int)n_ctrls, dt, tmax, mode, dout, d64, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, count * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && out64) e = cudaMemcpyAsync(out64, d64, count * 8, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(da, s);
    cudaFreeAsync(db, s);
    cudaFreeAsync(dt, s);
    cudaFreeAsync(dout, s);
    cudaFreeAsync(d64, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mi_compute");
    return FIU_OK;
}

int fiu_tables(fiu_ctx* ctx, const fiu_resident* res, unsigned order, const int32_t* combos, size_t count,
               uint32_t* cases_out, uint32_t* ctrls_out) {
    if (!ctx) return FIU_ERR_INVALID;
    Scope scope(ctx);
    if (!res || !combos || !cases_out || !ctrls_out || order < 1 || order > FIU_MAX_ORDER)
        return fail(ctx, FIU_ERR_INVALID, "invalid tables arguments");
    for (size_t q = 0; q < count * order; ++q)
        if (combos[q] < 0 || combos[q] >= res->d.snps) return fail(ctx, FIU_ERR_INVALID, "SNP index out of range");
    if (count == 0) return FIU_OK;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    size_t cells = 1;
    for (unsigned t = 0; t < order; ++t) cells *= 3;
    int* dc = nullptr;
    uint32_t* dout = nullptr;
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaMallocAsync((void**)&dc, count * order * 4, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dout, 2 * count * cells * 4, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dc, combos, count * order * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_tables(res->d, (int)order, dc, count, dout, dout + count * cells, nullptr, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cases_out, dout, count * cells * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctrls_out, dout + count * cells, count * cells * 4, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(dc, s);
    cudaFreeAsync(dout, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "tables");
    return FIU_OK;
}

int fiu_scan_tables(fiu_ctx* ctx, const fiu_resident* res, unsigned order, const fiu_distribution* distribution,
                    int kernel, uint32_t* out, size_t out_words) {
    if (!ctx) return FIU_ERR_INVALID;
    Scope scope(ctx);
    ScanWork w;
    int rc = make_work(ctx, res, order, distribution, 1, w);
    if (rc) return rc;
    size_t cells = 1;
    for (unsigned t = 0; t < order; ++t) cells *= 3;
    const size_t need = (size_t)w.n_prefixes * res->d.snps * 2 * cells;
    if (!out || out_words < need) return fail(ctx, FIU_ERR_INVALID, "output buffer too small");
    if (need == 0) return FIU_OK;
    if (need > ((size_t)1 << 31)) return fail(ctx, FIU_ERR_UNSUPPORTED, "scan too large to dump");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    int tp = (kernel >> 8) & 0x1ff;
    kernel &= 0xff;
    if (kernel == FIU_KERNEL_TENSOR) {
        if ((rc = choose_tile(ctx, res, w, kernel, kernel, tp, true))) return rc;
    } else {
        if ((rc = choose_kernel(ctx, res, order, kernel, kernel))) return rc;
        if (tp != 32 && tp != 64 && tp != 128 && tp != 256) tp = heuristic_tp(kernel, w);
        if (!tile_ok(kernel, tp, w)) return fail(ctx, FIU_ERR_UNSUPPORTED, "l-tile width not available for this request");
    }
    cudaStream_t s = ctx->stream;
    uint32_t* d = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&d, need * 4, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, out, need * 4, cudaMemcpyHostToDevice, s);
    CandSink sink{ctx->cand, ctx->ctl, ctx->ctl + 1, 0, (long long)0x7fffffffffffffffll, nullptr};
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->ctl, 0, 2 * sizeof(unsigned), s);
    if (e == cudaSuccess && kernel == FIU_KERNEL_TENSOR) {
        e = cudaMemsetAsync(ctx->ctl + 16, 0, sizeof(int), s);
        if (e == cudaSuccess)
            e = launch_tensor3(w, *res->t3, 0, tensor_units(*res->t3, w), sink, d, res->single, res->pairs,
                               res->triples, (int*)(ctx->ctl + 16), s, ctx->sms);
    } else if (e == cudaSuccess && e4_pair_major(kernel, res, w)) {
        if ((rc = ensure_e4_items(ctx, res))) {
            cudaFreeAsync(d, s);
            return rc;
        }
        e = launch_elided4p(w, res->e4_begin, 0, res->e4_items, sink, d, res->single, res->pairs, res->triples, s,
                            ctx->sms);
    } else if (e == cudaSuccess) {
        e = launch_kernel(kernel, tp, res, w, 0, w.n_prefixes, sink, d, s, ctx->sms);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, need * 4, cudaMemcpyDeviceToHost, s);
    int t_status = 0;  // a tensor kernel that gave up on a wait leaves incomplete tables: report it
    if (e == cudaSuccess && kernel == FIU_KERNEL_TENSOR)
        e = cudaMemcpyAsync(&t_status, ctx->ctl + 16, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scan tables");
    if (t_status) return fail(ctx, FIU_ERR_TIMEOUT, "tensor kernel: a tensor-memory wait ran past its limit");
    return FIU_OK;
}

int fiu_scan_digest(fiu_ctx* ctx, const fiu_resident* res, unsigned order, const fiu_distribution* distribution,
                    int kernel, uint64_t* digest, uint64_t* combinations) {
    if (!ctx) return FIU_ERR_INVALID;
    Scope scope(ctx);
    if (!digest || !combinations) return fail(ctx, FIU_ERR_INVALID, "null output pointer");
    *digest = 0;
    *combinations = 0;
    ScanWork w;
    int rc = make_work(ctx, res, order, distribution, 1, w);
    if (rc) return rc;
    if (w.n_prefixes == 0) return FIU_OK;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    int tp = 256;
    if ((rc = choose_tile(ctx, res, w, kernel ? kernel : ctx->kernel, kernel, tp, true))) return rc;
    if (kernel == FIU_KERNEL_FULL && order > 4)
        return fail(ctx, FIU_ERR_UNSUPPORTED, "the full-table kernel's digest covers orders 2-4");
    const bool tensor = kernel == FIU_KERNEL_TENSOR;
    const bool pair_major = e4_pair_major(kernel, res, w);
    const long long units = tensor ? tensor_units(*res->t3, w) : pair_major ? res->e4_items : w.n_prefixes;
    // order-4 and full-table kernels assemble each table in a per-thread row
    // (2 x 81 words) of scratch: room for every thread the launch can hold
    const bool scratch = order == 4 || kernel == FIU_KERNEL_FULL;
    const unsigned threads = scratch ? (unsigned)ctx->sms * 2048u : 0u;
    cudaStream_t s = ctx->stream;
    unsigned long long* d = nullptr;  // kDigestSlots sums, then the combination counter
    uint32_t* sc = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&d, (kDigestSlots + 1) * sizeof(unsigned long long), s);
    if (e == cudaSuccess && scratch) e = cudaMallocAsync((void**)&sc, (size_t)threads * 2 * 81 * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, (kDigestSlots + 1) * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->ctl, 0, 2 * sizeof(unsigned), s);
    int* t_status = (int*)(ctx->ctl + 16);
    if (e == cudaSuccess && tensor) e = cudaMemsetAsync(t_status, 0, sizeof(int), s);
    CandSink sink{ctx->cand, ctx->ctl, ctx->ctl + 1, 0, (long long)0x7fffffffffffffffll, d + kDigestSlots,
                  d, sc, threads};
    if (e == cudaSuccess) {
        if (tensor)
            e = launch_tensor3(w, *res->t3, 0, units, sink, nullptr, res->single, res->pairs, res->triples, t_status, s,
                               ctx->sms);
        else if (pair_major)
            e = launch_elided4p(w, res->e4_begin, 0, units, sink, nullptr, res->single, res->pairs, res->triples, s,
                                ctx->sms);
        else
            e = launch_kernel(kernel, tp, res, w, 0, units, sink, nullptr, s, ctx->sms);
    }
    std::vector<unsigned long long> h(kDigestSlots + 1, 0);
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && tensor) e = cudaMemcpyAsync(&st, t_status, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (sc) cudaFreeAsync(sc, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scan digest");
    if (st) return fail(ctx, FIU_ERR_TIMEOUT, "tensor kernel: a tensor-memory wait ran past its limit");
    unsigned long long sum = 0;
    for (int i = 0; i < kDigestSlots; ++i) sum += h[i];
    *digest = sum;
    *combinations = h[kDigestSlots];
    return FIU_OK;
}

}  // extern "C"
