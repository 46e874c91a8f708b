// Host-side internals shared by the C ABI translation units: the context and
// resident data set objects, error helpers and the single-scan driver.
#pragma once

#include <atomic>
#include <map>
#include <string>
#include <utility>

#include "../../include/fiuncho_gpu.h"
#include "internal.h"

struct fiu_ctx {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    unsigned long long launches = 0;
    // growable scratch of the search driver
    fiu::Cand* cand = nullptr;  // candidate buffer
    size_t cand_cap = 0;
    fiu::Cand* tmp = nullptr;   // select_top working space
    size_t tmp_cap = 0;
    unsigned* ctl = nullptr;  // [0] count, [1] overflow, [2..] select scratch (262)
    double* mi64 = nullptr;
    size_t mi64_cap = 0;
    unsigned* pinned = nullptr;  // host mirror of ctl[0..1]
    // optional timing of the counting kernels (CUDA events on `stream`)
    bool timing = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double count_ms = 0;
    unsigned long long count_launches = 0;
    unsigned long long* evaluated = nullptr;  // device counter of combinations evaluated
    int kernel = FIU_KERNEL_AUTO;
    // autotuner: (order, family, words bucket, snps bucket) -> (kernel, tp)
    bool autotune = true;
    int last_kernel = 0, last_tp = 0;  // tile of the last single-scan search
    std::map<unsigned long long, std::pair<int, int>> tuned;
    // batched-search arena (device) and its pinned host mirror
    char* arena = nullptr;
    size_t arena_cap = 0;
    char* host_arena = nullptr;
    size_t host_arena_cap = 0;
    // helper lanes of the batched search (own stream and scratch each), made on first use
    fiu_ctx* lanes[2] = {nullptr, nullptr};
    // set by another thread to stop the search running on this context after
    // its current chunk (FIU_ERR_CANCELLED)
    std::atomic<int> cancel{0};
    // searches on this context may be cancelled (the server's solo lanes):
    // their chunks are also kept under about a quarter second, so a cancel
    // takes effect soon.  Elsewhere the chunk schedule depends on the data only.
    bool cancellable = false;
};

struct fiu_resident {
    fiu::DevData d{};
    uint64_t* ref = nullptr;
    uint64_t* tr = nullptr;
    long long* ftab = nullptr;
    long long ftab_max = 0;
    int one_hot = 0;
    int device = 0;
    uint32_t* single = nullptr;  // single-SNP cores (elided kernels)
    uint4* pairs = nullptr;      // pair cores (elided order-3 and order-4 kernels)
    uint4* triples = nullptr;    // triple cores (elided order-4 kernel)
    long long* e4_begin = nullptr;  // pair-major order-4 work items: first item per second SNP j
    long long e4_items = 0;
    fiu::T3Plan* t3 = nullptr;  // operand planes and work items of the tensor order-3 kernel
};

namespace fiu {

struct Scope {  // routes launch counting of this thread to the context
    explicit Scope(fiu_ctx* c) { g_launch_counter = &c->launches; }
    ~Scope() { g_launch_counter = nullptr; }
};

#define CK(expr, what)                                          \
    do {                                                        \
        cudaError_t e_ = (expr);                                \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

int fail(fiu_ctx* ctx, int code, const std::string& msg);
int cuda_fail(fiu_ctx* ctx, cudaError_t e, const char* what);
int grow_bytes(fiu_ctx* ctx, char*& p, size_t& cap, size_t need);
int grow_host(fiu_ctx* ctx, size_t need);
int make_work(fiu_ctx* ctx, const fiu_resident* res, unsigned order, const fiu_distribution* dist,
              unsigned outputs, ScanWork& w);
int choose_kernel(fiu_ctx* ctx, const fiu_resident* res, unsigned order, int requested, int& kernel);
// Picks the counting kernel variant and l-tile width (threads per prefix) of a
// request: measured on a strided sample of its prefixes (cached per shape
// bucket) when autotuning is on and the request is large, else a heuristic.
int choose_tile(fiu_ctx* ctx, const fiu_resident* res, const ScanWork& w, int requested_kernel, int& kernel, int& tp,
                bool allow_tensor = false);
bool e4_pair_major(int kernel, const fiu_resident* res, const ScanWork& w);
cudaError_t launch_kernel(int kernel, int tp, const fiu_resident* res, const ScanWork& w, long long m0, long long m1,
                          const CandSink& sink, uint32_t* dump, cudaStream_t s, int sms);
// Data set upload in steps (api.cu): sizes check, allocation of the reference
// layout, then the derived device layouts once the layout is filled.
int check_sizes(fiu_ctx* ctx, uint64_t snps, uint64_t cases, uint64_t ctrls, uint64_t cw, uint64_t tw);
int new_resident(fiu_ctx* ctx, uint64_t snps, uint64_t cases, uint64_t ctrls, uint64_t cw, uint64_t tw,
                 fiu_resident** out);
int finish_resident(fiu_ctx* ctx, fiu_resident* r);
// shard / n_shards: the search covers the shard-th of n_shards contiguous
// ranges of the serving kernel's work units (tensor work items, pair-major
// items or prefix ordinals).
int search_impl(fiu_ctx* ctx, const fiu_resident* res, unsigned order, const fiu_distribution* dist,
                unsigned outputs, int32_t* out_comb, float* out_vals, double* out_vals64, unsigned* out_count,
                int kernel, unsigned shard = 0, unsigned n_shards = 1);
cudaError_t prepare_round_kernels(size_t smem);

}  // namespace fiu
