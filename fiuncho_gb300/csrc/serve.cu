// Served request stream with continuous batching (fiu_server_*).
//
// One worker thread owns a device context.  Scans are admitted from a FIFO
// queue while their device footprint fits the budget; every admitted scan
// occupies a slot of device-resident descriptors/state (ScanDesc/ScanState
// of batch.cu) and keeps its data set, candidate buffer and running top-N on
// the device until it completes.  Each loop iteration is one round over all
// admitted scans: the round kernels process every scan's next chunk of
// prefixes (chunks grow x4 per round, capped by a per-round work budget so a
// large scan does not hold small ones back), then one selection CTA per slot
// raises thresholds on the device.  Scans whose last chunk ran are finalised
// (FP64 re-score + top-N), copied out, and release their memory and slot;
// scans that arrived meanwhile are admitted before the next round.
//
// Scans that run best alone -- those served by the tensor-core kernels
// (one-hot orders 2-4) or the pair-major order-4 kernel, full-table scans
// above order 4, and any scan admitted while every slot is taken -- go to the
// solo lanes: kSoloLanes worker threads, each with its own context and
// stream, take them from one FIFO and run each through the single-scan path.
// The lanes run concurrently with one another and with the rounds, so the
// kernels of several scans share the device: a persistent kernel of one scan
// takes the SMs that another leaves idle (launch tails, the host gaps between
// a scan's chunks, its selection and re-scoring), and a small scan that
// arrives behind a large one starts at once instead of waiting for it.
// fiu_serve_stats.overlapped counts the scans whose device work overlapped
// another scan's.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "ctx.h"

using namespace fiu;
using Clock = std::chrono::steady_clock;

namespace {

constexpr int kSlots = 256;                // concurrently admitted scans
constexpr int kSoloLanes = 2;              // solo worker threads (one context and stream each)
constexpr double kRoundBudget = 1.5e11;    // combinations x samples per scan per round

struct ServeScan {
    uint64_t ticket = 0;
    std::vector<uint64_t> data;
    fiu_dataset host{};
    unsigned order = 0, outputs = 0;
    Clock::time_point submitted, done;
    fiu_resident* res = nullptr;
    int slot = -1;
    ScanWork w{};
    int kind = 0, tp = 256;
    unsigned keep = 0, cap = 0;
    long long cursor = 0, chunk = 1, max_chunk = 1;
    unsigned shard = 0, n_shards = 1;  // shard of the scan's work units (fiu_server_submit_shard)
    long long m_end = 0;               // end of the shard's prefix ordinals (round scans)
    size_t bytes = 0;
    double work = 0;  // combinations x samples of the scan (its shard): the shortest-first key
    char* buf = nullptr;
    size_t off_scored = 0, off_comb = 0, off_val = 0, off_val64 = 0;
    int status = FIU_OK;
    bool finished = false;
    bool overlap = false;  // its device work overlapped another scan's (under the server mutex)
    std::vector<int32_t> comb;
    std::vector<float> vals;
    std::vector<double> vals64;
    unsigned count = 0;
};

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t footprint(const ServeScan& s) {
    const size_t snps = s.host.snps, W = s.host.cases_words + s.host.ctrls_words;
    size_t b = 2 * snps * 3 * W * 8 + (64 * W + 1) * 8 + snps * 16;  // data set, transposed copy, c ln c table
    if (s.order >= 3) b += snps * (snps - 1) / 2 * 16;                     // pair cores
    if (s.order == 4) b += (size_t)binom((long long)snps, 3) * 32;         // triple cores
    // e4m3 operand planes of the tensor-core kernels: 2 rows per SNP, each class padded to 128 samples
    b += 2 * snps * 128 * ((s.host.cases_words + 1) / 2 + (s.host.ctrls_words + 1) / 2);
    const size_t keep = s.outputs + std::max(32u, s.outputs / 8);
    b += std::max<size_t>({32768, 16 * keep, snps + keep}) * sizeof(Cand) + keep * sizeof(ScoredRec) +
         (size_t)s.outputs * (4 * s.order + 12) + 4096;
    return b;
}

}  // namespace

struct fiu_server {
    fiu_ctx* ctx = nullptr;
    uint64_t budget = 0;
    int policy = FIU_SERVE_FIFO;  // order in which queued scans are admitted and solo lanes pick (under mu)
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ServeScan*> queue;
    std::vector<ServeScan*> active;
    std::map<uint64_t, ServeScan*> tickets;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread worker;
    // solo lanes
    fiu_ctx* solo_ctx[kSoloLanes] = {};
    std::deque<ServeScan*> solo_queue;
    std::condition_variable cv_solo;
    std::thread solo_worker[kSoloLanes];
    std::vector<ServeScan*> running;  // scans with device work in flight, any lane (under mu)
    ScanDesc* d_desc = nullptr;
    ScanState* d_state = nullptr;
    unsigned* d_zero = nullptr;
    unsigned long long* d_queue = nullptr;  // one work-queue cursor per round launch (family x tile width)
    RoundEntry* d_ents = nullptr;
    size_t ents_cap = 0;
    std::vector<int> free_slots;
    // statistics (under mu)
    uint64_t submitted = 0, completed = 0, failed = 0, rounds = 0, bytes_in_use = 0, solo = 0, overlapped = 0;
    uint64_t peak_bytes = 0;
    std::vector<double> lat_ms;
    double combos_samples = 0;
    int init_status = FIU_OK;
};

namespace {

// Frees what a scan holds on the device; ctx is the context of the calling lane.
void release(fiu_server* sv, ServeScan* s, fiu_ctx* ctx) {
    if (s->slot >= 0) {
        ScanDesc zero{};
        cudaMemcpyAsync(sv->d_desc + s->slot, &zero, sizeof(zero), cudaMemcpyHostToDevice, sv->ctx->stream);
        cudaStreamSynchronize(sv->ctx->stream);
        sv->free_slots.push_back(s->slot);
        s->slot = -1;
    }
    if (s->buf) cudaFree(s->buf);
    s->buf = nullptr;
    if (s->res) fiu_dataset_free(ctx, s->res);
    s->res = nullptr;
    std::vector<uint64_t>().swap(s->data);
}

// A scan's device work starts (called under sv->mu): it and every scan
// already in flight on any lane overlap.
void start_run(fiu_server* sv, ServeScan* s) {
    if (!sv->running.empty()) {
        s->overlap = true;
        for (ServeScan* o : sv->running) o->overlap = true;
    }
    sv->running.push_back(s);
}

void finish(fiu_server* sv, ServeScan* s, int status, fiu_ctx* ctx = nullptr) {
    s->status = status;
    release(sv, s, ctx ? ctx : sv->ctx);
    std::lock_guard<std::mutex> g(sv->mu);
    s->done = Clock::now();
    s->finished = true;
    sv->bytes_in_use -= s->bytes;
    sv->running.erase(std::remove(sv->running.begin(), sv->running.end(), s), sv->running.end());
    if (status == FIU_OK) {
        sv->completed++;
        if (s->overlap) sv->overlapped++;
        sv->lat_ms.push_back(std::chrono::duration<double, std::milli>(s->done - s->submitted).count());
        sv->combos_samples +=
            (double)binom(s->host.snps, s->order) / s->n_shards * (double)(s->host.cases + s->host.ctrls);
    } else {
        sv->failed++;
    }
    sv->cv_done.notify_all();
    sv->cv_work.notify_all();  // memory freed: the worker may admit the next scan
}

// Uploads and plans an admitted scan; returns false when it finished right away.
bool admit(fiu_server* sv, ServeScan* s) {
    fiu_ctx* ctx = sv->ctx;
    int rc = fiu_dataset_upload(ctx, &s->host, &s->res);
    if (rc) {
        finish(sv, s, rc);
        return false;
    }
    fiu_distribution dist{(int)s->host.snps, (int)s->order - 1, 1, 0};
    s->comb.assign((size_t)std::max(1u, s->outputs) * s->order, 0);
    s->vals.assign(std::max(1u, s->outputs), 0.f);
    s->vals64.assign(std::max(1u, s->outputs), 0.0);
    if ((rc = make_work(ctx, s->res, s->order, &dist, s->outputs, s->w))) {
        finish(sv, s, rc);
        return false;
    }
    if (s->outputs == 0 || s->w.n_prefixes == 0) {
        finish(sv, s, FIU_OK);
        return false;
    }
    {
        const long long P = s->w.n_prefixes, N = s->n_shards;
        s->cursor = P / N * s->shard + std::min<long long>(s->shard, P % N);
        s->m_end = s->cursor + P / N + ((long long)s->shard < P % N ? 1 : 0);
    }
    if ((rc = choose_tile(ctx, s->res, s->w, ctx->kernel, s->kind, s->tp, true))) {
        finish(sv, s, rc);
        return false;
    }
    if (s->kind == FIU_KERNEL_TENSOR || e4_pair_major(s->kind, s->res, s->w) ||
        (s->kind == FIU_KERNEL_FULL && s->order > 4) || sv->free_slots.empty()) {
        // outside the round kernels: the solo lane
        std::lock_guard<std::mutex> g(sv->mu);
        sv->solo_queue.push_back(s);
        sv->cv_solo.notify_one();
        return false;
    }
    s->keep = s->outputs + std::max(32u, s->outputs / 8);
    s->cap = (unsigned)std::max<size_t>({32768, (size_t)16 * s->keep, (size_t)s->host.snps + s->keep});
    size_t b = a256((size_t)s->cap * sizeof(Cand));
    s->off_scored = b;
    b = a256(b + (size_t)s->keep * sizeof(ScoredRec));
    s->off_comb = b;
    b = a256(b + (size_t)s->outputs * s->order * sizeof(int));
    s->off_val = b;
    b = a256(b + (size_t)s->outputs * sizeof(float));
    s->off_val64 = b;
    b = a256(b + (size_t)s->outputs * sizeof(double));
    if (cudaMalloc((void**)&s->buf, b) != cudaSuccess) {
        finish(sv, s, FIU_ERR_NOMEM);
        return false;
    }
    s->slot = sv->free_slots.back();
    sv->free_slots.pop_back();
    ScanDesc d{};
    d.w = s->w;
    d.kind = s->kind;
    d.tp = s->tp;
    d.keep = s->keep;
    d.cap = s->cap;
    d.outputs = s->outputs;
    d.single = s->res->single;
    d.pairs = s->res->pairs;
    d.triples = s->res->triples;
    d.cand = (Cand*)s->buf;
    d.scored = (ScoredRec*)(s->buf + s->off_scored);
    d.out_comb = (int*)(s->buf + s->off_comb);
    d.out_val = (float*)(s->buf + s->off_val);
    d.out_val64 = (double*)(s->buf + s->off_val64);
    const ScanState st0{0, 0, 0, 0, (long long)0x8000000000000000ull, 0};
    cudaMemcpyAsync(sv->d_desc + s->slot, &d, sizeof(d), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(sv->d_state + s->slot, &st0, sizeof(st0), cudaMemcpyHostToDevice, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        finish(sv, s, FIU_ERR_CUDA);
        return false;
    }
    const double per = (double)binom(s->w.dist_n, s->order) / std::max(1.0, (double)binom(s->w.dist_n, s->order - 1));
    s->chunk = std::max<long long>(1, (long long)(s->keep / std::max(1.0, per)));
    s->max_chunk = std::max<long long>(1, (long long)(kRoundBudget / std::max(1.0, per * (double)(s->host.cases + s->host.ctrls))));
    std::lock_guard<std::mutex> g(sv->mu);
    start_run(sv, s);
    return true;
}

// One round over the admitted scans; finalises the ones that completed.
int run_round(fiu_server* sv) {
    fiu_ctx* ctx = sv->ctx;
    cudaStream_t st = ctx->stream;
    std::vector<RoundEntry> ents;
    std::vector<std::pair<size_t, long long>> groups;  // (first entry, items) per family
    size_t smem = 0;
    for (ServeScan* s : sv->active) {
        ScanDesc d{};
        d.w = s->w;
        d.kind = s->kind;
        d.tp = s->tp;
        smem = std::max(smem, round_smem(d));
    }
    std::vector<long long> take(sv->active.size(), 0);
    for (size_t i = 0; i < sv->active.size(); ++i) {
        ServeScan* s = sv->active[i];
        take[i] = std::min({s->m_end - s->cursor, s->chunk, s->max_chunk});
    }
    // entries of a launch in decreasing work per prefix (words x last SNPs per
    // prefix): the device work queue hands out the long items first
    std::vector<size_t> by_cost(sv->active.size());
    std::vector<double> cost(sv->active.size());
    for (size_t i = 0; i < sv->active.size(); ++i) {
        const ScanWork& w = sv->active[i]->w;
        by_cost[i] = i;
        cost[i] = (double)(w.dist_n - w.order + 2) / w.order * (double)(w.d.cw + w.d.tw);
    }
    std::stable_sort(by_cost.begin(), by_cost.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<std::pair<int, int>> gkey;  // (family, tp) of each group
    for (int fam = 0; fam < kRoundFamilies; ++fam)
        for (int tp : {32, 64, 128, 256}) {
            const size_t first = ents.size();
            long long total = 0;
            for (size_t i : by_cost) {
                ServeScan* s = sv->active[i];
                if (!take[i] || round_family(s->kind, s->order) != fam || s->tp != tp) continue;
                ents.push_back(RoundEntry{s->slot, 0, s->cursor, total});
                total += take[i];
            }
            groups.push_back({first, total});
            gkey.push_back({fam, tp});
        }
    int rc = FIU_OK;
    if (ents.size() > sv->ents_cap) {
        cudaFree(sv->d_ents);
        sv->d_ents = nullptr;
        sv->ents_cap = 0;
        if (cudaMalloc((void**)&sv->d_ents, ents.size() * 2 * sizeof(RoundEntry)) != cudaSuccess) return FIU_ERR_NOMEM;
        sv->ents_cap = ents.size() * 2;
    }
    CK(prepare_round_kernels(smem), "kernel attributes");
    CK(cudaMemcpyAsync(sv->d_ents, ents.data(), ents.size() * sizeof(RoundEntry), cudaMemcpyHostToDevice, st),
       "round entries");
    CK(cudaMemsetAsync(sv->d_queue, 0, kRoundFamilies * 4 * sizeof(unsigned long long), st), "work queue");
    for (size_t g = 0; g < groups.size(); ++g) {
        const size_t first = groups[g].first;
        const size_t ne = (g + 1 < groups.size() ? groups[g + 1].first : ents.size()) - first;
        if (ne) CK(launch_round(gkey[g].first, gkey[g].second, sv->d_desc, sv->d_state, sv->d_ents + first, (int)ne,
                                groups[g].second, smem, ctx->sms, sv->d_queue + g, st), "round");
    }
    CK(launch_select_scans(sv->d_desc, sv->d_state, kSlots, 0, st), "selection");
    std::vector<ServeScan*> done, still;
    for (size_t i = 0; i < sv->active.size(); ++i) {
        ServeScan* s = sv->active[i];
        s->cursor += take[i];
        s->chunk *= 4;
        (s->cursor >= s->m_end ? done : still).push_back(s);
    }
    std::vector<ScanState> hs(done.size());
    for (size_t i = 0; i < done.size(); ++i) {
        ServeScan* s = done[i];
        CK(launch_select_scans(sv->d_desc + s->slot, sv->d_state + s->slot, 1, 1, st), "final selection");
        CK(launch_finish_scans(sv->d_desc + s->slot, sv->d_state + s->slot, sv->d_zero, 1, s->keep, st), "finish");
        CK(cudaMemcpyAsync(&hs[i], sv->d_state + s->slot, sizeof(ScanState), cudaMemcpyDeviceToHost, st), "state");
    }
    CK(cudaStreamSynchronize(st), "round");
    for (size_t i = 0; i < done.size(); ++i) {
        ServeScan* s = done[i];
        if (hs[i].overflow) {  // candidate buffer overflowed: redo alone on the adaptive path
            fiu_distribution dist{(int)s->host.snps, (int)s->order - 1, 1, 0};
            rc = search_impl(ctx, s->res, s->order, &dist, s->outputs, s->comb.data(), s->vals.data(),
                             s->vals64.data(), &s->count, 0, s->shard, s->n_shards);
            finish(sv, s, rc);
            continue;
        }
        s->count = std::min(hs[i].n_out, s->outputs);
        cudaMemcpy(s->comb.data(), s->buf + s->off_comb, (size_t)s->count * s->order * sizeof(int),
                   cudaMemcpyDeviceToHost);
        cudaMemcpy(s->vals.data(), s->buf + s->off_val, (size_t)s->count * sizeof(float), cudaMemcpyDeviceToHost);
        const cudaError_t e = cudaMemcpy(s->vals64.data(), s->buf + s->off_val64, (size_t)s->count * sizeof(double),
                                         cudaMemcpyDeviceToHost);
        finish(sv, s, e == cudaSuccess ? FIU_OK : FIU_ERR_CUDA);
    }
    sv->active.swap(still);
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->rounds++;
    }
    return FIU_OK;
}

// Position of the scan a queue hands out next: its head (FIFO) or, under
// FIU_SERVE_SHORTEST_FIRST, the scan of least work (the earliest of equals).
size_t next_of(const fiu_server* sv, const std::deque<ServeScan*>& q) {
    size_t best = 0;
    if (sv->policy == FIU_SERVE_SHORTEST_FIRST)
        for (size_t i = 1; i < q.size(); ++i)
            if (q[i]->work < q[best]->work) best = i;
    return best;
}

// A solo lane: takes scans that run alone from the shared queue (in the
// server's policy order) and runs each on the lane's own stream.
void solo_main(fiu_server* sv, int lane) {
    fiu_ctx* ctx = sv->solo_ctx[lane];
    Scope scope(ctx);
    for (;;) {
        ServeScan* s = nullptr;
        {
            std::unique_lock<std::mutex> g(sv->mu);
            sv->cv_solo.wait(g, [&] { return sv->stop || !sv->solo_queue.empty(); });
            if (sv->stop) return;
            const size_t at = next_of(sv, sv->solo_queue);
            s = sv->solo_queue[at];
            sv->solo_queue.erase(sv->solo_queue.begin() + (long)at);
            start_run(sv, s);
        }
        fiu_distribution dist{(int)s->host.snps, (int)s->order - 1, 1, 0};
        const int rc = search_impl(ctx, s->res, s->order, &dist, s->outputs, s->comb.data(), s->vals.data(),
                                   s->vals64.data(), &s->count, 0, s->shard, s->n_shards);
        {
            std::lock_guard<std::mutex> g(sv->mu);
            sv->solo++;
        }
        finish(sv, s, rc, ctx);
    }
}

void worker_main(fiu_server* sv) {
    Scope scope(sv->ctx);
    for (;;) {
        // admit while the next scan of the queue (policy order) fits the budget
        for (;;) {
            ServeScan* s = nullptr;
            {
                std::unique_lock<std::mutex> g(sv->mu);
                if (sv->stop) return;
                if (sv->queue.empty() || sv->free_slots.empty()) break;
                const size_t at = next_of(sv, sv->queue);
                ServeScan* h = sv->queue[at];
                // every admitted scan holds its footprint until it finishes, whether it runs
                // in the rounds or waits for / runs on a solo lane; a scan larger than the
                // budget left runs only when nothing else holds device memory
                if (sv->bytes_in_use + h->bytes > sv->budget && sv->bytes_in_use > 0) break;
                sv->queue.erase(sv->queue.begin() + (long)at);
                sv->bytes_in_use += h->bytes;
                sv->peak_bytes = std::max(sv->peak_bytes, sv->bytes_in_use);
                s = h;
            }
            if (admit(sv, s)) sv->active.push_back(s);
        }
        if (sv->active.empty()) {
            std::unique_lock<std::mutex> g(sv->mu);
            sv->cv_work.wait_for(g, std::chrono::milliseconds(50),
                                 [&] { return sv->stop || !sv->queue.empty(); });
            if (sv->stop) return;
            continue;
        }
        if (run_round(sv) != FIU_OK) {  // device error: fail every admitted scan
            for (ServeScan* s : sv->active) finish(sv, s, FIU_ERR_CUDA);
            sv->active.clear();
        }
    }
}

}  // namespace

extern "C" {

int fiu_server_create(int device, uint64_t budget_bytes, fiu_server** out) {
    if (!out) return FIU_ERR_INVALID;
    *out = nullptr;
    auto* sv = new fiu_server;
    int rc = fiu_create(device, &sv->ctx);
    if (rc) {
        delete sv;
        return rc;
    }
    sv->budget = budget_bytes ? budget_bytes : 120ull * 1000 * 1000 * 1000;
    for (int l = 0; l < kSoloLanes; ++l)
        if ((rc = fiu_create(device, &sv->solo_ctx[l]))) {
            for (int m = 0; m < l; ++m) fiu_destroy(sv->solo_ctx[m]);
            fiu_destroy(sv->ctx);
            delete sv;
            return rc;
        } else {
            sv->solo_ctx[l]->cancellable = true;
        }
    cudaSetDevice(device);
    if (cudaMalloc((void**)&sv->d_desc, kSlots * sizeof(ScanDesc)) != cudaSuccess ||
        cudaMalloc((void**)&sv->d_state, kSlots * sizeof(ScanState)) != cudaSuccess ||
        cudaMalloc((void**)&sv->d_zero, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc((void**)&sv->d_queue, kRoundFamilies * 4 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(sv->d_desc, 0, kSlots * sizeof(ScanDesc)) != cudaSuccess ||
        cudaMemset(sv->d_state, 0, kSlots * sizeof(ScanState)) != cudaSuccess ||
        cudaMemset(sv->d_zero, 0, sizeof(unsigned)) != cudaSuccess) {
        cudaFree(sv->d_desc);
        cudaFree(sv->d_state);
        cudaFree(sv->d_zero);
        cudaFree(sv->d_queue);
        for (fiu_ctx* c : sv->solo_ctx) fiu_destroy(c);
        fiu_destroy(sv->ctx);
        delete sv;
        return FIU_ERR_CUDA;
    }
    for (int i = kSlots - 1; i >= 0; --i) sv->free_slots.push_back(i);
    sv->worker = std::thread([sv] {
        cudaSetDevice(sv->ctx->device);
        worker_main(sv);
    });
    for (int l = 0; l < kSoloLanes; ++l)
        sv->solo_worker[l] = std::thread([sv, l] {
            cudaSetDevice(sv->ctx->device);
            solo_main(sv, l);
        });
    *out = sv;
    return FIU_OK;
}

int fiu_server_set_policy(fiu_server* sv, int policy) {
    if (!sv || (policy != FIU_SERVE_FIFO && policy != FIU_SERVE_SHORTEST_FIRST)) return FIU_ERR_INVALID;
    std::lock_guard<std::mutex> g(sv->mu);
    sv->policy = policy;
    return FIU_OK;
}

int fiu_server_submit(fiu_server* sv, const fiu_dataset* d, unsigned order, unsigned outputs, uint64_t* ticket) {
    return fiu_server_submit_shard(sv, d, order, outputs, 0, 1, ticket);
}

int fiu_server_submit_shard(fiu_server* sv, const fiu_dataset* d, unsigned order, unsigned outputs, unsigned shard,
                            unsigned n_shards, uint64_t* ticket) {
    if (!sv || !d || !d->data || !ticket) return FIU_ERR_INVALID;
    if (order < 2 || order > FIU_MAX_ORDER || outputs > FIU_MAX_OUTPUTS) return FIU_ERR_INVALID;
    if (n_shards == 0 || shard >= n_shards) return FIU_ERR_INVALID;
    auto* s = new ServeScan;
    s->shard = shard;
    s->n_shards = n_shards;
    const size_t words = (size_t)d->snps * 3 * (d->cases_words + d->ctrls_words);
    s->data.assign(d->data, d->data + words);
    s->host = *d;
    s->host.data = s->data.data();
    s->order = order;
    s->outputs = outputs;
    s->bytes = footprint(*s);
    s->work = (double)binom((long long)d->snps, (int)order) / n_shards * (double)(d->cases + d->ctrls);
    s->submitted = Clock::now();
    std::lock_guard<std::mutex> g(sv->mu);
    if (s->bytes > sv->budget) {
        delete s;
        return FIU_ERR_NOMEM;
    }
    s->ticket = sv->next_ticket++;
    sv->tickets[s->ticket] = s;
    sv->queue.push_back(s);
    sv->submitted++;
    *ticket = s->ticket;
    sv->cv_work.notify_one();
    return FIU_OK;
}

int fiu_server_poll(fiu_server* sv, uint64_t ticket, int wait_ms, int32_t* out_comb, float* out_vals,
                    double* out_vals64, unsigned* out_count, double* latency_ms) {
    if (!sv) return FIU_ERR_INVALID;
    std::unique_lock<std::mutex> g(sv->mu);
    auto it = sv->tickets.find(ticket);
    if (it == sv->tickets.end()) return FIU_ERR_INVALID;
    ServeScan* s = it->second;
    auto ready = [&] { return s->finished; };
    if (wait_ms < 0) sv->cv_done.wait(g, ready);
    else if (wait_ms > 0) sv->cv_done.wait_for(g, std::chrono::milliseconds(wait_ms), ready);
    if (!s->finished) return FIU_ERR_TIMEOUT;
    const int status = s->status;
    if (status == FIU_OK) {
        if (out_count) *out_count = s->count;
        if (out_comb) std::memcpy(out_comb, s->comb.data(), (size_t)s->count * s->order * sizeof(int32_t));
        if (out_vals) std::memcpy(out_vals, s->vals.data(), (size_t)s->count * sizeof(float));
        if (out_vals64) std::memcpy(out_vals64, s->vals64.data(), (size_t)s->count * sizeof(double));
    }
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(s->done - s->submitted).count();
    sv->tickets.erase(it);
    delete s;
    return status;
}

int fiu_server_stats(fiu_server* sv, fiu_serve_stats* out) {
    if (!sv || !out) return FIU_ERR_INVALID;
    std::lock_guard<std::mutex> g(sv->mu);
    *out = fiu_serve_stats{};
    out->submitted = sv->submitted;
    out->completed = sv->completed;
    out->failed = sv->failed;
    out->queued = sv->queue.size();
    out->active = sv->submitted - sv->completed - sv->failed - sv->queue.size();
    out->rounds = sv->rounds;
    out->solo = sv->solo;
    out->overlapped = sv->overlapped;
    out->bytes_in_use = sv->bytes_in_use;
    out->peak_bytes = sv->peak_bytes;
    out->combos_samples = sv->combos_samples;
    if (!sv->lat_ms.empty()) {
        std::vector<double> v = sv->lat_ms;
        std::sort(v.begin(), v.end());
        auto q = [&](double f) { return v[std::min(v.size() - 1, (size_t)(f * (v.size() - 1) + 0.5))]; };
        out->p50_ms = q(0.50);
        out->p99_ms = q(0.99);
        out->max_ms = v.back();
        double sum = 0;
        for (double x : v) sum += x;
        out->mean_ms = sum / v.size();
    }
    return FIU_OK;
}

void fiu_server_destroy(fiu_server* sv) {
    if (!sv) return;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->stop = true;
    }
    for (fiu_ctx* c : sv->solo_ctx)  // scans running on the solo lanes stop after their current chunk
        if (c) c->cancel.store(1);
    sv->cv_work.notify_all();
    sv->cv_solo.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    for (std::thread& t : sv->solo_worker)
        if (t.joinable()) t.join();
    cudaSetDevice(sv->ctx->device);
    for (ServeScan* s : sv->active) release(sv, s, sv->ctx);
    for (auto& kv : sv->tickets) {
        if (kv.second->res || kv.second->buf) release(sv, kv.second, sv->ctx);
        delete kv.second;
    }
    cudaFree(sv->d_desc);
    cudaFree(sv->d_state);
    cudaFree(sv->d_zero);
    cudaFree(sv->d_queue);
    cudaFree(sv->d_ents);
    for (fiu_ctx* c : sv->solo_ctx) fiu_destroy(c);
    fiu_destroy(sv->ctx);
    delete sv;
}

}  // extern "C"
