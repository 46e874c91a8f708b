// The batched form: fiu_search_batch runs many scans together in rounds
// (kernels in batch.cu).  Per-scan chunk schedules grow geometrically (the
// first chunk is sized to yield about `keep` combinations, then x4), so every
// scan gets a threshold early and later rounds admit few candidates.  A scan
// whose candidate buffer overflowed is re-run alone on the single-scan path
// (whose chunking adapts on the host), so results never depend on batching.
// Scans served by the tensor-core kernels (one-hot order 2, 3 or 4 over the whole
// data set) or by the pair-major order-4 kernel (one-hot, whole data set) are
// not split into rounds: each runs on the single-scan path, as in a loop of
// single calls, but on one of two helper lanes (a context with its own stream
// and scratch) concurrently with the rounds and with the other lane, and the
// calling thread joins them once its rounds are done.  Their kernels then
// share the device: the persistent kernels of one scan take the SMs another
// leaves idle (launch tails, the host steps between a scan's chunks).  The
// scans of one data set stay on one lane.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fiuncho_gpu.h"
#include "ctx.h"

using namespace fiu;

namespace {

struct Plan {
    int idx;           // index in the caller's array
    long long m_begin, m_end;  // owned prefix ordinals of the scan's shard
    ScanWork w;
    int kind, tp;
    unsigned keep, cap, outputs;
    const fiu_resident* res;
    size_t off_cand, off_scored, off_comb, off_val, off_val64;  // byte offsets in the arena
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" int fiu_search_batch(fiu_ctx* ctx, fiu_scan* scans, unsigned n_scans, int use_graph) {
    if (!ctx) return FIU_ERR_INVALID;
    Scope scope(ctx);
    if (!scans && n_scans) return fail(ctx, FIU_ERR_INVALID, "null scan array");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    std::vector<Plan> plans;
    std::vector<unsigned> single_path;  // scans the round kernel does not cover
    size_t bytes = 0;
    for (unsigned i = 0; i < n_scans; ++i) {
        fiu_scan& sc = scans[i];
        sc.out_count = 0;
        sc.status = FIU_OK;
        if (sc.outputs && (!sc.out_combinations || !sc.out_vals)) {
            sc.status = fail(ctx, FIU_ERR_INVALID, "null output pointer");
            continue;
        }
        ScanWork w;
        int rc = make_work(ctx, sc.res, sc.order, &sc.distribution, sc.outputs, w);
        if (rc) {
            sc.status = rc;
            continue;
        }
        const unsigned ns = sc.n_shards ? sc.n_shards : 1;
        if (sc.shard >= ns ||
            (ns > 1 && (w.dist_step != 1 || w.dist_offset != 0 || w.dist_n != sc.res->d.snps))) {
            sc.status = fail(ctx, FIU_ERR_INVALID, "shard out of range, or a shard of a distribution layer");
            continue;
        }
        if (sc.outputs == 0 || w.n_prefixes == 0) continue;
        int kind = 0, tp = 256;
        if ((rc = choose_tile(ctx, sc.res, w, ctx->kernel, kind, tp, true))) {
            sc.status = rc;
            continue;
        }
        // tensor-core and pair-major order-4 scans and full-table scans above order 4 run alone
        if (kind == FIU_KERNEL_TENSOR || e4_pair_major(kind, sc.res, w) || (kind == FIU_KERNEL_FULL && sc.order > 4)) {
            single_path.push_back(i);
            continue;
        }
        Plan p;
        p.idx = (int)i;
        p.m_begin = w.n_prefixes / ns * sc.shard + std::min<long long>(sc.shard, w.n_prefixes % ns);
        p.m_end = p.m_begin + w.n_prefixes / ns + (sc.shard < w.n_prefixes % ns ? 1 : 0);
        p.w = w;
        p.kind = kind;
        p.tp = tp;
        p.keep = sc.outputs + std::max(32u, sc.outputs / 8);
        p.cap = (unsigned)std::max<size_t>({32768, (size_t)16 * p.keep, (size_t)sc.res->d.snps + p.keep});
        p.outputs = sc.outputs;
        p.res = sc.res;
        p.off_cand = bytes;
        bytes = align256(bytes + (size_t)p.cap * sizeof(Cand));
        p.off_scored = bytes;
        bytes = align256(bytes + (size_t)p.keep * sizeof(ScoredRec));
        p.off_comb = bytes;
        bytes = align256(bytes + (size_t)p.outputs * sc.order * sizeof(int));
        p.off_val = bytes;
        bytes = align256(bytes + (size_t)p.outputs * sizeof(float));
        p.off_val64 = bytes;
        bytes = align256(bytes + (size_t)p.outputs * sizeof(double));
        plans.push_back(p);
    }
    const int n = (int)plans.size();
    // ---- scans that run alone: grouped by data set, taken by the helper lanes
    // (and by this thread after its rounds)
    std::vector<std::vector<unsigned>> alone;
    {
        std::map<const fiu_resident*, size_t> by_res;
        for (unsigned i : single_path) {
            auto it = by_res.find(scans[i].res);
            if (it == by_res.end()) {
                it = by_res.emplace(scans[i].res, alone.size()).first;
                alone.emplace_back();
            }
            alone[it->second].push_back(i);
        }
    }
    single_path.clear();  // from here on: round scans whose candidate buffer overflowed
    std::atomic<size_t> next_group{0};
    std::mutex err_mu;
    std::string lane_err;  // a lane's last error message, reported on this context after the join
    auto run_alone = [&](fiu_ctx* lc) {
        for (size_t g; (g = next_group.fetch_add(1)) < alone.size();)
            for (unsigned i : alone[g]) {
                fiu_scan& sc = scans[i];
                sc.status = search_impl(lc, sc.res, sc.order, &sc.distribution, sc.outputs, sc.out_combinations,
                                        sc.out_vals, sc.out_vals64, &sc.out_count, 0, sc.shard,
                                        sc.n_shards ? sc.n_shards : 1);
                if (sc.status && lc != ctx) {
                    std::lock_guard<std::mutex> g2(err_mu);
                    lane_err = lc->err;
                }
            }
    };
    std::vector<std::thread> lane_threads;
    std::vector<fiu_ctx*> used_lanes;
    std::vector<unsigned long long> lane_launches0;
    struct Joiner {  // every return below waits for the lanes first
        std::vector<std::thread>& t;
        ~Joiner() {
            for (std::thread& x : t)
                if (x.joinable()) x.join();
        }
    } joiner{lane_threads};
    const size_t helpers = std::min<size_t>(2, n > 0 ? alone.size() : (alone.empty() ? 0 : alone.size() - 1));
    for (size_t l = 0; l < helpers; ++l) {
        fiu_ctx*& lc = ctx->lanes[l];
        if (!lc && fiu_create(ctx->device, &lc) != FIU_OK) {
            lc = nullptr;
            break;  // fewer lanes: this thread takes what is left
        }
        lc->kernel = ctx->kernel;  // the same kernel choice and tuned tiles as this context
        lc->autotune = ctx->autotune;
        lc->tuned = ctx->tuned;
        used_lanes.push_back(lc);
        lane_launches0.push_back(lc->launches);
        lane_threads.emplace_back([lc, &run_alone] {
            cudaSetDevice(lc->device);
            Scope lane_scope(lc);
            run_alone(lc);
        });
    }
    if (n > 0) {
        // ---- round schedule: per round, the entries of each kernel family
        // (round_family) and l-tile width, each group with its own item space
        std::vector<RoundEntry> ents;
        std::vector<size_t> grp_first;      // entries of group g = [grp_first[g], grp_first[g+1])
        std::vector<long long> grp_total;   // items of group g
        std::vector<int> grp_family, grp_tp;
        std::vector<long long> cursor(n, 0), chunk(n);
        std::vector<double> cost(n);  // work of one prefix: words x last SNPs per prefix
        for (int s = 0; s < n; ++s) cursor[s] = plans[s].m_begin;
        for (int s = 0; s < n; ++s) {
            const auto& w = plans[s].w;
            const double per = (double)binom(w.dist_n, w.order) / std::max(1.0, (double)binom(w.dist_n, w.order - 1));
            chunk[s] = std::max<long long>(1, (long long)(plans[s].keep / std::max(1.0, per)));
            cost[s] = per * (double)(w.d.cw + w.d.tw);
        }
        // entries of a launch in decreasing cost per prefix: the work queue hands
        // out the long items first, the short ones fill the tail
        std::vector<int> by_cost(n);
        for (int s = 0; s < n; ++s) by_cost[s] = s;
        std::stable_sort(by_cost.begin(), by_cost.end(), [&](int a, int b) { return cost[a] > cost[b]; });
        int rounds = 0;
        for (bool more = true; more; ++rounds) {
            more = false;
            std::vector<long long> take(n, 0);
            for (int s = 0; s < n; ++s) {
                const long long left = plans[s].m_end - cursor[s];
                if (left > 0) take[s] = std::min(left, chunk[s]);
            }
            for (int fam = 0; fam < kRoundFamilies; ++fam)
                for (int tp : {32, 64, 128, 256}) {
                    long long total = 0;
                    grp_first.push_back(ents.size());
                    for (int s : by_cost) {
                        if (!take[s] || round_family(plans[s].kind, plans[s].w.order) != fam || plans[s].tp != tp)
                            continue;
                        ents.push_back(RoundEntry{s, 0, cursor[s], total});
                        total += take[s];
                    }
                    grp_total.push_back(total);
                    grp_family.push_back(fam);
                    grp_tp.push_back(tp);
                }
            for (int s = 0; s < n; ++s) {
                cursor[s] += take[s];
                chunk[s] *= 4;
                if (cursor[s] < plans[s].m_end) more = true;
            }
        }
        grp_first.push_back(ents.size());
        // ---- device arena: [descs][states][slot_begin][entries][queue cursors][per-scan buffers]
        const size_t n_groups = grp_first.size() - 1;
        const size_t off_desc = 0;
        const size_t off_state = align256(off_desc + n * sizeof(ScanDesc));
        const size_t off_slots = align256(off_state + n * sizeof(ScanState));
        const size_t off_ents = align256(off_slots + n * sizeof(unsigned));
        const size_t off_queue = align256(off_ents + ents.size() * sizeof(RoundEntry));
        const size_t off_bufs = align256(off_queue + n_groups * sizeof(unsigned long long));
        int rc = grow_bytes(ctx, ctx->arena, ctx->arena_cap, off_bufs + bytes);
        if (rc) return rc;
        char* base = ctx->arena;
        std::vector<ScanDesc> descs(n);
        std::vector<ScanState> states(n);
        std::vector<unsigned> slot_begin(n);
        unsigned total_slots = 0;
        size_t smem = 0;
        for (int s = 0; s < n; ++s) {
            const Plan& p = plans[s];
            ScanDesc& d = descs[s];
            d.w = p.w;
            d.kind = p.kind;
            d.tp = p.tp;
            d.keep = p.keep;
            d.cap = p.cap;
            d.outputs = p.outputs;
            d.single = p.res->single;
            d.pairs = p.res->pairs;
            d.triples = p.res->triples;
            d.cand = (Cand*)(base + off_bufs + p.off_cand);
            d.scored = (ScoredRec*)(base + off_bufs + p.off_scored);
            d.out_comb = (int*)(base + off_bufs + p.off_comb);
            d.out_val = (float*)(base + off_bufs + p.off_val);
            d.out_val64 = (double*)(base + off_bufs + p.off_val64);
            states[s] = ScanState{0, 0, 0, 0, (long long)0x8000000000000000ull, 0};
            slot_begin[s] = total_slots;
            total_slots += p.keep;
            smem = std::max(smem, round_smem(d));
        }
        cudaStream_t st = ctx->stream;
        CK(cudaMemcpyAsync(base + off_desc, descs.data(), n * sizeof(ScanDesc), cudaMemcpyHostToDevice, st), "upload");
        CK(cudaMemcpyAsync(base + off_state, states.data(), n * sizeof(ScanState), cudaMemcpyHostToDevice, st), "upload");
        CK(cudaMemcpyAsync(base + off_slots, slot_begin.data(), n * sizeof(unsigned), cudaMemcpyHostToDevice, st),
           "upload");
        CK(cudaMemcpyAsync(base + off_ents, ents.data(), ents.size() * sizeof(RoundEntry), cudaMemcpyHostToDevice, st),
           "upload");
        CK(cudaMemsetAsync(base + off_queue, 0, n_groups * sizeof(unsigned long long), st), "upload");
        CK(cudaStreamSynchronize(st), "upload");
        const ScanDesc* d_desc = (const ScanDesc*)(base + off_desc);
        ScanState* d_state = (ScanState*)(base + off_state);
        const unsigned* d_slots = (const unsigned*)(base + off_slots);
        const RoundEntry* d_ents = (const RoundEntry*)(base + off_ents);
        unsigned long long* d_queue = (unsigned long long*)(base + off_queue);
        // host mirror of results (pinned, so the copies can live in a graph)
        rc = grow_host(ctx, bytes + n * sizeof(ScanState));
        if (rc) return rc;
        char* hbuf = ctx->host_arena;
        auto enqueue = [&]() -> cudaError_t {
            cudaError_t e = cudaSuccess;
            for (size_t g = 0; g + 1 < grp_first.size() && e == cudaSuccess; ++g) {
                const int ne = (int)(grp_first[g + 1] - grp_first[g]);
                if (ne)
                    e = launch_round(grp_family[g], grp_tp[g], d_desc, d_state, d_ents + grp_first[g], ne,
                                     grp_total[g], smem, ctx->sms, d_queue + g, st);
                if (e == cudaSuccess && g % 8 == 7) e = launch_select_scans(d_desc, d_state, n, 0, st);
            }
            if (e == cudaSuccess) e = launch_select_scans(d_desc, d_state, n, 1, st);
            if (e == cudaSuccess) e = launch_finish_scans(d_desc, d_state, d_slots, n, total_slots, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(hbuf, base + off_bufs, bytes, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(hbuf + bytes, d_state, n * sizeof(ScanState), cudaMemcpyDeviceToHost, st);
            return e;
        };
        // kernel attributes are set outside any capture
        CK(prepare_round_kernels(smem), "kernel attributes");
        if (use_graph) {
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "graph capture");
            cudaError_t e = enqueue();
            cudaError_t e2 = cudaStreamEndCapture(st, &graph);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                return cuda_fail(ctx, e != cudaSuccess ? e : e2, "graph capture");
            }
            e = cudaGraphInstantiate(&exec, graph, 0);
            if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (exec) cudaGraphExecDestroy(exec);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "batch graph");
            count_launch(1);  // the graph launch itself
        } else {
            CK(enqueue(), "batch launches");
            CK(cudaStreamSynchronize(st), "batch");
        }
        const ScanState* hs = (const ScanState*)(hbuf + bytes);
        for (int s = 0; s < n; ++s) {
            const Plan& p = plans[s];
            fiu_scan& sc = scans[p.idx];
            if (hs[s].overflow) {
                single_path.push_back((unsigned)p.idx);
                continue;
            }
            const unsigned cnt = std::min(hs[s].n_out, p.outputs);
            std::memcpy(sc.out_combinations, hbuf + p.off_comb, (size_t)cnt * sc.order * sizeof(int));
            std::memcpy(sc.out_vals, hbuf + p.off_val, (size_t)cnt * sizeof(float));
            if (sc.out_vals64) std::memcpy(sc.out_vals64, hbuf + p.off_val64, (size_t)cnt * sizeof(double));
            sc.out_count = cnt;
        }
    }
    for (unsigned i : single_path) {
        fiu_scan& sc = scans[i];
        sc.status = search_impl(ctx, sc.res, sc.order, &sc.distribution, sc.outputs, sc.out_combinations,
                                sc.out_vals, sc.out_vals64, &sc.out_count, 0, sc.shard, sc.n_shards ? sc.n_shards : 1);
    }
    run_alone(ctx);
    for (std::thread& t : lane_threads) t.join();
    for (size_t l = 0; l < used_lanes.size(); ++l) ctx->launches += used_lanes[l]->launches - lane_launches0[l];
    if (!lane_err.empty()) ctx->err = lane_err;
    return FIU_OK;
}
