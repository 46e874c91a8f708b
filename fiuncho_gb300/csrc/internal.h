// Host-side declarations shared by the library's translation units.
#pragma once

#include <cuda.h>

#include <mutex>
#include <vector>

#include "common.cuh"

namespace fiu {

// Where the counting kernels append top-N candidates: every combination whose
// fixed-point key is >= thr goes to buf[atomicAdd(count, 1)] while below cap;
// past cap the kernel only raises *overflow.
struct CandSink {
    Cand* buf;
    unsigned* count;
    unsigned* overflow;
    unsigned cap;
    long long thr;
    unsigned long long* evaluated;  // optional: += combinations evaluated
    // Digest mode (fiu_scan_digest; off when null): every valid combination
    // gets its exact tables and adds its term (digest.cuh) to one of the
    // kDigestSlots sums at digest.  The order-4 kernels assemble a table in
    // dscratch (2 x 81 words per thread of the grid, dscratch_threads threads;
    // a thread beyond them adds a wrong term, so the digest cannot match).
    unsigned long long* digest;
    uint32_t* dscratch;
    unsigned dscratch_threads;
};

// ---- multi-scan engine (batch.cu, engine.cu) ----------------------------------
struct ScoredRec {  // a re-scored candidate (FP64 MI, combination code, fixed-point key)
    double v;
    unsigned long long code;
    long long key;
};

struct ScanDesc {  // per scan, read-only on the device
    ScanWork w;
    int kind;          // FIU_KERNEL_FULL / _ELIDED_POPC / _ELIDED_HS
    int tp;            // threads per prefix (l-tile width): 32, 64, 128 or 256
    unsigned keep;     // candidates kept between rounds (outputs + margin)
    unsigned cap;      // candidate buffer capacity
    unsigned outputs;
    const uint32_t* single;
    const uint4* pairs;
    const uint4* triples;  // order-4 reduced-work kernel only
    Cand* cand;        // [cap]
    ScoredRec* scored; // [keep]
    int* out_comb;     // [outputs * order]
    float* out_val;    // [outputs]
    double* out_val64; // [outputs]
};

struct ScanState {  // per scan, updated on the device between rounds
    unsigned count;     // candidates held in cand
    unsigned overflow;  // a round dropped candidates (cap exceeded)
    unsigned have;      // kept candidates after the last selection
    unsigned n_out;     // results written by the final pass
    long long thr;      // current admission threshold (fixed-point key)
    unsigned long long evaluated;  // combinations evaluated
};

struct RoundEntry {  // owned prefix ordinals [m0, m0 + n) of scan `scan`, items [begin, begin + n)
    int scan;
    int pad;
    long long m0;
    long long begin;
};

// batch.cu
size_t round_smem(const ScanDesc& sd);
// family: 0 reduced-work kernels (orders 2-3), 1 full table (orders 2-4), 2 reduced-work
// kernel at order 4; tp as in ScanDesc.
constexpr int kRoundFamilies = 3;
inline int round_family(int kind, int order) { return kind == FIU_KERNEL_FULL_ID ? 1 : order == 4 ? 2 : 0; }
// queue: the launch's work-queue cursor (device, zero before the launch).
cudaError_t launch_round(int family, int tp, const ScanDesc* scans, ScanState* states, const RoundEntry* ents,
                         int n_ents, long long total, size_t smem, int sms, unsigned long long* queue,
                         cudaStream_t s);
cudaError_t launch_select_scans(const ScanDesc* scans, ScanState* states, int n_scans, int final_pass,
                                cudaStream_t s);
cudaError_t launch_finish_scans(const ScanDesc* scans, ScanState* states, const unsigned* slot_begin, int n_scans,
                                unsigned total_slots, cudaStream_t s);

// Synchronises the TP threads of group `grp` of a 256-thread block: the whole
// block, one warp, or a named barrier (ids 1..8) for 64 / 128 threads.
template <int TP>
__device__ __forceinline__ void group_sync(int grp) {
    if (TP >= 256) {
        __syncthreads();
    } else if (TP == 32) {
        __syncwarp();
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(grp + 1), "r"(TP) : "memory");
    }
}

// Launch-count bookkeeping (kernels of this library only).
extern thread_local unsigned long long* g_launch_counter;
inline void count_launch(unsigned n = 1) {
    if (g_launch_counter) *g_launch_counter += n;
}

// Largest dynamic shared memory a counting kernel may use (all groups).
constexpr size_t kMaxGroupSmem = 200 * 1024;

// Launch configuration of one kernel, cached and safe to share between host
// threads (the served form runs two): the dynamic shared-memory limit only
// grows, so a launch prepared by one thread is never invalidated by another;
// resident blocks per SM are looked up again when the size changes.
struct LaunchCache {
    std::mutex mu;
    size_t attr = 0;
    size_t occ_smem = ~(size_t)0;
    int occ = 0;
};
template <class F>
cudaError_t blocks_per_sm(LaunchCache& c, F* fn, int threads, size_t smem, int& out) {
    std::lock_guard<std::mutex> g(c.mu);
    if (smem > c.attr) {
        const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        c.attr = smem;
    }
    if (c.occ_smem != smem) {
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.occ, fn, threads, smem);
        if (e != cudaSuccess) return e;
        if (c.occ < 1) c.occ = 1;
        c.occ_smem = smem;
    }
    out = c.occ;
    return cudaSuccess;
}

// count.cu -- generic full 3^k table kernel (any data, orders 2..8) with the
// fused fixed-point MI and the candidate filter; tp = threads per prefix
// (32, 64, 128 or 256; orders above 5 always use 256).
cudaError_t launch_count(int tp, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                         uint32_t* dump, cudaStream_t s, int sms);

// elided.cu -- reduced-work kernels for one-hot data, orders 2 and 3.
cudaError_t build_cores(const DevData& d, uint32_t* single, uint4* pairs, int sms, cudaStream_t s);
size_t elided_smem(int order, int cw, int tw);
cudaError_t launch_elided(bool hs, int tp, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                          uint32_t* dump, const uint32_t* single, const uint4* pairs, cudaStream_t s, int sms);

// elided4.cu -- reduced-work kernel for one-hot data, order 4 (reads triple cores).
size_t triples_bytes(int snps);
cudaError_t build_triples(const DevData& d, uint4* triples, int sms, cudaStream_t s);
size_t elided4_smem(int cw, int tw);
cudaError_t launch_elided4(bool hs, int tp, const ScanWork& w, long long m0, long long m1, const CandSink& sink,
                           uint32_t* dump, const uint32_t* single, const uint4* pairs, const uint4* triples,
                           cudaStream_t s, int sms);
// Pair-major schedule of a whole-data-set order-4 scan: work items g in [g0, g1)
// of the table begin[0..snps] (e4p_item_begin).
std::vector<long long> e4p_item_begin(int snps);
size_t e4p_smem(int cw, int tw);
cudaError_t launch_elided4p(const ScanWork& w, const long long* begin, long long g0, long long g1,
                            const CandSink& sink, uint32_t* dump, const uint32_t* single, const uint4* pairs,
                            const uint4* triples, cudaStream_t s, int sms);

// tensor3.cu -- order-2 and order-3 core cells on tcgen05 (one-hot data, whole data set, one worker).
// Device state of the tensor kernel for one data set: the e4m3 operand planes
// (row 2*snp+g = "genotype of snp == g" per sample, cases then controls, each
// class padded to a multiple of 128 samples), their TMA descriptors and the
// work-item prefix sums.
struct T3Plan {
    std::mutex items_mu;  // guards the order-3 / order-4 item tables made on first use
    uint8_t* planes = nullptr;
    int pack = 0;         // log2 of the control weight W when one accumulator holds both classes (else 0)
    double item_combos = 0;  // combinations per work item, about 32 x L / 2
    int pitch = 0;        // bytes per plane row
    int k_cases = 0;      // padded case samples (= byte offset of the control region)
    bool pair3 = false;   // order 3, packed classes: pair items (i, 64 j, 128 l) of the CTA-pair kernel
    struct T3Layers* layers = nullptr;  // order 3, packed: work items of Distribution layers (tensor3.cu)
    long long* item_begin = nullptr;
    long long total = 0;  // work items
    CUtensorMap map_l;    // box 128 B x 192 rows (256 when packed), 128-byte swizzle (l operand)
    CUtensorMap map_j;    // box 128 B x 64 rows, 128-byte swizzle (j rows of the (i,j) operand)
    CUtensorMap map_i;    // box 128 B x 2 rows, 128-byte swizzle (i rows)
    // order 2: work items (64 i, 128 j) over i-tiles, or pair items (2 x 64 i, 128 j) of the
    // CTA-pair kernel (pair2)
    bool pair2 = false;
    long long* item2_begin = nullptr;
    long long total2 = 0;
    int n_itiles = 0;
    double item2_combos = 0;
    CUtensorMap map_a2;   // box 128 B x 128 rows (i rows)
    CUtensorMap map_b2;   // box 128 B x 256 rows (j rows)
    // order 4: work items (i, j, 16 k, 128 l) (64 l when the classes do not pack); item4_begin[j]
    // = first item of the pairs with second SNP j, item4_per[j] = items per such pair
    long long* item4_begin = nullptr;
    long long* item4_per = nullptr;
    long long total4 = 0;
    double item4_combos = 0;
    CUtensorMap map_k4;   // box 128 B x 32 rows (k rows)
};
// log2 of the control weight W = 4^h when both classes fit one FP32 accumulator
// (n_cases < W, n_cases + W * n_ctrls < 2^24), else 0.
int tensor_pack(int n_cases, int n_ctrls);
// Work units of a request on the tensor kernels (w's order and Distribution
// layer; a layer's items must have been made by tensor3_layer), and the
// combinations of an average unit.
long long tensor_units(const T3Plan& plan, const ScanWork& w);
double tensor_item_combos(const T3Plan& plan, const ScanWork& w);
// Whether the tensor kernels serve the Distribution layer of w (order 3,
// classes that pack, the layer of all SNPs), and the layer's work items,
// made on first use (host enumeration of the owned prefixes; the operand
// planes ordered by SNP residue mod the layer's step, copied on stream s).
bool tensor_layer_ok(const T3Plan& plan, const ScanWork& w);
cudaError_t tensor3_layer(T3Plan& plan, const ScanWork& w, cudaStream_t s);
cudaError_t tensor3_prepare(const DevData& d, T3Plan& plan, cudaStream_t s);
// The whole data set's work items at order 3 or 4, made on first use (thread-safe).
cudaError_t tensor3_order_items(T3Plan& plan, const DevData& d, int order);
void tensor3_release(T3Plan& plan);
cudaError_t launch_tensor3(const ScanWork& w, const T3Plan& plan, long long g0, long long g1, const CandSink& sink,
                           uint32_t* dump, const uint32_t* single, const uint4* pairs, const uint4* triples,
                           int* status, cudaStream_t s, int sms);
// tensor4.cu -- order 4 on tcgen05 (one-hot data, the whole data set or a Distribution layer of it).
std::vector<long long> t4_item_table(int n, bool pack, std::vector<long long>& per);
long long t4_layer_items(int n, int step, long long offset, bool pack, std::vector<long long>& pbegin,
                         std::vector<int4>& pinfo, long long& combos);
// pinfo / n_pairs: a layer's pair tables (begin = their first items, per unused; map_k over the
// residue-ordered planes), else nullptr
cudaError_t launch_tensor4(const ScanWork& w, const CUtensorMap& map_l256, const CUtensorMap& map_l128,
                           const CUtensorMap& map_k, const CUtensorMap& map_i, const long long* begin,
                           const long long* per, int k_cases, int pack, long long g0, long long g1,
                           const CandSink& sink, uint32_t* dump, const uint32_t* single, const uint4* pairs,
                           const uint4* triples, int* status, cudaStream_t s, int sms, const int4* pinfo = nullptr,
                           int n_pairs = 0);
// Largest absolute error of the kernel's single-precision log2 over all its inputs (counts <= max_c).
cudaError_t probe_lg2_error(unsigned max_c, double* max_abs_err, cudaStream_t s);
cudaError_t probe_wait_limit(unsigned limit_us, int arrive, int* completed, double* elapsed_ms, cudaStream_t s);

// layout.cu -- device layouts of a data set.
cudaError_t launch_transpose(const uint64_t* ref, uint64_t* tr, int snps, int rows, cudaStream_t s);
cudaError_t launch_onehot_check(const uint64_t* ref, int snps, int cw, int tw, int n_cases, int n_ctrls,
                                int* bad, cudaStream_t s);
cudaError_t launch_combine(const uint64_t* t1, int size1, const uint64_t* t2, int cw, int tw, uint64_t* out,
                           cudaStream_t s);
// Sustained AND+POPC+ADD word-op rate of this GPU (in-bounds microbenchmark).
cudaError_t probe_popc_rate(int sms, cudaStream_t s, double* word_ops_per_s);
cudaError_t launch_combine_popcnt(const uint64_t* t1, int size1, const uint64_t* t2, int cw, int tw,
                                  uint32_t* cases_out, uint32_t* ctrls_out, int ct_size, cudaStream_t s);

// topn.cu -- top-N selection, FP64 rescoring, tables of given combinations.
// Keeps the best `keep` of buf[0..M) (key desc, code asc) in buf[0..min(M,keep)),
// sorted best first.  tmp must hold M + 8192 entries; scratch >= 262 words.
cudaError_t select_top(Cand* buf, unsigned M, unsigned keep, Cand* tmp, unsigned* scratch, cudaStream_t s);
// FP64 MI of candidates (recomputing their full tables), then sorts
// (mi64 desc, code asc) in place; out_mi64[i] matches cands[i] after the sort.
cudaError_t rescore_sort(const DevData& d, int order, int bits, Cand* cands, unsigned n, double* mi64,
                         cudaStream_t s);
cudaError_t launch_tables(const DevData& d, int order, const int* combos, size_t count, uint32_t* cases_out,
                          uint32_t* ctrls_out, double* mi64, cudaStream_t s);
cudaError_t launch_mi(const uint32_t* cases, const uint32_t* ctrls, size_t cells, size_t count, int n_cases,
                      int n_ctrls, const long long* ftab, long long ftab_max, int mode, float* out, double* out64,
                      cudaStream_t s);

}  // namespace fiu
