// Order-4 contingency tables on the 5th-generation tensor cores (tcgen05).
//
// For one-hot data the 16 core cells of a combination (i, j, k, l) --
// genotypes x, y, z, w in {0, 1} -- are dot products over the samples:
//     core[x][y][z][w] = sum_s a_ix(s) a_jy(s) a_kz(s) a_lw(s).
// A work item is (i, j, 16 consecutive k, 128 consecutive l); it is one GEMM
//     D[(k,x,y,z), (l,w)] = sum_s A[(k,x,y,z), s] B[(l,w), s]   (M 128, N 256)
// over the e4m3 operand planes of tensor3.cu, both classes in one FP32
// accumulator (control samples weighted by W = 4^h, exact while
// n_cases < W and n_cases + W * n_ctrls < 2^24).  Classes that do not pack
// take the split form: 64 l per item, the case samples accumulate into one
// N 128 region and the control samples into another, two such pairs
// alternating between items (measured against 128 l per item with one N 256
// region per class and no alternation: 16.9 vs 18.4 ms at 150 SNPs x
// 5 900/9 000 samples).  B rows are plane rows 2l+w
// by TMA; A rows are the bytewise AND of the i, j and k plane rows, built in
// shared memory by two producer warps from the TMA-staged rows (i AND j once
// per stage, then AND each k row).  Two accumulator regions alternate between
// items so the next item's GEMM overlaps the epilogue.
//
// Epilogue.  Each thread reads the accumulators of one row (k, x, y, z); a
// swizzled shared-memory transpose gives each lane the 16 core counts of one
// combination.  The 81-cell tables follow exactly (slice by slice, from the
// triple, pair and single cores, as in the CUDA-core order-4 kernels).  A
// bounded estimate of the MI key -- single-precision c*lg2(c) terms summed
// pairwise per 27-cell slice, slices summed in 64-bit fixed point -- rejects
// the combinations that cannot reach the threshold; the others get the exact
// 64-bit fixed-point key from the integer c*ln(c) table.
//
// Reference semantics: GenotypeTable::combine_and_popcnt for order 4
// (src/base/gt_popcnt.cpp:4-35) and MutualInformation::compute
// (src/base/mi_compute.cpp:16-41) over the combinations
// ThreadedSearch visits (include/fiuncho/ThreadedSearch.h:157-180) with one
// worker.
#include <algorithm>
#include <cmath>

#include "elided4_prefix.cuh"
#include "tensor_common.cuh"

namespace fiu {

constexpr int kT4K = 16, kT4L = 128;                // k and l SNPs per work item (64 l in the split form)
constexpr int kT4M = 8 * kT4K, kT4N = 2 * kT4L;     // 128 x 256 GEMM tile
// Two A builders keep pace with the MMA (about 130 instructions per builder
// thread and k-step against ~640 tensor cycles).  The epilogue warps (a
// multiple of 4: each reads the tensor-memory lane quarter warp % 4) share an
// item's column groups of 8 l round-robin within their quarter.  12 warps in
// all (three per SM sub-partition) leave 168 registers a thread, which the
// epilogue's derivation needs: 12 epilogue warps (16 in all, 128 registers,
// ~100 bytes of spills) took 137 instead of 82 ms for 300 SNPs x 4 000/4 000
// and 173 instead of 166 ms for 400 SNPs x 558/1 012.
constexpr int kT4BuildWarps = 2, kT4EpiWarps = 8;
constexpr int kT4Threads = 32 * (2 + kT4BuildWarps + kT4EpiWarps);
static_assert(kT4EpiWarps % 4 == 0, "epilogue warps cover the four lane quarters evenly");
constexpr int kT4BuildRows = 2 * kT4K / (4 * kT4BuildWarps);          // k rows per builder thread and stage
static_assert(2 * kT4K % (4 * kT4BuildWarps) == 0, "builder threads split the k rows evenly");
constexpr int kT4Stages = 3;
constexpr int kT4SB = kT4N * kT3KB;                 // 32 KB  l rows
constexpr int kT4SA = kT4M * kT3KB;                 // 16 KB  A (k, x, y, z)
constexpr int kT4SK = 2 * kT4K * kT3KB;             //  4 KB  k rows
constexpr int kT4SI = 1024;                         // i rows (2 x 128 B) in a 1 KB slot
constexpr int kT4SJ = 1024;                         // j rows
constexpr int kT4Stage = kT4SB + kT4SA + kT4SK + kT4SI + kT4SJ;  // 54 KB, a multiple of 1 KB
constexpr int kT4Ebuf = 2048;                       // per epilogue warp: 32 combinations x 8 (x,y,z) x 8 B

// Sources of the epilogue that depend on one of k or l only, copied into
// shared memory by the epilogue threads (cp.async: global to shared without
// registers) one item ahead, into two alternating buffers: the triple
// (i, j, l), pair (i, l), (j, l) and single l cores of every l of the item,
// and the triple (i, j, k), pair (i, k), (j, k) and single k cores of every k
// with the pair (i, j) and singles i, j (the prefix star tables follow from
// these in the epilogue).
struct T4Item {
    uint4 tijl[2][kT4L];  // [cases, controls][l]: 16-byte stride across the lanes' l
    uint4 pil[kT4L], pjl[kT4L], sl[kT4L];
    uint4 tijk[2][kT4K];
    uint4 pik[kT4K], pjk[kT4K], sk[kT4K];
    uint4 pij, si, sj;
};
constexpr size_t kT4Smem =
    1024 + (size_t)kT4Stages * kT4Stage + (size_t)kT4EpiWarps * kT4Ebuf + 2 * sizeof(T4Item);
// instruction descriptor: e4m3 x e4m3 -> FP32, M 128, N 256 (packed) or 128 (split)
constexpr uint32_t t4_idesc(int N) { return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kT4M >> 4) << 24); }
static_assert(kT4Smem <= 227 * 1024 - 256, "order-4 tensor kernel shared memory");
static_assert(2 * kT4N <= 512, "order-4 tensor kernel tensor memory");

struct T4Maps {
    CUtensorMap l, k, i;  // boxes of 2 L (256 or 128), 32 and 2 plane rows
};

// Items of one pair (i, j): for k-tiles k0 = j + 1 + 16 a (k0 <= n - 2),
// ceil((n - 1 - k0) / L) l-tiles l0 = k0 + 1 + L b.
inline long long t4_items_per_pair(int n, int j, int L) {
    long long c = 0;
    for (int k0 = j + 1; k0 <= n - 2; k0 += kT4K) c += (n - 1 - k0 + L - 1) / L;
    return c;
}

// Item g -> (i, j, k0, l0).  begin[j]: first item of the pairs with second
// element j (j pairs of per[j] items each).
template <int L>
__device__ __forceinline__ void t4_decode(const long long* __restrict__ begin, const long long* __restrict__ per,
                                          int n, long long g, int& i, int& j, int& k0, int& l0) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(begin + mid) <= g) lo = mid;
        else hi = mid - 1;
    }
    j = lo;
    const long long pj = __ldg(per + j);
    const long long rel = g - __ldg(begin + j);
    i = (int)(rel / pj);
    long long q = rel - (long long)i * pj;
    for (int k = j + 1;; k += kT4K) {
        const long long nl = (n - 1 - k + L - 1) / L;
        if (q < nl) {
            k0 = k;
            l0 = k + 1 + L * (int)q;
            return;
        }
        q -= nl;
    }
}

// Distribution layers of order-4 scans: the owned prefixes (i, j, k) of a pair
// (i, j) are k = kf + step m (their ranks triple_index(i, j, j + 1) + k - j - 1
// step through the layer's offset class), consecutive rows of the operand
// planes ordered by residue mod step.  A layer item is (i, j, 16 owned k from
// kf + 16 step a, L l from that first k + 1); pbegin[p] = first item of listed
// pair p, pinfo[p] = (i, j, kf).
template <int L>
__device__ __forceinline__ void t4l_decode(const long long* __restrict__ pbegin, const int4* __restrict__ pinfo,
                                           int n_pairs, int n, int step, long long g, int& i, int& j, int& k0,
                                           int& l0) {
    int lo = 0, hi = n_pairs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(pbegin + mid) <= g) lo = mid;
        else hi = mid - 1;
    }
    const int4 f = __ldg(pinfo + lo);
    i = f.x;
    j = f.y;
    long long q = g - __ldg(pbegin + lo);
    for (int k = f.z;; k += kT4K * step) {
        const long long nl = (n - 1 - k + L - 1) / L;
        if (q < nl) {
            k0 = k;
            l0 = k + 1 + L * (int)q;
            return;
        }
        q -= nl;
    }
}

// Item g of a scan of the whole data set (t4_decode) or of a layer (t4l_decode).
template <int L, bool LAYER>
__device__ __forceinline__ void t4_item(const long long* __restrict__ begin, const long long* __restrict__ per,
                                        const int4* __restrict__ pinfo, int n_pairs, const ScanWork& w, long long g,
                                        int& i, int& j, int& k0, int& l0) {
    if (LAYER) t4l_decode<L>(begin, pinfo, n_pairs, w.d.snps, w.dist_step, g, i, j, k0, l0);
    else t4_decode<L>(begin, per, w.d.snps, g, i, j, k0, l0);
}

// 8-byte slot of the epilogue transpose buffer holding (cases w0 | w1 << 16,
// controls w0 | w1 << 16) of row (kk, xyz) for the column ll of a group;
// conflict-free for the row-wise writes (fixed ll) and the combination-wise
// reads (fixed xyz): each half-warp covers the 32 banks once.
__device__ __forceinline__ int t4_slot(int kk, int ll, int xyz) { return kk * 64 + (ll ^ (kk & 1)) * 8 + (xyz ^ ll); }

// The cores of one combination that depend on both k and l: triples (i,k,l)
// and (j,k,l) (cases, controls) and pair (k,l), loaded from global memory at
// the start of a column group so that their latency overlaps the
// accumulator reads.
struct T4KL {
    uint4 ikl_c, ikl_t, jkl_c, jkl_t, kl;
};

__device__ __forceinline__ T4KL t4_load_kl(const uint4* __restrict__ pairs, const uint4* __restrict__ triples, int i,
                                           int j, int k, int l, int n) {
    const uint4* tik = triples + 2 * triple_index(i, k, l, n);
    const uint4* tjk = triples + 2 * triple_index(j, k, l, n);
    T4KL v;
    v.ikl_c = __ldg(tik);
    v.ikl_t = __ldg(tik + 1);
    v.jkl_c = __ldg(tjk);
    v.jkl_t = __ldg(tjk + 1);
    v.kl = __ldg(pairs + pair_index(k, l, n));
    return v;
}

// Estimate of the key minus the base in units of 2^-16 bits, cell by cell
// over both classes in one packed derivation (the totals as their sum):
// within t4_margin.  l-only and prefix sources come from the item's
// shared-memory stage, (k, l) sources from registers.
__device__ __forceinline__ long long t4_estimate(const uint32_t (&cp)[2][8], const T4Item& it, int kk, int ll,
                                                 const T4KL& kl, uint32_t nn) {
    E4Both wd;
    wd.tc[0] = it.tijl[0][ll];
    wd.tt[0] = it.tijl[1][ll];
    wd.tc[1] = kl.ikl_c;
    wd.tt[1] = kl.ikl_t;
    wd.tc[2] = kl.jkl_c;
    wd.tt[2] = kl.jkl_t;
    wd.pil = it.pil[ll];
    wd.pjl = it.pjl[ll];
    wd.pkl = kl.kl;
    wd.sl = it.sl[ll];
    E4PrefixStarPacked ps;
    ps.tc = it.tijk[0][kk];
    ps.tt = it.tijk[1][kk];
    ps.pij = it.pij;
    ps.pik = it.pik[kk];
    ps.pjk = it.pjk[kk];
    ps.si = it.si;
    ps.sj = it.sj;
    ps.sk = it.sk[kk];
    ps.nn = nn;
    long long acc = 0;
    e4_slices_packed(cp, wd, ps, [&](int, const uint32_t* t) { acc += e4_slice_estimate_packed(t); });
    return acc;
}

// 16-byte asynchronous copy global -> shared (both addresses 16-byte aligned).
__device__ __forceinline__ void t4_cp16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

// Copies item g's k-only and l-only sources into it (epilogue thread et of
// 256), then commits this thread's copy group.
template <int L, bool LAYER>
__device__ __forceinline__ void t4_stage(T4Item& it, long long g, int et, const long long* __restrict__ begin,
                                         const long long* __restrict__ per, const int4* __restrict__ pinfo,
                                         int n_pairs, const ScanWork& w, const uint32_t* __restrict__ single,
                                         const uint4* __restrict__ pairs, const uint4* __restrict__ triples) {
    const int n = w.d.snps, kstep = LAYER ? w.dist_step : 1;
    int i, j, k0, l0;
    t4_item<L, LAYER>(begin, per, pinfo, n_pairs, w, g, i, j, k0, l0);
    const uint4* single4 = reinterpret_cast<const uint4*>(single);
    if (et < L) {
        const int l = l0 + et;
        if (l < n) {
            const uint4* t = triples + 2 * triple_index(i, j, l, n);
            t4_cp16(&it.tijl[0][et], t);
            t4_cp16(&it.tijl[1][et], t + 1);
            t4_cp16(&it.pil[et], pairs + pair_index(i, l, n));
            t4_cp16(&it.pjl[et], pairs + pair_index(j, l, n));
            t4_cp16(&it.sl[et], single4 + l);
        }
    } else if (et >= kT4L && et < kT4L + kT4K) {
        const int kk = et - kT4L, k = k0 + kstep * kk;
        if (k < n) {
            const uint4* t = triples + 2 * triple_index(i, j, k, n);
            t4_cp16(&it.tijk[0][kk], t);
            t4_cp16(&it.tijk[1][kk], t + 1);
            t4_cp16(&it.pik[kk], pairs + pair_index(i, k, n));
            t4_cp16(&it.pjk[kk], pairs + pair_index(j, k, n));
            t4_cp16(&it.sk[kk], single4 + k);
        }
    } else if (et == kT4L + kT4K) {
        t4_cp16(&it.pij, pairs + pair_index(i, j, n));
        t4_cp16(&it.si, single4 + i);
        t4_cp16(&it.sj, single4 + j);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// Exact key of one combination (and its tables when o): the rare path, kept
// out of line so that its registers do not weigh on the estimate.
__device__ __noinline__ long long t4_exact(const ScanWork& w, const uint32_t (&cp)[2][8], int i, int j, int k, int l,
                                           const uint32_t* __restrict__ single, const uint4* __restrict__ pairs,
                                           const uint4* __restrict__ triples, uint32_t* o) {
    const DevData& d = w.d;
    const int n = d.snps;
    const uint4* single4 = reinterpret_cast<const uint4*>(single);
    E4Src src;
    src.tij = triples + 2 * triple_index(i, j, l, n);
    src.tik = triples + 2 * triple_index(i, k, l, n);
    src.tjk = triples + 2 * triple_index(j, k, l, n);
    src.pil = pairs + pair_index(i, l, n);
    src.pjl = pairs + pair_index(j, l, n);
    src.pkl = pairs + pair_index(k, l, n);
    src.sl = single4 + l;
    E4Prefix pre;
    pre.tijk = triples + 2 * triple_index(i, j, k, n);
    pre.pij = pairs + pair_index(i, j, n);
    pre.pik = pairs + pair_index(i, k, n);
    pre.pjk = pairs + pair_index(j, k, n);
    pre.si = single4 + i;
    pre.sj = single4 + j;
    pre.sk = single4 + k;
    long long key = e4p_pass<0>(cp, src, pre, d.ftab, d.n_cases, o);
    key += e4p_pass<1>(cp, src, pre, d.ftab, d.n_ctrls, o);
    key -= e4p_pass<2>(cp, src, pre, d.ftab, d.n_cases + d.n_ctrls, o);
    return key;
}

template <bool DIGEST>
__device__ __forceinline__ void t4_eval(const ScanWork& w, const CandSink& sink, long long thr_q, uint32_t* dump,
                                        const uint32_t* __restrict__ single, const uint4* __restrict__ pairs,
                                        const uint4* __restrict__ triples, const T4Item& it,
                                        const uint32_t (&cp)[2][8], const T4KL& kl, int i, int j, int kk, int l0,
                                        int k, int l, bool valid, int lane) {
    const DevData& d = w.d;
    const int n = d.snps;
    long long key = w.base_key;
    bool pass = false;
    unsigned long long dg = 0;
    if (valid) {
        bool cand = DIGEST || dump != nullptr;
        if (!cand) {
            const int ll = l - l0;
            const long long est = t4_estimate(cp, it, kk, ll, kl, d.n_cases | d.n_ctrls << 16);
            cand = est >= thr_q;
        }
        if (cand) {
            // owned prefix ordinal of (i, j, k): rank offset + m * step
            const size_t m = (size_t)((triple_index(i, j, k, n) - w.dist_offset) / w.dist_step);
            uint32_t* o = dump ? dump + (m * n + l) * 2 * 81 : nullptr;
            const unsigned gt = blockIdx.x * blockDim.x + threadIdx.x;
            if (DIGEST && gt < sink.dscratch_threads) o = sink.dscratch + (size_t)gt * 2 * 81;
            key += t4_exact(w, cp, i, j, k, l, single, pairs, triples, o);
            pass = key >= sink.thr;
            if (DIGEST) {
                const int cmb[4] = {i, j, k, l};
                dg = o ? dg_table(cmb, 4, n, o, 81) : 0;
            }
        }
    }
    if (DIGEST) dg_warp_add(sink.digest, dg);
    if (sink.evaluated) {
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
        if (lane == 0 && vm) atomicAdd(sink.evaluated, (unsigned long long)__popc(vm));
    }
    const unsigned mask = __ballot_sync(0xffffffffu, pass);
    if (mask) {
        const int leader = __ffs(mask) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(sink.count, (unsigned)__popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (pass) {
            const unsigned idx = base + __popc(mask & ((1u << lane) - 1u));
            if (idx < sink.cap) {
                const int c[4] = {i, j, k, l};
                sink.buf[idx] = Cand{key, pack_code(c, 4, w.bits)};
            } else {
                atomicOr(sink.overflow, 1u);
            }
        }
    }
}

// 16 consecutive accumulator columns of this warp's 32 lanes (one per thread).
__device__ __forceinline__ void t4_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
}

// DIGEST: the digest mode of fiu_scan_digest (every valid combination's tables hashed), compiled
// separately so that the search's instantiation carries none of its code.
// LAYER: a Distribution layer (t4l_decode; maps.k then covers the residue-ordered planes, begin /
// pinfo / n_pairs are the layer's pair tables).
template <bool PACK, bool DIGEST, bool LAYER>
__global__ void __launch_bounds__(kT4Threads, 1)
    tensor4p_kernel(const __grid_constant__ T4Maps maps, ScanWork w, const long long* __restrict__ begin,
                    const long long* __restrict__ per, long long g0, long long g1, int k_cases, int pack,
                    CandSink sink, long long thr_q, uint32_t* dump, const uint32_t* __restrict__ single,
                    const uint4* __restrict__ pairs, const uint4* __restrict__ triples, int* status,
                    const int4* __restrict__ pinfo, int n_pairs) {
    extern __shared__ uint8_t smraw[];
    __shared__ __align__(8) uint64_t full_t[kT4Stages], full_a[kT4Stages], empty[kT4Stages];
    __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2], done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);  // stages: B | A | k | i | j
    uint32_t* ebuf_all = reinterpret_cast<uint32_t*>(sm + kT4Stages * kT4Stage);
    volatile int* abort = &abort_flag;
    const DevData& d = w.d;
    const int n = d.snps;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ks_c = k_cases / kT3KB;
    const int ksteps = ks_c + (d.tw + 1) / 2;
    constexpr int L = PACK ? kT4L : kT4L / 2;                     // l per item
    constexpr int NR = 2 * L;                                       // N of one accumulator region
    constexpr uint32_t kTx = NR * kT3KB + kT4SK + 2 * 2 * kT3KB;  // bytes the TMA brings per stage
    constexpr int NG = L / 8;                                       // column groups of 8 l per item
    constexpr int H = kT4EpiWarps / 4;                              // epilogue warps per lane quarter

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < kT4Stages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_t[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_a[s])), "r"(kT4BuildWarps));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_full[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&acc_empty[b])), "r"(kT4EpiWarps));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;");
        abort_flag = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    bool ok = true;

    if (warp == 0) {
        // ---------------------------------------------------------------- TMA producer
        if (lane == 0) {
            long long step = 0;
            for (long long g = g0 + blockIdx.x; g < g1 && ok; g += gridDim.x) {
                int i, j, k0, l0;
                t4_item<L, LAYER>(begin, per, pinfo, n_pairs, w, g, i, j, k0, l0);
                const int krow = LAYER ? residue_row(k0, w.dist_step, n) : k0;  // first row of the k tile
                for (int ks = 0; ks < ksteps; ++ks) {
                    const int s = (int)(step % kT4Stages);
                    const long long u = step / kT4Stages;
                    if (u > 0 && !t3_wait(smem_u32(&empty[s]), (uint32_t)((u - 1) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    const int kb = ks < ks_c ? ks * kT3KB : k_cases + (ks - ks_c) * kT3KB;
                    uint8_t* st = sm + s * kT4Stage;
                    const uint32_t bar = smem_u32(&full_t[s]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kTx)
                                 : "memory");
                    t3_tma(smem_u32(st), &maps.l, kb, 2 * l0, bar);
                    t3_tma(smem_u32(st + kT4SB + kT4SA), &maps.k, kb, 2 * krow, bar);
                    t3_tma(smem_u32(st + kT4SB + kT4SA + kT4SK), &maps.i, kb, 2 * i, bar);
                    t3_tma(smem_u32(st + kT4SB + kT4SA + kT4SK + kT4SI), &maps.i, kb, 2 * j, bar);
                    ++step;
                }
            }
            for (int s = 0; s < kT4Stages; ++s) {
                if (step <= s) continue;
                const long long last = s + ((step - 1 - s) / kT4Stages) * kT4Stages;
                if (!t3_drain(smem_u32(&full_t[s]), (uint32_t)((last / kT4Stages) & 1))) ok = false;
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0) {
            long long step = 0, item = 0;
            for (long long g = g0 + blockIdx.x; g < g1 && ok; g += gridDim.x, ++item) {
                const int buf = (int)(item & 1);
                if (item >= 2 && !t3_wait(smem_u32(&acc_empty[buf]), (uint32_t)(((item >> 1) - 1) & 1), abort)) {
                    ok = false;
                    break;
                }
                // the MMA costs in proportion to N (from N 64 up): an item whose l run is cut
                // short by the last SNP multiplies only the columns of its valid l, rounded up
                // to 8 l (the epilogue's column groups), N 64 at least
                int ii, jj, kk0, l0;
                t4_item<L, LAYER>(begin, per, pinfo, n_pairs, w, g, ii, jj, kk0, l0);
                const int vl = min(L, n - l0);
                const uint32_t idesc = t4_idesc(min(NR, max(64, (2 * vl + 15) / 16 * 16)));
                for (int ks = 0; ks < ksteps; ++ks, ++step) {
                    // packed: one region of N 256 per buffer; split: cases in the
                    // buffer's first N 128 columns, controls in its second
                    const bool ctrl = !PACK && ks >= ks_c;
                    const uint32_t dcol = tmem + (uint32_t)(kT4N * buf + (ctrl ? NR : 0));
                    const bool first = ks == 0 || (!PACK && ks == ks_c);
                    const int s = (int)(step % kT4Stages);
                    if (!t3_wait(smem_u32(&full_a[s]), (uint32_t)((step / kT4Stages) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t sb = smem_u32(sm + s * kT4Stage), sa = sb + kT4SB;
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const uint64_t ad = t3_desc(sa + 32 * kk), bd = t3_desc(sb + 32 * kk);
                        const uint32_t acc = (first && kk == 0) ? 0u : 1u;
                        asm volatile(
                            "{.reg .pred p; setp.ne.b32 p, %4, 0;\n"
                            "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;}\n" ::"r"(dcol),
                            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                        smem_u32(&empty[s])));
                }
                if (!ok) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    smem_u32(&acc_full[buf])));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&done)));
            if (!t3_drain(smem_u32(&done), 0)) ok = false;
        }
    } else if (warp < 2 + kT4BuildWarps) {
        // ---------------------------------------------------------------- A builders (shared memory)
        const int t = tid - 64;  // 0 .. 32 * kT4BuildWarps - 1
        const int c = t & 7;     // 16-byte chunk; 8 consecutive threads cover one 128-byte row
        long long step = 0;
        for (long long g = g0 + blockIdx.x; g < g1 && ok; g += gridDim.x) {
            for (int ks = 0; ks < ksteps; ++ks, ++step) {
                const int s = (int)(step % kT4Stages);
                if (!t3_wait(smem_u32(&full_t[s]), (uint32_t)((step / kT4Stages) & 1), abort)) {
                    ok = false;
                    break;
                }
                uint8_t* st = sm + s * kT4Stage;
                uint8_t* sA = st + kT4SB;
                const uint8_t* sK = sA + kT4SA;
                const uint8_t* sI = sK + kT4SK;
                const uint8_t* sJ = sI + kT4SI;
                // 128-byte swizzle: chunk c of box row r sits at chunk c ^ (r & 7)
                // every load of the stage first, then the ANDs and stores: the loads
                // overlap instead of waiting one by one behind the stores
                const uint4 i0 = *reinterpret_cast<const uint4*>(sI + (c << 4));
                const uint4 i1 = *reinterpret_cast<const uint4*>(sI + 128 + ((c ^ 1) << 4));
                const uint4 j0 = *reinterpret_cast<const uint4*>(sJ + (c << 4));
                const uint4 j1 = *reinterpret_cast<const uint4*>(sJ + 128 + ((c ^ 1) << 4));
                uint4 kv[kT4BuildRows];
#pragma unroll
                for (int u = 0; u < kT4BuildRows; ++u) {  // k row r = (kk, z)
                    const int r = (t >> 3) + 4 * kT4BuildWarps * u;
                    kv[u] = *reinterpret_cast<const uint4*>(sK + r * 128 + ((c ^ (r & 7)) << 4));
                }
                uint4 ij[4];  // (x, y) = (0,0), (0,1), (1,0), (1,1)
                ij[0] = make_uint4(i0.x & j0.x, i0.y & j0.y, i0.z & j0.z, i0.w & j0.w);
                ij[1] = make_uint4(i0.x & j1.x, i0.y & j1.y, i0.z & j1.z, i0.w & j1.w);
                ij[2] = make_uint4(i1.x & j0.x, i1.y & j0.y, i1.z & j0.z, i1.w & j0.w);
                ij[3] = make_uint4(i1.x & j1.x, i1.y & j1.y, i1.z & j1.z, i1.w & j1.w);
#pragma unroll
                for (int u = 0; u < kT4BuildRows; ++u) {
                    const int r = (t >> 3) + 4 * kT4BuildWarps * u;
                    const int kk = r >> 1, z = r & 1;
#pragma unroll
                    for (int xy = 0; xy < 4; ++xy) {
                        const int m = kk * 8 + xy * 2 + z;  // A row (kk, x, y, z)
                        const uint4 v =
                            make_uint4(ij[xy].x & kv[u].x, ij[xy].y & kv[u].y, ij[xy].z & kv[u].z, ij[xy].w & kv[u].w);
                        *reinterpret_cast<uint4*>(sA + m * 128 + ((c ^ (m & 7)) << 4)) = v;
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_a[s])) : "memory");
            }
        }
    } else {
        // ---------------------------------------------------------------- epilogue
        const int e = warp - (2 + kT4BuildWarps);  // 0 .. kT4EpiWarps - 1
        const int q = warp & 3;                     // tensor-memory lane quarter this warp may access
        const int hh = e >> 2;                      // column groups hh, hh + H, ...: l offsets 8 gi + [0, 8)
        uint32_t* ebuf = ebuf_all + e * (kT4Ebuf / 4);
        const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
        const uint32_t wmask = PACK ? (1u << pack) - 1u : 0xffffffffu;
        const int kkw = lane >> 3, xyz = lane & 7;  // this thread's accumulator row (4 q + kkw, xyz)
        const int kkc = lane >> 3, llc = lane & 7;  // this lane's combination in a column group
        const int et = tid - 32 * (2 + kT4BuildWarps);  // 0 .. 32 kT4EpiWarps - 1
        T4Item* items = reinterpret_cast<T4Item*>(ebuf_all + kT4EpiWarps * (kT4Ebuf / 4));  // two buffers
        long long item = 0;
        if (g0 + blockIdx.x < g1)
            t4_stage<L, LAYER>(items[0], g0 + blockIdx.x, et, begin, per, pinfo, n_pairs, w, single, pairs, triples);
        for (long long g = g0 + blockIdx.x; g < g1 && ok; g += gridDim.x, ++item) {
            int i, j, k0, l0;
            t4_item<L, LAYER>(begin, per, pinfo, n_pairs, w, g, i, j, k0, l0);
            const int buf = (int)(item & 1);
            const int k = k0 + (LAYER ? w.dist_step : 1) * (4 * q + kkc);
            // this thread's copies of the item's sources have landed; the named
            // barrier (the epilogue threads) makes everyone's visible and
            // frees the other buffer (every thread is done with the previous item)
            asm volatile("cp.async.wait_group 0;" ::: "memory");
            asm volatile("bar.sync 1, %0;" ::"n"(32 * kT4EpiWarps) : "memory");
            if (g + gridDim.x < g1)
                t4_stage<L, LAYER>(items[buf ^ 1], g + gridDim.x, et, begin, per, pinfo, n_pairs, w, single, pairs,
                                   triples);
            const T4Item& it = items[buf];
            if (!t3_wait(smem_u32(&acc_full[buf]), (uint32_t)((item >> 1) & 1), abort)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
            for (int gi = hh; gi < NG; gi += H) {
                const int l = l0 + 8 * gi + llc;  // the warps of a quarter interleave
                const bool valid = k < n && l < n && l > k;
                const bool last = gi + H >= NG;  // this warp's last column group of the item
                // a column group without a valid combination in this warp is skipped
                // (its accumulators are never read); the region is still released
                if (!__any_sync(0xffffffffu, valid)) {
                    if (last) {
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0)
                            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[buf]))
                                         : "memory");
                    }
                    continue;
                }
                T4KL kl{};
                if (valid && !dump) kl = t4_load_kl(pairs, triples, i, j, k, l, n);
                {
                    const uint32_t col = (uint32_t)(kT4N * buf + 16 * gi);
                    uint32_t v[16], vt[16];
                    t4_ld16(lane_base + col, v);
                    if (!PACK) t4_ld16(lane_base + col + NR, vt);  // control counts of the same rows / columns
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (last) {  // this warp's last read of the item's accumulators
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0)
                            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[buf]))
                                         : "memory");
                    }
#pragma unroll
                    for (int ll = 0; ll < 8; ++ll) {
                        const uint32_t u0 = __float2uint_rn(__uint_as_float(v[2 * ll]));
                        const uint32_t u1 = __float2uint_rn(__uint_as_float(v[2 * ll + 1]));
                        uint2 c2;
                        if (PACK) {
                            c2 = make_uint2((u0 & wmask) | (u1 & wmask) << 16, (u0 >> pack) | (u1 >> pack) << 16);
                        } else {
                            c2 = make_uint2(u0 | u1 << 16, __float2uint_rn(__uint_as_float(vt[2 * ll])) |
                                                               __float2uint_rn(__uint_as_float(vt[2 * ll + 1])) << 16);
                        }
                        *reinterpret_cast<uint2*>(ebuf + 2 * t4_slot(kkw, ll, xyz)) = c2;
                    }
                }
                __syncwarp();
                uint32_t cp[2][8];
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const uint2 c2 = *reinterpret_cast<const uint2*>(ebuf + 2 * t4_slot(kkc, llc, r));
                    cp[0][r] = c2.x;
                    cp[1][r] = c2.y;
                }
                __syncwarp();
                t4_eval<DIGEST>(w, sink, thr_q, dump, single, pairs, triples, it, cp, kl, i, j, 4 * q + kkc, l0,
                                valid ? k : 2,
                        valid ? l : 3, valid, lane);
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");  // no copy in flight at exit (after an abort)
    }
    if (!ok) *abort = 1;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0 && abort_flag) atomicOr(status, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// Bound (in bits) on |estimate - exact key / (ln2 * 2^32)|, N samples: each
// sample lies in exactly one of the 81 cells, so sum (a+b) over the cells is
// N and sum (a+b) lg2 (a+b) <= N lg2 N.  Per cell the three products and two
// additions of g round at most 5 times by 2^-24 of at most (a+b) lg2 (a+b);
// lg2.approx is within 2^-18 of log2 on every input the kernel can see
// (checked exhaustively by fiu_probe_lg2_error), which moves g by at most
// 2 (a+b) 2^-18; the c + 2^-20 shift moves each of the 243 products by at
// most 2^-20 / ln 2 and its rounding each logarithm by at most 2^-24 / ln 2;
// a 27-term pairwise sum rounds 5 times by 2^-24 of at most sum |g| <= N;
// each of the 3 slice sums rounds by 2^-17 in fixed point; the integer table
// rounds each of the 243 exact terms by 1/2 of 2^-32 nats.  Doubled.
double t4_margin(int n_samples) {
    const double N = n_samples, lgN = std::log2(std::max(2.0, N));
    const double u = std::ldexp(1.0, -24), e20 = std::ldexp(1.0, -20), e_lg2 = std::ldexp(1.0, -18);
    const double T = 243;
    const double err = 5 * u * N * lgN + 2 * N * e_lg2 + T * e20 / std::log(2.0) + 2 * N * u / std::log(2.0) +
                       5 * u * N + 3 * std::ldexp(1.0, -17) + T * 0.5 / (std::log(2.0) * 4294967296.0);
    return 2 * err + 1e-3;
}

std::vector<long long> t4_item_table(int n, bool pack, std::vector<long long>& per) {
    std::vector<long long> begin((size_t)n + 1, 0);
    per.assign((size_t)std::max(n, 1), 0);
    for (int j = 0; j < n; ++j) {
        per[j] = t4_items_per_pair(n, j, pack ? kT4L : kT4L / 2);
        begin[j + 1] = begin[j] + (long long)j * per[j];
    }
    return begin;
}

// Pair tables of a Distribution layer of an order-4 scan (host): the listed pairs (i, j) with at
// least one item, their first owned k and first item.  Returns the items; combos = combinations.
long long t4_layer_items(int n, int step, long long offset, bool pack, std::vector<long long>& pbegin,
                         std::vector<int4>& pinfo, long long& combos) {
    const int L = pack ? kT4L : kT4L / 2;
    pbegin.clear();
    pinfo.clear();
    combos = 0;
    long long total = 0;
    for (int i = 0; i + 3 < n; ++i)
        for (int j = i + 1; j + 2 < n; ++j) {
            const long long base = triple_index(i, j, j + 1, n), cnt = n - 1 - j;  // ranks base .. base + cnt - 1
            long long t = std::max(0ll, offset - base);
            t += ((offset - base - t) % step + step) % step;  // first t with base + t = offset (mod step)
            if (t >= cnt) continue;
            const int kf = j + 1 + (int)t;
            long long items = 0;
            for (long long k = kf; k <= n - 2; k += (long long)kT4K * step) items += (n - 1 - k + L - 1) / L;
            for (long long k = kf; k < n; k += step) combos += n - 1 - k;
            if (items == 0) continue;
            pbegin.push_back(total);
            pinfo.push_back(make_int4(i, j, kf, 0));
            total += items;
        }
    pbegin.push_back(total);
    return total;
}

cudaError_t launch_tensor4(const ScanWork& w, const CUtensorMap& map_l256, const CUtensorMap& map_l128,
                           const CUtensorMap& map_k, const CUtensorMap& map_i, const long long* begin,
                           const long long* per, int k_cases, int pack, long long g0, long long g1,
                           const CandSink& sink, uint32_t* dump, const uint32_t* single, const uint4* pairs,
                           const uint4* triples, int* status, cudaStream_t s, int sms, const int4* pinfo,
                           int n_pairs) {
    const bool layer = pinfo != nullptr;
    if (!triples || !pairs || !single || !begin || (!per && !layer)) return cudaErrorInvalidValue;
    static LaunchCache cache[8];
    const bool dg = sink.digest != nullptr;
    using Fn = decltype(&tensor4p_kernel<true, true, true>);
    static const Fn fns[8] = {tensor4p_kernel<false, false, false>, tensor4p_kernel<false, true, false>,
                              tensor4p_kernel<true, false, false>,  tensor4p_kernel<true, true, false>,
                              tensor4p_kernel<false, false, true>,  tensor4p_kernel<false, true, true>,
                              tensor4p_kernel<true, false, true>,   tensor4p_kernel<true, true, true>};
    const int v = (layer ? 4 : 0) + (pack ? 2 : 0) + (dg ? 1 : 0);
    const Fn fn = fns[v];
    int per_sm = 1;
    cudaError_t e = blocks_per_sm(cache[v], fn, kT4Threads, kT4Smem, per_sm);
    if (e != cudaSuccess) return e;
    const long long items = g1 - g0;
    if (items <= 0) return cudaSuccess;
    // threshold of the estimate in units of 2^-16 bits
    const double scale = 65536.0 / (std::log(2.0) * 4294967296.0);
    const double thr = ((double)sink.thr - (double)w.base_key) * scale - t4_margin(w.d.n_cases + w.d.n_ctrls) * 65536.0;
    const long long thr_q = (long long)std::floor(std::max(-9.0e18, std::min(9.0e18, thr)));
    const unsigned grid = (unsigned)(items < sms ? items : sms);
    const T4Maps maps{pack ? map_l256 : map_l128, map_k, map_i};
    fn<<<grid, kT4Threads, kT4Smem, s>>>(maps, w, begin, per, g0, g1, k_cases, pack, sink, thr_q, dump, single, pairs,
                                         triples, status, pinfo, n_pairs);
    count_launch();
    return cudaGetLastError();
}

}  // namespace fiu
