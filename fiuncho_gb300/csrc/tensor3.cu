// Order-3 and order-2 contingency tables on the 5th-generation tensor cores
// (tcgen05).  Kernels: tensor3x_kernel (order 3, classes that pack into one
// accumulator, CTA pairs), tensor3_kernel (order 3, one accumulator per
// class, described first below), tensor2x_kernel (order 2, classes that
// pack, CTA pairs) and tensor2_kernel (order 2, per class).
//
// For one-hot data the 8 core cells of a combination (i, j, l) -- genotypes
// x, y, z in {0, 1} -- are dot products over the samples of one class:
//     core[x][y][z] = sum_s a_ix(s) a_jy(s) a_lz(s),
// where a_gx(s) is 1 when sample s has genotype x at SNP g.  A work item is
// (i, 32 consecutive j, 96 consecutive l); per class it is one GEMM
//     D[(j,x,y), (l,z)] = sum_s A[(j,x,y), s] B[(l,z), s]    (M 128, N 192),
// accumulated exactly in FP32 in tensor memory.
//
// Operands.  Each data set is expanded once into e4m3 operand planes in HBM:
// row 2*snp+g holds 0x38 (1.0) where the sample has genotype g, else 0; cases
// then controls, each class padded to a multiple of 128 samples.  B rows are
// plane rows 2l+z, loaded by TMA with 128-byte swizzle straight into the
// layout tcgen05 reads (K-major, SWIZZLE_128B descriptor).  A rows are the
// bytewise AND of the i and j plane rows (0x38 & 0x38 = 0x38): four producer
// warps read the TMA-staged j and i rows from shared memory, AND them in
// registers and write the result to tensor memory (tcgen05.st; one thread per
// row, 4 e4m3 per 32-bit column), where the MMA reads A from (the [a-tmem]
// form of tcgen05.mma): A never touches shared memory, whose bandwidth is the
// kernel's bound.
//
// Warp roles (448 threads, one CTA per SM): warp 0 issues the TMA copies,
// warp 1 issues tcgen05.mma (kind::f8f6f4, K 32 per instruction, 4 per
// 128-sample stage) and commits, warps 2-5 build A, warps 6-13 run the
// epilogue.  Four stages are handed over with mbarriers.  Tensor memory
// (512 columns): case accumulators in columns 0-191, control accumulators in
// 192-383, the A ring (4 stages x 32 columns) in 384-511.  As soon as an
// item's case GEMM is done the epilogue packs its counts to 16 bits in shared
// memory and frees columns 0-191, so the next item's case GEMM overlaps the
// current item's epilogue.
//
// Epilogue.  Each thread reads the accumulators of one row (j, x, y); a
// swizzled shared-memory transpose gives each thread the 16 core counts of one
// combination.  The full 27-cell tables are derived exactly from the pair and
// single cores (inclusion-exclusion, as the CUDA-core reduced-work kernel
// does).  A single-precision estimate of the fixed-point MI key (lg2.approx)
// with a proven error bound rejects the combinations that cannot reach the
// current threshold; the others get the exact 64-bit fixed-point key from the
// integer c*ln(c) table, so the kept set is exactly the one of the exact key.
//
// Reference semantics: GenotypeTable::combine_and_popcnt for order 3
// (src/base/gt_popcnt.cpp:4-35) and MutualInformation::compute
// (src/base/mi_compute.cpp:16-41) over the combinations ThreadedSearch
// visits (include/fiuncho/ThreadedSearch.h:157-180) with one worker.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <mutex>

#include "tensor_common.cuh"

namespace fiu {

constexpr int kT3J = 32, kT3L = 96;              // SNPs per tile
constexpr int kT3M = 4 * kT3J, kT3N = 2 * kT3L;  // 128 x 192 GEMM tile
constexpr int kT3Stages = 4;
constexpr int kT3SB = kT3N * kT3KB;              // 24 KB  l rows (1 KB multiple)
constexpr int kT3SJ = 2 * kT3J * kT3KB;          //  8 KB  staged j rows
constexpr int kT3SI = 1024;                      // i rows of a stage (2 x 128 B, 128-byte swizzle: the two
                                                 // rows' chunk c sit in different banks)
constexpr int kT3EpiWarps = 8, kT3BuildWarps = 4;
constexpr int kT3Threads = 32 * (2 + kT3BuildWarps + kT3EpiWarps);  // 448
constexpr int kT3Ebuf = 2048;                    // per epilogue warp: 256 transpose slots of 8 B
constexpr int kT3Stash = 32 * (kT3L / 2) * 4;    // per epilogue warp: 32 rows x 48 words (16-bit case pairs)
constexpr size_t kT3Smem = 1024 + (size_t)kT3Stages * (kT3SB + kT3SJ + kT3SI) +
                           (size_t)kT3EpiWarps * (kT3Ebuf + kT3Stash);
constexpr int kT3ColCtrl = kT3N, kT3ColA = 2 * kT3N;  // tensor-memory column bases
constexpr uint32_t kT3Idesc = (1u << 4) | ((uint32_t)(kT3N >> 3) << 17) | ((uint32_t)(kT3M >> 4) << 24);

static_assert(kT3Smem <= 227 * 1024 - 256, "tensor kernel shared memory");
static_assert(kT3ColA + 32 * kT3Stages <= 512, "tensor memory columns");

// Work items of one i: J-tile a starts at j0 = i+1+32a and has
// ceil((n-1-j0)/L) L-tiles starting at l0 = j0+1+L*b.
template <int L>
__device__ __forceinline__ void t3_decode(const long long* __restrict__ item_begin, int n, long long g, int& i,
                                          int& j0, int& l0) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (item_begin[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    i = lo;
    long long q = g - item_begin[i];
    for (int a = 0;; ++a) {
        const int j = i + 1 + kT3J * a;
        const long long nl = (n - 1 - j + L - 1) / L;
        if (q < nl) {
            j0 = j;
            l0 = j + 1 + L * (int)q;
            return;
        }
        q -= nl;
    }
}

// List mode (a Distribution layer): the owned j of each i are listed in
// jlist[jl_begin[i] .. jl_begin[i+1]); an item takes J consecutive entries
// from p0 (= jl_begin[i] + J a) and an l-tile l0 = jlist[p0] + 1 + L b.
template <int J, int L>
__device__ __forceinline__ void t3l_decode(const long long* __restrict__ item_begin,
                                           const long long* __restrict__ jl_begin, const int* __restrict__ jlist,
                                           int n, long long g, int& i, long long& p0, int& l0) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (item_begin[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    i = lo;
    long long q = g - item_begin[i];
    for (long long p = jl_begin[i];; p += J) {
        const int jf = jlist[p];
        const long long nl = (n - 1 - jf + L - 1) / L;
        if (q < nl) {
            p0 = p;
            l0 = jf + 1 + L * (int)q;
            return;
        }
        q -= nl;
    }
}

// The j of row jj (0..31) of a CTA's 32 j of an item: j0 + jj, or in list mode
// the listed entry p0 + jj (n when the list of i ends before it).
template <bool LIST>
__device__ __forceinline__ int t3x_j(int j0, long long p0, long long p_end, const int* __restrict__ jlist, int jj,
                                     int n) {
    if (!LIST) return j0 + jj;
    const long long p = p0 + jj;
    return p < p_end ? __ldg(jlist + p) : n;
}

// 8-byte slot of the order-3 epilogue transpose buffer holding the counts
// (cases z0 | z1 << 16, controls z0 | z1 << 16) of row (jl, xy) and column
// group k; the XOR makes both the row-wise writes (lanes (jl, xy), fixed k)
// and the combination-wise reads (lanes (jl, k / 2), fixed xy) cover the 32
// banks once per half-warp.
__device__ __forceinline__ int t3_slot(int jl, int k, int xy) {
    return ((jl * 8 + k) * 4 + xy) ^ ((jl & 3) | (((jl ^ (k >> 1)) & 3) << 2));
}

// Float view of the packed 16-bit pair cores [class][x][y].
__device__ __forceinline__ float pcf(const uint4& v, int k) {
    const uint32_t w = (&v.x)[k >> 1];
    return u2f((k & 1) ? (w >> 16) : (w & 0xffffu));
}

// Full 27-cell table of one class in single precision (every value an exact
// integer), the derivation of expand3: core[(x*2+y)*2+z], pair cores of
// (i,j), (i,l), (j,l), singles of i, j, l, class size.
__device__ __forceinline__ void expand3f(const float* core, const uint4& pij, const uint4& pil, const uint4& pjl,
                                         const float* si, const float* sj, const float* sl, float ncls, int cls,
                                         float* t) {
    const int o = 4 * cls;
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
            t[(x * 3 + y) * 3 + 0] = core[(x * 2 + y) * 2 + 0];
            t[(x * 3 + y) * 3 + 1] = core[(x * 2 + y) * 2 + 1];
            t[(x * 3 + y) * 3 + 2] = pcf(pij, o + x * 2 + y);
        }
#pragma unroll
    for (int x = 0; x < 2; ++x) {
#pragma unroll
        for (int z = 0; z < 2; ++z) t[(x * 3 + 2) * 3 + z] = pcf(pil, o + x * 2 + z);
        t[(x * 3 + 2) * 3 + 2] = si[x];
    }
#pragma unroll
    for (int y = 0; y < 2; ++y) {
#pragma unroll
        for (int z = 0; z < 2; ++z) t[(2 * 3 + y) * 3 + z] = pcf(pjl, o + y * 2 + z);
        t[(2 * 3 + y) * 3 + 2] = sj[y];
    }
    t[24] = sl[0];
    t[25] = sl[1];
    t[26] = ncls;
#pragma unroll
    for (int xy = 0; xy < 9; ++xy) t[xy * 3 + 2] -= t[xy * 3 + 0] + t[xy * 3 + 1];
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int z = 0; z < 3; ++z) t[(x * 3 + 2) * 3 + z] -= t[(x * 3 + 0) * 3 + z] + t[(x * 3 + 1) * 3 + z];
#pragma unroll
    for (int yz = 0; yz < 9; ++yz) t[18 + yz] -= t[yz] + t[9 + yz];
}

// Evaluates combination (i, j, l) whose 16 core counts (cases z0, z1, controls z0, z1 of each
// (x, y)) sit in column group k of this warp's transpose buffer: exact 27-cell tables, the
// bounded single-precision prefilter, the exact fixed-point key for survivors, and the
// warp-aggregated append of candidates (warp-synchronous: every lane calls it).
// When stage is given it holds the item's pair cores (i, l0 + ll) at [ll] and
// single cores of l0 + ll at [128 + ll] (shared memory).
__device__ __forceinline__ void t3_eval(const ScanWork& w, const CandSink& sink, float thr_f, uint32_t* dump,
                                        const uint32_t* __restrict__ single, const uint4* __restrict__ pairs,
                                        const uint32_t* ebuf, int jl, int k, int i, int j, int l, bool j_ok,
                                        const uint4& pij, const float (&si)[2][2], const float (&sj)[2][2],
                                        int lane, const uint4* stage = nullptr, int l0 = 0) {
    const DevData& d = w.d;
    const int n = d.snps;
    const uint32_t ncls[2] = {(uint32_t)d.n_cases, (uint32_t)d.n_ctrls};
    const float ncf[2] = {(float)d.n_cases, (float)d.n_ctrls};
    const float tiny = 9.5367431640625e-07f;  // 2^-20: x*lg2(x + tiny) = 0 at x = 0
    const bool valid = j_ok && l < n && l > j;
    float core[2][8];
#pragma unroll
    for (int x4 = 0; x4 < 4; ++x4) {
        const uint2 c2 = *reinterpret_cast<const uint2*>(ebuf + 2 * t3_slot(jl, k, x4));
        core[0][2 * x4] = u2f(c2.x & 0xffffu);
        core[0][2 * x4 + 1] = u2f(c2.x >> 16);
        core[1][2 * x4] = u2f(c2.y & 0xffffu);
        core[1][2 * x4 + 1] = u2f(c2.y >> 16);
    }
    uint4 pil = make_uint4(0, 0, 0, 0), pjl = pil, sl4 = pil;
    if (valid) {
        pjl = __ldg(pairs + pair_index(j, l, n));
        if (stage) {
            pil = stage[l - l0];
            sl4 = stage[128 + l - l0];
        } else {
            pil = __ldg(pairs + pair_index(i, l, n));
            sl4 = __ldg(reinterpret_cast<const uint4*>(single) + l);
        }
    }
    const float sl[2][2] = {{u2f(sl4.x), u2f(sl4.y)}, {u2f(sl4.z), u2f(sl4.w)}};
    float t[2][27];
#pragma unroll
    for (int cls = 0; cls < 2; ++cls)
        expand3f(core[cls], pij, pil, pjl, si[cls], sj[cls], sl[cls], ncf[cls], cls, t[cls]);
    // single-precision estimate of sum over cells of T[a] + T[b] - T[a+b], in units of ln2 * 2^32
    float kf = 0.f;
#pragma unroll
    for (int c = 0; c < 27; ++c) {
        const float a = t[0][c], bb = t[1][c], s = a + bb;
        kf = fmaf(a, t3_lg2(a + tiny), kf);
        kf = fmaf(bb, t3_lg2(bb + tiny), kf);
        kf = fmaf(-s, t3_lg2(s + tiny), kf);
    }
    const bool cand = valid && (dump != nullptr || sink.digest != nullptr || kf >= thr_f);
    long long key = w.base_key;
    bool pass = false;
    unsigned long long dg = 0;
    if (cand) {
#pragma unroll
        for (int c = 0; c < 27; ++c) {
            const uint32_t a = min(f2u(fmaxf(t[0][c], 0.f)), ncls[0]);
            const uint32_t bb = min(f2u(fmaxf(t[1][c], 0.f)), ncls[1]);
            key += __ldg(d.ftab + a) + __ldg(d.ftab + bb) - __ldg(d.ftab + a + bb);
        }
        pass = key >= sink.thr;
        if (dump) {
            // owned prefix ordinal m of (i, j): rank offset + m * step
            const size_t m = (size_t)((pair_index(i, j, n) - w.dist_offset) / w.dist_step);
            uint32_t* o = dump + (m * n + l) * 54;
#pragma unroll
            for (int c = 0; c < 27; ++c) {
                o[c] = f2u(t[0][c]);
                o[27 + c] = f2u(t[1][c]);
            }
        }
        if (sink.digest) {
            const int cmb[3] = {i, j, l};
            dg = dg_begin(cmb, 3, n);
#pragma unroll
            for (int c = 0; c < 27; ++c) dg = dg_cell(dg, f2u(t[0][c]), f2u(t[1][c]));
        }
    }
    if (sink.digest) dg_warp_add(sink.digest, dg);
    if (sink.evaluated) {
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        if (lane == 0 && vmask) atomicAdd(sink.evaluated, (unsigned long long)__popc(vmask));
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
                const int cmb[3] = {i, j, l};
                sink.buf[idx] = Cand{key, pack_code(cmb, 3, w.bits)};
            } else {
                atomicOr(sink.overflow, 1u);
            }
        }
    }
}

// Per-item constants of one j: the pair cores of (i, j) and the single cores of i and j as floats.
__device__ __forceinline__ void t3_item_consts(const uint32_t* __restrict__ single, const uint4* __restrict__ pairs,
                                               int i, int j, int n, bool j_ok, uint4& pij, float (&si)[2][2],
                                               float (&sj)[2][2]) {
    const uint4 a = __ldg(reinterpret_cast<const uint4*>(single) + i);
    uint4 b = make_uint4(0, 0, 0, 0);
    pij = make_uint4(0, 0, 0, 0);
    if (j_ok) {
        b = __ldg(reinterpret_cast<const uint4*>(single) + j);
        pij = __ldg(pairs + pair_index(i, j, n));
    }
    si[0][0] = u2f(a.x);
    si[0][1] = u2f(a.y);
    si[1][0] = u2f(a.z);
    si[1][1] = u2f(a.w);
    sj[0][0] = u2f(b.x);
    sj[0][1] = u2f(b.y);
    sj[1][0] = u2f(b.z);
    sj[1][1] = u2f(b.w);
}

struct T3Maps {
    CUtensorMap l, j, i;
};

// LIST: a Distribution layer (t3l_decode; maps.j covers the residue-ordered planes, where the
// listed j of one i are consecutive rows).
template <bool LIST>
__global__ void __launch_bounds__(kT3Threads, 1)
    tensor3_kernel(const __grid_constant__ T3Maps maps, ScanWork w, const long long* __restrict__ item_begin,
                   long long g0, long long g1, int k_cases, CandSink sink, float thr_f, uint32_t* dump,
                   const uint32_t* __restrict__ single, const uint4* __restrict__ pairs, int* status,
                   const long long* __restrict__ jl_begin, const int* __restrict__ jlist) {
    extern __shared__ uint8_t smraw[];
    __shared__ __align__(8) uint64_t full_t[kT3Stages], full_a[kT3Stages], empty[kT3Stages];
    __shared__ __align__(8) uint64_t case_full, case_empty, ctrl_full, ctrl_empty, done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);  // B ring
    uint8_t* sj_base = sm + kT3Stages * kT3SB;                                 // j ring
    uint8_t* si_base = sj_base + kT3Stages * kT3SJ;                            // i ring
    uint32_t* ebuf_all = reinterpret_cast<uint32_t*>(si_base + kT3Stages * kT3SI);
    uint4* stash_all = reinterpret_cast<uint4*>(ebuf_all + kT3EpiWarps * (kT3Ebuf / 4));
    volatile int* abort = &abort_flag;
    const DevData& d = w.d;
    const int n = d.snps;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ks_c = k_cases / kT3KB;     // 128-sample steps of the case class
    const int ks_t = (d.tw + 1) / 2;      // ... of the control class
    const int ksteps = ks_c + ks_t;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < kT3Stages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_t[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_a[s])), "r"(kT3BuildWarps));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&case_full)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&case_empty)), "r"(kT3EpiWarps));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&ctrl_full)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&ctrl_empty)), "r"(kT3EpiWarps));
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
                int i, j0, l0;  // LIST: j0 = the first listed j's row in the residue-ordered planes
                if (LIST) {
                    long long p0;
                    t3l_decode<kT3J, kT3L>(item_begin, jl_begin, jlist, n, g, i, p0, l0);
                    j0 = residue_row(jlist[p0], w.dist_step, n);
                } else {
                    t3_decode<kT3L>(item_begin, n, g, i, j0, l0);
                }
                for (int ks = 0; ks < ksteps; ++ks) {
                    const int s = (int)(step % kT3Stages);
                    const long long u = step / kT3Stages;
                    if (u > 0 && !t3_wait(smem_u32(&empty[s]), (uint32_t)((u - 1) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    const int k0 = ks < ks_c ? ks * kT3KB : k_cases + (ks - ks_c) * kT3KB;
                    const uint32_t bar = smem_u32(&full_t[s]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                                 "r"((uint32_t)(kT3SB + kT3SJ + 2 * kT3KB))
                                 : "memory");
                    t3_tma(smem_u32(sm + s * kT3SB), &maps.l, k0, 2 * l0, bar);
                    t3_tma(smem_u32(sj_base + s * kT3SJ), &maps.j, k0, 2 * j0, bar);
                    t3_tma(smem_u32(si_base + s * kT3SI), &maps.i, k0, 2 * i, bar);
                    ++step;
                }
            }
            // no copy may be in flight when the CTA exits: wait for the last use of every stage
            for (int s = 0; s < kT3Stages; ++s) {
                if (step <= s) continue;
                const long long last = s + ((step - 1 - s) / kT3Stages) * kT3Stages;
                if (!t3_drain(smem_u32(&full_t[s]), (uint32_t)((last / kT3Stages) & 1))) ok = false;
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0) {
            long long step = 0, item = 0;
            for (long long g = g0 + blockIdx.x; g < g1 && ok; g += gridDim.x, ++item) {
                for (int ks = 0; ks < ksteps; ++ks, ++step) {
                    const int cls = ks >= ks_c;
                    if (item > 0 && (ks == 0 || ks == ks_c)) {  // accumulator columns free again?
                        if (!t3_wait(smem_u32(cls ? &ctrl_empty : &case_empty), (uint32_t)((item - 1) & 1), abort)) {
                            ok = false;
                            break;
                        }
                    }
                    const int s = (int)(step % kT3Stages);
                    if (!t3_wait(smem_u32(&full_a[s]), (uint32_t)((step / kT3Stages) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t sb = smem_u32(sm + s * kT3SB);
                    const uint32_t acol = tmem + (uint32_t)(kT3ColA + 32 * s);
                    const uint32_t dcol = tmem + (cls ? (uint32_t)kT3ColCtrl : 0u);
                    const bool first = ks == 0 || ks == ks_c;
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {  // A: 8 columns (32 e4m3) per instruction
                        const uint64_t bd = t3_desc(sb + 32 * kk);
                        const uint32_t acc = (first && kk == 0) ? 0u : 1u;
                        asm volatile(
                            "{.reg .pred p; setp.ne.b32 p, %4, 0;\n"
                            "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [%1], %2, %3, p;}\n" ::"r"(dcol),
                            "r"(acol + 8 * kk), "l"(bd), "r"(kT3Idesc), "r"(acc));
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                        smem_u32(&empty[s])));
                    if (ks == ks_c - 1 || ks == ksteps - 1)
                        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                            smem_u32(ks == ks_c - 1 ? &case_full : &ctrl_full)));
                }
            }
            // every MMA of this thread complete before the tensor memory is released
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&done)));
            if (!t3_drain(smem_u32(&done), 0)) ok = false;
        }
    } else if (warp < 2 + kT3BuildWarps) {
        // ---------------------------------------------------------------- A builders
        // thread = tensor-memory lane = A row m = (jj, x, y) of this warp's lane quarter
        const int m = 32 * (warp & 3) + lane;
        const int r = 2 * (m >> 2) + (m & 1), x = (m >> 1) & 1;  // staged j row (jj, y), i row x
        const uint32_t a_lane = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)kT3ColA;
        long long step = 0;
        for (long long g = g0 + blockIdx.x; g < g1 && ok; g += gridDim.x) {
            for (int ks = 0; ks < ksteps; ++ks, ++step) {
                const int s = (int)(step % kT3Stages);
                if (!t3_wait(smem_u32(&full_t[s]), (uint32_t)((step / kT3Stages) & 1), abort)) {
                    ok = false;
                    break;
                }
                const uint8_t* sJ = sj_base + s * kT3SJ + r * 128;
                const uint8_t* sI = si_base + s * kT3SI + x * 128;
                uint32_t a[32];
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const uint4 jv = *reinterpret_cast<const uint4*>(sJ + ((c ^ (r & 7)) << 4));
                    const uint4 iv = *reinterpret_cast<const uint4*>(sI + ((c ^ x) << 4));
                    a[4 * c + 0] = jv.x & iv.x;
                    a[4 * c + 1] = jv.y & iv.y;
                    a[4 * c + 2] = jv.z & iv.z;
                    a[4 * c + 3] = jv.w & iv.w;
                }
                // slot s of the A ring is free: the TMA of this step waited for the MMAs of its last use
                asm volatile(
                    "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%"
                    "16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(a_lane +
                                                                                               (uint32_t)(32 * s)),
                    "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]),
                    "r"(a[9]), "r"(a[10]), "r"(a[11]), "r"(a[12]), "r"(a[13]), "r"(a[14]), "r"(a[15]), "r"(a[16]),
                    "r"(a[17]), "r"(a[18]), "r"(a[19]), "r"(a[20]), "r"(a[21]), "r"(a[22]), "r"(a[23]), "r"(a[24]),
                    "r"(a[25]), "r"(a[26]), "r"(a[27]), "r"(a[28]), "r"(a[29]), "r"(a[30]), "r"(a[31]));
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                asm volatile("tcgen05.fence::before_thread_sync;");
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_a[s])) : "memory");
            }
        }
    } else {
        // ---------------------------------------------------------------- epilogue
        const int e = warp - (2 + kT3BuildWarps);  // 0..7
        const int q = warp & 3;                    // tensor-memory lane quarter this warp may access
        const int hh = e >> 2;                     // column groups 2 cc + hh: l offsets 16 cc + 8 hh + [0, 8)
        uint32_t* ebuf = ebuf_all + e * (kT3Ebuf / 4);
        uint4* stash = stash_all + e * (kT3Stash / 16);  // [word quad][lane]: conflict-free
        const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
        // row (writer) view: jl = lane/4, xy = lane%4; combination (reader) view: jl = lane/4, kp = lane%4
        const int jl = lane >> 2, xy = lane & 3, kp = lane & 3;
        long long item = 0;
        for (long long g = g0 + blockIdx.x; g < g1 && ok; g += gridDim.x, ++item) {
            int i, j0 = 0, l0;
            long long p0 = 0, p_end = 0;
            if (LIST) {
                t3l_decode<kT3J, kT3L>(item_begin, jl_begin, jlist, n, g, i, p0, l0);
                p_end = jl_begin[i + 1];
            } else {
                t3_decode<kT3L>(item_begin, n, g, i, j0, l0);
            }
            // ---- phase 1: case counts -> 16-bit stash, case columns free for the next item
            if (!t3_wait(smem_u32(&case_full), (uint32_t)(item & 1), abort)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
            for (int cc = 0; cc < 6; ++cc) {
                const uint32_t col = (uint32_t)(32 * cc + 16 * hh);
                uint32_t v[16], p[8];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15])
                    : "r"(lane_base + col));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    p[k] = f2u(__uint_as_float(v[2 * k])) | (f2u(__uint_as_float(v[2 * k + 1])) << 16);
                stash[(2 * cc) * 32 + lane] = make_uint4(p[0], p[1], p[2], p[3]);
                stash[(2 * cc + 1) * 32 + lane] = make_uint4(p[4], p[5], p[6], p[7]);
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&case_empty)) : "memory");
            // ---- per-item constants of this thread's j
            const int j = t3x_j<LIST>(j0, p0, p_end, jlist, 8 * q + jl, n);
            const bool j_ok = j < n;
            uint4 pij;
            float si[2][2], sj[2][2];
            t3_item_consts(single, pairs, i, j, n, j_ok, pij, si, sj);
            // ---- phase 2: control counts + stash -> transpose -> tables -> keys
            if (!t3_wait(smem_u32(&ctrl_full), (uint32_t)(item & 1), abort)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
            for (int cc = 0; cc < 6; ++cc) {
                // a group without a valid combination for this warp is skipped (the two warps
                // of a lane quarter interleave over the l range); the columns are still released
                const int lg = l0 + 16 * cc + 8 * hh;
                if (!__any_sync(0xffffffffu, j_ok && lg + 7 > j && lg < n)) {
                    if (cc == 5) {
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0)
                            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&ctrl_empty))
                                         : "memory");
                    }
                    continue;
                }
                {
                    const uint32_t col = (uint32_t)(32 * cc + 16 * hh);
                    uint32_t vt[16];
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%"
                        "15}, [%16];"
                        : "=r"(vt[0]), "=r"(vt[1]), "=r"(vt[2]), "=r"(vt[3]), "=r"(vt[4]), "=r"(vt[5]), "=r"(vt[6]),
                          "=r"(vt[7]), "=r"(vt[8]), "=r"(vt[9]), "=r"(vt[10]), "=r"(vt[11]), "=r"(vt[12]),
                          "=r"(vt[13]), "=r"(vt[14]), "=r"(vt[15])
                        : "r"(lane_base + (uint32_t)kT3ColCtrl + col));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    const uint4 s0 = stash[(2 * cc) * 32 + lane], s1 = stash[(2 * cc + 1) * 32 + lane];
                    const uint32_t su[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
                    if (cc == 5) {  // last read of this item's accumulators: control columns free
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0)
                            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&ctrl_empty))
                                         : "memory");
                    }
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const uint32_t t0 = f2u(__uint_as_float(vt[2 * k]));
                        const uint32_t t1 = f2u(__uint_as_float(vt[2 * k + 1]));
                        *reinterpret_cast<uint2*>(ebuf + 2 * t3_slot(jl, k, xy)) = make_uint2(su[k], t0 | t1 << 16);
                    }
                }
                __syncwarp();
#pragma unroll 1
                for (int b = 0; b < 2; ++b)
                    t3_eval(w, sink, thr_f, dump, single, pairs, ebuf, jl, 2 * kp + b, i, j, lg + 2 * kp + b, j_ok,
                            pij, si, sj, lane);
                __syncwarp();
            }
        }
    }
    if (!ok) *abort = 1;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0 && abort_flag) atomicOr(status, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// ---------------------------------------------------------------------------
// Packed classes.  When both classes fit one FP32 accumulator -- control
// samples weighted by W = 4^h: the operand planes hold 2^h instead of 1.0 in
// the control region, every control product is 2^h * 2^h = W, and an
// accumulator holds cases + W * controls, exact while n_cases < W and
// n_cases + W * n_ctrls < 2^24 -- an item needs one tensor-memory region of
// N columns instead of two.  N = 256 (128 l per item; the MMA costs the same
// for every N up to 256) and two regions alternate between items, so the next
// item's GEMM runs while the epilogue reads the last one.  A is built in
// shared memory (tensor memory is full) by six producer warps.
constexpr int kPL = 128, kPN = 2 * kPL;                  // 128 l, N 256
constexpr int kPBuildWarps = 6;                           // producer warps (the A build is on the critical path)
constexpr int kPThreads = 32 * (2 + kPBuildWarps + kT3EpiWarps);  // 512: 128 registers fill the register file
constexpr int kPSA = kT3M * kT3KB;                        // 16 KB  (i,j) rows, 128-byte swizzle
static_assert(2 * kPN <= 512, "packed tensor kernel tensor memory");

// ---------------------------------------------------------------------------
// Packed-class order-3 kernel on CTA pairs.  A cluster of two CTAs (the two
// SMs of a TPC) runs one GEMM of M 256 x N 256 per work item (i, 64 j, 128 l)
// with tcgen05.mma.cta_group::2: CTA r builds the A tile of its 32 j
// (j0 + 32 r ..) in its own shared memory and stages half r of the l rows
// (64 l x 2 rows); CTA 0 issues the MMAs, which read both CTAs' shared memory
// and leave each CTA's 128 accumulator rows -- its own (j, x, y) rows x the
// item's 256 (l, z) columns -- in its own tensor memory.  The shared memory
// of an SM then takes 82 instead of 114 KB per 128-sample stage (the l-row
// TMA writes and MMA operand reads halve; the single-CTA kernel keeps the
// SM's shared memory at its bank limit), and 4 stages of 41 KB fit.  (Split
// into a 5-slot TMA ring and a 3-slot A ring it ran 18 % slower: the A build
// then has too little slack.)
// Handover: each CTA's TMA completes on its own `full_t`; its producer warps
// build A once their rows landed and arrive on CTA 0's `full_a` (12 arrivals:
// both CTAs' rows and A tiles are then in place); the MMA commits go to both
// CTAs' `empty`, `acc_full` and `done`; both CTAs' epilogue warps arrive on
// CTA 0's `acc_empty` (16 arrivals).  Every wait is bounded; both CTAs meet
// at a cluster barrier before tensor memory is released.
constexpr int kPxJ = 2 * kT3J;                                     // 64 j per pair item
constexpr int kPxStages = 4;
constexpr int kPxBRows = kPN / 2;                                  // this CTA's l rows (64 l x 2)
constexpr int kPxSB = kPxBRows * kT3KB;                            // 16 KB
constexpr int kPxStage = kPxSB + kPSA + kT3SJ + kT3SI;             // 41 KB, a multiple of 1 KB
constexpr size_t kPxSmem = 1024 + (size_t)kPxStages * kPxStage + (size_t)kT3EpiWarps * kT3Ebuf + 2 * kPL * 16;
constexpr uint32_t kPxIdesc = (1u << 4) | ((uint32_t)(kPN >> 3) << 17) | ((uint32_t)((2 * kT3M) >> 4) << 24);
static_assert(kPxSmem <= 227 * 1024 - 256, "paired order-3 tensor kernel shared memory");

// Pair items of one i: J-tile a starts at j0 = i+1+64a and has
// ceil((n-1-j0)/128) L-tiles starting at l0 = j0+1+128b.
__device__ __forceinline__ void t3x_decode(const long long* __restrict__ item_begin, int n, long long g, int& i,
                                           int& j0, int& l0) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (item_begin[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    i = lo;
    long long q = g - item_begin[i];
    for (int a = 0;; ++a) {
        const int j = i + 1 + kPxJ * a;
        const long long nl = (n - 1 - j + kPL - 1) / kPL;
        if (q < nl) {
            j0 = j;
            l0 = j + 1 + kPL * (int)q;
            return;
        }
        q -= nl;
    }
}

// LIST: the list mode above (maps.j then covers the residue-ordered planes,
// where the listed j of one i are consecutive rows).
template <bool LIST>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kPThreads, 1)
    tensor3x_kernel(const __grid_constant__ T3Maps maps, const __grid_constant__ CUtensorMap map_lh, ScanWork w,
                    const long long* __restrict__ item_begin, long long g0, long long g1, int k_cases, int pack,
                    CandSink sink, float thr_f, uint32_t* dump, const uint32_t* __restrict__ single,
                    const uint4* __restrict__ pairs, int* status, const long long* __restrict__ jl_begin,
                    const int* __restrict__ jlist) {
    extern __shared__ uint8_t smraw[];
    __shared__ __align__(8) uint64_t full_t[kPxStages], full_a[kPxStages], empty[kPxStages];
    __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2], done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);  // stages: B half | A | j | i
    uint32_t* ebuf_all = reinterpret_cast<uint32_t*>(sm + kPxStages * kPxStage);
    volatile int* abort = &abort_flag;
    const DevData& d = w.d;
    const int n = d.snps;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ks_c = k_cases / kT3KB;
    const int ksteps = ks_c + (d.tw + 1) / 2;
    const uint32_t rank = cluster_rank();  // 0 issues the MMAs
    const long long cid = cluster_id(), ncl = cluster_count();

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < kPxStages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_t[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_a[s])),
                         "r"(2 * kPBuildWarps));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_full[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&acc_empty[b])),
                         "r"(2 * kT3EpiWarps));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;");
        abort_flag = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    cluster_sync_all();  // both CTAs' barriers exist before either signals the other
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    bool ok = true;

    if (warp == 0) {
        // ---------------------------------------------------------------- TMA producer (both CTAs)
        if (lane == 0) {
            long long step = 0;
            for (long long g = g0 + cid; g < g1 && ok; g += ncl) {
                int i, j0 = 0, l0;
                if (LIST) {
                    long long p0;
                    t3l_decode<kPxJ, kPL>(item_begin, jl_begin, jlist, n, g, i, p0, l0);
                    // this CTA's 32 listed j: consecutive residue-ordered rows from its first one (rows
                    // past the end of i's list are loaded too and ignored by the epilogue)
                    p0 += kT3J * (int)rank;
                    j0 = p0 < jl_begin[i + 1] ? residue_row(jlist[p0], w.dist_step, n) : 0;
                } else {
                    t3x_decode(item_begin, n, g, i, j0, l0);
                    j0 += kT3J * (int)rank;
                }
                for (int ks = 0; ks < ksteps; ++ks) {
                    const int s = (int)(step % kPxStages);
                    const long long u = step / kPxStages;
                    if (u > 0 && !t3_wait_cl(smem_u32(&empty[s]), (uint32_t)((u - 1) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    const int k0 = ks < ks_c ? ks * kT3KB : k_cases + (ks - ks_c) * kT3KB;
                    uint8_t* st = sm + s * kPxStage;
                    const uint32_t bar = smem_u32(&full_t[s]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                                 "r"((uint32_t)(kPxSB + kT3SJ + 2 * kT3KB))
                                 : "memory");
                    t3_tma(smem_u32(st), &map_lh, k0, 2 * l0 + kPxBRows * (int)rank, bar);
                    t3_tma(smem_u32(st + kPxSB + kPSA), &maps.j, k0, 2 * j0, bar);
                    t3_tma(smem_u32(st + kPxSB + kPSA + kT3SJ), &maps.i, k0, 2 * i, bar);
                    ++step;
                }
            }
            if (lane == 0)
                for (int s = 0; s < kPxStages; ++s) {
                    if (step <= s) continue;
                    const long long last = s + ((step - 1 - s) / kPxStages) * kPxStages;
                    if (!t3_drain(smem_u32(&full_t[s]), (uint32_t)((last / kPxStages) & 1))) ok = false;
                }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------------- MMA issuer (CTA 0)
        if (lane == 0 && rank == 0) {
            long long step = 0, item = 0;
            for (long long g = g0 + cid; g < g1 && ok; g += ncl, ++item) {
                const int buf = (int)(item & 1);
                if (item >= 2 && !t3_wait_cl(smem_u32(&acc_empty[buf]), (uint32_t)(((item >> 1) - 1) & 1), abort)) {
                    ok = false;
                    break;
                }
                const uint32_t dcol = tmem + (uint32_t)(kPN * buf);
                // (N stays 256: with cta_group::2 each CTA supplies N / 2 of the B rows, so a
                // narrower N would move the split point off the CTAs' l halves)
                for (int ks = 0; ks < ksteps; ++ks, ++step) {
                    const int s = (int)(step % kPxStages);
                    // both CTAs' rows landed and both A tiles are built
                    if (!t3_wait_cl(smem_u32(&full_a[s]), (uint32_t)((step / kPxStages) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t sb = smem_u32(sm + s * kPxStage), sa = sb + kPxSB;
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const uint64_t ad = t3_desc(sa + 32 * kk), bd = t3_desc(sb + 32 * kk);
                        const uint32_t acc = (ks == 0 && kk == 0) ? 0u : 1u;
                        asm volatile(
                            "{.reg .pred p; setp.ne.b32 p, %4, 0;\n"
                            "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;}\n" ::"r"(dcol),
                            "l"(ad), "l"(bd), "r"(kPxIdesc), "r"(acc));
                    }
                    commit_pair(smem_u32(&empty[s]));
                }
                if (!ok) break;
                commit_pair(smem_u32(&acc_full[buf]));
            }
            commit_pair(smem_u32(&done));
        }
        // neither CTA releases shared or tensor memory before the pair's MMAs are
        // done (CTA 1 waits once its own work is over, below: waiting here would
        // span its whole launch, longer than the bound on a single wait)
        if (lane == 0 && rank == 0 && !t3_drain_cl(smem_u32(&done), 0)) ok = false;
    } else if (warp < 2 + kPBuildWarps) {
        // ---------------------------------------------------------------- A builders (both CTAs)
        const int t = tid - 64;
        const int c = t & 7;
        uint32_t full_a0[kPxStages];
#pragma unroll
        for (int s = 0; s < kPxStages; ++s) full_a0[s] = cluster_addr(smem_u32(&full_a[s]), 0);
        long long step = 0;
        for (long long g = g0 + cid; g < g1 && ok; g += ncl) {
            for (int ks = 0; ks < ksteps; ++ks, ++step) {
                const int s = (int)(step % kPxStages);
                if (!t3_wait(smem_u32(&full_t[s]), (uint32_t)((step / kPxStages) & 1), abort)) {
                    ok = false;
                    break;
                }
                uint8_t* st = sm + s * kPxStage;
                uint8_t* sA = st + kPxSB;
                const uint8_t* sJ = sA + kPSA;
                const uint8_t* sI = sJ + kT3SJ;
                const uint4 i0 = *reinterpret_cast<const uint4*>(sI + (c << 4));
                const uint4 i1 = *reinterpret_cast<const uint4*>(sI + 128 + ((c ^ 1) << 4));
                constexpr int kRows = (2 * kT3J + 4 * kPBuildWarps - 1) / (4 * kPBuildWarps);
                uint4 jrow[kRows];
#pragma unroll
                for (int u = 0; u < kRows; ++u) {
                    const int r = (t >> 3) + 4 * kPBuildWarps * u;
                    if (r < 2 * kT3J) jrow[u] = *reinterpret_cast<const uint4*>(sJ + r * 128 + ((c ^ (r & 7)) << 4));
                }
#pragma unroll
                for (int u = 0; u < kRows; ++u) {
                    const int r = (t >> 3) + 4 * kPBuildWarps * u;
                    if (r >= 2 * kT3J) break;
                    const uint4 jv = jrow[u];
                    const int m0 = 4 * (r >> 1) + (r & 1), m1 = m0 + 2;
                    uint4 v;
                    v.x = jv.x & i0.x;
                    v.y = jv.y & i0.y;
                    v.z = jv.z & i0.z;
                    v.w = jv.w & i0.w;
                    *reinterpret_cast<uint4*>(sA + m0 * 128 + ((c ^ (m0 & 7)) << 4)) = v;
                    v.x = jv.x & i1.x;
                    v.y = jv.y & i1.y;
                    v.z = jv.z & i1.z;
                    v.w = jv.w & i1.w;
                    *reinterpret_cast<uint4*>(sA + m1 * 128 + ((c ^ (m1 & 7)) << 4)) = v;
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) arrive_cl(full_a0[s]);
            }
        }
    } else {
        // ---------------------------------------------------------------- epilogue (both CTAs)
        const int e = warp - (2 + kPBuildWarps);
        const int q = warp & 3;
        const int hh = e >> 2;
        uint32_t* ebuf = ebuf_all + e * (kT3Ebuf / 4);
        const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
        const uint32_t wmask = (1u << pack) - 1u;
        const int jl = lane >> 2, xy = lane & 3, kp = lane & 3;
        const int et = tid - 32 * (2 + kPBuildWarps);
        const uint32_t acc_empty0[2] = {cluster_addr(smem_u32(&acc_empty[0]), 0),
                                        cluster_addr(smem_u32(&acc_empty[1]), 0)};
        uint4* stage = reinterpret_cast<uint4*>(ebuf_all + kT3EpiWarps * (kT3Ebuf / 4));
        long long item = 0;
        for (long long g = g0 + cid; g < g1 && ok; g += ncl, ++item) {
            int i, j0 = 0, l0;
            long long p0 = 0, p_end = 0;
            if (LIST) {
                t3l_decode<kPxJ, kPL>(item_begin, jl_begin, jlist, n, g, i, p0, l0);
                p0 += kT3J * (int)rank;
                p_end = jl_begin[i + 1];
            } else {
                t3x_decode(item_begin, n, g, i, j0, l0);
                j0 += kT3J * (int)rank;
            }
            const int buf = (int)(item & 1);
            asm volatile("bar.sync 1, %0;" ::"n"(32 * kT3EpiWarps) : "memory");
            {
                const int ll = et & (kPL - 1), l = l0 + ll;
                if (l < n) {
                    if (et < kPL) stage[ll] = __ldg(pairs + pair_index(i, l, n));
                    else stage[kPL + ll] = __ldg(reinterpret_cast<const uint4*>(single) + l);
                }
            }
            asm volatile("bar.sync 1, %0;" ::"n"(32 * kT3EpiWarps) : "memory");
            const int j = t3x_j<LIST>(j0, p0, p_end, jlist, 8 * q + jl, n);
            const bool j_ok = j < n;
            uint4 pij;
            float si[2][2], sj[2][2];
            t3_item_consts(single, pairs, i, j, n, j_ok, pij, si, sj);
            if (!t3_wait_cl(smem_u32(&acc_full[buf]), (uint32_t)((item >> 1) & 1), abort)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
            for (int cc = 0; cc < 8; ++cc) {
                const int lg = l0 + 16 * cc + 8 * hh;
                if (!__any_sync(0xffffffffu, j_ok && lg + 7 > j && lg < n)) {
                    if (cc == 7) {
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0) arrive_cl(acc_empty0[buf]);
                    }
                    continue;
                }
                {
                    const uint32_t col = (uint32_t)(kPN * buf + 32 * cc + 16 * hh);
                    uint32_t v[16];
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%"
                        "15}, [%16];"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                          "=r"(v[14]), "=r"(v[15])
                        : "r"(lane_base + col));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (cc == 7) {
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0) arrive_cl(acc_empty0[buf]);
                    }
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const uint32_t u0 = __float2uint_rn(__uint_as_float(v[2 * k]));
                        const uint32_t u1 = __float2uint_rn(__uint_as_float(v[2 * k + 1]));
                        *reinterpret_cast<uint2*>(ebuf + 2 * t3_slot(jl, k, xy)) =
                            make_uint2((u0 & wmask) | (u1 & wmask) << 16, (u0 >> pack) | (u1 >> pack) << 16);
                    }
                }
                __syncwarp();
#pragma unroll 1
                for (int b = 0; b < 2; ++b)
                    t3_eval(w, sink, thr_f, dump, single, pairs, ebuf, jl, 2 * kp + b, i, j, lg + 2 * kp + b, j_ok,
                            pij, si, sj, lane, stage, l0);
                __syncwarp();
            }
        }
    }
    if (!ok) *abort = 1;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // CTA 1: its epilogue has read the last accumulators, so the pair's final
    // commit to this CTA's `done` lands soon; it must land before the CTA exits
    if (rank == 1 && warp == 1 && lane == 0 && !t3_drain_cl(smem_u32(&done), 0)) *abort = 1;
    cluster_sync_all();  // the other CTA is done with this CTA's shared and tensor memory
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0 && abort_flag) atomicOr(status, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// ---------------------------------------------------------------------------
// Order 2.  The 4 core cells of a pair (i, j) are plain dot products of two
// plane rows, core[x][y] = sum_s a_ix(s) a_jy(s): a work item (64 i, 128 j)
// is one GEMM D[(i,x), (j,y)] (M 128 x N 256) with both operands straight
// from the operand planes by TMA -- no producer warps.  Both classes in one
// accumulator when they pack (two alternating tensor-memory regions), else
// cases in columns 0-255 and controls in 256-511 (the MMA then waits for the
// epilogue between items).  4 stages of 48 KB; 8 epilogue warps.
// Reference semantics: GenotypeTable::combine_and_popcnt for order 2
// (src/base/gt_popcnt.cpp:4-35) over the pairs ThreadedSearch visits
// (include/fiuncho/ThreadedSearch.h:157-180) with one worker.
constexpr int kT2I = 64, kT2L = 128;                     // SNPs per tile
constexpr int kT2M = 2 * kT2I, kT2N = 2 * kT2L;          // 128 x 256
constexpr int kT2Stages = 4;
constexpr int kT2SA = kT2M * kT3KB, kT2SB = kT2N * kT3KB;  // 16 KB, 32 KB
constexpr int kT2Stage = kT2SA + kT2SB;                    // 48 KB
constexpr int kT2Threads = 32 * (2 + kT3EpiWarps);         // 320
constexpr size_t kT2Smem = 1024 + (size_t)kT2Stages * kT2Stage + (size_t)kT3EpiWarps * kT3Ebuf;
constexpr uint32_t kT2Idesc = (1u << 4) | ((uint32_t)(kT2N >> 3) << 17) | ((uint32_t)(kT2M >> 4) << 24);
static_assert(kT2Smem <= 227 * 1024 - 256, "order-2 tensor kernel shared memory");

// Work items.  i-tiles a (i0 = 64 a) are grouped in bands of kT2Band; j-tiles
// are global (j0 = 128 b).  Band r covers i-tiles [8 r, 8 r + 8) and j-tiles
// b >= 4 r (the first j-tile holding a j > i of the band) and lists its items
// j-tile by j-tile, i-tile fastest: the CTAs working at the same time share
// a band's eight A tiles and each B tile, so the operands stream from HBM
// about once per band instead of once per item (items left of the diagonal
// are masked in the epilogue).  item_begin[r] = first item of band r.
constexpr int kT2Band = 8;
__device__ __forceinline__ void t2_decode(const long long* __restrict__ item_begin, int n_itiles, long long g, int& i0,
                                          int& j0) {
    const int n_bands = (n_itiles + kT2Band - 1) / kT2Band;
    int lo = 0, hi = n_bands - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (item_begin[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    const int ca = min(kT2Band, n_itiles - kT2Band * lo);  // i-tiles in the band
    const long long idx = g - item_begin[lo];
    const int b = kT2Band * kT2I / kT2L * lo + (int)(idx / ca);
    i0 = kT2I * (kT2Band * lo + (int)(idx % ca));
    j0 = kT2L * b;
}

// 8-byte slot of the order-2 transpose buffer holding (cases y0 | y1 << 16,
// controls y0 | y1 << 16) of row (ii, x) and column group k; each half-warp
// covers the 32 banks once for the row-wise writes (lanes (ii, x), fixed k)
// and the pair-wise reads (lanes (ii, kh), fixed x, k = 4 kh + kk).
__device__ __forceinline__ int t2_slot(int ii, int k, int x) {
    return ((((ii >> 3) * 4 + (k & 3)) * 2 + (k >> 2)) * 16) + (((ii & 7) << 1) | (x ^ (k >> 2)));
}

// Distribution layers of order-2 scans: the owned prefixes are the SNPs
// i = offset + step m, consecutive rows m of the operand planes ordered by
// residue mod step (from row residue_row(offset)).  A layer tile is IT
// consecutive owned i (positions p0 = IT a ..); tiles are grouped in bands of
// BT (512 owned i), and a band lists its items j-tile by j-tile, tile fastest,
// from the j-tile holding the band's first i + 1 (as the whole scan's bands:
// the CTAs at work share a band's A tiles and each B tile in L2).
// item_begin[r] = first item of band r.
template <int IT, int BT>
__device__ __forceinline__ void t2l_decode(const long long* __restrict__ item_begin, int n_tiles, const ScanWork& w,
                                           long long g, int& p0, int& j0) {
    const int n_bands = (n_tiles + BT - 1) / BT;
    int lo = 0, hi = n_bands - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (item_begin[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    const int ca = min(BT, n_tiles - BT * lo);  // tiles in the band
    const long long idx = g - item_begin[lo];
    const int i_first = w.dist_offset + w.dist_step * (IT * BT * lo);
    p0 = IT * (BT * lo + (int)(idx % ca));
    j0 = kT2L * ((i_first + 1) / kT2L + (int)(idx / ca));
}

// Evaluates pair (i, j) from its transpose chunks: exact 9-cell tables from the
// cores and the single cores, the bounded single-precision prefilter, the exact
// fixed-point key for survivors, warp-aggregated append (every lane calls it).
__device__ __forceinline__ void t2_eval(const ScanWork& w, const CandSink& sink, float thr_f, uint32_t* dump,
                                        const uint4& sjp, const uint32_t* ebuf, int ii, int k, int i, int j,
                                        bool i_ok, const float (&si)[2][2], int lane) {
    const DevData& d = w.d;
    const int n = d.snps;
    const uint32_t ncls[2] = {(uint32_t)d.n_cases, (uint32_t)d.n_ctrls};
    const float ncf[2] = {(float)d.n_cases, (float)d.n_ctrls};
    const float tiny = 9.5367431640625e-07f;  // 2^-20: x*lg2(x + tiny) = 0 at x = 0
    const bool valid = i_ok && j < n && j > i;
    float t[2][9];
#pragma unroll
    for (int x = 0; x < 2; ++x) {
        const uint2 c2 = *reinterpret_cast<const uint2*>(ebuf + 2 * t2_slot(ii, k, x));
        t[0][x * 3 + 0] = u2f(c2.x & 0xffffu);
        t[0][x * 3 + 1] = u2f(c2.x >> 16);
        t[1][x * 3 + 0] = u2f(c2.y & 0xffffu);
        t[1][x * 3 + 1] = u2f(c2.y >> 16);
    }
    // single cores of j = jg + k, loaded by lane k of the warp for the column group
    uint4 sj4;
    sj4.x = __shfl_sync(0xffffffffu, sjp.x, k);
    sj4.y = __shfl_sync(0xffffffffu, sjp.y, k);
    sj4.z = __shfl_sync(0xffffffffu, sjp.z, k);
    sj4.w = __shfl_sync(0xffffffffu, sjp.w, k);
    const float sj[2][2] = {{u2f(sj4.x), u2f(sj4.y)}, {u2f(sj4.z), u2f(sj4.w)}};
#pragma unroll
    for (int c = 0; c < 2; ++c) {
#pragma unroll
        for (int x = 0; x < 2; ++x) t[c][x * 3 + 2] = si[c][x] - t[c][x * 3] - t[c][x * 3 + 1];
#pragma unroll
        for (int y = 0; y < 2; ++y) t[c][6 + y] = sj[c][y] - t[c][y] - t[c][3 + y];
        t[c][8] = ncf[c] - si[c][0] - si[c][1] - t[c][6] - t[c][7];
    }
    float kf = 0.f;
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        const float a = t[0][c], bb = t[1][c], s = a + bb;
        kf = fmaf(a, t3_lg2(a + tiny), kf);
        kf = fmaf(bb, t3_lg2(bb + tiny), kf);
        kf = fmaf(-s, t3_lg2(s + tiny), kf);
    }
    const bool cand = valid && (dump != nullptr || sink.digest != nullptr || kf >= thr_f);
    long long key = w.base_key;
    bool pass = false;
    unsigned long long dg = 0;
    if (cand) {
#pragma unroll
        for (int c = 0; c < 9; ++c) {
            const uint32_t a = min(f2u(fmaxf(t[0][c], 0.f)), ncls[0]);
            const uint32_t bb = min(f2u(fmaxf(t[1][c], 0.f)), ncls[1]);
            key += __ldg(d.ftab + a) + __ldg(d.ftab + bb) - __ldg(d.ftab + a + bb);
        }
        pass = key >= sink.thr;
        if (dump) {
            // owned prefix ordinal m of i: rank offset + m * step
            uint32_t* o = dump + ((size_t)((i - w.dist_offset) / w.dist_step) * n + j) * 18;
#pragma unroll
            for (int c = 0; c < 9; ++c) {
                o[c] = f2u(t[0][c]);
                o[9 + c] = f2u(t[1][c]);
            }
        }
        if (sink.digest) {
            const int cmb[2] = {i, j};
            dg = dg_begin(cmb, 2, n);
#pragma unroll
            for (int c = 0; c < 9; ++c) dg = dg_cell(dg, f2u(t[0][c]), f2u(t[1][c]));
        }
    }
    if (sink.digest) dg_warp_add(sink.digest, dg);
    if (sink.evaluated) {
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        if (lane == 0 && vmask) atomicAdd(sink.evaluated, (unsigned long long)__popc(vmask));
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
                const int cmb[2] = {i, j};
                sink.buf[idx] = Cand{key, pack_code(cmb, 2, w.bits)};
            } else {
                atomicOr(sink.overflow, 1u);
            }
        }
    }
}

struct T2Maps {
    CUtensorMap a, b;
};

// LAYER: a Distribution layer (t2l_decode; maps.a covers the residue-ordered
// planes, item_begin / n_itiles are the layer's tiles).
template <bool LAYER>
__global__ void __launch_bounds__(kT2Threads, 1)
    tensor2_kernel(const __grid_constant__ T2Maps maps, ScanWork w, const long long* __restrict__ item_begin,
                   int n_itiles, long long g0, long long g1, int k_cases, int pack, CandSink sink, float thr_f,
                   uint32_t* dump, const uint32_t* __restrict__ single, int* status) {
    extern __shared__ uint8_t smraw[];
    __shared__ __align__(8) uint64_t full[kT2Stages], empty[kT2Stages];
    __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2], done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);  // stages: A | B
    uint32_t* ebuf_all = reinterpret_cast<uint32_t*>(sm + kT2Stages * kT2Stage);
    volatile int* abort = &abort_flag;
    const DevData& d = w.d;
    const int n = d.snps;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ks_c = k_cases / kT3KB;
    const int ksteps = ks_c + (d.tw + 1) / 2;
    const int nbuf = pack ? 2 : 1;  // accumulator regions that alternate between items

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < kT2Stages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_full[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&acc_empty[b])), "r"(kT3EpiWarps));
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
                int i0, j0;  // LAYER: i0 = the tile's first row in the residue-ordered planes
                if (LAYER) {
                    int p0;
                    t2l_decode<kT2I, 8>(item_begin, n_itiles, w, g, p0, j0);
                    i0 = residue_row(w.dist_offset, w.dist_step, n) + p0;
                } else {
                    t2_decode(item_begin, n_itiles, g, i0, j0);
                }
                for (int ks = 0; ks < ksteps; ++ks) {
                    const int s = (int)(step % kT2Stages);
                    const long long u = step / kT2Stages;
                    if (u > 0 && !t3_wait(smem_u32(&empty[s]), (uint32_t)((u - 1) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    const int k0 = ks < ks_c ? ks * kT3KB : k_cases + (ks - ks_c) * kT3KB;
                    uint8_t* st = sm + s * kT2Stage;
                    const uint32_t bar = smem_u32(&full[s]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                                 "r"((uint32_t)kT2Stage)
                                 : "memory");
                    t3_tma(smem_u32(st), &maps.a, k0, 2 * i0, bar);
                    t3_tma(smem_u32(st + kT2SA), &maps.b, k0, 2 * j0, bar);
                    ++step;
                }
            }
            for (int s = 0; s < kT2Stages; ++s) {
                if (step <= s) continue;
                const long long last = s + ((step - 1 - s) / kT2Stages) * kT2Stages;
                if (!t3_drain(smem_u32(&full[s]), (uint32_t)((last / kT2Stages) & 1))) ok = false;
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0) {
            long long step = 0, item = 0;
            for (long long g = g0 + blockIdx.x; g < g1 && ok; g += gridDim.x, ++item) {
                const int buf = (int)(item % nbuf);
                if (item >= nbuf &&
                    !t3_wait(smem_u32(&acc_empty[buf]), (uint32_t)(((item / nbuf) - 1) & 1), abort)) {
                    ok = false;
                    break;
                }
                for (int ks = 0; ks < ksteps; ++ks, ++step) {
                    const int s = (int)(step % kT2Stages);
                    if (!t3_wait(smem_u32(&full[s]), (uint32_t)((step / kT2Stages) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t sa = smem_u32(sm + s * kT2Stage), sb = sa + kT2SA;
                    const int cls = ks >= ks_c;
                    const uint32_t dcol = tmem + (uint32_t)(pack ? kT2N * buf : kT2N * cls);
                    const bool first = pack ? ks == 0 : (ks == 0 || ks == ks_c);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const uint64_t ad = t3_desc(sa + 32 * kk), bd = t3_desc(sb + 32 * kk);
                        const uint32_t acc = (first && kk == 0) ? 0u : 1u;
                        asm volatile(
                            "{.reg .pred p; setp.ne.b32 p, %4, 0;\n"
                            "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;}\n" ::"r"(dcol),
                            "l"(ad), "l"(bd), "r"(kT2Idesc), "r"(acc));
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
    } else {
        // ---------------------------------------------------------------- epilogue
        const int e = warp - 2;     // 0..7
        const int q = warp & 3;     // tensor-memory lane quarter this warp may access
        const int hh = e >> 2;      // column groups 2 cc + hh: j offsets 16 cc + 8 hh + [0, 8)
        uint32_t* ebuf = ebuf_all + e * (kT3Ebuf / 4);
        const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
        const uint32_t wmask = pack ? (1u << pack) - 1u : 0xffffffffu;
        const int ii = lane >> 1, x = lane & 1, kh = lane & 1;  // row (ii, x); pairs k = 4 kh + kk
        long long item = 0;
        for (long long g = g0 + blockIdx.x; g < g1 && ok; g += gridDim.x, ++item) {
            int i0, j0, istep = 1;
            if (LAYER) {
                int p0;
                t2l_decode<kT2I, 8>(item_begin, n_itiles, w, g, p0, j0);
                i0 = w.dist_offset + w.dist_step * p0;
                istep = w.dist_step;
            } else {
                t2_decode(item_begin, n_itiles, g, i0, j0);
            }
            const int buf = (int)(item % nbuf);
            const int i = i0 + istep * (16 * q + ii);
            const bool i_ok = i < n;
            float si[2][2];
            {
                uint4 a = make_uint4(0, 0, 0, 0);
                if (i_ok) a = __ldg(reinterpret_cast<const uint4*>(single) + i);
                si[0][0] = u2f(a.x);
                si[0][1] = u2f(a.y);
                si[1][0] = u2f(a.z);
                si[1][1] = u2f(a.w);
            }
            if (!t3_wait(smem_u32(&acc_full[buf]), (uint32_t)((item / nbuf) & 1), abort)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
            for (int cc = 0; cc < 8; ++cc) {
                // the two warps of a lane quarter interleave over the j range; a group without
                // a valid pair for this warp (left of the diagonal, past the last SNP) is skipped
                const int jg = j0 + 16 * cc + 8 * hh;
                if (!__any_sync(0xffffffffu, i_ok && jg + 7 > i && jg < n)) {
                    if (cc == 7) {
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0)
                            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[buf]))
                                         : "memory");
                    }
                    continue;
                }
                // the group's 8 single cores of j: lane t loads j = jg + (t & 7) before the
                // accumulator reads, so that its latency overlaps them
                const int jl = jg + (lane & 7);
                const uint4 sjp = jl < n ? __ldg(reinterpret_cast<const uint4*>(single) + jl) : make_uint4(0, 0, 0, 0);
                {
                    const uint32_t col = (uint32_t)((pack ? kT2N * buf : 0) + 32 * cc + 16 * hh);
                    uint32_t v[16], vt[16];
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%"
                        "15}, [%16];"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                          "=r"(v[14]), "=r"(v[15])
                        : "r"(lane_base + col));
                    if (!pack)
                        asm volatile(
                            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%"
                            "14,%15}, [%16];"
                            : "=r"(vt[0]), "=r"(vt[1]), "=r"(vt[2]), "=r"(vt[3]), "=r"(vt[4]), "=r"(vt[5]),
                              "=r"(vt[6]), "=r"(vt[7]), "=r"(vt[8]), "=r"(vt[9]), "=r"(vt[10]), "=r"(vt[11]),
                              "=r"(vt[12]), "=r"(vt[13]), "=r"(vt[14]), "=r"(vt[15])
                            : "r"(lane_base + (uint32_t)kT2N + col));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (cc == 7) {  // last read of this item's accumulators
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0)
                            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[buf]))
                                         : "memory");
                    }
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        uint2 c2;
                        if (pack) {
                            const uint32_t u0 = __float2uint_rn(__uint_as_float(v[2 * k]));
                            const uint32_t u1 = __float2uint_rn(__uint_as_float(v[2 * k + 1]));
                            c2 = make_uint2((u0 & wmask) | (u1 & wmask) << 16, (u0 >> pack) | (u1 >> pack) << 16);
                        } else {
                            c2 = make_uint2(f2u(__uint_as_float(v[2 * k])) | f2u(__uint_as_float(v[2 * k + 1])) << 16,
                                            f2u(__uint_as_float(vt[2 * k])) | f2u(__uint_as_float(vt[2 * k + 1])) << 16);
                        }
                        *reinterpret_cast<uint2*>(ebuf + 2 * t2_slot(ii, k, x)) = c2;
                    }
                }
                __syncwarp();
#pragma unroll 1
                for (int kk = 0; kk < 4; ++kk) {
                    const int k = 4 * kh + kk;
                    t2_eval(w, sink, thr_f, dump, sjp, ebuf, ii, k, i, jg + k, i_ok, si, lane);
                }
                __syncwarp();
            }
        }
    }
    if (!ok) *abort = 1;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0 && abort_flag) atomicOr(status, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// ---------------------------------------------------------------------------
// Order 2 on CTA pairs.  A cluster of two CTAs (the two SMs of a TPC) runs one
// GEMM D[(i,x), (j,y)] of M 256 x N 256 per work item with
// tcgen05.mma.cta_group::2: CTA r stages its own A tile (64 i x 2 rows, i-tile
// 2p + r of the band) and half r of the B tile (64 j x 2 rows); CTA 0 issues
// the MMAs, which read both CTAs' shared memory and leave each CTA's 128
// accumulator rows in its own tensor memory.  Per SM a stage then moves 32
// instead of 48 KB through shared memory (TMA writes and MMA operand reads of
// B halve), which is what bounded the single-CTA kernel.
// Handover: CTA 0's `full` barriers take one arrival with the transaction
// bytes of both CTAs' copies (CTA 1's copies complete on them through the
// .cta_group::2 TMA form); the MMA commits go to both CTAs' `empty`,
// `acc_full` and `done`; both CTAs' epilogue warps arrive on CTA 0's
// `acc_empty` (16 arrivals).  Every wait is bounded as in the other kernels;
// both CTAs meet at a cluster barrier before tensor memory is released.
constexpr int kT2xStages = 5;
constexpr int kT2xSA = kT2M * kT3KB;        // 16 KB: this CTA's 64 i x 2 rows
constexpr int kT2xSB = kT2M * kT3KB;        // 16 KB: this CTA's half of the 128 j x 2 rows
constexpr int kT2xStage = kT2xSA + kT2xSB;  // 32 KB
constexpr size_t kT2xSmem = 1024 + (size_t)kT2xStages * kT2xStage + (size_t)kT3EpiWarps * kT3Ebuf;
constexpr uint32_t kT2xIdesc = (1u << 4) | ((uint32_t)(kT2N >> 3) << 17) | ((uint32_t)((2 * kT2M) >> 4) << 24);
static_assert(kT2xSmem <= 227 * 1024 - 256, "paired order-2 tensor kernel shared memory");

// Pair items: band r (i-tiles [8 r, 8 r + 8), j-tiles b >= 4 r) lists, j-tile by
// j-tile, its i-tile pairs (2 p, 2 p + 1); i0 = first i of the pair.
__device__ __forceinline__ void t2x_decode(const long long* __restrict__ item_begin, int n_itiles, long long g,
                                           int& i0, int& j0) {
    const int n_bands = (n_itiles + kT2Band - 1) / kT2Band;
    int lo = 0, hi = n_bands - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (item_begin[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    const int ca = min(kT2Band, n_itiles - kT2Band * lo);
    const int cp = (ca + 1) >> 1;  // i-tile pairs in the band
    const long long idx = g - item_begin[lo];
    const int b = kT2Band * kT2I / kT2L * lo + (int)(idx / cp);
    i0 = kT2I * (kT2Band * lo + 2 * (int)(idx % cp));
    j0 = kT2L * b;
}

// LAYER: a Distribution layer (t2l_decode over tile pairs, as tensor2_kernel).
template <bool LAYER>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kT2Threads, 1)
    tensor2x_kernel(const __grid_constant__ T2Maps maps, ScanWork w, const long long* __restrict__ item_begin,
                    int n_itiles, long long g0, long long g1, int k_cases, int pack, CandSink sink, float thr_f,
                    uint32_t* dump, const uint32_t* __restrict__ single, int* status) {
    extern __shared__ uint8_t smraw[];
    __shared__ __align__(8) uint64_t full[kT2xStages], empty[kT2xStages];
    __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2], done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);  // stages: A | B half
    uint32_t* ebuf_all = reinterpret_cast<uint32_t*>(sm + kT2xStages * kT2xStage);
    volatile int* abort = &abort_flag;
    const DevData& d = w.d;
    const int n = d.snps;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ks_c = k_cases / kT3KB;
    const int ksteps = ks_c + (d.tw + 1) / 2;
    const int nbuf = pack ? 2 : 1;
    const uint32_t rank = cluster_rank();  // 0 issues the MMAs
    const long long cid = cluster_id(), ncl = cluster_count();

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < kT2xStages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_full[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&acc_empty[b])),
                         "r"(2 * kT3EpiWarps));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;");
        abort_flag = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    cluster_sync_all();  // both CTAs' barriers exist before either signals the other
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    bool ok = true;

    if (warp == 0) {
        // ---------------------------------------------------------------- TMA producer (both CTAs)
        if (lane == 0) {
            long long step = 0;
            for (long long g = g0 + cid; g < g1 && ok; g += ncl) {
                int i0, j0;  // LAYER: i0 = the pair's first row in the residue-ordered planes
                if (LAYER) {
                    int p0;
                    t2l_decode<2 * kT2I, 4>(item_begin, n_itiles, w, g, p0, j0);
                    i0 = residue_row(w.dist_offset, w.dist_step, n) + p0;
                } else {
                    t2x_decode(item_begin, n_itiles, g, i0, j0);
                }
                for (int ks = 0; ks < ksteps; ++ks) {
                    const int s = (int)(step % kT2xStages);
                    const long long u = step / kT2xStages;
                    if (u > 0 && !t3_wait_cl(smem_u32(&empty[s]), (uint32_t)((u - 1) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    const int k0 = ks < ks_c ? ks * kT3KB : k_cases + (ks - ks_c) * kT3KB;
                    uint8_t* st = sm + s * kT2xStage;
                    const uint32_t bar = cluster_addr(smem_u32(&full[s]), 0);
                    if (rank == 0)
                        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&full[s])),
                                     "r"((uint32_t)(2 * kT2xStage))
                                     : "memory");
                    t3_tma_pair(smem_u32(st), &maps.a, k0, 2 * (i0 + kT2I * (int)rank), bar);
                    t3_tma_pair(smem_u32(st + kT2xSA), &maps.b, k0, 2 * j0 + kT2M * (int)rank, bar);
                    ++step;
                }
            }
            // copies in flight land before the pair is released: CTA 0 sees every copy of
            // both CTAs complete on its `full` barriers, CTA 1 sees its stages consumed
            for (int s = 0; s < kT2xStages; ++s) {
                if (step <= s) continue;
                const long long last = s + ((step - 1 - s) / kT2xStages) * kT2xStages;
                const uint32_t par = (uint32_t)((last / kT2xStages) & 1);
                if (!(rank == 0 ? t3_drain_cl(smem_u32(&full[s]), par) : t3_drain_cl(smem_u32(&empty[s]), par)))
                    ok = false;
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------------- MMA issuer (CTA 0)
        if (lane == 0 && rank == 0) {
            long long step = 0, item = 0;
            for (long long g = g0 + cid; g < g1 && ok; g += ncl, ++item) {
                const int buf = (int)(item % nbuf);
                if (item >= nbuf &&
                    !t3_wait_cl(smem_u32(&acc_empty[buf]), (uint32_t)(((item / nbuf) - 1) & 1), abort)) {
                    ok = false;
                    break;
                }
                for (int ks = 0; ks < ksteps; ++ks, ++step) {
                    const int s = (int)(step % kT2xStages);
                    if (!t3_wait_cl(smem_u32(&full[s]), (uint32_t)((step / kT2xStages) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t sa = smem_u32(sm + s * kT2xStage), sb = sa + kT2xSA;
                    const int cls = ks >= ks_c;
                    const uint32_t dcol = tmem + (uint32_t)(pack ? kT2N * buf : kT2N * cls);
                    const bool first = pack ? ks == 0 : (ks == 0 || ks == ks_c);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const uint64_t ad = t3_desc(sa + 32 * kk), bd = t3_desc(sb + 32 * kk);
                        const uint32_t acc = (first && kk == 0) ? 0u : 1u;
                        asm volatile(
                            "{.reg .pred p; setp.ne.b32 p, %4, 0;\n"
                            "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;}\n" ::"r"(dcol),
                            "l"(ad), "l"(bd), "r"(kT2xIdesc), "r"(acc));
                    }
                    commit_pair(smem_u32(&empty[s]));
                }
                if (!ok) break;
                commit_pair(smem_u32(&acc_full[buf]));
            }
            commit_pair(smem_u32(&done));
        }
        // neither CTA releases shared or tensor memory before the pair's MMAs are
        // done (CTA 1 waits once its own work is over, below: waiting here would
        // span its whole launch, longer than the bound on a single wait)
        if (lane == 0 && rank == 0 && !t3_drain_cl(smem_u32(&done), 0)) ok = false;
    } else {
        // ---------------------------------------------------------------- epilogue (both CTAs)
        const int e = warp - 2;
        const int q = warp & 3;
        const int hh = e >> 2;
        uint32_t* ebuf = ebuf_all + e * (kT3Ebuf / 4);
        const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
        const uint32_t wmask = pack ? (1u << pack) - 1u : 0xffffffffu;
        const int ii = lane >> 1, x = lane & 1, kh = lane & 1;
        const uint32_t acc_empty0[2] = {cluster_addr(smem_u32(&acc_empty[0]), 0),
                                        cluster_addr(smem_u32(&acc_empty[1]), 0)};
        long long item = 0;
        for (long long g = g0 + cid; g < g1 && ok; g += ncl, ++item) {
            int i0, j0, istep = 1;
            if (LAYER) {
                int p0;
                t2l_decode<2 * kT2I, 4>(item_begin, n_itiles, w, g, p0, j0);
                i0 = w.dist_offset + w.dist_step * (p0 + kT2I * (int)rank);
                istep = w.dist_step;
            } else {
                t2x_decode(item_begin, n_itiles, g, i0, j0);
                i0 += kT2I * (int)rank;
            }
            const int buf = (int)(item % nbuf);
            const int i = i0 + istep * (16 * q + ii);
            const bool i_ok = i < n;
            float si[2][2];
            {
                uint4 a = make_uint4(0, 0, 0, 0);
                if (i_ok) a = __ldg(reinterpret_cast<const uint4*>(single) + i);
                si[0][0] = u2f(a.x);
                si[0][1] = u2f(a.y);
                si[1][0] = u2f(a.z);
                si[1][1] = u2f(a.w);
            }
            if (!t3_wait_cl(smem_u32(&acc_full[buf]), (uint32_t)((item / nbuf) & 1), abort)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
            for (int cc = 0; cc < 8; ++cc) {
                const int jg = j0 + 16 * cc + 8 * hh;
                if (!__any_sync(0xffffffffu, i_ok && jg + 7 > i && jg < n)) {
                    if (cc == 7) {
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0) arrive_cl(acc_empty0[buf]);
                    }
                    continue;
                }
                const int jl = jg + (lane & 7);
                const uint4 sjp = jl < n ? __ldg(reinterpret_cast<const uint4*>(single) + jl) : make_uint4(0, 0, 0, 0);
                {
                    const uint32_t col = (uint32_t)((pack ? kT2N * buf : 0) + 32 * cc + 16 * hh);
                    uint32_t v[16], vt[16];
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%"
                        "15}, [%16];"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                          "=r"(v[14]), "=r"(v[15])
                        : "r"(lane_base + col));
                    if (!pack)
                        asm volatile(
                            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%"
                            "14,%15}, [%16];"
                            : "=r"(vt[0]), "=r"(vt[1]), "=r"(vt[2]), "=r"(vt[3]), "=r"(vt[4]), "=r"(vt[5]),
                              "=r"(vt[6]), "=r"(vt[7]), "=r"(vt[8]), "=r"(vt[9]), "=r"(vt[10]), "=r"(vt[11]),
                              "=r"(vt[12]), "=r"(vt[13]), "=r"(vt[14]), "=r"(vt[15])
                            : "r"(lane_base + (uint32_t)kT2N + col));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (cc == 7) {
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncwarp();
                        if (lane == 0) arrive_cl(acc_empty0[buf]);
                    }
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        uint2 c2;
                        if (pack) {
                            const uint32_t u0 = __float2uint_rn(__uint_as_float(v[2 * k]));
                            const uint32_t u1 = __float2uint_rn(__uint_as_float(v[2 * k + 1]));
                            c2 = make_uint2((u0 & wmask) | (u1 & wmask) << 16, (u0 >> pack) | (u1 >> pack) << 16);
                        } else {
                            c2 = make_uint2(f2u(__uint_as_float(v[2 * k])) | f2u(__uint_as_float(v[2 * k + 1])) << 16,
                                            f2u(__uint_as_float(vt[2 * k])) | f2u(__uint_as_float(vt[2 * k + 1])) << 16);
                        }
                        *reinterpret_cast<uint2*>(ebuf + 2 * t2_slot(ii, k, x)) = c2;
                    }
                }
                __syncwarp();
#pragma unroll 1
                for (int kk = 0; kk < 4; ++kk) {
                    const int k = 4 * kh + kk;
                    t2_eval(w, sink, thr_f, dump, sjp, ebuf, ii, k, i, jg + k, i_ok, si, lane);
                }
                __syncwarp();
            }
        }
    }
    if (!ok) *abort = 1;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // CTA 1: its epilogue has read the last accumulators, so the pair's final
    // commit to this CTA's `done` lands soon; it must land before the CTA exits
    if (rank == 1 && warp == 1 && lane == 0 && !t3_drain_cl(smem_u32(&done), 0)) *abort = 1;
    cluster_sync_all();  // the other CTA is done with this CTA's shared and tensor memory
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0 && abort_flag) atomicOr(status, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// Operand planes: one thread per 16 output bytes (16 samples of one row).
__global__ void t3_planes_kernel(DevData d, uint8_t* planes, int pitch, int k_cases, uint32_t ctrl_byte) {
    const long long chunks = (long long)pitch / 16;
    const long long total = 2ll * d.snps * chunks;
    const size_t per_snp = 3 * (size_t)(d.cw + d.tw);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long row = e / chunks;
        const int ch = (int)(e - row * chunks);
        const int snp = (int)(row >> 1), g = (int)(row & 1);
        const int o = 16 * ch;
        const bool ctrl = o >= k_cases;
        const int k = ctrl ? o - k_cases : o;
        const int W = ctrl ? d.tw : d.cw;
        const int word = k >> 6;
        uint32_t bits = 0;
        if (word < W)
            bits = (uint32_t)(__ldg(d.ref + (size_t)snp * per_snp + (ctrl ? 3 * (size_t)d.cw : 0) + (size_t)g * W +
                                    word) >>
                              (k & 63)) &
                   0xffffu;
        uint4 v;
        uint32_t* pv = &v.x;
#pragma unroll
        for (int qd = 0; qd < 4; ++qd)
            pv[qd] = (((bits >> (4 * qd)) & 0xfu) * 0x00204081u & 0x01010101u) * (ctrl ? ctrl_byte : 0x38u);
        *reinterpret_cast<uint4*>(planes + (size_t)row * pitch + o) = v;
    }
}

// Order-2 items (host): prefix sums over the bands of t2_decode; returns the
// total and the number of i-tiles.
static long long t2_items(int n, std::vector<long long>& item_begin, int& n_itiles) {
    n_itiles = std::max(1, (n - 1 + kT2I - 1) / kT2I);
    const int n_bands = (n_itiles + kT2Band - 1) / kT2Band;
    const int nb = (n + kT2L - 1) / kT2L;  // global j-tiles
    item_begin.assign((size_t)n_bands + 1, 0);
    long long total = 0;
    for (int r = 0; r < n_bands; ++r) {
        item_begin[r] = total;
        const int ca = std::min(kT2Band, n_itiles - kT2Band * r);
        const int b0 = kT2Band * kT2I / kT2L * r;
        if (nb > b0) total += (long long)ca * (nb - b0);
    }
    item_begin[n_bands] = total;
    return total;
}

// Pair items of tensor2x_kernel (host): prefix sums over the bands of t2x_decode.
static long long t2x_items(int n, std::vector<long long>& item_begin, int& n_itiles) {
    n_itiles = std::max(1, (n - 1 + kT2I - 1) / kT2I);
    const int n_bands = (n_itiles + kT2Band - 1) / kT2Band;
    const int nb = (n + kT2L - 1) / kT2L;
    item_begin.assign((size_t)n_bands + 1, 0);
    long long total = 0;
    for (int r = 0; r < n_bands; ++r) {
        item_begin[r] = total;
        const int ca = std::min(kT2Band, n_itiles - kT2Band * r);
        const int b0 = kT2Band * kT2I / kT2L * r;
        if (nb > b0) total += (long long)((ca + 1) / 2) * (nb - b0);
    }
    item_begin[n_bands] = total;
    return total;
}

// Items per i (host): prefix sums item_begin[0..n], item_begin[n] = total;
// J j per item (kT3J, or kPxJ for the pair items of tensor3x_kernel).
static long long t3_items(int n, int L, std::vector<long long>& item_begin, int J = kT3J) {
    item_begin.assign((size_t)n + 1, 0);
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        item_begin[i] = total;
        for (int j = i + 1; j < n - 1; j += J) total += (n - 1 - j + L - 1) / L;
    }
    item_begin[n] = total;
    return total;
}

static PFN_cuTensorMapEncodeTiled_v12000 t3_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (PFN_cuTensorMapEncodeTiled_v12000)p;
        return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }();
    return fn;
}

static cudaError_t t3_map(CUtensorMap* m, uint8_t* base, int rows, int pitch, int box_rows, bool swizzle) {
    auto enc = t3_encoder();
    if (!enc) return cudaErrorNotSupported;
    cuuint64_t dims[2] = {(cuuint64_t)pitch, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)pitch};
    cuuint32_t box[2] = {(cuuint32_t)kT3KB, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, base, dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE,
                           swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// One accumulator for both classes when some W = 4^h (h <= 8, so 2^h is an
// e4m3 power of two) has n_cases < W and n_cases + W * n_ctrls < 2^24 (every
// count exact in FP32).
int tensor_pack(int n_cases, int n_ctrls) {
    for (int h = 1; h <= 8; ++h) {
        const long long W = 1ll << (2 * h);
        if (W > n_cases && n_cases + W * (long long)n_ctrls < (1ll << 24)) return 2 * h;
    }
    return 0;
}

cudaError_t tensor3_prepare(const DevData& d, T3Plan& plan, cudaStream_t s) {
    plan.pack = tensor_pack(d.n_cases, d.n_ctrls);
    const int L = plan.pack ? kPL : kT3L;
    // packed classes: CTA-pair items
    plan.pair3 = plan.pack != 0;
    const int J = plan.pair3 ? kPxJ : kT3J;
    plan.item_combos = J * L / 2.0;
    plan.k_cases = kT3KB * ((d.cw + 1) / 2);
    plan.pitch = plan.k_cases + kT3KB * ((d.tw + 1) / 2);
    (void)L;
    cudaError_t e = cudaMalloc((void**)&plan.planes, (size_t)2 * d.snps * plan.pitch);
    if (e != cudaSuccess) return e;
    const long long total = 2ll * d.snps * (plan.pitch / 16);
    const int grid = (int)std::min<long long>((total + 255) / 256, 4096);
    const uint32_t ctrl_byte = plan.pack ? (uint32_t)((plan.pack / 2 + 7) << 3) : 0x38u;  // e4m3 2^h
    t3_planes_kernel<<<grid, 256, 0, s>>>(d, plan.planes, plan.pitch, plan.k_cases, ctrl_byte);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int rows = 2 * d.snps;
    if ((e = t3_map(&plan.map_l, plan.planes, rows, plan.pitch, plan.pack ? kPN : kT3N, true)) != cudaSuccess)
        return e;
    if ((e = t3_map(&plan.map_j, plan.planes, rows, plan.pitch, 2 * kT3J, true)) != cudaSuccess) return e;
    if ((e = t3_map(&plan.map_i, plan.planes, rows, plan.pitch, 2, true)) != cudaSuccess) return e;
    // order 2: CTA-pair items when the classes pack (per class the MMA waits for the epilogue between
    // items, and the single-CTA kernel measured 2 % faster there)
    std::vector<long long> ib2;
    plan.pair2 = plan.pack != 0;
    plan.total2 = plan.pair2 ? t2x_items(d.snps, ib2, plan.n_itiles) : t2_items(d.snps, ib2, plan.n_itiles);
    plan.item2_combos = (double)d.snps * (d.snps - 1) / 2 / std::max(1ll, plan.total2);
    e = cudaMalloc((void**)&plan.item2_begin, ib2.size() * sizeof(long long));
    if (e == cudaSuccess)
        e = cudaMemcpy(plan.item2_begin, ib2.data(), ib2.size() * sizeof(long long), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    if ((e = t3_map(&plan.map_a2, plan.planes, rows, plan.pitch, kT2M, true)) != cudaSuccess) return e;
    return t3_map(&plan.map_b2, plan.planes, rows, plan.pitch, kT2N, true);
}

// The work items of the whole data set at order 3 or 4, made on the first
// search of that order (the host enumeration grows as n^2 / 16 at order 4:
// about 0.1 s at 40 000 SNPs, which a search of another order need not pay).
cudaError_t tensor3_order_items(T3Plan& plan, const DevData& d, int order) {
    std::lock_guard<std::mutex> g(plan.items_mu);
    cudaError_t e = cudaSuccess;
    if (order == 3 && !plan.item_begin) {
        const int L = plan.pack ? kPL : kT3L, J = plan.pair3 ? kPxJ : kT3J;
        std::vector<long long> ib;
        const long long total = t3_items(d.snps, L, ib, J);
        long long* p = nullptr;
        e = cudaMalloc((void**)&p, ib.size() * sizeof(long long));
        if (e == cudaSuccess) e = cudaMemcpy(p, ib.data(), ib.size() * sizeof(long long), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(p);
            return e;
        }
        plan.total = total;
        plan.item_begin = p;
    }
    if (order == 4 && !plan.item4_begin && d.snps >= 4) {
        std::vector<long long> per4;
        const std::vector<long long> ib4 = t4_item_table(d.snps, plan.pack != 0, per4);
        long long *pb = nullptr, *pp = nullptr;
        e = t3_map(&plan.map_k4, plan.planes, 2 * d.snps, plan.pitch, 32, true);
        if (e == cudaSuccess) e = cudaMalloc((void**)&pb, ib4.size() * sizeof(long long));
        if (e == cudaSuccess) e = cudaMalloc((void**)&pp, per4.size() * sizeof(long long));
        if (e == cudaSuccess) e = cudaMemcpy(pb, ib4.data(), ib4.size() * sizeof(long long), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(pp, per4.data(), per4.size() * sizeof(long long), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(pb);
            cudaFree(pp);
            return e;
        }
        plan.total4 = ib4.back();
        const double n = d.snps;
        plan.item4_combos = n * (n - 1) * (n - 2) * (n - 3) / 24.0 / std::max(1ll, plan.total4);
        plan.item4_per = pp;
        plan.item4_begin = pb;
    }
    return e;
}

// Work items of Distribution layers of order-3 scans (the pair kernel's list
// mode), one entry per (step, offset) used on the data set.  The owned j of
// one i are the j > i of one residue mod step (pair ranks base(i) + j - i - 1
// step through the layer's offset class), so in a copy of the operand planes
// ordered by residue -- SNPs r, r + step, r + 2 step, .. for r = 0, 1, .. --
// they are consecutive rows, and one tiled TMA copy per stage loads an item's
// j rows as in the scan of all prefixes.
struct T3Layer {
    long long* item_begin = nullptr;  // order 3: [n + 1] first item of each i; order 2: [tiles + 1] of each tile
    long long* jl_begin = nullptr;    // order 3: [n + 1] first listed j of each i
    int* jlist = nullptr;             // order 3: owned j of each i, ascending
    long long total = 0;
    double item_combos = 0;
    int n_tiles = 0;                  // order 2: tiles of owned i; order 4: listed pairs
    int4* pinfo = nullptr;            // order 4: (i, j, first owned k) of each listed pair
    CUtensorMap map_jr;               // order 3: box 128 B x 64 rows over the residue-ordered planes
    CUtensorMap map_ar;               // order 2: box 128 B x 128 rows over the residue-ordered planes
    CUtensorMap map_kr;               // order 4: box 128 B x 32 rows over the residue-ordered planes
};
struct T3Layers {
    std::mutex mu;
    std::map<std::tuple<int, int, int>, T3Layer> by;  // (order, step, offset)
    std::map<int, uint8_t*> by_residue;              // residue-ordered operand planes per step
};


static bool is_layer(const ScanWork& w) { return w.dist_step != 1 || w.dist_offset != 0; }

bool tensor_layer_ok(const T3Plan& plan, const ScanWork& w) {
    return (w.order == 2 || w.order == 3 || (w.order == 4 && w.d.snps >= 4)) && w.dist_n == w.d.snps;
}

static const T3Layer* find_layer(const T3Plan& plan, const ScanWork& w) {
    if (!plan.layers) return nullptr;
    std::lock_guard<std::mutex> g(plan.layers->mu);
    auto it = plan.layers->by.find(std::make_tuple(w.order, w.dist_step, w.dist_offset));
    return it == plan.layers->by.end() ? nullptr : &it->second;
}

cudaError_t tensor3_layer(T3Plan& plan, const ScanWork& w, cudaStream_t s) {
    if (!tensor_layer_ok(plan, w)) return cudaErrorInvalidValue;
    if (!plan.layers) plan.layers = new T3Layers;
    std::lock_guard<std::mutex> g(plan.layers->mu);
    const auto key = std::make_tuple(w.order, w.dist_step, w.dist_offset);
    if (plan.layers->by.count(key)) return cudaSuccess;
    uint8_t*& perm = plan.layers->by_residue[w.dist_step];
    if (!perm) {
        // residue class r holds SNPs r + step m, m < ceil((n - r) / step), each as its 2 plane rows
        const int n = w.d.snps, step = w.dist_step;
        const size_t row2 = (size_t)2 * plan.pitch;
        cudaError_t e = cudaMalloc((void**)&perm, (size_t)n * row2);
        for (int r = 0; r < step && r < n && e == cudaSuccess; ++r)
            e = cudaMemcpy2DAsync(perm + (size_t)residue_row(r, step, n) * row2, row2, plan.planes + (size_t)r * row2,
                                  (size_t)step * row2, row2, (size_t)((n - r + step - 1) / step),
                                  cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            cudaFree(perm);
            plan.layers->by_residue.erase(w.dist_step);
            return e;
        }
    }
    const int n = w.d.snps;
    const long long step = w.dist_step, offset = w.dist_offset;
    if (w.order == 4) {
        std::vector<long long> pb;
        std::vector<int4> pi;
        long long combos = 0;
        const long long total = t4_layer_items(n, (int)step, offset, plan.pack != 0, pb, pi, combos);
        T3Layer L;
        L.total = total;
        L.n_tiles = (int)pi.size();
        L.item_combos = (double)combos / std::max(1ll, total);
        cudaError_t e = t3_map(&L.map_kr, perm, 2 * n, plan.pitch, 32, true);
        if (e == cudaSuccess) e = cudaMalloc((void**)&L.item_begin, pb.size() * sizeof(long long));
        if (e == cudaSuccess) e = cudaMalloc((void**)&L.pinfo, std::max<size_t>(1, pi.size()) * sizeof(int4));
        if (e == cudaSuccess)
            e = cudaMemcpy(L.item_begin, pb.data(), pb.size() * sizeof(long long), cudaMemcpyHostToDevice);
        if (e == cudaSuccess && !pi.empty())
            e = cudaMemcpy(L.pinfo, pi.data(), pi.size() * sizeof(int4), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(L.item_begin);
            cudaFree(L.pinfo);
            return e;
        }
        plan.layers->by[key] = L;
        return cudaSuccess;
    }
    if (w.order == 2) {
        // owned prefixes: SNPs i = offset + m step; tiles of IT consecutive owned i (a CTA pair's two
        // i-tiles when the classes pack) in bands of BT (t2l_decode)
        const int IT = plan.pack ? 2 * kT2I : kT2I, BT = plan.pack ? 4 : 8;
        const long long count = offset < n ? (n - offset + step - 1) / step : 0;
        const int tiles = (int)((count + IT - 1) / IT);
        const int bands = (tiles + BT - 1) / BT;
        const int nb = (n + kT2L - 1) / kT2L;
        std::vector<long long> tb((size_t)bands + 1);
        long long total = 0, combos = 0;
        for (int r = 0; r < bands; ++r) {
            tb[r] = total;
            const long long i_first = offset + step * (long long)IT * BT * r;
            const int ca = std::min(BT, tiles - BT * r);
            total += (long long)ca * std::max(0ll, (long long)nb - (i_first + 1) / kT2L);
        }
        tb[bands] = total;
        for (long long i = offset; i < n; i += step) combos += n - 1 - i;
        T3Layer L;
        L.total = total;
        L.n_tiles = tiles;
        L.item_combos = (double)combos / std::max(1ll, total);
        cudaError_t e = t3_map(&L.map_ar, perm, 2 * n, plan.pitch, kT2M, true);
        if (e == cudaSuccess) e = cudaMalloc((void**)&L.item_begin, tb.size() * sizeof(long long));
        if (e == cudaSuccess)
            e = cudaMemcpy(L.item_begin, tb.data(), tb.size() * sizeof(long long), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(L.item_begin);
            return e;
        }
        plan.layers->by[key] = L;
        return cudaSuccess;
    }
    // order 3: owned prefixes (i, j): lexicographic ranks offset + m * step; the pairs
    // (i, j > i) have ranks base(i) + (j - i - 1), base(i) = i (n-1) - i (i-1) / 2
    std::vector<long long> ib((size_t)n + 1), jb((size_t)n + 1);
    std::vector<int> jl;
    long long total = 0, combos = 0;
    for (int i = 0; i < n; ++i) {
        ib[i] = total;
        jb[i] = (long long)jl.size();
        const long long base = (long long)i * (n - 1) - (long long)i * (i - 1) / 2, cnt = n - 1 - i;
        long long t = std::max(0ll, offset - base);
        t += ((offset - base - t) % step + step) % step;  // first t with base + t = offset (mod step)
        for (; t < cnt; t += step) {
            jl.push_back(i + 1 + (int)t);
            combos += n - 2 - i - t;
        }
        // items of J listed j and L l: the pair kernel's (classes that pack) or the per-class kernel's
        const int J = plan.pair3 ? kPxJ : kT3J, L = plan.pair3 ? kPL : kT3L;
        for (size_t a = (size_t)jb[i]; a < jl.size(); a += J) total += (n - 1 - jl[a] + L - 1) / L;
    }
    ib[n] = total;
    jb[n] = (long long)jl.size();
    T3Layer L;
    L.total = total;
    L.item_combos = (double)combos / std::max(1ll, total);
    cudaError_t e = t3_map(&L.map_jr, perm, 2 * n, plan.pitch, 2 * kT3J, true);
    if (e == cudaSuccess) e = cudaMalloc((void**)&L.item_begin, ib.size() * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc((void**)&L.jl_begin, jb.size() * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc((void**)&L.jlist, std::max<size_t>(1, jl.size()) * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(L.item_begin, ib.data(), ib.size() * sizeof(long long), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(L.jl_begin, jb.data(), jb.size() * sizeof(long long), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !jl.empty())
        e = cudaMemcpy(L.jlist, jl.data(), jl.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(L.item_begin);
        cudaFree(L.jl_begin);
        cudaFree(L.jlist);
        return e;
    }
    plan.layers->by[key] = L;
    return cudaSuccess;
}

long long tensor_units(const T3Plan& plan, const ScanWork& w) {
    if (is_layer(w)) {
        const T3Layer* L = find_layer(plan, w);
        return L ? L->total : 0;
    }
    return w.order == 2 ? plan.total2 : w.order == 4 ? plan.total4 : plan.total;
}
double tensor_item_combos(const T3Plan& plan, const ScanWork& w) {
    if (is_layer(w)) {
        const T3Layer* L = find_layer(plan, w);
        return L ? L->item_combos : 1.0;
    }
    return w.order == 2 ? plan.item2_combos : w.order == 4 ? plan.item4_combos : plan.item_combos;
}

void tensor3_release(T3Plan& plan) {
    if (plan.layers) {
        for (auto& kv : plan.layers->by) {
            cudaFree(kv.second.item_begin);
            cudaFree(kv.second.jl_begin);
            cudaFree(kv.second.jlist);
            cudaFree(kv.second.pinfo);
        }
        for (auto& kv : plan.layers->by_residue) cudaFree(kv.second);
        delete plan.layers;
        plan.layers = nullptr;
    }
    cudaFree(plan.planes);
    cudaFree(plan.item_begin);
    cudaFree(plan.item2_begin);
    cudaFree(plan.item4_begin);
    cudaFree(plan.item4_per);
    plan.planes = nullptr;
    plan.item_begin = nullptr;
    plan.item2_begin = nullptr;
    plan.item4_begin = nullptr;
    plan.item4_per = nullptr;
}

// Bound on |single-precision estimate - exact key / (ln2 * 2^32)| over the 81
// terms of one combination: with N the number of samples every partial sum is
// at most 2 N lg2 N (81 roundings of at most 2^-24 of it), lg2.approx is
// within 2^-18 of log2 on every input the kernel can see (measured worst case
// 1.93e-6, checked exhaustively against FP64 by fiu_probe_lg2_error), the
// x + 2^-20 shift moves each term by at most 2^-20 / ln 2 (counts below 16)
// or one rounding of the count, and the integer table rounds each term by
// 1/2.  Doubled.
static double t3_margin(int n_samples) {
    const double N = n_samples, lgN = std::log2(std::max(2.0, N)), B = 2 * N * lgN;
    const double u = std::ldexp(1.0, -24), e20 = std::ldexp(1.0, -20), e_lg2 = std::ldexp(1.0, -18);
    const double err = 81 * u * B + 2 * N * (18 * u + e_lg2) + 81 * e20 / std::log(2.0) +
                       2 * N * std::ldexp(1.0, -23) / std::log(2.0) + 81 * 0.5 / (std::log(2.0) * 4294967296.0);
    return 2 * err + 1e-3;
}

// Self-check of the bounded mbarrier wait the tensor kernels use: one thread
// initialises an mbarrier (one arrival expected), arrives on it first when
// `arrive` is set, then waits for phase 0 with the given limit in the same
// try-wait loop as t3_wait.  Without the arrival nothing completes the phase
// and the wait must give up after the limit; out[0] = 1 if it completed,
// out[1] = elapsed ns.
__global__ void t3_wait_probe_kernel(unsigned long long limit_ns, int arrive, unsigned long long* out) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (arrive) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&bar)) : "memory");
    const unsigned long long t0 = t3_now();
    bool done = false;
    for (;;) {
        if (t3_try(smem_u32(&bar), 0)) {
            done = true;
            break;
        }
        if (t3_now() - t0 > limit_ns) break;
    }
    out[0] = done ? 1 : 0;
    out[1] = t3_now() - t0;
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bar)) : "memory");
}

cudaError_t probe_wait_limit(unsigned limit_us, int arrive, int* completed, double* elapsed_ms, cudaStream_t s) {
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&d, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    unsigned long long h[2] = {0, 0};
    t3_wait_probe_kernel<<<1, 32, 0, s>>>((unsigned long long)limit_us * 1000ull, arrive, d);
    count_launch();
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    *completed = (int)h[0];
    *elapsed_ms = (double)h[1] / 1e6;
    return e;
}

// Every input of t3_lg2 in the kernel is x = (float)(c + 2^-20) for an integer
// count c in [0, max_c]; largest |t3_lg2(x) - log2(x)| over them, log2 in FP64.
__global__ void t3_lg2_probe_kernel(unsigned max_c, unsigned long long* worst_bits) {
    double worst = 0;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c <= max_c; c += gridDim.x * blockDim.x) {
        const float x = (float)c + 9.5367431640625e-07f;
        const double err = fabs((double)t3_lg2(x) - log2((double)x));
        worst = fmax(worst, err);
    }
    atomicMax(worst_bits, (unsigned long long)__double_as_longlong(worst));  // non-negative doubles order as integers
}

cudaError_t probe_lg2_error(unsigned max_c, double* max_abs_err, cudaStream_t s) {
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&d, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    unsigned long long h = 0;
    e = cudaMemsetAsync(d, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        t3_lg2_probe_kernel<<<256, 256, 0, s>>>(max_c, d);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    double v;
    memcpy(&v, &h, sizeof(v));
    *max_abs_err = v;
    return e;
}

// Clusters of two CTAs of a pair kernel that fit on the device at once (a TPC
// each); 0 when the occupancy query is not available.
template <class K>
static int pair_clusters(K* kernel, int threads, size_t smem) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(2, 1, 1);
    cfg.blockDim = dim3(threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int c = 0;
    if (cudaOccupancyMaxActiveClusters(&c, kernel, &cfg) != cudaSuccess || c < 1) {
        cudaGetLastError();
        c = 0;
    }
    return c;
}

cudaError_t launch_tensor3(const ScanWork& w, const T3Plan& plan, long long g0, long long g1, const CandSink& sink,
                           uint32_t* dump, const uint32_t* single, const uint4* pairs, const uint4* triples,
                           int* status, cudaStream_t s, int sms) {
    if (w.order == 4) {
        if (is_layer(w)) {
            const T3Layer* L = find_layer(plan, w);
            if (!L || !tensor_layer_ok(plan, w)) return cudaErrorInvalidValue;
            return launch_tensor4(w, plan.map_l, plan.map_a2, L->map_kr, plan.map_i, L->item_begin, nullptr,
                                  plan.k_cases, plan.pack, g0, g1, sink, dump, single, pairs, triples, status, s, sms,
                                  L->pinfo, L->n_tiles);
        }
        return launch_tensor4(w, plan.map_l, plan.map_a2, plan.map_k4, plan.map_i, plan.item4_begin, plan.item4_per,
                              plan.k_cases, plan.pack, g0, g1, sink, dump, single, pairs, triples, status, s, sms);
    }
    // set once, by whichever host thread comes first (thread-safe static initialisation)
    static const cudaError_t attr = [] {
        cudaError_t e = cudaFuncSetAttribute(tensor3_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kT3Smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(tensor3_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kT3Smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(tensor2_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kT2Smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(tensor2_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kT2Smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(tensor2x_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kT2xSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(tensor2x_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kT2xSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(tensor3x_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPxSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(tensor3x_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPxSmem);
        return e;
    }();
    if (attr != cudaSuccess) return attr;
    const long long items = g1 - g0;
    if (items <= 0) return cudaSuccess;
    const double scale = 1.0 / (std::log(2.0) * 4294967296.0);
    const double thr = ((double)sink.thr - (double)w.base_key) * scale - t3_margin(w.d.n_cases + w.d.n_ctrls);
    const float thr_f = (float)std::max(-3.0e38, std::min(3.0e38, thr));
    const unsigned grid = (unsigned)(items < sms ? items : sms);
    if (w.order == 2) {
        // a Distribution layer: A rows from the residue-ordered planes, the layer's tiles
        const T3Layer* L = is_layer(w) ? find_layer(plan, w) : nullptr;
        if (is_layer(w) && (!L || !tensor_layer_ok(plan, w))) return cudaErrorInvalidValue;
        const long long* ib = L ? L->item_begin : plan.item2_begin;
        const int nt = L ? L->n_tiles : plan.n_itiles;
        if (plan.pair2) {
            static const int max_clusters = pair_clusters(tensor2x_kernel<false>, kT2Threads, kT2xSmem);
            const long long clusters = std::min<long long>(items, max_clusters > 0 ? max_clusters : sms / 2);
            const unsigned grid2 = (unsigned)(2 * std::max(1ll, clusters));
            const T2Maps maps2{L ? L->map_ar : plan.map_a2, plan.map_a2};  // both boxes 128 rows
            if (L)
                tensor2x_kernel<true><<<grid2, kT2Threads, kT2xSmem, s>>>(maps2, w, ib, nt, g0, g1, plan.k_cases,
                                                                         plan.pack, sink, thr_f, dump, single, status);
            else
                tensor2x_kernel<false><<<grid2, kT2Threads, kT2xSmem, s>>>(maps2, w, ib, nt, g0, g1, plan.k_cases,
                                                                          plan.pack, sink, thr_f, dump, single, status);
        } else {
            const T2Maps maps2{L ? L->map_ar : plan.map_a2, plan.map_b2};
            if (L)
                tensor2_kernel<true><<<grid, kT2Threads, kT2Smem, s>>>(maps2, w, ib, nt, g0, g1, plan.k_cases,
                                                                       plan.pack, sink, thr_f, dump, single, status);
            else
                tensor2_kernel<false><<<grid, kT2Threads, kT2Smem, s>>>(maps2, w, ib, nt, g0, g1, plan.k_cases,
                                                                        plan.pack, sink, thr_f, dump, single, status);
        }
        count_launch();
        return cudaGetLastError();
    }
    T3Maps maps{plan.map_l, plan.map_j, plan.map_i};
    if (plan.pair3) {
        static const int max_clusters = pair_clusters(tensor3x_kernel<false>, kPThreads, kPxSmem);
        const long long clusters = std::min<long long>(items, max_clusters > 0 ? max_clusters : sms / 2);
        const unsigned grid2 = (unsigned)(2 * std::max(1ll, clusters));
        if (is_layer(w)) {
            const T3Layer* L = find_layer(plan, w);
            if (!L || !tensor_layer_ok(plan, w)) return cudaErrorInvalidValue;
            const T3Maps lmaps{plan.map_l, L->map_jr, plan.map_i};
            tensor3x_kernel<true><<<grid2, kPThreads, kPxSmem, s>>>(lmaps, plan.map_a2, w, L->item_begin, g0, g1,
                                                                    plan.k_cases, plan.pack, sink, thr_f, dump, single,
                                                                    pairs, status, L->jl_begin, L->jlist);
        } else {
            tensor3x_kernel<false><<<grid2, kPThreads, kPxSmem, s>>>(maps, plan.map_a2, w, plan.item_begin, g0, g1,
                                                                     plan.k_cases, plan.pack, sink, thr_f, dump,
                                                                     single, pairs, status, nullptr, nullptr);
        }
        count_launch();
        return cudaGetLastError();
    }
    if (is_layer(w)) {
        const T3Layer* L = find_layer(plan, w);
        if (!L || !tensor_layer_ok(plan, w)) return cudaErrorInvalidValue;
        const T3Maps lmaps{plan.map_l, L->map_jr, plan.map_i};
        tensor3_kernel<true><<<grid, kT3Threads, kT3Smem, s>>>(lmaps, w, L->item_begin, g0, g1, plan.k_cases, sink,
                                                               thr_f, dump, single, pairs, status, L->jl_begin,
                                                               L->jlist);
    } else {
        tensor3_kernel<false><<<grid, kT3Threads, kT3Smem, s>>>(maps, w, plan.item_begin, g0, g1, plan.k_cases, sink,
                                                                thr_f, dump, single, pairs, status, nullptr, nullptr);
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace fiu
