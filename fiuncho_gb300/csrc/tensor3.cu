// Order-3 contingency tables on the 5th-generation tensor cores (tcgen05).
//
// For one-hot data the 8 core cells of a combination (i, j, l) -- genotypes
// x, y, z in {0, 1} -- are dot products over the samples of one class:
//     core[x][y][z] = sum_s a_ix(s) a_jy(s) a_lz(s),
// where a_gx(s) is bit "genotype of SNP g == x" of sample s.  A work item is
// (i, 32 consecutive j, 128 consecutive l); it is one GEMM per class
//     D[(j,x,y), (l,z)] = sum_s A[(j,x,y), s] B[(l,z), s],
// with A = a_ix & a_jy (128 rows) and B = a_lz (256 rows) expanded from bits
// to e4m3 0/1 (0x38 = 1.0) in shared memory, in the canonical K-major
// no-swizzle core-matrix layout (8 rows x 16 bytes per core matrix), and
// accumulated exactly in FP32 in tensor memory: cases in columns 0-255,
// controls in columns 256-511 (M = 128, N = 256, K = 32 per instruction).
// Two shared-memory stages of 128 samples pipeline the bit expansion of step
// s+1 against the MMAs of step s (one mbarrier per stage, committed by the
// issuing thread).  The epilogue reads the accumulators with tcgen05.ld,
// transposes each quad of rows (x, y) through shared memory so that one
// thread sees the 8 cells of a combination, and derives the full 27-cell
// table exactly with the pair/single cores (as the reduced-work CUDA-core
// kernel does), then the fixed-point MI and the top-N filter.
//
// Reference semantics: GenotypeTable::combine_and_popcnt for order 3
// (src/base/gt_popcnt.cpp:4-35) over the combinations ThreadedSearch visits
// (include/fiuncho/ThreadedSearch.h:157-180) with one worker.
#include "elided_prefix.cuh"

namespace fiu {

constexpr int kT3Threads = 256;
constexpr int kT3J = 32, kT3L = 128;          // SNPs per tile
constexpr int kT3M = 4 * kT3J, kT3N = 2 * kT3L;  // 128 x 256 GEMM tile
constexpr int kT3KB = 128;                    // samples (= e4m3 bytes) per stage
constexpr int kT3StageA = kT3M * kT3KB, kT3StageB = kT3N * kT3KB;
constexpr int kT3Stage = kT3StageA + kT3StageB;  // 48 KB
constexpr int kT3Lut = 256 * 8;
constexpr int kT3Ebuf = 8 * 1024 * 4;            // per-warp transpose buffers
constexpr size_t kT3Smem = 2 * kT3Stage + kT3Lut + kT3Ebuf;  // 130 KB: one CTA per SM
constexpr unsigned kT3Spin = 1u << 24;           // bounded mbarrier waits

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory descriptor: start >> 4, leading (K-direction core
// matrix) byte offset >> 4 at bit 16, stride (8-row group) byte offset >> 4 at
// bit 32, descriptor version 1 at bit 46, no swizzle.
__device__ __forceinline__ uint64_t t3_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)((8 * 128) >> 4) << 32) |
           ((uint64_t)1 << 46);
}

// Instruction descriptor, kind::f8f6f4: D = F32 (bit 4), A = B = E4M3 (0),
// both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t kT3Idesc = (1u << 4) | ((uint32_t)(kT3N >> 3) << 17) | ((uint32_t)(kT3M >> 4) << 24);

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (unsigned it = 0; it < kT3Spin; ++it) {
        uint32_t ok;
        asm volatile("{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p;}"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}

// Work items of one i: J-tile a starts at j0 = i+1+32a and has
// ceil((n-1-j0)/128) L-tiles starting at l0 = j0+1+128b.
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
        const long long nl = (n - 1 - j + kT3L - 1) / kT3L;
        if (q < nl) {
            j0 = j;
            l0 = j + 1 + kT3L * (int)q;
            return;
        }
        q -= nl;
    }
}

__global__ void __launch_bounds__(kT3Threads, 1)
    tensor3_kernel(ScanWork w, const long long* __restrict__ item_begin, long long g0, long long g1, CandSink sink,
                   uint32_t* dump, const uint32_t* __restrict__ single, const uint4* __restrict__ pairs,
                   int* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    const DevData& d = w.d;
    const int n = d.snps, cw = d.cw, tw = d.tw;
    const size_t per_snp = 3 * (size_t)(cw + tw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint64_t* lut = reinterpret_cast<uint64_t*>(smem + 2 * kT3Stage);
    uint32_t* ebuf = reinterpret_cast<uint32_t*>(smem + 2 * kT3Stage + kT3Lut) + warp * 1024;
    for (int e = tid; e < 256; e += kT3Threads) {
        uint64_t v = 0;
        for (int b = 0; b < 8; ++b)
            if ((e >> b) & 1) v |= 0x38ull << (8 * b);
        lut[e] = v;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar[0])), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar[1])), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const int ks_c = (cw + 1) / 2, ks_t = (tw + 1) / 2;  // K-steps (2 words = 128 samples) per class
    unsigned step = 0;                                  // K-steps issued by this CTA
    bool ok = true;
    const uint32_t n_cls[2] = {(uint32_t)d.n_cases, (uint32_t)d.n_ctrls};

    for (long long g = g0 + blockIdx.x; g < g1; g += gridDim.x) {
        int i, j0, l0;
        t3_decode(item_begin, n, g, i, j0, l0);
        // ---- GEMMs: cases then controls
        for (int ks = 0; ks < ks_c + ks_t; ++ks, ++step) {
            const int cls = ks >= ks_c;
            const int W = cls ? tw : cw;
            const int wb = 2 * (cls ? ks - ks_c : ks);
            const size_t roff = cls ? 3 * (size_t)cw : 0;
            const int s = step & 1;
            uint8_t* sA = smem + s * kT3Stage;
            uint8_t* sB = sA + kT3StageA;
            if (step >= 2 && !mbar_wait(smem_u32(&mbar[s]), ((step >> 1) - 1) & 1)) ok = false;
            // expand: task t -> (row, word half); 8 consecutive tasks fill one 128-byte core-matrix column
            for (int t = tid; t < (kT3M + kT3N) * 2; t += kT3Threads) {
                const int isB = t >= kT3M * 2;
                const int tt = isB ? t - kT3M * 2 : t;
                const int r = (tt & 7) + 8 * (tt >> 4), h = (tt >> 3) & 1;
                const int word = wb + h;
                uint64_t bits = 0;
                if (word < W) {
                    if (isB) {
                        const int l = l0 + (r >> 1), z = r & 1;
                        if (l < n) bits = __ldg(d.ref + (size_t)l * per_snp + roff + (size_t)z * W + word);
                    } else {
                        const int j = j0 + (r >> 2), x = (r >> 1) & 1, y = r & 1;
                        if (j < n)
                            bits = __ldg(d.ref + (size_t)i * per_snp + roff + (size_t)x * W + word) &
                                   __ldg(d.ref + (size_t)j * per_snp + roff + (size_t)y * W + word);
                    }
                }
                uint8_t* base = (isB ? sB : sA) + (r >> 3) * 1024 + (r & 7) * 16 + h * 512;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    uint4 v;
                    const uint64_t lo = lut[(bits >> (16 * c)) & 0xff], hi = lut[(bits >> (16 * c + 8)) & 0xff];
                    v.x = (uint32_t)lo;
                    v.y = (uint32_t)(lo >> 32);
                    v.z = (uint32_t)hi;
                    v.w = (uint32_t)(hi >> 32);
                    *reinterpret_cast<uint4*>(base + c * 128) = v;
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t dcol = tmem + (cls ? 256u : 0u);
                const int first = cls ? ks == ks_c : ks == 0;
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const uint64_t ad = t3_desc(smem_u32(sA) + kk * 256), bd = t3_desc(smem_u32(sB) + kk * 256);
                    const uint32_t acc = (first && kk == 0) ? 0u : 1u;
                    asm volatile("{.reg .pred p; setp.ne.b32 p, %4, 0;\n"
                                 "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;}\n" ::"r"(dcol),
                                 "l"(ad), "l"(bd), "r"(kT3Idesc), "r"(acc));
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    smem_u32(&mbar[s])));
            }
        }
        // ---- all MMAs of the item done (commits track every earlier MMA of the thread)
        if (!mbar_wait(smem_u32(&mbar[(step - 1) & 1]), ((step - 1) >> 1) & 1)) ok = false;
        asm volatile("tcgen05.fence::after_thread_sync;");
        // ---- epilogue: warp w reads TMEM lanes 32(w%4).. (rows), l columns [64(w/4), 64(w/4)+64)
        const int q = warp & 3, hh = warp >> 2;
        const int jl = lane >> 2, xy = lane & 3;
        for (int cc = 0; cc < 8; ++cc) {
            const uint32_t col = (uint32_t)(128 * hh + 16 * cc);
            uint32_t vc[16], vt[16];
            const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + col;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(vc[0]), "=r"(vc[1]), "=r"(vc[2]), "=r"(vc[3]), "=r"(vc[4]), "=r"(vc[5]), "=r"(vc[6]),
                  "=r"(vc[7]), "=r"(vc[8]), "=r"(vc[9]), "=r"(vc[10]), "=r"(vc[11]), "=r"(vc[12]), "=r"(vc[13]),
                  "=r"(vc[14]), "=r"(vc[15])
                : "r"(ta));
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(vt[0]), "=r"(vt[1]), "=r"(vt[2]), "=r"(vt[3]), "=r"(vt[4]), "=r"(vt[5]), "=r"(vt[6]),
                  "=r"(vt[7]), "=r"(vt[8]), "=r"(vt[9]), "=r"(vt[10]), "=r"(vt[11]), "=r"(vt[12]), "=r"(vt[13]),
                  "=r"(vt[14]), "=r"(vt[15])
                : "r"(ta + 256u));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            // transpose: ebuf[((jl*8 + k)*2 + cls)*8 + xy*2 + z]  (FP32 accumulators hold exact integers)
#pragma unroll
            for (int k = 0; k < 8; ++k)
#pragma unroll
                for (int z = 0; z < 2; ++z) {
                    ebuf[((jl * 8 + k) * 2 + 0) * 8 + xy * 2 + z] = (uint32_t)__uint_as_float(vc[2 * k + z]);
                    ebuf[((jl * 8 + k) * 2 + 1) * 8 + xy * 2 + z] = (uint32_t)__uint_as_float(vt[2 * k + z]);
                }
            __syncwarp();
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int ci = lane + 32 * u, cj = ci >> 3, k = ci & 7;
                const int j = j0 + 8 * q + cj, l = l0 + 64 * hh + 8 * cc + k;
                const bool valid = j < n && l < n && l > j;
                long long key = w.base_key;
                if (valid) {
                    uint32_t core[2][8];
#pragma unroll
                    for (int cls = 0; cls < 2; ++cls) {
                        const uint4 a = *reinterpret_cast<const uint4*>(ebuf + ((cj * 8 + k) * 2 + cls) * 8);
                        const uint4 b = *reinterpret_cast<const uint4*>(ebuf + ((cj * 8 + k) * 2 + cls) * 8 + 4);
                        core[cls][0] = a.x; core[cls][1] = a.y; core[cls][2] = a.z; core[cls][3] = a.w;
                        core[cls][4] = b.x; core[cls][5] = b.y; core[cls][6] = b.z; core[cls][7] = b.w;
                    }
                    const uint4 pij = __ldg(pairs + pair_index(i, j, n)), pil = __ldg(pairs + pair_index(i, l, n)),
                                pjl = __ldg(pairs + pair_index(j, l, n));
                    uint32_t t[2][27];
#pragma unroll
                    for (int cls = 0; cls < 2; ++cls)
                        expand3(core[cls], pij, pil, pjl, __ldg(single + i * 4 + cls * 2),
                                __ldg(single + i * 4 + cls * 2 + 1), __ldg(single + j * 4 + cls * 2),
                                __ldg(single + j * 4 + cls * 2 + 1), __ldg(single + l * 4 + cls * 2),
                                __ldg(single + l * 4 + cls * 2 + 1), n_cls[cls], cls, t[cls]);
#pragma unroll
                    for (int c = 0; c < 27; ++c) {
                        const uint32_t a = min(t[0][c], n_cls[0]), b = min(t[1][c], n_cls[1]);
                        key += __ldg(d.ftab + a) + __ldg(d.ftab + b) - __ldg(d.ftab + a + b);
                    }
                    if (dump) {
                        uint32_t* o = dump + ((size_t)pair_index(i, j, n) * n + l) * 54;
#pragma unroll
                        for (int c = 0; c < 27; ++c) {
                            o[c] = t[0][c];
                            o[27 + c] = t[1][c];
                        }
                    }
                }
                const unsigned vmask = __ballot_sync(0xffffffffu, valid);
                if (sink.evaluated && lane == 0 && vmask) atomicAdd(sink.evaluated, (unsigned long long)__popc(vmask));
                const bool pass = valid && key >= sink.thr;
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
            __syncwarp();
        }
        // the next item's first MMA overwrites the accumulators: all reads done first
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
    }
    if (!ok) atomicOr(status, 1);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// Items per i (host): prefix sums item_begin[0..n], item_begin[n] = total.
long long tensor3_items(int n, std::vector<long long>& item_begin) {
    item_begin.assign((size_t)n + 1, 0);
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        item_begin[i] = total;
        for (int j = i + 1; j < n - 1; j += kT3J) total += (n - 1 - j + kT3L - 1) / kT3L;
    }
    item_begin[n] = total;
    return total;
}

cudaError_t launch_tensor3(const ScanWork& w, const long long* item_begin, long long g0, long long g1,
                           const CandSink& sink, uint32_t* dump, const uint32_t* single, const uint4* pairs,
                           int* status, cudaStream_t s, int sms) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(tensor3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kT3Smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long long items = g1 - g0;
    if (items <= 0) return cudaSuccess;
    const unsigned grid = (unsigned)(items < sms ? items : sms);
    tensor3_kernel<<<grid, kT3Threads, kT3Smem, s>>>(w, item_begin, g0, g1, sink, dump, single, pairs, status);
    count_launch();
    return cudaGetLastError();
}

}  // namespace fiu
