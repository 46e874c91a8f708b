// Device helpers shared by the tcgen05 kernels (tensor3.cu: orders 2 and 3,
// tensor4.cu: order 4): bounded mbarrier waits, TMA copies, shared-memory
// matrix descriptors, exact integer <-> float views and the fast log2.
#pragma once

#include <cudaTypedefs.h>

#include "elided_prefix.cuh"

namespace fiu {

constexpr int kT3KB = 128;                                // samples (= e4m3 bytes) per pipeline stage
constexpr unsigned long long kT3LimitNs = 2000000000ull;  // 2 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long t3_now() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool t3_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p;}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase.  A wait that runs past the limit raises
// the CTA's abort flag; every other waiter then gives up at once.
__device__ __forceinline__ bool t3_wait(uint32_t bar, uint32_t parity, volatile int* abort) {
    const unsigned long long t0 = t3_now();
    for (;;) {
        if (t3_try(bar, parity)) return true;
        if (*abort) return false;
        if (t3_now() - t0 > kT3LimitNs) {
            *abort = 1;
            return false;
        }
    }
}

// Bounded wait that ignores the abort flag (draining copies and MMAs in flight).
__device__ __forceinline__ bool t3_drain(uint32_t bar, uint32_t parity) {
    const unsigned long long t0 = t3_now();
    for (;;) {
        if (t3_try(bar, parity)) return true;
        if (t3_now() - t0 > kT3LimitNs) return false;
    }
}

// ---- CTA pairs (cluster of two CTAs, tcgen05 cta_group::2) ----------------
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_id() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_count() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
// Shared::cluster address of the variable at shared address `a` in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t cluster_addr(uint32_t a, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
// Every thread of both CTAs (release / acquire at cluster scope).
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ bool t3_try_cl(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p;}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// t3_wait for a barrier that the other CTA of the pair (or its MMA commits) completes.
__device__ __forceinline__ bool t3_wait_cl(uint32_t bar, uint32_t parity, volatile int* abort) {
    const unsigned long long t0 = t3_now();
    for (;;) {
        if (t3_try_cl(bar, parity)) return true;
        if (*abort) return false;
        if (t3_now() - t0 > kT3LimitNs) {
            *abort = 1;
            return false;
        }
    }
}
__device__ __forceinline__ bool t3_drain_cl(uint32_t bar, uint32_t parity) {
    const unsigned long long t0 = t3_now();
    for (;;) {
        if (t3_try_cl(bar, parity)) return true;
        if (t3_now() - t0 > kT3LimitNs) return false;
    }
}
// Arrival on an mbarrier of either CTA of the pair (cluster address).
__device__ __forceinline__ void arrive_cl(uint32_t cluster_bar) {
    asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(cluster_bar) : "memory");
}
// TMA tile load into this CTA's shared memory whose completion is counted on an
// mbarrier of either CTA of the pair (cluster address).
__device__ __forceinline__ void t3_tma_pair(uint32_t dst, const CUtensorMap* m, int x, int y, uint32_t cluster_bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, "
        "{%2, %3}], [%4];" ::"r"(dst),
        "l"((uint64_t)m), "r"(x), "r"(y), "r"(cluster_bar)
        : "memory");
}
// Arrival, once the MMAs issued so far by this thread completed, on the mbarrier
// at shared address `bar` of both CTAs of the pair.
__device__ __forceinline__ void commit_pair(uint32_t bar) {
    const uint16_t both = 3;
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(bar),
        "h"(both));
}

__device__ __forceinline__ void t3_tma(uint32_t dst, const CUtensorMap* m, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(dst),
        "l"((uint64_t)m), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// tcgen05 shared-memory descriptor, K-major with 128-byte swizzle: start >> 4,
// leading byte offset 16 (unused for swizzled K-major), stride byte offset
// 1024 (8 rows of 128 bytes), version 1 at bit 46, layout SWIZZLE_128B (2) at
// bits 61-63.  Within the 128-byte swizzle atom the K offset is added to the
// start address (tiles are 1024-byte aligned).
__device__ __forceinline__ uint64_t t3_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ float u2f(uint32_t v) {  // exact for v < 2^23
    return __uint_as_float(0x4B000000u | v) - 8388608.0f;
}

__device__ __forceinline__ uint32_t f2u(float f) {  // f an exact integer in [0, 2^23)
    return __float_as_uint(f + 8388608.0f) & 0x7FFFFFu;
}

// Row (SNP position) of SNP j in the operand planes ordered by residue mod
// step (SNPs r, r + step, .. for r = 0, 1, ..; residue r holds
// n / step + (r < n % step) SNPs).
__host__ __device__ __forceinline__ int residue_row(int j, int step, int n) {
    const int r = j % step;
    return r * (n / step) + min(r, n % step) + j / step;
}

__device__ __forceinline__ float t3_lg2(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

}  // namespace fiu
