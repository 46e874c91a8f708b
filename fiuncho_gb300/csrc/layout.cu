// Device layouts of a data set and the stand-alone combine kernels.
#include "internal.h"

namespace fiu {

// ref [snps][rows] -> tr [rows][snps] (uint64), 32x32 tiles through shared memory.
__global__ void transpose_kernel(const uint64_t* __restrict__ ref, uint64_t* __restrict__ tr, int snps, int rows) {
    __shared__ uint64_t tile[32][33];
    const int r0 = blockIdx.x * 32, s0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int s = s0 + i, r = r0 + threadIdx.x;
        if (s < snps && r < rows) tile[i][threadIdx.x] = ref[(size_t)s * rows + r];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, s = s0 + threadIdx.x;
        if (s < snps && r < rows) tr[(size_t)r * snps + s] = tile[threadIdx.x][i];
    }
}

cudaError_t launch_transpose(const uint64_t* ref, uint64_t* tr, int snps, int rows, cudaStream_t s) {
    dim3 grid((rows + 31) / 32, (snps + 31) / 32), block(32, 8);
    if (grid.y > 65535) return cudaErrorInvalidValue;
    transpose_kernel<<<grid, block, 0, s>>>(ref, tr, snps, rows);
    count_launch();
    return cudaGetLastError();
}

// One-hot check (tests/dataset.cpp:25-44 of the reference asserts the
// per-class popcount; this asks for the stronger exact form): for every SNP and
// class the three rows are pairwise disjoint and their union is exactly the
// bit set of the class's samples (full words, then the right-aligned partial
// word, then zero padding).  Sets *bad on any violation.
__global__ void onehot_kernel(const uint64_t* __restrict__ ref, int snps, int cw, int tw, int n_cases, int n_ctrls,
                              int* bad) {
    const size_t per_snp = 3 * (size_t)(cw + tw);
    const long long total = (long long)snps * (cw + tw);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int snp = (int)(e / (cw + tw));
        int w = (int)(e - (long long)snp * (cw + tw));
        const bool cls = w >= cw;
        const int W = cls ? tw : cw;
        const int n = cls ? n_ctrls : n_cases;
        if (cls) w -= cw;
        const uint64_t* base = ref + snp * per_snp + (cls ? 3 * (size_t)cw : 0);
        const uint64_t r0 = base[w], r1 = base[W + w], r2 = base[2 * W + w];
        const int full = n / 64, rem = n % 64;
        const uint64_t want = w < full ? ~0ull : (w == full && rem ? ((1ull << rem) - 1) : 0ull);
        if (((r0 & r1) | (r0 & r2) | (r1 & r2)) != 0 || (r0 | r1 | r2) != want) atomicOr(bad, 1);
    }
}

cudaError_t launch_onehot_check(const uint64_t* ref, int snps, int cw, int tw, int n_cases, int n_ctrls, int* bad,
                                cudaStream_t s) {
    const long long total = (long long)snps * (cw + tw);
    const int grid = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
    onehot_kernel<<<grid > 0 ? grid : 1, 256, 0, s>>>(ref, snps, cw, tw, n_cases, n_ctrls, bad);
    count_launch();
    return cudaGetLastError();
}

// GenotypeTable::combine (src/base/gt_combine.cpp:3-27), both classes:
// out[(i*3+j)*W + w] = t1[i*W + w] & t2[j*W + w].
__global__ void combine_kernel(const uint64_t* __restrict__ t1, int size1, const uint64_t* __restrict__ t2, int cw,
                               int tw, uint64_t* __restrict__ out) {
    const long long nc = 3ll * size1 * cw, total = nc + 3ll * size1 * tw;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const bool cls = e >= nc;
        const int W = cls ? tw : cw;
        const long long f = cls ? e - nc : e;
        const long long row = f / W;
        const int w = (int)(f - row * W);
        const int i = (int)(row / 3), j = (int)(row % 3);
        const uint64_t* a = t1 + (cls ? (size_t)size1 * cw : 0);
        const uint64_t* b = t2 + (cls ? 3 * (size_t)cw : 0);
        out[e] = a[(size_t)i * W + w] & b[(size_t)j * W + w];
    }
}

cudaError_t launch_combine(const uint64_t* t1, int size1, const uint64_t* t2, int cw, int tw, uint64_t* out,
                           cudaStream_t s) {
    combine_kernel<<<1024, 256, 0, s>>>(t1, size1, t2, cw, tw, out);
    count_launch();
    return cudaGetLastError();
}

// GenotypeTable::combine_and_popcnt (src/base/gt_popcnt.cpp:4-35): one warp per
// cell, lanes over words; cells 3*size1 .. ct_size-1 are zeroed.
__global__ void combine_popcnt_kernel(const uint64_t* __restrict__ t1, int size1, const uint64_t* __restrict__ t2,
                                      int cw, int tw, uint32_t* __restrict__ cases_out,
                                      uint32_t* __restrict__ ctrls_out, int ct_size) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int q = warp; q < 2 * ct_size; q += nwarps) {
        const int cls = q >= ct_size, cell = cls ? q - ct_size : q;
        uint32_t* o = cls ? ctrls_out : cases_out;
        if (cell >= 3 * size1) {
            if (lane == 0) o[cell] = 0;
            continue;
        }
        const int W = cls ? tw : cw;
        const uint64_t* a = t1 + (cls ? (size_t)size1 * cw : 0) + (size_t)(cell / 3) * W;
        const uint64_t* b = t2 + (cls ? 3 * (size_t)cw : 0) + (size_t)(cell % 3) * W;
        uint32_t acc = 0;
        for (int w = lane; w < W; w += 32) acc += __popcll(a[w] & b[w]);
        for (int o2 = 16; o2; o2 >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o2);
        if (lane == 0) o[cell] = acc;
    }
}

cudaError_t launch_combine_popcnt(const uint64_t* t1, int size1, const uint64_t* t2, int cw, int tw,
                                  uint32_t* cases_out, uint32_t* ctrls_out, int ct_size, cudaStream_t s) {
    combine_popcnt_kernel<<<256, 256, 0, s>>>(t1, size1, t2, cw, tw, cases_out, ctrls_out, ct_size);
    count_launch();
    return cudaGetLastError();
}

// AND+POPC+ADD throughput probe: every thread loops over 16 independent
// accumulators on register data; reads 1024 words, writes one word per thread.
__global__ void popc_probe_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int iters) {
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t v[16], acc[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        v[k] = in[(tid + k * 37) & 1023];
        acc[k] = 0;
    }
    uint32_t x = in[tid & 1023] | 1u;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 16; ++k) acc[k] += __popc(v[k] & x);
        x = x * 1664525u + 1013904223u;
    }
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) s += acc[k];
    out[tid] = s;
}

cudaError_t probe_popc_rate(int sms, cudaStream_t s, double* rate) {
    const int blocks = sms * 4, threads = 256, iters = 40000;
    uint32_t *in = nullptr, *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&in, 1024 * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&out, (size_t)blocks * threads * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(in, 0x5a, 1024 * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
        cudaEventRecord(e0, s);
        popc_probe_kernel<<<blocks, threads, 0, s>>>(in, out, iters);
        count_launch();
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        float ms = 0;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && ms < best) best = ms;
    }
    if (e == cudaSuccess) *rate = (double)blocks * threads * iters * 16.0 / (best * 1e-3);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFreeAsync(in, s);
    cudaFreeAsync(out, s);
    return e;
}

}  // namespace fiu
