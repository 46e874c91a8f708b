// MutualInformation::compute for callers that cannot allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc once they are running:
// applications that hand all device memory to their own pool at start-up and
// forbid later allocations, latency-critical pipelines that cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree imply, and plugin hosts
// (JNI, embedded interpreters) whose memory policy belongs to the host.  For
// them, fiu_mi_compute_noalloc evaluates the search's fixed-point MI over
// caller-owned device tables without allocating anything: its only scratch --
// the c*ln(c) fixed-point table -- lives in the file-scope device array below,
// sized for data sets of at most FIU_NOALLOC_MAX_SAMPLES samples (512 KiB,
// held by every GPU that loads this library until the process exits).
#include <mutex>

#include "../../include/fiuncho_gpu.h"
#include "internal.h"

namespace fiu {

static __device__ __align__(256) long long g_noalloc_ftab[FIU_NOALLOC_MAX_SAMPLES + 1];

// g_noalloc_ftab[c] = round(c * ln(c) * 2^32) for c in [0, n]; every entry
// the MI kernel reads (0..n) is rewritten by each call.
__global__ void noalloc_fill_kernel(long long* __restrict__ ftab, long long n) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c <= n; c += (long long)gridDim.x * blockDim.x)
        ftab[c] = c < 2 ? 0 : llrint((double)c * log((double)c) * 4294967296.0);
}

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_lock;
long long* g_noalloc_addr[kMaxDevices] = {};

// Device address of the table on the current device, looked up once per device.
cudaError_t noalloc_table(long long** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> guard(g_noalloc_lock);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_ftab);
        if (e != cudaSuccess) return e;
        g_noalloc_addr[dev] = static_cast<long long*>(p);
    }
    *out = g_noalloc_addr[dev];
    return cudaSuccess;
}
}  // namespace

}  // namespace fiu

extern "C" int fiu_mi_compute_noalloc(const uint32_t* d_cases, const uint32_t* d_ctrls, size_t cells, size_t count,
                                      unsigned n_cases, unsigned n_ctrls, float* d_out, void* stream) {
    using namespace fiu;
    if (!d_cases || !d_ctrls || !d_out || cells == 0 || n_cases + (unsigned long long)n_ctrls == 0)
        return FIU_ERR_INVALID;
    if ((unsigned long long)n_cases + n_ctrls > FIU_NOALLOC_MAX_SAMPLES) return FIU_ERR_UNSUPPORTED;
    if (count == 0) return FIU_OK;
    long long* ftab = nullptr;
    if (noalloc_table(&ftab) != cudaSuccess) return FIU_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long n = (long long)n_cases + n_ctrls;
    noalloc_fill_kernel<<<(unsigned)((n + 256) / 256), 256, 0, s>>>(ftab, n);
    if (cudaGetLastError() != cudaSuccess) return FIU_ERR_CUDA;
    // counts above n (tables that are not one-hot) are evaluated in FP64 by the kernel
    if (launch_mi(d_cases, d_ctrls, cells, count, (int)n_cases, (int)n_ctrls, ftab, n, 0, d_out, nullptr, s) !=
        cudaSuccess)
        return FIU_ERR_CUDA;
    return FIU_OK;
}
