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
//
// The table's entries are computed on the host with the same expression as the
// allocating entry points (round(c ln c 2^32) in double precision), so both
// give bit-identical results, and copied into the array once per device at
// set-up; calls afterwards only read it.
#include <cmath>
#include <mutex>

#include "../../include/fiuncho_gpu.h"
#include "internal.h"

namespace fiu {

static __device__ __align__(256) long long g_noalloc_ftab[FIU_NOALLOC_MAX_SAMPLES + 1];

namespace {
constexpr int kMaxDevices = 64;
constexpr size_t kTabBytes = sizeof(long long) * (FIU_NOALLOC_MAX_SAMPLES + 1);
std::mutex g_noalloc_lock;
long long g_host_tab[FIU_NOALLOC_MAX_SAMPLES + 1];  // filled once, then read-only
bool g_host_tab_ready = false;
struct DeviceTable {
    void* context = nullptr;  // the CUDA context the set-up ran in
    long long* addr = nullptr;
};
DeviceTable g_noalloc_dev[kMaxDevices];

typedef int (*CtxGetCurrentFn)(void**);
CtxGetCurrentFn ctx_get_current() {
    static const CtxGetCurrentFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuCtxGetCurrent", &p, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (CtxGetCurrentFn)p;
        return (CtxGetCurrentFn) nullptr;
    }();
    return fn;
}

// Device address of the filled table on the current device.  Set-up, with the
// device current, the first time a device (or a new context on it, e.g. after
// a cudaDeviceReset) is seen: cudaGetSymbolAddress -- the array's name is only
// a host-side stand-in in host code -- and a synchronous copy of the table.
cudaError_t noalloc_table(long long** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    e = cudaSetDevice(dev);  // initialises the device's primary context if no call has yet
    if (e != cudaSuccess) return e;
    void* ctx = nullptr;
    const CtxGetCurrentFn get = ctx_get_current();
    if (!get || get(&ctx) != 0 || !ctx) return cudaErrorInitializationError;
    std::lock_guard<std::mutex> guard(g_noalloc_lock);
    DeviceTable& t = g_noalloc_dev[dev];
    if (t.context != ctx || !t.addr) {
        if (!g_host_tab_ready) {
            for (long long c = 0; c <= FIU_NOALLOC_MAX_SAMPLES; ++c)
                g_host_tab[c] = c < 2 ? 0 : (long long)llround((double)c * std::log((double)c) * 4294967296.0);
            g_host_tab_ready = true;
        }
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_ftab);
        if (e != cudaSuccess) return e;
        e = cudaMemcpy(p, g_host_tab, kTabBytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
        t.context = ctx;
        t.addr = static_cast<long long*>(p);
    }
    *out = t.addr;
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
    // counts above n (tables that are not one-hot) are evaluated in FP64 by the kernel
    if (launch_mi(d_cases, d_ctrls, cells, count, (int)n_cases, (int)n_ctrls, ftab, n, 0, d_out, nullptr, s) !=
        cudaSuccess)
        return FIU_ERR_CUDA;
    return FIU_OK;
}
