// noalloc.cu — the exclusive scan for callers that cannot allocate device
// memory.
//
// sr_exclusive_scan_i32 takes its look-back scratch from cudaMallocAsync.
// Some callers cannot allow that: a host that hands all device memory to
// its own allocator or runs under a hard memory budget forbids third-party
// allocations, and a frame loop with a fixed latency budget cannot risk an
// allocation call that may wait on the device.  This variant runs the same
// kernel with its scratch in a fixed array compiled into the library: every
// GPU that loads the library holds SR_NOALLOC_SCAN_SCRATCH_BYTES of it until
// the process exits.
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/sr.h"
#include "kernels.h"

namespace sr {
sr_status report_error(sr_status s, const char* msg);   // api.cu
}

namespace {

// Look-back words for the largest scan, then the tile counter
// (scan_status_words(n) + 1 words of 8 bytes, with a few to spare).
constexpr size_t kNoallocWords = SR_NOALLOC_SCAN_SCRATCH_BYTES / sizeof(uint64_t);

static __device__ __align__(256) uint64_t g_noalloc_scan_scratch[kNoallocWords];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
uint64_t* g_scratch_addr[kMaxDevices] = {};
uint32_t* g_status_addr[kMaxDevices] = {};

// Device addresses, on the current device, of the scratch array and of the
// standalone scans' status word, looked up once per device (the array's
// name in host code is only a stand-in).  A cudaDeviceReset unloads the
// library's device code, so these addresses do not survive one.
sr_status scratch_on_current_device(uint64_t** scratch, uint32_t** status) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sr::report_error(SR_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return sr::report_error(SR_ERR_INVALID_ARG, "device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
        if (e != cudaSuccess || !p) return sr::report_error(SR_ERR_CUDA, cudaGetErrorString(e));
        uint32_t* w = nullptr;
        e = sr::standalone_scan_status(&w);
        if (e != cudaSuccess || !w) return sr::report_error(SR_ERR_CUDA, cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<uint64_t*>(p);
        g_status_addr[dev] = w;
    }
    *scratch = g_scratch_addr[dev];
    *status = g_status_addr[dev];
    return SR_OK;
}

}  // namespace

extern "C" sr_status sr_exclusive_scan_i32_noalloc(const int32_t* d_in, int32_t* d_out, int64_t n, void* stream) {
    if (n < 0 || n > SR_NOALLOC_SCAN_MAX_N) {
        char msg[160];
        snprintf(msg, sizeof msg, "scan length %lld outside 0..%lld (the fixed scratch of the allocation-free scan)",
                 (long long)n, (long long)SR_NOALLOC_SCAN_MAX_N);
        return sr::report_error(SR_ERR_INVALID_ARG, msg);
    }
    if (!d_out || (n > 0 && !d_in)) return sr::report_error(SR_ERR_INVALID_ARG, "NULL device pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint64_t* scratch = nullptr;
    uint32_t* status = nullptr;
    sr_status s = scratch_on_current_device(&scratch, &status);
    if (s != SR_OK) return s;
    cudaError_t e;
    if (n == 0) {
        e = cudaMemsetAsync(d_out, 0, sizeof(int32_t), st);
        return e == cudaSuccess ? SR_OK : sr::report_error(SR_ERR_CUDA, cudaGetErrorString(e));
    }
    const size_t words = sr::scan_status_words(n) + 1;
    if (words > kNoallocWords) return sr::report_error(SR_ERR_INTERNAL, "scan scratch too small");
    // the previous call's look-back words and tile counter stay in the
    // array: clear the part this call uses.  A look-back that gives up sets
    // a bit in the status word, which sr_scan_status reports.
    e = cudaMemsetAsync(scratch, 0, words * sizeof(uint64_t), st);
    if (e != cudaSuccess) return sr::report_error(SR_ERR_CUDA, cudaGetErrorString(e));
    uint32_t* counter = reinterpret_cast<uint32_t*>(scratch + words - 1);
    sr::launch_exclusive_scan_i32(d_in, d_out, n, scratch, counter, status, st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return sr::report_error(SR_ERR_CUDA, cudaGetErrorString(e));
    return SR_OK;
}
