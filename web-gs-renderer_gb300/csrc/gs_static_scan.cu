// gs_static_scan.cu -- gs_exclusive_scan_static: the decoupled-lookback exclusive scan with its
// scratch memory in a fixed device array, for callers that must not allocate.
//
// gs_exclusive_scan allocates its scratch (lookback words, a counter block, a staging copy) on the
// context. Some callers cannot allow that: cudaMalloc and cudaFree may synchronize the whole device,
// which stalls a real-time frame loop that owns the GPU, and hosts that manage device memory
// themselves (engine-side arenas, plugin sandboxes) forbid a library from allocating behind their
// back. This entry point takes the caller's device buffers and a stream, and its scratch lives in
// g_static_scan below: about 74 KB per GPU that loads the library, held until the process exits.
#include <cstdint>
#include <mutex>

#include "../../include/gs.h"
#include "gs_kernels.h"

namespace {

using gs::FrameCtl;

// Largest n accepted: 2^24 entries = 8192 scan partitions of 2048 entries.
constexpr uint32_t kStaticScanMaxN = 1u << 24;
constexpr uint32_t kStaticScanWords = kStaticScanMaxN / gs::kScanPartition;

struct StaticScanScratch {
    FrameCtl ctl;                       // tickets, sequence number and status word of the scan
    uint32_t total;                     // receives the sum when the caller passes no total pointer
    uint32_t pad[63];
    uint64_t words[kStaticScanWords];   // lookback words, tagged with the call's sequence number
};

// The scratch. In host code this name is only a host-side stand-in: kernels get the device address
// that cudaGetSymbolAddress returns for the current device (see scratch_for_current_device).
static __device__ __align__(256) StaticScanScratch g_static_scan;

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
StaticScanScratch* g_scratch_ptr[kMaxDevices] = {};

// Set-up, once per device, with that device current: looks up the device address of the scratch
// and clears it (lookback words must not start with a stale sequence number). Neither step
// allocates memory.
cudaError_t scratch_for_current_device(StaticScanScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        StaticScanScratch* p = nullptr;
        e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_static_scan);
        if (e != cudaSuccess) return e;
        e = cudaMemset(p, 0, sizeof(StaticScanScratch));
        if (e != cudaSuccess) return e;
        e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int gs_exclusive_scan_static(const uint32_t* d_in, uint32_t* d_out, uint32_t n, uint32_t* d_total,
                                        void* stream) {
    if (n > kStaticScanMaxN) return GS_ERR_INVALID;  // beyond the fixed scratch: 2^24 entries at most
    if ((!d_in || !d_out) && n) return GS_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    StaticScanScratch* scratch = nullptr;
    if (scratch_for_current_device(&scratch) != cudaSuccess) return GS_ERR_CUDA;
    if (n && d_in != d_out &&
        cudaMemcpyAsync(d_out, d_in, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return GS_ERR_CUDA;
    // the counters the scan relies on start at zero on every call (the lookback words do not need
    // clearing: each call tags them with a new sequence number)
    gs::launch_frame_begin(&scratch->ctl, s);
    uint32_t* total = d_total ? d_total : &scratch->total;
    gs::launch_exclusive_scan(d_out, n, total, &scratch->ctl, scratch->words, 0, s);
    if (cudaGetLastError() != cudaSuccess) return GS_ERR_CUDA;
    uint32_t status = 0;
    if (cudaMemcpyAsync(&status, &scratch->ctl.status, sizeof(status), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GS_ERR_CUDA;
    return (status & gs::kDevTimeout) ? GS_ERR_TIMEOUT : GS_OK;
}
