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

// The scratch, zero-filled when the module loads. In host code this name is only a host-side
// stand-in: kernels get the device address that cudaGetSymbolAddress returns for the current device.
static __device__ __align__(256) StaticScanScratch g_static_scan;

// Device address of the scratch on the current device. Looked up on every call, not cached: after
// the application resets the device, the module is loaded again and a cached address would be stale.
// The lookup allocates nothing; the first one on a device loads the module, which is why the first
// call must come before any stream capture.
cudaError_t scratch_address(StaticScanScratch** out) {
    return cudaGetSymbolAddress(reinterpret_cast<void**>(out), g_static_scan);
}

}  // namespace

namespace gs {

// Test hook behind gs_debug_set_sequence(NULL, seq): sets the scan's sequence number on the current
// device (synchronous), so a test can make the lookback-word tags wrap without 2^26 calls.
cudaError_t static_scan_set_sequence(uint32_t seq) {
    StaticScanScratch* scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess) return e;
    return cudaMemcpy(&scratch->ctl.seq, &seq, sizeof(seq), cudaMemcpyHostToDevice);
}

}  // namespace gs

extern "C" int gs_exclusive_scan_static(const uint32_t* d_in, uint32_t* d_out, uint32_t n, uint32_t* d_total,
                                        void* stream) {
    if (n > kStaticScanMaxN) return GS_ERR_INVALID;  // beyond the fixed scratch: 2^24 entries at most
    if ((!d_in || !d_out) && n) return GS_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaGetLastError();  // an error left behind by earlier, unrelated work is not this call's failure
    StaticScanScratch* scratch = nullptr;
    if (scratch_address(&scratch) != cudaSuccess) return GS_ERR_CUDA;
    // once work is queued, a failure waits for the stream before returning, so the caller never
    // reuses d_out or d_total while the scan may still write them
    auto fail_after_queue = [s]() {
        cudaStreamSynchronize(s);
        cudaGetLastError();
        return GS_ERR_CUDA;
    };
    if (n && d_in != d_out &&
        cudaMemcpyAsync(d_out, d_in, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return fail_after_queue();
    // the counters start at zero on every call; the lookback words are tagged with the call's sequence
    // number instead, and cleared only on the call where those tags wrap
    gs::launch_frame_begin(&scratch->ctl, scratch->words, kStaticScanWords, s);
    uint32_t* total = d_total ? d_total : &scratch->total;
    gs::launch_exclusive_scan(d_out, n, total, &scratch->ctl, scratch->words, 0, s);
    if (cudaGetLastError() != cudaSuccess) return fail_after_queue();
    uint32_t status = 0;
    if (cudaMemcpyAsync(&status, &scratch->ctl.status, sizeof(status), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return fail_after_queue();
    if (cudaStreamSynchronize(s) != cudaSuccess) return GS_ERR_CUDA;
    return (status & gs::kDevTimeout) ? GS_ERR_TIMEOUT : GS_OK;
}
