// gs_kernels.h -- launch wrappers of the splat kernels (host side), used by the C ABI in gs_api.cu.
#pragma once
#include <cstdint>
#include <utility>
#include <cuda_runtime.h>

#include "gs_common.cuh"

namespace gs {

// Per-Gaussian raster record written by preprocess (three float4 per Gaussian):
//   r0 = (pixel.x, pixel.y, conic.x, conic.y)
//   r1 = (conic.z, opacity, color.r, color.g)
//   r2 = (color.b, power cut-off below which alpha < 1/255 for sure, 0, 0)
constexpr int kRecFloat4 = 3;

// ---- scene layout -------------------------------------------------------------------------
// packed (reference layout, preprocess.wgsl:16-24) -> rows of the structure-of-arrays layout.
void launch_pack_to_rows(const float* packed, uint32_t n, uint32_t stride, float* rows, cudaStream_t s);
// rows -> packed (used for gradients).

// Launches kernel k on stream s as a programmatic dependent of the kernel before it on s: k's launch
// is set up while that kernel runs and its CTAs start as that kernel's CTAs exit, instead of after the
// whole grid has drained (inside a captured graph the edge stays programmatic). k must call pdl_wait()
// before anything else.
template <typename... Params, typename... Args>
inline void launch_pdl(void (*k)(Params...), dim3 grid, dim3 block, cudaStream_t s, Args&&... args) {
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// ---- frame ----------------------------------------------------------------------------------
// Resets the frame control block and, when given, clears the frame's tile ranges (range_words words,
// every pair to (0xFFFFFFFF, 0): see launch_onesweep).
// flags / flag_words: every lookback word the kernels of this control block use; they are cleared on
// the one frame in 2^26 where the words' 30-bit sequence tags start again at zero.
void launch_frame_begin(FrameCtl* ctl, uint64_t* flags, uint32_t flag_words, cudaStream_t s,
                        uint32_t* ranges = nullptr, uint32_t range_words = 0);

// Up to kMaxMultiViews views of one scene for launch_preprocess_multi: each view's block and frame
// outputs.
constexpr uint32_t kMaxMultiViews = 16;
struct MultiViewFrames {
    const ViewBlock* view[kMaxMultiViews];
    float4* rec[kMaxMultiViews];
    uint4* meta[kMaxMultiViews];
    uint32_t* counts[kMaxMultiViews];
    FrameCtl* ctl[kMaxMultiViews];
    uint32_t* ranges[kMaxMultiViews];  // tile ranges, cleared by launch_frame_begin_multi
    uint32_t range_words[kMaxMultiViews];
    uint64_t* flags[kMaxMultiViews];   // lookback words of each view's frame (see launch_frame_begin)
    uint32_t flag_words[kMaxMultiViews];
    uint32_t count;
};
// launch_frame_begin for every view of mv in one launch (one row of CTAs per view).
void launch_frame_begin_multi(const MultiViewFrames& mv, cudaStream_t s);
// The preprocess of several views of one scene in one pass over the scene's attribute rows (each
// view's FrameCtl must have been reset by launch_frame_begin).
void launch_preprocess_multi(const float* rows, uint32_t stride, uint32_t n, uint32_t tile, const MultiViewFrames& mv,
                             cudaStream_t s);
void launch_preprocess(const float* rows, uint32_t stride, uint32_t n, const ViewBlock* view, uint32_t tile,
                       float4* rec, uint4* meta, uint32_t* counts, FrameCtl* ctl, cudaStream_t s);

// Offset scan (each partition sums its predecessors' published aggregates) fused with emit and the
// sort's digit histograms.
constexpr uint32_t kScanItems = 8;
constexpr uint32_t kScanThreads = 256;
constexpr uint32_t kScanPartition = kScanItems * kScanThreads;
void launch_scan_emit(const uint32_t* counts, const uint4* meta, uint32_t n, uint32_t tiles_x, uint32_t max_instance,
                      uint32_t digit_bits, uint32_t passes, uint32_t* offsets, uint32_t* keys, uint32_t* vals,
                      FrameCtl* ctl, uint64_t* flags, uint32_t slot, cudaStream_t s);

// Onesweep LSD radix pass. n comes from *n_dev when non-null, else n_host. flags must hold
// onesweep_flag_words(partitions, radix) words for the largest partition count the pass can see (the
// partitions' digit totals and the aggregate tree above them, 8 nodes per parent).
inline size_t onesweep_flag_words(size_t parts, uint32_t radix) {
    size_t words = 0;
    for (size_t rows = parts;; rows = (rows + 7) / 8) {
        words += rows * radix;
        if (rows <= 1) break;
    }
    return words;
}
constexpr uint32_t kSortThreads = 256;
constexpr uint32_t kSortItems = 16;                            // keys per thread of the largest block
constexpr uint32_t kSortPartition = kSortThreads * kSortItems; // largest sort block (4096 keys)
constexpr uint32_t kSortPartitionMin = kSortThreads * 8;       // smallest sort block (2048 keys)
// Per-device kernel attributes (shared-memory carveout of the sort); call once per context.
void configure_sort_kernels();
void launch_onesweep(uint32_t digit_bits, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                     uint32_t* vals_out, const uint32_t* n_dev, uint32_t n_host, uint32_t max_n, uint32_t shift,
                     uint32_t dmask, const uint32_t* hist, FrameCtl* ctl, uint64_t* flags, uint32_t slot,
                     int grid_cap, cudaStream_t s, uint32_t block = kSortPartition, uint32_t split = 0,
                     bool early = false, uint32_t* ranges = nullptr, uint32_t tiles = 0);
// early: *n_dev (or n_host), hist, ctl->seq and the ticket counter were written at least two kernels
// back on the stream, so they are read before the programmatic-launch wait for the previous kernel.
// ranges (the last pass of a frame's sort only): each tile's (first, last + 1) in the sorted keys is
// combined into ranges[2 tile], ranges[2 tile + 1] by atomic min / max over the CTAs; the ranges must
// hold (0xFFFFFFFF, 0) before the pass (launch_frame_begin) and launch_tile_order, which reads them
// next, puts (0, 0) into the tiles left empty.
// Digit histograms of all passes over the low key_bits bits, for a standalone sort.
void launch_digit_hist(const uint32_t* keys, uint32_t n, uint32_t digit_bits, uint32_t key_bits, uint32_t* hist,
                       cudaStream_t s);
// Standalone exclusive scan (decoupled lookback); total written to *total_dev. grid 0: one CTA per
// partition (the normal case); a smaller grid leaves partitions unprocessed (failure-path checks).
void launch_exclusive_scan(uint32_t* data, uint32_t n, uint32_t* total_dev, FrameCtl* ctl, uint64_t* flags,
                           uint32_t slot, cudaStream_t s, uint32_t grid = 0);

// Tiles by decreasing range length (a permutation of 0..tiles-1) for the raster launches: two
// kernels over slices of 1024 tiles. slice_hist holds 64 words per slice (tile_order_slices), fully
// rewritten by every call.
uint32_t tile_order_slices(uint32_t tiles);
void launch_tile_order(uint32_t* ranges, uint32_t tiles, uint32_t* slice_hist, uint32_t* order, uint32_t* status,
                       cudaStream_t s);

// Checked builds: verifies the canary pads of up to kCanaryListMax buffers (head and tail pad of
// kCanaryBytes each, filled with kCanaryWord) and sets kDevCanary in *status if any word changed.
constexpr uint32_t kCanaryBytes = 256;
constexpr uint32_t kCanaryWord = 0xA5A5A5A5u;
constexpr uint32_t kCanaryListMax = 64;
struct CanaryList {
    const uint32_t* head[kCanaryListMax];
    const uint32_t* tail[kCanaryListMax];
    uint32_t count;
};
void launch_check_canaries(const CanaryList& list, uint32_t* status, cudaStream_t s);


struct RasterOut {
    uint32_t* rgba8;     // W*H packed rgba8 or null
    float* rgb;          // W*H*3 or null
    float* final_t;      // W*H or null
    uint32_t* n_contrib; // W*H or null
};
// ctl (optional) bounds every range by the sorted count; n bounds the Gaussian indices; order
// (optional) is the tile each CTA renders (launch_tile_order), else CTA i renders tile i.
void launch_raster(uint32_t tile, uint32_t batch, const uint32_t* ranges, const uint32_t* vals, const float4* rec,
                   uint32_t n, const FrameCtl* ctl, uint32_t width, uint32_t height, uint32_t tiles_x,
                   uint32_t tiles_y, const RasterOut& out, const uint32_t* order, cudaStream_t s);

// y = the pinned exp of x (raster: the raster's exp, defined on [-5.6, 0]).
void launch_exp(const float* x, float* y, uint32_t n, cudaStream_t s, bool raster = false);
// y = o * exp(x) as the raster forms it, before the 0.99 clamp (x at or above o's cut-off).
void launch_raster_alpha(const float* o, const float* x, float* y, uint32_t n, cudaStream_t s);

}  // namespace gs
struct gs_camera;
namespace gs {
// Camera.getUniform() for n cameras on the device (gs_camera.cu): out[i] gets camera i's 176-byte
// block, the same bits as gs_camera_view. out must be 16-byte aligned.
void launch_camera_views(const gs_camera* cams, uint32_t n, ViewBlock* out, cudaStream_t s);

// Sets the sequence number of gs_exclusive_scan_static's scratch on the current device (a test hook).
cudaError_t static_scan_set_sequence(uint32_t seq);

// ---- backward ---------------------------------------------------------------------------------
// grad2d: 9 floats per Gaussian, dL/d(pixel.x, pixel.y, conic.x, conic.y, conic.z, opacity, r, g, b),
// accumulated with atomics (zero it first).
void launch_raster_backward(uint32_t tile, uint32_t batch, const uint32_t* ranges, const uint32_t* vals,
                            const float4* rec, uint32_t n, const FrameCtl* ctl, uint32_t width, uint32_t height,
                            uint32_t tiles_x, uint32_t tiles_y, const float* final_t, const uint32_t* n_contrib,
                            const float* dl_drgb, float* grad2d, const uint32_t* order, cudaStream_t s);
// Up to kMaxMultiViews views of one scene for launch_preprocess_backward_multi.
struct MultiViewGrads {
    const ViewBlock* view[kMaxMultiViews];
    const uint32_t* counts[kMaxMultiViews];
    float* grad2d[kMaxMultiViews];  // cleared after use (the raster backward accumulates into zeros)
    uint32_t count;
};
// Sum over the views of their dL/d(attributes), written in the packed layout into `out` (add: added
// to what `out` holds). Call configure_backward_kernels once per device first.
void configure_backward_kernels();
void launch_preprocess_backward_multi(const float* rows, uint32_t stride, uint32_t n, const MultiViewGrads& mv,
                                      float* out, bool add, uint32_t* status, cudaStream_t s);

// grad2d -> dL/d(attributes), one thread per Gaussian, stored into `out` in the packed input layout
// (59*n floats, zeros for invisible Gaussians).
void launch_preprocess_backward(const float* rows, uint32_t stride, uint32_t n, const ViewBlock* view,
                                const uint32_t* counts, float* grad2d, float* out, uint32_t* status,
                                cudaStream_t s);

// ---- L1 + SSIM loss -----------------------------------------------------------------------------
size_t loss_scratch_floats(uint32_t width, uint32_t height);
size_t loss_sum_doubles(uint32_t width, uint32_t height);
// sums (loss_sum_doubles entries): [0] = sum of the SSIM map, [1] = sum |x - y| (both over W*H*3),
// then per-block partials; dl may be null.
void launch_loss_l1_ssim(const float* x, const float* y, uint32_t width, uint32_t height, float lambda,
                         float* scratch, double* sums, float* dl, cudaStream_t s);

}  // namespace gs
