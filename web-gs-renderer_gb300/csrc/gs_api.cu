// gs_api.cu -- the C ABI of libwebgs.so (include/gs.h).
//
// Replaces the reference Renderer (src/renderer/renderer.js): the context owns one CUDA stream and
// per-view frame state (buffers sized from count * MAX_INSTANCE_FACTOR like renderer.js:531-577,
// grown on demand and kept). gs_forward sequences the passes of renderer.js:822-932 on that stream,
// replayed from one CUDA graph per (scene, resolution, output set); gs_forward_batch captures many
// views, forked over side streams, into one graph. No pass reads a count back to the host: the
// instance count travels in FrameCtl, which every later kernel reads on the device (the role of the
// reference's indirect dispatch, indirect_arg.wgsl).
#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gs.h"
#include "gs_camera.h"
#include "gs_kernels.h"

using namespace gs;

namespace {

const char* kNoCtxError = "invalid context";

// A device buffer that grows on demand. In checked builds every allocation carries a canary pad of
// kCanaryBytes (kCanaryWord repeated) on either side, which k_check_canaries verifies after frames.
template <class T> struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;  // elements
#ifdef GS_CHECKED
    char* raw = nullptr;
#endif
    cudaError_t reserve(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        release();
        const size_t want = std::max<size_t>(n, 1);
#ifdef GS_CHECKED
        const size_t bytes = want * sizeof(T);
        cudaError_t e = cudaMalloc(&raw, bytes + 2 * kCanaryBytes);
        if (e != cudaSuccess) { raw = nullptr; return e; }
        e = cudaMemset(raw, 0xA5, kCanaryBytes);
        if (e == cudaSuccess) e = cudaMemset(raw + kCanaryBytes + bytes, 0xA5, kCanaryBytes);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) { cudaFree(raw); raw = nullptr; return e; }
        p = reinterpret_cast<T*>(raw + kCanaryBytes);
#else
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e != cudaSuccess) { p = nullptr; return e; }
#endif
        cap = want;
        return cudaSuccess;
    }
    void release() {
#ifdef GS_CHECKED
        if (raw) cudaFree(raw);
        raw = nullptr;
#else
        if (p) cudaFree(p);
#endif
        p = nullptr;
        cap = 0;
    }
    // checked builds: appends this buffer's two pads to the list
    void pads(CanaryList& l) const {
#ifdef GS_CHECKED
        if (!raw || l.count >= kCanaryListMax) return;
        l.head[l.count] = reinterpret_cast<const uint32_t*>(raw);
        l.tail[l.count] = reinterpret_cast<const uint32_t*>(raw + kCanaryBytes + cap * sizeof(T));
        ++l.count;
#else
        (void)l;
#endif
    }
};

uint32_t bitlen(uint32_t v) { return v == 0 ? 0u : 32u - (uint32_t)__builtin_clz(v); }

constexpr int kViewSlots = 16;
constexpr int kSideStreams = 16;
enum Pass { kPassBegin, kPassPreprocess, kPassScanEmit, kPassSort, kPassRanges, kPassRaster, kPassCount };
const char* kPassLabel[kPassCount] = {"frame begin", "preprocess", "scan+emit", "sort", "tile order", "raster"};

// Everything one view's frame needs on the device, and what the last frame on it was.
struct Frame {
    DevBuf<FrameCtl> ctl;
    FrameCtl* h_ctl = nullptr;  // pinned readback of the counters
    DevBuf<ViewBlock> view;
    DevBuf<float4> rec;
    DevBuf<uint4> meta;
    DevBuf<uint32_t> counts, offsets;
    DevBuf<uint32_t> keys[2], vals[2];
    DevBuf<uint64_t> flags;
    DevBuf<uint32_t> ranges;
    DevBuf<uint32_t> order;  // tiles by decreasing range length: the raster CTAs' tile order
    DevBuf<uint32_t> order_hist;  // per-slice bin counts of the tile order (64 words per 1024 tiles)
    DevBuf<uint32_t> rgba8, n_contrib;
    DevBuf<float> rgb, final_t;
    DevBuf<float> grad2d, dl_stage;
    bool grad2d_zero = false;  // grad2d holds zeros (cleared by the last preprocess backward)
    // the last frame rendered into these buffers
    const gs_scene* scene = nullptr;
    const ViewBlock* view_used = nullptr;  // device view block the last frame read
    uint32_t n = 0, width = 0, height = 0, tiles_x = 0, tiles_y = 0, passes = 0, max_instance = 0;
    int sorted_buf = 0;
    bool valid = false;
    bool direct_rgba8 = false, direct_rgb = false;  // the raster writes the caller's host buffer itself

    cudaError_t init(cudaStream_t s) {
        cudaError_t e = ctl.reserve(1);
        if (e == cudaSuccess) e = view.reserve(1);
        if (e == cudaSuccess) e = cudaMallocHost(&h_ctl, sizeof(FrameCtl));
        if (e == cudaSuccess) e = cudaMemsetAsync(ctl.p, 0, sizeof(FrameCtl), s);
        return e;
    }
    void pads(CanaryList& l) const {
        ctl.pads(l); view.pads(l); rec.pads(l); meta.pads(l); counts.pads(l); offsets.pads(l);
        for (int b = 0; b < 2; ++b) { keys[b].pads(l); vals[b].pads(l); }
        flags.pads(l); ranges.pads(l); order.pads(l); order_hist.pads(l); rgba8.pads(l); n_contrib.pads(l);
        rgb.pads(l); final_t.pads(l); grad2d.pads(l); dl_stage.pads(l);
    }
    void release() {
        ctl.release(); view.release(); rec.release(); meta.release(); counts.release(); offsets.release();
        for (int b = 0; b < 2; ++b) { keys[b].release(); vals[b].release(); }
        flags.release(); ranges.release(); rgba8.release(); n_contrib.release(); rgb.release(); final_t.release();
        order.release(); order_hist.release(); grad2d.release(); dl_stage.release();
        if (h_ctl) cudaFreeHost(h_ctl);
        h_ctl = nullptr;
    }
};

// Launch description of one frame.
struct FrameArgs {
    const gs_scene* scene;
    const ViewBlock* view;  // device copy of the view block
    uint32_t n, w, h, tiles_x, tiles_y, passes, max_instance;
    RasterOut out;
};

struct GraphKey {
    std::vector<const void*> ptrs;
    std::vector<uint32_t> dims;
    uint64_t alloc_gen = 0;
    bool operator==(const GraphKey& o) const { return ptrs == o.ptrs && dims == o.dims && alloc_gen == o.alloc_gen; }
};

}  // namespace

struct gs_scene {
    gs_ctx* ctx = nullptr;
    uint32_t n = 0;
    uint32_t stride = 0;
    float* rows = nullptr;  // 59 rows x stride floats (structure of arrays)
};

struct gs_ctx {
    gs_config cfg{};
    cudaStream_t stream = nullptr;
    cudaStream_t side[kSideStreams] = {};
    cudaEvent_t fork = nullptr, join[kSideStreams] = {};
    cudaEvent_t group_done[kSideStreams] = {};  // a batch's per-scene preprocess, one per group
    std::string err;

    Frame main;                  // gs_forward / gs_backward
    std::vector<Frame*> batch;   // gs_forward_batch / gs_backward_batch, one per view
    uint32_t batch_count = 0;    // views of the last batch
    uint64_t alloc_gen = 0;      // changes whenever a frame buffer is reallocated

    DevBuf<FrameCtl> aux_ctl;
    DevBuf<uint64_t> aux_flags;
    DevBuf<uint32_t> aux_u32;
    DevBuf<float> aux_f32;
    DevBuf<float> grad_stage, loss_scratch, loss_io;
    DevBuf<double> loss_sums;
    FrameCtl* h_aux = nullptr;

    // graph caches
    cudaGraphExec_t exec = nullptr, exec_batch = nullptr;
    GraphKey key, key_batch;

    // pinned view blocks: a frame's H2D copy reads a slot that is not rewritten before the copy has
    // completed (slot_done), so frames never block the host
    ViewBlock* h_views = nullptr;
    cudaEvent_t slot_done[kViewSlots] = {};
    uint32_t next_slot = 0;
    ViewBlock* h_bviews = nullptr;  // batch view blocks (pinned), capacity bviews_cap
    gs_camera* h_bcams = nullptr;   // batch cameras (pinned), capacity bviews_cap
    uint32_t bviews_cap = 0;
    cudaEvent_t bviews_done = nullptr;
    DevBuf<ViewBlock> d_bviews;
    DevBuf<gs_camera> d_bcams;

    // profiling
    cudaEvent_t ev[kPassCount + 1] = {};
    float pass_ms[kPassCount] = {};
    bool have_timing = false;
    cudaEvent_t bev[3] = {};  // raster backward / preprocess backward of the last gs_backward
    bool have_bwd = false;
};

namespace {

int fail(gs_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}
int cuda_fail(gs_ctx* ctx, cudaError_t e, const char* what) {
    return fail(ctx, GS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define GS_CK(call)                                                   \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);      \
    } while (0)

// Checked builds: enqueues the canary check of a frame's buffers and the context's shared ones; a
// damaged pad sets kDevCanary in the frame's status word. Product builds: nothing.
void check_canaries(gs_ctx* ctx, const Frame& f, cudaStream_t s) {
#ifdef GS_CHECKED
    CanaryList l{};
    f.pads(l);
    ctx->aux_ctl.pads(l); ctx->aux_flags.pads(l); ctx->aux_u32.pads(l); ctx->aux_f32.pads(l);
    ctx->grad_stage.pads(l); ctx->loss_scratch.pads(l); ctx->loss_io.pads(l); ctx->loss_sums.pads(l);
    ctx->d_bviews.pads(l); ctx->d_bcams.pads(l);
    launch_check_canaries(l, &f.ctl.p->status, s);
#else
    (void)ctx; (void)f; (void)s;
#endif
}

int status_to_code(gs_ctx* ctx, uint32_t status) {
    if (status & (kDevBounds | kDevCanary))
        return fail(ctx, GS_ERR_MEMORY, status & kDevBounds ? "a store index fell outside its buffer (checked build)"
                                                             : "a canary pad around a device buffer was overwritten");
    if (status & kDevTimeout) return fail(ctx, GS_ERR_TIMEOUT, "a device-side wait hit its iteration limit");
    if (status & kDevOverflow)
        return fail(ctx, GS_ERR_OVERFLOW, "instance count exceeded max_instance; output truncated");
    return GS_OK;
}

bool valid_config(const gs_config& c) {
    const bool tile_ok = c.tile_size == 8 || c.tile_size == 16 || c.tile_size == 32;
    const bool digit_ok = c.digit_bits == 4 || c.digit_bits == 8;
    const bool batch_ok = c.raster_batch == 32 || c.raster_batch == 64 || c.raster_batch == 128 || c.raster_batch == 256;
    const bool block_ok = c.sort_block == kSortPartition || c.sort_block == kSortPartitionMin;
    return tile_ok && digit_ok && batch_ok && block_ok && c.max_instance_factor >= 1;
}

// Checks a view block and derives the frame's sizes.
int frame_args(gs_ctx* ctx, const gs_scene* scene, const gs_view* view, FrameArgs* a) {
    if (!scene || scene->ctx != ctx || !view) return fail(ctx, GS_ERR_INVALID, "null scene or view");
    const float fw = view->texture_size[0], fh = view->texture_size[1];
    if (!(fw >= 1.0f) || !(fh >= 1.0f) || !(fw <= 65536.0f) || !(fh <= 65536.0f))
        return fail(ctx, GS_ERR_INVALID, "texture size out of range");
    const uint32_t w = (uint32_t)fw, h = (uint32_t)fh, tile = ctx->cfg.tile_size;
    const uint32_t tiles_x = (w + tile - 1) / tile, tiles_y = (h + tile - 1) / tile;
    const uint64_t tiles = (uint64_t)tiles_x * tiles_y;
    if (tiles > 65536u) return fail(ctx, GS_ERR_INVALID, "more than 65536 tiles do not fit the key's 16-bit tile field");
    a->scene = scene;
    a->view = nullptr;
    a->n = scene->n;
    a->w = w;
    a->h = h;
    a->tiles_x = tiles_x;
    a->tiles_y = tiles_y;
    a->max_instance = scene->n * ctx->cfg.max_instance_factor;
    const uint32_t key_bits = 16u + bitlen((uint32_t)tiles - 1u);
    a->passes = (key_bits + ctx->cfg.digit_bits - 1) / ctx->cfg.digit_bits;
    return GS_OK;
}

// Grows a frame's buffers for the frame described by a.
int ensure_frame(gs_ctx* ctx, Frame& f, const FrameArgs& a) {
    const uint32_t radix = 1u << ctx->cfg.digit_bits;
    const void* before[] = {f.rec.p, f.meta.p, f.counts.p, f.offsets.p, f.keys[0].p, f.keys[1].p, f.vals[0].p,
                            f.vals[1].p, f.flags.p, f.ranges.p, f.rgba8.p, f.rgb.p, f.final_t.p, f.n_contrib.p,
                            f.order.p, f.order_hist.p};
    GS_CK(f.rec.reserve((size_t)a.n * kRecFloat4));
    GS_CK(f.meta.reserve(a.n));
    GS_CK(f.counts.reserve(((size_t)a.n + 1 + 7) / 8 * 8));
    GS_CK(f.offsets.reserve((size_t)a.n + 1));
    for (int b = 0; b < 2; ++b) {
        GS_CK(f.keys[b].reserve(a.max_instance));
        GS_CK(f.vals[b].reserve(a.max_instance));
    }
    const size_t sort_parts = ((size_t)a.max_instance + ctx->cfg.sort_block - 1) / ctx->cfg.sort_block;
    const size_t scan_parts = ((size_t)a.n + 1 + kScanPartition - 1) / kScanPartition;
    const size_t words = std::max(onesweep_flag_words(sort_parts, radix), scan_parts);
    if (words > f.flags.cap || !f.flags.p) {
        GS_CK(f.flags.reserve(words));
        GS_CK(cudaMemsetAsync(f.flags.p, 0, f.flags.cap * sizeof(uint64_t), ctx->stream));
    }
    GS_CK(f.ranges.reserve((size_t)a.tiles_x * a.tiles_y * 2));
    GS_CK(f.order.reserve((size_t)a.tiles_x * a.tiles_y));
    GS_CK(f.order_hist.reserve((size_t)tile_order_slices(a.tiles_x * a.tiles_y) * 64));
    const size_t pix = (size_t)a.w * a.h;
    GS_CK(f.rgba8.reserve(pix));
    GS_CK(f.rgb.reserve(pix * 3));
    GS_CK(f.final_t.reserve(pix));
    GS_CK(f.n_contrib.reserve(pix));
    const void* after[] = {f.rec.p, f.meta.p, f.counts.p, f.offsets.p, f.keys[0].p, f.keys[1].p, f.vals[0].p,
                           f.vals[1].p, f.flags.p, f.ranges.p, f.rgba8.p, f.rgb.p, f.final_t.p, f.n_contrib.p,
                            f.order.p, f.order_hist.p};
    if (std::memcmp(before, after, sizeof(before)) != 0) ++ctx->alloc_gen;
    return GS_OK;
}

// Raster outputs of a frame: caller device buffers, or the frame's own buffers for host outputs and
// for the state a differentiable context keeps (final T and last contributor).
// The device address of a host buffer the GPU can write directly (pinned / registered memory), or
// null for pageable memory, which is reached through a staging copy.
void* mapped_host(const void* p) {
    cudaPointerAttributes attr{};
    if (!p || cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return attr.type == cudaMemoryTypeHost ? attr.devicePointer : nullptr;
}

RasterOut raster_out(const gs_ctx* ctx, Frame& f, const gs_image* out) {
    const bool dev = out && out->location == GS_MEM_DEVICE;
    const bool keep = (ctx->cfg.flags & GS_FLAG_DIFFERENTIABLE) != 0;
    RasterOut ro{};
    f.direct_rgba8 = f.direct_rgb = false;
    if (out) {
        // host images in pinned memory are written by the raster over the host link (no staging copy)
        void* h8 = !dev && out->rgba8 ? mapped_host(out->rgba8) : nullptr;
        void* hrgb = !dev && out->rgb ? mapped_host(out->rgb) : nullptr;
        f.direct_rgba8 = h8 != nullptr;
        f.direct_rgb = hrgb != nullptr;
        ro.rgba8 = out->rgba8 ? (dev ? reinterpret_cast<uint32_t*>(out->rgba8)
                                     : h8 ? static_cast<uint32_t*>(h8) : f.rgba8.p)
                              : nullptr;
        ro.rgb = out->rgb ? (dev ? out->rgb : hrgb ? static_cast<float*>(hrgb) : f.rgb.p) : nullptr;
    }
    if (keep) {
        ro.final_t = f.final_t.p;
        ro.n_contrib = f.n_contrib.p;
    } else if (out) {
        ro.final_t = out->final_t ? (dev ? out->final_t : f.final_t.p) : nullptr;
        ro.n_contrib = out->n_contrib ? (dev ? out->n_contrib : f.n_contrib.p) : nullptr;
    }
    return ro;
}

// Enqueues one frame (renderer.js:822-932) on stream s; preprocessed: its frame control block was
// reset and its preprocess done already (by a multi-view preprocess of its scene).
void enqueue_frame(gs_ctx* ctx, Frame& f, const FrameArgs& a, cudaStream_t s, bool profile, bool preprocessed = false) {
    const uint32_t bits = ctx->cfg.digit_bits, radix = 1u << bits;
    FrameCtl* ctl = f.ctl.p;
    if (profile) cudaEventRecord(ctx->ev[0], s);
    if (!preprocessed) launch_frame_begin(ctl, f.flags.p, (uint32_t)f.flags.cap, s, f.ranges.p, a.tiles_x * a.tiles_y * 2u);
    if (profile) cudaEventRecord(ctx->ev[1], s);
    if (!preprocessed) {
        launch_preprocess(a.scene->rows, a.scene->stride, a.n, a.view, ctx->cfg.tile_size, f.rec.p, f.meta.p,
                          f.counts.p, ctl, s);
    }
    if (profile) cudaEventRecord(ctx->ev[2], s);
    launch_scan_emit(f.counts.p, f.meta.p, a.n, a.tiles_x, a.max_instance, bits, a.passes, f.offsets.p, f.keys[0].p,
                     f.vals[0].p, ctl, f.flags.p, 0, s);
    if (profile) cudaEventRecord(ctx->ev[3], s);
    int cur = 0;
    const uint32_t key_bits = 16u + bitlen(a.tiles_x * a.tiles_y - 1u);
    for (uint32_t p = 0; p < a.passes; ++p) {
        // the tile digits arrive in depth order, nearly all distinct within a warp: their ranking
        // matches the high half of the digit and separates the low half by ballots (w/2 of a w-bit
        // digit, from 2 bits up); the depth digits keep the plain match
        const uint32_t w = std::min(bits, key_bits - p * bits);
        const uint32_t split = p * bits >= 16u && w / 2u >= 2u ? w / 2u : 0u;
        launch_onesweep(bits, f.keys[cur].p, f.vals[cur].p, f.keys[cur ^ 1].p, f.vals[cur ^ 1].p, &ctl->sorted_count,
                        0, a.max_instance, p * bits, radix - 1u, ctl->hist + p * radix, ctl, f.flags.p, 1 + p, 0, s,
                        ctx->cfg.sort_block, split, p > 0,  // the emit right before the first pass writes its inputs
                        p + 1 == a.passes ? f.ranges.p : nullptr, a.tiles_x * a.tiles_y);  // the last pass: ranges
        cur ^= 1;
    }
    if (profile) cudaEventRecord(ctx->ev[4], s);
    launch_tile_order(f.ranges.p, a.tiles_x * a.tiles_y, f.order_hist.p, f.order.p, &ctl->status, s);
    if (profile) cudaEventRecord(ctx->ev[5], s);
    launch_raster(ctx->cfg.tile_size, ctx->cfg.raster_batch, f.ranges.p, f.vals[cur].p, f.rec.p, a.n, ctl, a.w, a.h,
                  a.tiles_x, a.tiles_y, a.out, f.order.p, s);
    if (profile) cudaEventRecord(ctx->ev[6], s);
}

void remember(Frame& f, const FrameArgs& a) {
    f.scene = a.scene;
    f.view_used = a.view;
    f.n = a.n;
    f.width = a.w;
    f.height = a.h;
    f.tiles_x = a.tiles_x;
    f.tiles_y = a.tiles_y;
    f.passes = a.passes;
    f.max_instance = a.max_instance;
    f.sorted_buf = (int)(a.passes & 1u);
    f.valid = true;
}

// Copies a frame's requested outputs out of its own buffers after the frame (stream-ordered).
int copy_outputs(gs_ctx* ctx, Frame& f, const gs_image* out, cudaStream_t s) {
    const size_t pix = (size_t)f.width * f.height;
    if (out->location == GS_MEM_DEVICE) {
        if (ctx->cfg.flags & GS_FLAG_DIFFERENTIABLE) {
            if (out->final_t) GS_CK(cudaMemcpyAsync(out->final_t, f.final_t.p, pix * 4, cudaMemcpyDeviceToDevice, s));
            if (out->n_contrib)
                GS_CK(cudaMemcpyAsync(out->n_contrib, f.n_contrib.p, pix * 4, cudaMemcpyDeviceToDevice, s));
        }
        return GS_OK;
    }
    if (out->rgba8 && !f.direct_rgba8) GS_CK(cudaMemcpyAsync(out->rgba8, f.rgba8.p, pix * 4, cudaMemcpyDeviceToHost, s));
    if (out->rgb && !f.direct_rgb) GS_CK(cudaMemcpyAsync(out->rgb, f.rgb.p, pix * 12, cudaMemcpyDeviceToHost, s));
    if (out->final_t) GS_CK(cudaMemcpyAsync(out->final_t, f.final_t.p, pix * 4, cudaMemcpyDeviceToHost, s));
    if (out->n_contrib) GS_CK(cudaMemcpyAsync(out->n_contrib, f.n_contrib.p, pix * 4, cudaMemcpyDeviceToHost, s));
    return GS_OK;
}

// A batch whose view blocks are built on the device: the graph's first kernel fills `views` from
// `cams` (count cameras) before any frame reads them.
struct CameraPrologue {
    const gs_camera* cams = nullptr;
    ViewBlock* views = nullptr;
    uint32_t count = 0;
};

int capture_and_launch(gs_ctx* ctx, cudaGraphExec_t* exec, GraphKey* cached, const GraphKey& key,
                       const std::vector<Frame*>& frames, const std::vector<FrameArgs>& args,
                       const CameraPrologue& prologue = CameraPrologue{}) {
    if (!*exec || !(key == *cached)) {
        if (*exec) cudaGraphExecDestroy(*exec);
        *exec = nullptr;
        cudaGraph_t g = nullptr;
        GS_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        if (prologue.cams) launch_camera_views(prologue.cams, prologue.count, prologue.views, ctx->stream);
        if (frames.size() == 1) {
            enqueue_frame(ctx, *frames[0], args[0], ctx->stream, false);
        } else {
            // views are independent: fork them over the side streams so small views fill the GPU
            // together. Views of one scene are preprocessed together (one pass over the scene's
            // attributes per group of up to 16 views) on the stream of the group's first view, so the
            // groups' preprocesses run side by side; a view on another stream waits for its group.
            cudaEventRecord(ctx->fork, ctx->stream);
            const int used = (int)std::min<size_t>(frames.size(), kSideStreams);
            for (int s = 0; s < used; ++s) cudaStreamWaitEvent(ctx->side[s], ctx->fork, 0);
            std::vector<int> group_of(frames.size(), -1);
            int groups = 0;
            for (size_t i = 0; i < frames.size() && groups < kSideStreams; ++i) {
                if (group_of[i] >= 0) continue;
                std::vector<size_t> members;
                for (size_t j = i; j < frames.size(); ++j)
                    if (group_of[j] < 0 && args[j].scene == args[i].scene) members.push_back(j);
                if (members.size() < 2) continue;
                for (size_t c0 = 0; c0 < members.size() && groups < kSideStreams; c0 += kMaxMultiViews) {
                    MultiViewFrames mv{};
                    mv.count = (uint32_t)std::min<size_t>(kMaxMultiViews, members.size() - c0);
                    for (uint32_t v = 0; v < mv.count; ++v) {
                        const size_t j = members[c0 + v];
                        Frame& f = *frames[j];
                        mv.view[v] = args[j].view;
                        mv.rec[v] = f.rec.p;
                        mv.meta[v] = f.meta.p;
                        mv.counts[v] = f.counts.p;
                        mv.ctl[v] = f.ctl.p;
                        mv.ranges[v] = f.ranges.p;
                        mv.range_words[v] = args[j].tiles_x * args[j].tiles_y * 2u;
                        mv.flags[v] = f.flags.p;
                        mv.flag_words[v] = (uint32_t)f.flags.cap;
                        group_of[j] = groups;
                    }
                    cudaStream_t gs = ctx->side[members[c0] % used];
                    launch_frame_begin_multi(mv, gs);
                    launch_preprocess_multi(args[i].scene->rows, args[i].scene->stride, args[i].n,
                                            ctx->cfg.tile_size, mv, gs);
                    cudaEventRecord(ctx->group_done[groups], gs);
                    ++groups;
                }
            }
            for (size_t i = 0; i < frames.size(); ++i) {
                cudaStream_t s = ctx->side[i % used];
                const int g = group_of[i];
                if (g >= 0) cudaStreamWaitEvent(s, ctx->group_done[g], 0);
                enqueue_frame(ctx, *frames[i], args[i], s, false, g >= 0);
            }
            for (int s = 0; s < used; ++s) {
                cudaEventRecord(ctx->join[s], ctx->side[s]);
                cudaStreamWaitEvent(ctx->stream, ctx->join[s], 0);
            }
        }
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "graph capture");
        e = cudaGraphInstantiate(exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            *exec = nullptr;
            return cuda_fail(ctx, e, "graph instantiate");
        }
        *cached = key;
    }
    GS_CK(cudaGraphLaunch(*exec, ctx->stream));
    return GS_OK;
}

void drop_graphs_of_scene(gs_ctx* ctx, const gs_scene* scene) {
    auto uses = [&](const GraphKey& k) { return std::find(k.ptrs.begin(), k.ptrs.end(), scene) != k.ptrs.end(); };
    if (ctx->exec && uses(ctx->key)) {
        cudaGraphExecDestroy(ctx->exec);
        ctx->exec = nullptr;
        ctx->key = GraphKey{};
    }
    if (ctx->exec_batch && uses(ctx->key_batch)) {
        cudaGraphExecDestroy(ctx->exec_batch);
        ctx->exec_batch = nullptr;
        ctx->key_batch = GraphKey{};
    }
}

}  // namespace

// =====================================================================================================
extern "C" {

const char* gs_version(void) { return "webgs-gb300 0.2 (sm_103a)"; }

void gs_config_default(gs_config* cfg) {
    if (!cfg) return;
    cfg->tile_size = 16;            // TILE_SIZE_X/Y, renderer.js:25-26
    cfg->digit_bits = 8;            // RADIX_DIGITS = 256, renderer.js:67
    cfg->raster_batch = 256;        // TIlE_SIZE batch, raseter.wgsl:21-23
    cfg->max_instance_factor = 64;  // MAX_INSTANCE_FACTOR, renderer.js:16
    cfg->flags = 0;
    cfg->device = 0;
    cfg->sort_block = 4096;         // keys per sort partition (the reference sorts 256-key blocks)
}

int gs_ctx_create(const gs_config* cfg, gs_ctx** out) {
    if (!out) return GS_ERR_INVALID;
    *out = nullptr;
    gs_config c;
    gs_config_default(&c);
    if (cfg) c = *cfg;
    if (!valid_config(c)) return GS_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || c.device < 0 || c.device >= ndev) {
        cudaGetLastError();
        return GS_ERR_CUDA;
    }
    if (cudaSetDevice(c.device) != cudaSuccess) return GS_ERR_CUDA;
    configure_sort_kernels();
    configure_backward_kernels();
    gs_ctx* ctx = new gs_ctx();
    ctx->cfg = c;
    bool ok = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) == cudaSuccess;
    for (int s = 0; ok && s < kSideStreams; ++s)
        ok = cudaStreamCreateWithFlags(&ctx->side[s], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&ctx->join[s], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&ctx->group_done[s], cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&ctx->bviews_done, cudaEventDisableTiming) == cudaSuccess &&
         ctx->main.init(ctx->stream) == cudaSuccess && ctx->aux_ctl.reserve(1) == cudaSuccess &&
         cudaMallocHost(&ctx->h_aux, sizeof(FrameCtl)) == cudaSuccess &&
         cudaMallocHost(&ctx->h_views, sizeof(ViewBlock) * kViewSlots) == cudaSuccess;
    if (!ok) {
        gs_ctx_destroy(ctx);
        return GS_ERR_OOM;
    }
    cudaMemsetAsync(ctx->aux_ctl.p, 0, sizeof(FrameCtl), ctx->stream);
    for (auto& e : ctx->ev) cudaEventCreate(&e);
    for (auto& e : ctx->bev) cudaEventCreate(&e);
    for (auto& e : ctx->slot_done) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        gs_ctx_destroy(ctx);
        return GS_ERR_CUDA;
    }
    *out = ctx;
    return GS_OK;
}

int gs_ctx_destroy(gs_ctx* ctx) {
    if (!ctx) return GS_ERR_INVALID;
    cudaSetDevice(ctx->cfg.device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->exec) cudaGraphExecDestroy(ctx->exec);
    if (ctx->exec_batch) cudaGraphExecDestroy(ctx->exec_batch);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : ctx->bev)
        if (e) cudaEventDestroy(e);
    for (auto& e : ctx->slot_done)
        if (e) cudaEventDestroy(e);
    for (int s = 0; s < kSideStreams; ++s) {
        if (ctx->side[s]) cudaStreamDestroy(ctx->side[s]);
        if (ctx->join[s]) cudaEventDestroy(ctx->join[s]);
        if (ctx->group_done[s]) cudaEventDestroy(ctx->group_done[s]);
    }
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    if (ctx->bviews_done) cudaEventDestroy(ctx->bviews_done);
    if (ctx->h_views) cudaFreeHost(ctx->h_views);
    if (ctx->h_bviews) cudaFreeHost(ctx->h_bviews);
    if (ctx->h_bcams) cudaFreeHost(ctx->h_bcams);
    if (ctx->h_aux) cudaFreeHost(ctx->h_aux);
    ctx->main.release();
    for (Frame* f : ctx->batch) {
        f->release();
        delete f;
    }
    ctx->aux_ctl.release(); ctx->aux_flags.release(); ctx->aux_u32.release(); ctx->aux_f32.release();
    ctx->grad_stage.release(); ctx->loss_scratch.release(); ctx->loss_io.release();
    ctx->loss_sums.release(); ctx->d_bviews.release(); ctx->d_bcams.release();
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GS_OK;
}

const char* gs_last_error(const gs_ctx* ctx) { return ctx ? ctx->err.c_str() : kNoCtxError; }

void* gs_ctx_stream(gs_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int gs_ctx_synchronize(gs_ctx* ctx) {
    if (!ctx) return GS_ERR_INVALID;
    GS_CK(cudaStreamSynchronize(ctx->stream));
    return GS_OK;
}

// ---- scenes ----------------------------------------------------------------------------------------
static int upload_rows(gs_ctx* ctx, gs_scene* sc, const float* packed, int32_t location) {
    const size_t bytes = (size_t)sc->n * kRows * sizeof(float);
    const float* src = packed;
    float* staging = nullptr;
    if (location == GS_MEM_HOST && sc->n) {
        GS_CK(cudaMalloc(&staging, bytes));
        cudaError_t e = cudaMemcpyAsync(staging, packed, bytes, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) { cudaFree(staging); return cuda_fail(ctx, e, "scene upload"); }
        src = staging;
    }
    launch_pack_to_rows(src, sc->n, sc->stride, sc->rows, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (staging) cudaFree(staging);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scene upload");
    GS_CK(cudaGetLastError());
    return GS_OK;
}

int gs_scene_upload(gs_ctx* ctx, const float* packed, uint32_t count, int32_t location, gs_scene** out) {
    if (!ctx) return GS_ERR_INVALID;
    if (!out || (!packed && count) || (location != GS_MEM_HOST && location != GS_MEM_DEVICE))
        return fail(ctx, GS_ERR_INVALID, "gs_scene_upload: bad argument");
    if ((uint64_t)count * ctx->cfg.max_instance_factor > 0xFFFFFFFFull)
        return fail(ctx, GS_ERR_INVALID, "gs_scene_upload: count * max_instance_factor exceeds 2^32-1");
    *out = nullptr;
    GS_CK(cudaSetDevice(ctx->cfg.device));
    gs_scene* sc = new gs_scene();
    sc->ctx = ctx;
    sc->n = count;
    sc->stride = std::max<uint32_t>(64u, (count + 63u) / 64u * 64u);
    cudaError_t e = cudaMalloc(&sc->rows, (size_t)sc->stride * kRows * sizeof(float));
    if (e != cudaSuccess) {
        delete sc;
        return fail(ctx, GS_ERR_OOM, "gs_scene_upload: device allocation failed");
    }
    const int rc = upload_rows(ctx, sc, packed, location);
    if (rc != GS_OK) {
        cudaFree(sc->rows);
        delete sc;
        return rc;
    }
    *out = sc;
    return GS_OK;
}

int gs_scene_update(gs_ctx* ctx, gs_scene* scene, const float* packed, int32_t location) {
    if (!ctx) return GS_ERR_INVALID;
    if (!scene || scene->ctx != ctx || (!packed && scene->n) || (location != GS_MEM_HOST && location != GS_MEM_DEVICE))
        return fail(ctx, GS_ERR_INVALID, "gs_scene_update: bad argument");
    GS_CK(cudaSetDevice(ctx->cfg.device));
    return upload_rows(ctx, scene, packed, location);
}

int gs_scene_destroy(gs_scene* scene) {
    if (!scene) return GS_ERR_INVALID;
    gs_ctx* ctx = scene->ctx;
    if (ctx) {
        cudaSetDevice(ctx->cfg.device);
        cudaStreamSynchronize(ctx->stream);
        drop_graphs_of_scene(ctx, scene);
        if (ctx->main.scene == scene) ctx->main.valid = false;
        for (Frame* f : ctx->batch)
            if (f->scene == scene) f->valid = false;
    }
    if (scene->rows) cudaFree(scene->rows);
    delete scene;
    return GS_OK;
}

uint32_t gs_scene_count(const gs_scene* scene) { return scene ? scene->n : 0u; }

// ---- forward ---------------------------------------------------------------------------------------
int gs_forward(gs_ctx* ctx, const gs_scene* scene, const gs_view* view, const gs_image* out) {
    if (!ctx) return GS_ERR_INVALID;
    if (!out) return fail(ctx, GS_ERR_INVALID, "gs_forward: null output");
    if (out->location != GS_MEM_HOST && out->location != GS_MEM_DEVICE)
        return fail(ctx, GS_ERR_INVALID, "gs_forward: bad output location");
    FrameArgs a;
    int rc = frame_args(ctx, scene, view, &a);
    if (rc != GS_OK) return rc;
    GS_CK(cudaSetDevice(ctx->cfg.device));
    Frame& f = ctx->main;
    rc = ensure_frame(ctx, f, a);
    if (rc != GS_OK) return rc;
    a.view = f.view.p;
    a.out = raster_out(ctx, f, out);
    {
        const uint32_t slot = ctx->next_slot;
        ctx->next_slot = (slot + 1) % kViewSlots;
        GS_CK(cudaEventSynchronize(ctx->slot_done[slot]));
        std::memcpy(&ctx->h_views[slot], view, sizeof(ViewBlock));
        GS_CK(cudaMemcpyAsync(f.view.p, &ctx->h_views[slot], sizeof(ViewBlock), cudaMemcpyHostToDevice, ctx->stream));
        GS_CK(cudaEventRecord(ctx->slot_done[slot], ctx->stream));
    }
    const bool profile = (ctx->cfg.flags & GS_FLAG_PROFILE) != 0;
    const bool use_graph = !profile && (ctx->cfg.flags & GS_FLAG_NO_GRAPH) == 0;
    if (use_graph) {
        GraphKey k;
        k.ptrs = {scene, a.out.rgba8, a.out.rgb, a.out.final_t, a.out.n_contrib};
        k.dims = {a.n, a.w, a.h};
        k.alloc_gen = ctx->alloc_gen;
        rc = capture_and_launch(ctx, &ctx->exec, &ctx->key, k, {&f}, {a});
        if (rc != GS_OK) return rc;
    } else {
        enqueue_frame(ctx, f, a, ctx->stream, profile);
    }
    GS_CK(cudaGetLastError());
    remember(f, a);
    ctx->have_timing = false;
    ctx->have_bwd = false;
    check_canaries(ctx, f, ctx->stream);
    GS_CK(cudaMemcpyAsync(f.h_ctl, f.ctl.p, offsetof(FrameCtl, tickets), cudaMemcpyDeviceToHost, ctx->stream));
    rc = copy_outputs(ctx, f, out, ctx->stream);
    if (rc != GS_OK) return rc;
    if (out->location == GS_MEM_HOST) {
        GS_CK(cudaStreamSynchronize(ctx->stream));
        if (profile) {
            for (int p = 0; p < kPassCount; ++p) cudaEventElapsedTime(&ctx->pass_ms[p], ctx->ev[p], ctx->ev[p + 1]);
            ctx->have_timing = true;
        }
        return status_to_code(ctx, f.h_ctl->status);
    }
    return GS_OK;
}

// gs_forward_batch and gs_forward_batch_cameras: with cams, the view blocks of `views` are ignored
// (only their texture sizes are read on the host) and built on the device from cams.
static int forward_batch(gs_ctx* ctx, const gs_batch_view* views, uint32_t count, const gs_camera* cams) {
    const int32_t loc = views[0].out.location;
    for (uint32_t i = 0; i < count; ++i)
        if (views[i].out.location != loc || (loc != GS_MEM_HOST && loc != GS_MEM_DEVICE))
            return fail(ctx, GS_ERR_INVALID, "gs_forward_batch: every view must use the same valid output location");
    GS_CK(cudaSetDevice(ctx->cfg.device));
    while (ctx->batch.size() < count) {
        Frame* f = new Frame();
        if (f->init(ctx->stream) != cudaSuccess) {
            f->release();
            delete f;
            return fail(ctx, GS_ERR_OOM, "gs_forward_batch: frame allocation failed");
        }
        ctx->batch.push_back(f);
        ++ctx->alloc_gen;
    }
    if (count > ctx->bviews_cap) {
        GS_CK(cudaStreamSynchronize(ctx->stream));
        if (ctx->h_bviews) cudaFreeHost(ctx->h_bviews);
        if (ctx->h_bcams) cudaFreeHost(ctx->h_bcams);
        ctx->h_bviews = nullptr;
        ctx->h_bcams = nullptr;
        ctx->bviews_cap = 0;
        GS_CK(cudaMallocHost(&ctx->h_bviews, sizeof(ViewBlock) * count));
        GS_CK(cudaMallocHost(&ctx->h_bcams, sizeof(gs_camera) * count));
        ctx->bviews_cap = count;
        const void* before[2] = {ctx->d_bviews.p, ctx->d_bcams.p};
        GS_CK(ctx->d_bviews.reserve(count));
        GS_CK(ctx->d_bcams.reserve(count));
        if (before[0] != ctx->d_bviews.p || before[1] != ctx->d_bcams.p) ++ctx->alloc_gen;
    }
    std::vector<FrameArgs> args(count);
    std::vector<Frame*> frames(ctx->batch.begin(), ctx->batch.begin() + count);
    GraphKey k;
    for (uint32_t i = 0; i < count; ++i) {
        int rc = frame_args(ctx, views[i].scene, &views[i].view, &args[i]);
        if (rc != GS_OK) return fail(ctx, rc, "gs_forward_batch: view " + std::to_string(i) + ": " + ctx->err);
        rc = ensure_frame(ctx, *frames[i], args[i]);
        if (rc != GS_OK) return rc;
    }
    for (uint32_t i = 0; i < count; ++i) {
        args[i].view = ctx->d_bviews.p + i;
        args[i].out = raster_out(ctx, *frames[i], &views[i].out);
        k.ptrs.insert(k.ptrs.end(), {views[i].scene, args[i].out.rgba8, args[i].out.rgb, args[i].out.final_t,
                                     args[i].out.n_contrib});
        k.dims.insert(k.dims.end(), {args[i].n, args[i].w, args[i].h});
    }
    k.dims.push_back(cams ? 1u : 0u);  // a graph that builds its view blocks is a different graph
    k.alloc_gen = ctx->alloc_gen;
    GS_CK(cudaEventSynchronize(ctx->bviews_done));
    CameraPrologue prologue;
    if (cams) {
        std::memcpy(ctx->h_bcams, cams, sizeof(gs_camera) * count);
        GS_CK(cudaMemcpyAsync(ctx->d_bcams.p, ctx->h_bcams, sizeof(gs_camera) * count, cudaMemcpyHostToDevice,
                              ctx->stream));
        prologue.cams = ctx->d_bcams.p;
        prologue.views = ctx->d_bviews.p;
        prologue.count = count;
    } else {
        for (uint32_t i = 0; i < count; ++i) std::memcpy(&ctx->h_bviews[i], &views[i].view, sizeof(ViewBlock));
        GS_CK(cudaMemcpyAsync(ctx->d_bviews.p, ctx->h_bviews, sizeof(ViewBlock) * count, cudaMemcpyHostToDevice,
                              ctx->stream));
    }
    GS_CK(cudaEventRecord(ctx->bviews_done, ctx->stream));
    int rc = capture_and_launch(ctx, &ctx->exec_batch, &ctx->key_batch, k, frames, args, prologue);
    if (rc != GS_OK) return rc;
    GS_CK(cudaGetLastError());
    for (uint32_t i = 0; i < count; ++i) {
        remember(*frames[i], args[i]);
        check_canaries(ctx, *frames[i], ctx->stream);
        GS_CK(cudaMemcpyAsync(frames[i]->h_ctl, frames[i]->ctl.p, offsetof(FrameCtl, tickets), cudaMemcpyDeviceToHost,
                              ctx->stream));
        rc = copy_outputs(ctx, *frames[i], &views[i].out, ctx->stream);
        if (rc != GS_OK) return rc;
    }
    ctx->batch_count = count;
    if (loc == GS_MEM_HOST) {
        GS_CK(cudaStreamSynchronize(ctx->stream));
        uint32_t status = 0;
        for (uint32_t i = 0; i < count; ++i) status |= frames[i]->h_ctl->status;
        return status_to_code(ctx, status);
    }
    return GS_OK;
}

int gs_forward_batch(gs_ctx* ctx, const gs_batch_view* views, uint32_t count) {
    if (!ctx) return GS_ERR_INVALID;
    if (!views || count == 0) return fail(ctx, GS_ERR_INVALID, "gs_forward_batch: no views");
    return forward_batch(ctx, views, count, nullptr);
}

int gs_forward_batch_cameras(gs_ctx* ctx, const gs_batch_camera* views, uint32_t count) {
    if (!ctx) return GS_ERR_INVALID;
    if (!views || count == 0) return fail(ctx, GS_ERR_INVALID, "gs_forward_batch_cameras: no views");
    std::vector<gs_batch_view> bv(count);
    std::vector<gs_camera> cams(count);
    for (uint32_t i = 0; i < count; ++i) {
        if (!gs_cam::camera_valid(views[i].camera))
            return fail(ctx, GS_ERR_INVALID, "gs_forward_batch_cameras: view " + std::to_string(i) + ": bad camera");
        cams[i] = views[i].camera;
        bv[i].scene = views[i].scene;
        bv[i].out = views[i].out;
        std::memset(&bv[i].view, 0, sizeof(gs_view));
        bv[i].view.texture_size[0] = (float)views[i].camera.width;
        bv[i].view.texture_size[1] = (float)views[i].camera.height;
    }
    return forward_batch(ctx, bv.data(), count, cams.data());
}

int gs_camera_views(gs_ctx* ctx, const gs_camera* cams, uint32_t n, gs_view* out, int32_t location) {
    if (!ctx) return GS_ERR_INVALID;
    if ((!cams || !out) && n) return fail(ctx, GS_ERR_INVALID, "gs_camera_views: null buffer");
    if (location != GS_MEM_HOST && location != GS_MEM_DEVICE) return fail(ctx, GS_ERR_INVALID, "gs_camera_views: bad location");
    for (uint32_t i = 0; i < n; ++i)
        if (!gs_cam::camera_valid(cams[i])) return fail(ctx, GS_ERR_INVALID, "gs_camera_views: bad camera");
    if (n == 0) return GS_OK;
    GS_CK(cudaSetDevice(ctx->cfg.device));
    // staging in the aux float buffer: the cameras, then (host output) the blocks
    const size_t cam_floats = ((size_t)n * sizeof(gs_camera) + 15) / 16 * 4;
    const size_t view_floats = (size_t)n * sizeof(ViewBlock) / 4;
    GS_CK(ctx->aux_f32.reserve(cam_floats + view_floats));
    gs_camera* d_cams = reinterpret_cast<gs_camera*>(ctx->aux_f32.p);
    ViewBlock* d_views = location == GS_MEM_DEVICE ? reinterpret_cast<ViewBlock*>(out)
                                                   : reinterpret_cast<ViewBlock*>(ctx->aux_f32.p + cam_floats);
    if (reinterpret_cast<uintptr_t>(d_views) % 16u != 0u)
        return fail(ctx, GS_ERR_INVALID, "gs_camera_views: device output must be 16-byte aligned");
    GS_CK(cudaMemcpyAsync(d_cams, cams, (size_t)n * sizeof(gs_camera), cudaMemcpyHostToDevice, ctx->stream));
    launch_camera_views(d_cams, n, d_views, ctx->stream);
    GS_CK(cudaGetLastError());
    if (location == GS_MEM_DEVICE) return GS_OK;
    GS_CK(cudaMemcpyAsync(out, d_views, (size_t)n * sizeof(ViewBlock), cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    return GS_OK;
}

static int fill_info(gs_ctx* ctx, const Frame& f, gs_frame_info* info) {
    const FrameCtl& c = *f.h_ctl;
    info->instance_count = c.instance_count;
    info->sorted_count = c.sorted_count;
    info->max_instance = f.max_instance;
    info->visible = c.visible;
    info->near_pass = c.near_pass;
    info->tiles_x = f.tiles_x;
    info->tiles_y = f.tiles_y;
    info->status = c.status;
    info->sort_passes = f.passes;
    (void)ctx;
    return GS_OK;
}

int gs_get_frame_info(gs_ctx* ctx, gs_frame_info* info) {
    if (!ctx) return GS_ERR_INVALID;
    if (!info) return fail(ctx, GS_ERR_INVALID, "gs_get_frame_info: null info");
    if (!ctx->main.valid) return fail(ctx, GS_ERR_STATE, "gs_get_frame_info: no frame rendered");
    GS_CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->cfg.flags & GS_FLAG_PROFILE && !ctx->have_timing) {
        for (int p = 0; p < kPassCount; ++p) cudaEventElapsedTime(&ctx->pass_ms[p], ctx->ev[p], ctx->ev[p + 1]);
        ctx->have_timing = true;
    }
    return fill_info(ctx, ctx->main, info);
}

int gs_get_batch_frame_info(gs_ctx* ctx, uint32_t index, gs_frame_info* info) {
    if (!ctx) return GS_ERR_INVALID;
    if (!info) return fail(ctx, GS_ERR_INVALID, "gs_get_batch_frame_info: null info");
    if (index >= ctx->batch_count || !ctx->batch[index]->valid)
        return fail(ctx, GS_ERR_STATE, "gs_get_batch_frame_info: no such view in the last batch");
    GS_CK(cudaStreamSynchronize(ctx->stream));
    return fill_info(ctx, *ctx->batch[index], info);
}

int gs_get_debug(gs_ctx* ctx, const gs_debug* dbg) {
    if (!ctx) return GS_ERR_INVALID;
    if (!dbg) return fail(ctx, GS_ERR_INVALID, "gs_get_debug: null argument");
    Frame& f = ctx->main;
    if (!f.valid) return fail(ctx, GS_ERR_STATE, "gs_get_debug: no frame rendered");
    GS_CK(cudaStreamSynchronize(ctx->stream));
    const uint32_t n = f.n;
    if (dbg->tiles_touched) GS_CK(cudaMemcpy(dbg->tiles_touched, f.counts.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
    if (dbg->meta) GS_CK(cudaMemcpy(dbg->meta, f.meta.p, (size_t)n * 16, cudaMemcpyDeviceToHost));
    if (dbg->conic_opacity || dbg->pixel || dbg->color) {
        std::vector<float> rec((size_t)n * kRecFloat4 * 4);
        if (n) GS_CK(cudaMemcpy(rec.data(), f.rec.p, rec.size() * 4, cudaMemcpyDeviceToHost));
        for (size_t g = 0; g < n; ++g) {
            const float* r = rec.data() + g * 12;
            if (dbg->pixel) { dbg->pixel[2 * g] = r[0]; dbg->pixel[2 * g + 1] = r[1]; }
            if (dbg->conic_opacity) {
                dbg->conic_opacity[4 * g] = r[2];
                dbg->conic_opacity[4 * g + 1] = r[3];
                dbg->conic_opacity[4 * g + 2] = r[4];
                dbg->conic_opacity[4 * g + 3] = r[5];
            }
            if (dbg->color) {
                dbg->color[4 * g] = r[6];
                dbg->color[4 * g + 1] = r[7];
                dbg->color[4 * g + 2] = r[8];
                dbg->color[4 * g + 3] = 0.0f;
            }
        }
    }
    if (dbg->offsets) GS_CK(cudaMemcpy(dbg->offsets, f.offsets.p, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost));
    const uint32_t sorted = f.h_ctl->sorted_count;
    const size_t kc = std::min<uint64_t>(sorted, dbg->capacity);
    if (dbg->keys && kc) GS_CK(cudaMemcpy(dbg->keys, f.keys[f.sorted_buf].p, kc * 4, cudaMemcpyDeviceToHost));
    if (dbg->vals && kc) GS_CK(cudaMemcpy(dbg->vals, f.vals[f.sorted_buf].p, kc * 4, cudaMemcpyDeviceToHost));
    if (dbg->ranges)
        GS_CK(cudaMemcpy(dbg->ranges, f.ranges.p, (size_t)f.tiles_x * f.tiles_y * 8, cudaMemcpyDeviceToHost));
    return GS_OK;
}

int gs_get_timings(gs_ctx* ctx, gs_timing* rows, int32_t max_rows, int32_t* n_rows) {
    if (!ctx) return GS_ERR_INVALID;
    if (!rows || !n_rows || max_rows < 0) return fail(ctx, GS_ERR_INVALID, "gs_get_timings: bad argument");
    if (!(ctx->cfg.flags & GS_FLAG_PROFILE)) return fail(ctx, GS_ERR_STATE, "gs_get_timings: context not profiling");
    if (!ctx->main.valid) return fail(ctx, GS_ERR_STATE, "gs_get_timings: no frame rendered");
    if (!ctx->have_timing) {
        GS_CK(cudaStreamSynchronize(ctx->stream));
        for (int p = 0; p < kPassCount; ++p) cudaEventElapsedTime(&ctx->pass_ms[p], ctx->ev[p], ctx->ev[p + 1]);
        ctx->have_timing = true;
    }
    int k = 0;
    float total = 0;
    for (int p = 0; p < kPassCount && k < max_rows; ++p, ++k) {
        std::snprintf(rows[k].label, sizeof(rows[k].label), "%s", kPassLabel[p]);
        rows[k].ms = ctx->pass_ms[p];
        total += ctx->pass_ms[p];
    }
    if (k < max_rows) {
        std::snprintf(rows[k].label, sizeof(rows[k].label), "TOTAL");
        rows[k].ms = total;
        ++k;
    }
    if (ctx->have_bwd) {  // the last gs_backward, after the forward rows
        GS_CK(cudaStreamSynchronize(ctx->stream));
        const char* labels[2] = {"raster backward", "preprocess backward"};
        for (int p = 0; p < 2 && k < max_rows; ++p, ++k) {
            std::snprintf(rows[k].label, sizeof(rows[k].label), "%s", labels[p]);
            cudaEventElapsedTime(&rows[k].ms, ctx->bev[p], ctx->bev[p + 1]);
        }
    }
    *n_rows = k;
    return GS_OK;
}

// ---- backward --------------------------------------------------------------------------------------
// Raster backward of frame f into f.grad2d (dL/d of its per-Gaussian 2D quantities).
static int enqueue_raster_backward(gs_ctx* ctx, Frame& f, const gs_scene* scene, const float* dl, cudaStream_t s,
                                   cudaEvent_t* ev = nullptr) {
    const float* before = f.grad2d.p;
    GS_CK(f.grad2d.reserve((size_t)scene->n * 9 + 4));  // + 4: the preprocess backward copies whole 16-byte units
    if (f.grad2d.p != before) f.grad2d_zero = false;
    // the preprocess backward clears what it read, so a buffer that went through one needs no memset
    if (scene->n && !f.grad2d_zero) GS_CK(cudaMemsetAsync(f.grad2d.p, 0, f.grad2d.cap * sizeof(float), s));
    f.grad2d_zero = false;
    if (ev) cudaEventRecord(ev[0], s);
    launch_raster_backward(ctx->cfg.tile_size, ctx->cfg.raster_batch, f.ranges.p, f.vals[f.sorted_buf].p, f.rec.p,
                           scene->n, f.ctl.p, f.width, f.height, f.tiles_x, f.tiles_y, f.final_t.p, f.n_contrib.p, dl,
                           f.grad2d.p, f.order.p, s);
    if (ev) cudaEventRecord(ev[1], s);
    GS_CK(cudaGetLastError());
    return GS_OK;
}

// Raster backward of frame f into f.grad2d, then the preprocess backward into `out` in the packed
// layout.
static int enqueue_backward(gs_ctx* ctx, Frame& f, const gs_scene* scene, const float* dl, float* out, cudaStream_t s,
                            cudaEvent_t* ev = nullptr) {
    const int rc = enqueue_raster_backward(ctx, f, scene, dl, s, ev);
    if (rc != GS_OK) return rc;
    launch_preprocess_backward(scene->rows, scene->stride, scene->n, f.view_used, f.counts.p, f.grad2d.p, out,
                               &f.ctl.p->status, s);
    if (ev) cudaEventRecord(ev[2], s);
    GS_CK(cudaGetLastError());
    f.grad2d_zero = true;
    return GS_OK;
}

int gs_backward(gs_ctx* ctx, const gs_scene* scene, const float* dl_drgb, float* grad_packed, int32_t location) {
    if (!ctx) return GS_ERR_INVALID;
    if (!scene || !dl_drgb || !grad_packed || (location != GS_MEM_HOST && location != GS_MEM_DEVICE))
        return fail(ctx, GS_ERR_INVALID, "gs_backward: bad argument");
    if (!(ctx->cfg.flags & GS_FLAG_DIFFERENTIABLE))
        return fail(ctx, GS_ERR_STATE, "gs_backward: context was created without GS_FLAG_DIFFERENTIABLE");
    Frame& f = ctx->main;
    if (!f.valid || f.scene != scene || f.n != scene->n)
        return fail(ctx, GS_ERR_STATE, "gs_backward: the last gs_forward on this context was not on this scene");
    GS_CK(cudaSetDevice(ctx->cfg.device));
    const size_t nfloats = (size_t)scene->n * kRows;
    const float* dl = dl_drgb;
    float* out = grad_packed;
    if (location == GS_MEM_HOST) {
        const size_t pix = (size_t)f.width * f.height;
        GS_CK(f.dl_stage.reserve(pix * 3));
        GS_CK(cudaMemcpyAsync(f.dl_stage.p, dl_drgb, pix * 12, cudaMemcpyHostToDevice, ctx->stream));
        dl = f.dl_stage.p;
        GS_CK(ctx->grad_stage.reserve(nfloats));
        out = ctx->grad_stage.p;
    }
    const bool profile = (ctx->cfg.flags & GS_FLAG_PROFILE) != 0;
    const int rc = enqueue_backward(ctx, f, scene, dl, out, ctx->stream, profile ? ctx->bev : nullptr);
    if (rc != GS_OK) return rc;
    ctx->have_bwd = profile;
    check_canaries(ctx, f, ctx->stream);
    GS_CK(cudaMemcpyAsync(&f.h_ctl->status, &f.ctl.p->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    if (location == GS_MEM_DEVICE) return GS_OK;
    if (nfloats) GS_CK(cudaMemcpyAsync(grad_packed, out, nfloats * 4, cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    // an overflow was reported by the forward
    return status_to_code(ctx, f.h_ctl->status & (kDevTimeout | kDevBounds | kDevCanary));
}

int gs_backward_batch(gs_ctx* ctx, const gs_scene* scene, const float* const* dl_drgb, uint32_t count,
                      float* grad_packed, int32_t location) {
    if (!ctx) return GS_ERR_INVALID;
    if (!scene || !dl_drgb || !grad_packed || count == 0 || (location != GS_MEM_HOST && location != GS_MEM_DEVICE))
        return fail(ctx, GS_ERR_INVALID, "gs_backward_batch: bad argument");
    if (!(ctx->cfg.flags & GS_FLAG_DIFFERENTIABLE))
        return fail(ctx, GS_ERR_STATE, "gs_backward_batch: context was created without GS_FLAG_DIFFERENTIABLE");
    if (count > ctx->batch_count) return fail(ctx, GS_ERR_STATE, "gs_backward_batch: more views than the last batch");
    for (uint32_t i = 0; i < count; ++i) {
        const Frame& f = *ctx->batch[i];
        if (!dl_drgb[i]) return fail(ctx, GS_ERR_INVALID, "gs_backward_batch: null dL/drgb");
        if (!f.valid || f.scene != scene || f.n != scene->n)
            return fail(ctx, GS_ERR_STATE, "gs_backward_batch: view " + std::to_string(i) + " of the last batch is not of this scene");
    }
    GS_CK(cudaSetDevice(ctx->cfg.device));
    const size_t nfloats = (size_t)scene->n * kRows;
    float* out = grad_packed;
    if (location == GS_MEM_HOST) {
        GS_CK(ctx->grad_stage.reserve(nfloats));
        out = ctx->grad_stage.p;
    }
    std::vector<const float*> dls(count);
    for (uint32_t i = 0; i < count; ++i) {
        Frame& f = *ctx->batch[i];
        dls[i] = dl_drgb[i];
        if (location == GS_MEM_HOST) {
            const size_t pix = (size_t)f.width * f.height;
            GS_CK(f.dl_stage.reserve(pix * 3));
            GS_CK(cudaMemcpyAsync(f.dl_stage.p, dl_drgb[i], pix * 12, cudaMemcpyHostToDevice, ctx->stream));
            dls[i] = f.dl_stage.p;
        }
    }
    // the views' raster backwards run concurrently on the side streams, each into its own frame's 2D
    // gradients; one preprocess backward per group of up to 16 views then reads the scene once and
    // sums the views' attribute gradients in the packed layout
    GS_CK(cudaEventRecord(ctx->fork, ctx->stream));
    const int used = (int)std::min<uint32_t>(count, kSideStreams);
    for (int s = 0; s < used; ++s) GS_CK(cudaStreamWaitEvent(ctx->side[s], ctx->fork, 0));
    for (uint32_t i = 0; i < count; ++i) {
        const int rc = enqueue_raster_backward(ctx, *ctx->batch[i], scene, dls[i], ctx->side[i % used]);
        if (rc != GS_OK) return rc;
    }
    for (int s = 0; s < used; ++s) {
        GS_CK(cudaEventRecord(ctx->join[s], ctx->side[s]));
        GS_CK(cudaStreamWaitEvent(ctx->stream, ctx->join[s], 0));
    }
    for (uint32_t g0 = 0; g0 < count; g0 += kMaxMultiViews) {
        MultiViewGrads mv{};
        mv.count = std::min<uint32_t>(kMaxMultiViews, count - g0);
        for (uint32_t v = 0; v < mv.count; ++v) {
            Frame& f = *ctx->batch[g0 + v];
            mv.view[v] = f.view_used;
            mv.counts[v] = f.counts.p;
            mv.grad2d[v] = f.grad2d.p;
        }
        launch_preprocess_backward_multi(scene->rows, scene->stride, scene->n, mv, out, g0 != 0,
                                         &ctx->batch[g0]->ctl.p->status, ctx->stream);
    }
    GS_CK(cudaGetLastError());
    for (uint32_t i = 0; i < count; ++i) ctx->batch[i]->grad2d_zero = true;
    for (uint32_t i = 0; i < count; ++i) {
        Frame& f = *ctx->batch[i];
        check_canaries(ctx, f, ctx->stream);
        GS_CK(cudaMemcpyAsync(&f.h_ctl->status, &f.ctl.p->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (location == GS_MEM_DEVICE) return GS_OK;
    if (nfloats) GS_CK(cudaMemcpyAsync(grad_packed, out, nfloats * 4, cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    uint32_t status = 0;
    for (uint32_t i = 0; i < count; ++i) status |= ctx->batch[i]->h_ctl->status;
    return status_to_code(ctx, status & (kDevTimeout | kDevBounds | kDevCanary));  // an overflow was reported by the forward
}

int gs_loss_l1_ssim(gs_ctx* ctx, const float* rgb, const float* target, uint32_t width, uint32_t height,
                    float lambda, double* loss, float* dl_drgb, int32_t location) {
    if (!ctx) return GS_ERR_INVALID;
    if (!rgb || !target || width == 0 || height == 0 || height > 65535u ||
        (location != GS_MEM_HOST && location != GS_MEM_DEVICE))
        return fail(ctx, GS_ERR_INVALID, "gs_loss_l1_ssim: bad argument");
    GS_CK(cudaSetDevice(ctx->cfg.device));
    const size_t pix = (size_t)width * height;
    GS_CK(ctx->loss_scratch.reserve(loss_scratch_floats(width, height)));
    GS_CK(ctx->loss_sums.reserve(loss_sum_doubles(width, height)));
    const float* x = rgb;
    const float* y = target;
    float* dl = dl_drgb;
    if (location == GS_MEM_HOST) {
        GS_CK(ctx->loss_io.reserve(pix * 9));
        float* dx = ctx->loss_io.p;
        GS_CK(cudaMemcpyAsync(dx, rgb, pix * 12, cudaMemcpyHostToDevice, ctx->stream));
        GS_CK(cudaMemcpyAsync(dx + pix * 3, target, pix * 12, cudaMemcpyHostToDevice, ctx->stream));
        x = dx;
        y = dx + pix * 3;
        dl = dl_drgb ? dx + pix * 6 : nullptr;
    }
    launch_loss_l1_ssim(x, y, width, height, lambda, ctx->loss_scratch.p, ctx->loss_sums.p, dl, ctx->stream);
    GS_CK(cudaGetLastError());
    if (location == GS_MEM_HOST && dl_drgb)
        GS_CK(cudaMemcpyAsync(dl_drgb, dl, pix * 12, cudaMemcpyDeviceToHost, ctx->stream));
    if (loss || location == GS_MEM_HOST) {
        double sums[2] = {0.0, 0.0};
        GS_CK(cudaMemcpyAsync(sums, ctx->loss_sums.p, sizeof(sums), cudaMemcpyDeviceToHost, ctx->stream));
        GS_CK(cudaStreamSynchronize(ctx->stream));
        const double cnt = 3.0 * (double)pix;
        if (loss) *loss = sums[1] / cnt + (double)lambda * (1.0 - sums[0] / cnt);
    }
    return GS_OK;
}

// ---- autotuner -------------------------------------------------------------------------------------
int gs_autotune_scenes(const gs_config* base, const float* const* packed, const uint32_t* counts, uint32_t n_scenes,
                       const gs_view* views, const uint32_t* view_scene, uint32_t n_views, uint32_t iters,
                       gs_config* best, float* best_ms) {
    if (!packed || !counts || n_scenes == 0 || !views || n_views == 0 || !best) return GS_ERR_INVALID;
    for (uint32_t s = 0; s < n_scenes; ++s)
        if (!packed[s] && counts[s]) return GS_ERR_INVALID;
    for (uint32_t i = 0; i < n_views; ++i)
        if (view_scene && view_scene[i] >= n_scenes) return GS_ERR_INVALID;
    gs_config b;
    gs_config_default(&b);
    if (base) b = *base;
    // times one configuration on the whole batch (its own context and scene copies): ms per batch
    auto time_config = [&](const gs_config& c, uint32_t reps, float* ms) -> int {
        gs_ctx* ctx = nullptr;
        if (gs_ctx_create(&c, &ctx) != GS_OK) return GS_ERR_CUDA;
        std::vector<gs_scene*> scs(n_scenes, nullptr);
        int rc = GS_OK;
        for (uint32_t s = 0; rc == GS_OK && s < n_scenes; ++s)
            rc = gs_scene_upload(ctx, packed[s], counts[s], GS_MEM_HOST, &scs[s]);
        std::vector<gs_batch_view> bv(n_views);
        std::vector<uint32_t*> imgs(n_views, nullptr);
        for (uint32_t i = 0; rc == GS_OK && i < n_views; ++i) {
            const size_t pix = (size_t)views[i].texture_size[0] * (size_t)views[i].texture_size[1];
            if (cudaMalloc(&imgs[i], pix * 4) != cudaSuccess) rc = GS_ERR_OOM;
            bv[i].scene = scs[view_scene ? view_scene[i] : 0];
            bv[i].view = views[i];
            bv[i].out = gs_image{GS_MEM_DEVICE, reinterpret_cast<uint8_t*>(imgs[i]), nullptr, nullptr, nullptr};
        }
        *ms = 0.0f;
        if (rc == GS_OK) {
            for (int w = 0; w < 2 && (rc == GS_OK || rc == GS_ERR_OVERFLOW); ++w)
                rc = gs_forward_batch(ctx, bv.data(), n_views);
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            cudaEventRecord(e0, ctx->stream);
            for (uint32_t k = 0; k < reps && (rc == GS_OK || rc == GS_ERR_OVERFLOW); ++k)
                rc = gs_forward_batch(ctx, bv.data(), n_views);
            cudaEventRecord(e1, ctx->stream);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(ms, e0, e1);
            *ms /= (float)reps;
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            if (rc == GS_OK || rc == GS_ERR_OVERFLOW) rc = gs_ctx_synchronize(ctx);
        }
        for (uint32_t* p : imgs)
            if (p) cudaFree(p);
        for (gs_scene* sc : scs)
            if (sc) gs_scene_destroy(sc);
        gs_ctx_destroy(ctx);
        return rc == GS_ERR_OVERFLOW ? GS_OK : rc;
    };
    // every candidate with `iters` timed batches, then the three fastest again with four times as
    // many: a close second of the first sweep is often the faster one
    const uint32_t tiles[] = {8, 16, 32};
    const uint32_t digits[] = {4, 8};
    const uint32_t batches[] = {32, 64, 128, 256};
    const uint32_t blocks[] = {kSortPartitionMin, kSortPartition};
    const uint32_t reps = std::max(iters, 1u);
    std::vector<std::pair<float, gs_config>> timed;
    for (uint32_t t : tiles)
        for (uint32_t d : digits)
            for (uint32_t r : batches)
                for (uint32_t sb : blocks) {
                    gs_config c = b;
                    c.tile_size = t;
                    c.digit_bits = d;
                    c.raster_batch = r;
                    c.sort_block = sb;
                    c.flags &= ~(GS_FLAG_PROFILE | GS_FLAG_DIFFERENTIABLE);
                    float ms = 0.0f;
                    const int rc = time_config(c, reps, &ms);
                    if (rc != GS_OK) return rc;
                    timed.emplace_back(ms, c);
                }
    std::sort(timed.begin(), timed.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
    float best_t = 3.0e38f;
    gs_config best_c = b;
    for (size_t k = 0; k < std::min<size_t>(3, timed.size()); ++k) {
        float ms = 0.0f;
        const int rc = time_config(timed[k].second, 4 * reps, &ms);
        if (rc != GS_OK) return rc;
        if (ms < best_t) {
            best_t = ms;
            best_c = timed[k].second;
        }
    }
    best_c.flags = b.flags;
    *best = best_c;
    if (best_ms) *best_ms = best_t;
    return GS_OK;
}

int gs_autotune(const gs_config* base, const float* packed, uint32_t count, const gs_view* views, uint32_t n_views,
                uint32_t iters, gs_config* best, float* best_ms) {
    if (!packed && count) return GS_ERR_INVALID;
    return gs_autotune_scenes(base, &packed, &count, 1, views, nullptr, n_views, iters, best, best_ms);
}

// ---- building blocks -------------------------------------------------------------------------------
int gs_sort_pairs(gs_ctx* ctx, uint32_t* keys, uint32_t* vals, uint32_t n, uint32_t key_bits, int32_t location) {
    if (!ctx) return GS_ERR_INVALID;
    if ((!keys || !vals) && n) return fail(ctx, GS_ERR_INVALID, "gs_sort_pairs: null buffer");
    if (key_bits == 0 || key_bits > 32 || (location != GS_MEM_HOST && location != GS_MEM_DEVICE))
        return fail(ctx, GS_ERR_INVALID, "gs_sort_pairs: bad argument");
    if (n == 0) return GS_OK;
    GS_CK(cudaSetDevice(ctx->cfg.device));
    const uint32_t bits = ctx->cfg.digit_bits, radix = 1u << bits;
    const uint32_t passes = (key_bits + bits - 1) / bits;
    GS_CK(ctx->aux_u32.reserve((size_t)n * 4));
    uint32_t* k0 = ctx->aux_u32.p;
    uint32_t* v0 = k0 + n;
    uint32_t* k1 = v0 + n;
    uint32_t* v1 = k1 + n;
    const size_t words = onesweep_flag_words(((size_t)n + ctx->cfg.sort_block - 1) / ctx->cfg.sort_block, radix);
    if (words > ctx->aux_flags.cap || !ctx->aux_flags.p) {
        GS_CK(ctx->aux_flags.reserve(words));
        GS_CK(cudaMemsetAsync(ctx->aux_flags.p, 0, ctx->aux_flags.cap * 8, ctx->stream));
    }
    const cudaMemcpyKind kin = location == GS_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    GS_CK(cudaMemcpyAsync(k0, keys, (size_t)n * 4, kin, ctx->stream));
    GS_CK(cudaMemcpyAsync(v0, vals, (size_t)n * 4, kin, ctx->stream));
    FrameCtl* ctl = ctx->aux_ctl.p;
    launch_frame_begin(ctl, ctx->aux_flags.p, (uint32_t)ctx->aux_flags.cap, ctx->stream);
    launch_digit_hist(k0, n, bits, key_bits, ctl->hist, ctx->stream);
    uint32_t* kb[2] = {k0, k1};
    uint32_t* vb[2] = {v0, v1};
    int cur = 0;
    for (uint32_t p = 0; p < passes; ++p) {
        const uint32_t left = key_bits - p * bits;
        const uint32_t dmask = left >= bits ? radix - 1u : (1u << left) - 1u;
        launch_onesweep(bits, kb[cur], vb[cur], kb[cur ^ 1], vb[cur ^ 1], nullptr, n, n, p * bits, dmask,
                        ctl->hist + p * radix, ctl, ctx->aux_flags.p, 1 + p, 0, ctx->stream, ctx->cfg.sort_block);
        cur ^= 1;
    }
    GS_CK(cudaGetLastError());
    const cudaMemcpyKind kout = location == GS_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    GS_CK(cudaMemcpyAsync(keys, kb[cur], (size_t)n * 4, kout, ctx->stream));
    GS_CK(cudaMemcpyAsync(vals, vb[cur], (size_t)n * 4, kout, ctx->stream));
    GS_CK(cudaMemcpyAsync(ctx->h_aux, ctl, offsetof(FrameCtl, tickets), cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    return status_to_code(ctx, ctx->h_aux->status);
}

int gs_exclusive_scan(gs_ctx* ctx, uint32_t* data, uint32_t n, uint32_t* total, int32_t location) {
    if (!ctx) return GS_ERR_INVALID;
    if ((!data && n) || (location != GS_MEM_HOST && location != GS_MEM_DEVICE))
        return fail(ctx, GS_ERR_INVALID, "gs_exclusive_scan: bad argument");
    GS_CK(cudaSetDevice(ctx->cfg.device));
    GS_CK(ctx->aux_u32.reserve((size_t)n + 1));
    uint32_t* d = ctx->aux_u32.p;
    const size_t words = ((size_t)n + kScanPartition - 1) / kScanPartition + 1;
    if (words > ctx->aux_flags.cap || !ctx->aux_flags.p) {
        GS_CK(ctx->aux_flags.reserve(words));
        GS_CK(cudaMemsetAsync(ctx->aux_flags.p, 0, ctx->aux_flags.cap * 8, ctx->stream));
    }
    const cudaMemcpyKind kin = location == GS_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (n) GS_CK(cudaMemcpyAsync(d, data, (size_t)n * 4, kin, ctx->stream));
    FrameCtl* ctl = ctx->aux_ctl.p;
    launch_frame_begin(ctl, ctx->aux_flags.p, (uint32_t)ctx->aux_flags.cap, ctx->stream);
    GS_CK(cudaMemsetAsync(d + n, 0, 4, ctx->stream));
    launch_exclusive_scan(d, n, d + n, ctl, ctx->aux_flags.p, 0, ctx->stream);
    GS_CK(cudaGetLastError());
    const cudaMemcpyKind kout = location == GS_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (n) GS_CK(cudaMemcpyAsync(data, d, (size_t)n * 4, kout, ctx->stream));
    uint32_t tot = 0;
    GS_CK(cudaMemcpyAsync(ctx->h_aux, ctl, offsetof(FrameCtl, tickets), cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaMemcpyAsync(&tot, d + n, 4, cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    if (total) *total = tot;
    return status_to_code(ctx, ctx->h_aux->status);
}

int gs_check_wait_timeout(gs_ctx* ctx) {
    if (!ctx) return GS_ERR_INVALID;
    GS_CK(cudaSetDevice(ctx->cfg.device));
    // a two-partition scan run by one CTA that is handed the second partition's ticket: its lookback
    // waits for the first partition's word, which nothing writes
    const uint32_t n = 2 * kScanPartition;
    GS_CK(ctx->aux_u32.reserve((size_t)n + 1));
    const size_t words = (size_t)n / kScanPartition + 1;
    if (words > ctx->aux_flags.cap || !ctx->aux_flags.p) {
        GS_CK(ctx->aux_flags.reserve(words));
        GS_CK(cudaMemsetAsync(ctx->aux_flags.p, 0, ctx->aux_flags.cap * 8, ctx->stream));
    }
    GS_CK(cudaMemsetAsync(ctx->aux_u32.p, 0, ((size_t)n + 1) * 4, ctx->stream));
    FrameCtl* ctl = ctx->aux_ctl.p;
    launch_frame_begin(ctl, ctx->aux_flags.p, (uint32_t)ctx->aux_flags.cap, ctx->stream);
    static const uint32_t kOne = 1u;
    GS_CK(cudaMemcpyAsync(&ctl->tickets[0], &kOne, sizeof(kOne), cudaMemcpyHostToDevice, ctx->stream));
    launch_exclusive_scan(ctx->aux_u32.p, n, ctx->aux_u32.p + n, ctl, ctx->aux_flags.p, 0, ctx->stream, 1);
    GS_CK(cudaGetLastError());
    GS_CK(cudaMemcpyAsync(ctx->h_aux, ctl, offsetof(FrameCtl, tickets), cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    return status_to_code(ctx, ctx->h_aux->status);
}

int gs_debug_set_sequence(gs_ctx* ctx, uint32_t seq) {
    if (!ctx) return static_scan_set_sequence(seq) == cudaSuccess ? GS_OK : GS_ERR_CUDA;
    GS_CK(cudaSetDevice(ctx->cfg.device));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    std::vector<FrameCtl*> ctls = {ctx->main.ctl.p, ctx->aux_ctl.p};
    for (Frame* f : ctx->batch) ctls.push_back(f->ctl.p);
    for (FrameCtl* c : ctls)
        if (c) GS_CK(cudaMemcpy(&c->seq, &seq, sizeof(seq), cudaMemcpyHostToDevice));
    return GS_OK;
}

int gs_checked_build(void) {
#ifdef GS_CHECKED
    return 1;
#else
    return 0;
#endif
}

int gs_debug_damage_canary(gs_ctx* ctx) {
    if (!ctx) return GS_ERR_INVALID;
#ifdef GS_CHECKED
    Frame& f = ctx->main;
    if (!f.keys[0].raw) return fail(ctx, GS_ERR_STATE, "gs_debug_damage_canary: no frame rendered");
    GS_CK(cudaSetDevice(ctx->cfg.device));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    const uint32_t zero = 0u;
    // the first word of the tail pad: allocated memory, outside the buffer the kernels may write
    GS_CK(cudaMemcpy(f.keys[0].raw + kCanaryBytes + f.keys[0].cap * sizeof(uint32_t), &zero, sizeof(zero),
                     cudaMemcpyHostToDevice));
    return GS_OK;
#else
    return fail(ctx, GS_ERR_UNSUPPORTED, "gs_debug_damage_canary: product build (no canaries)");
#endif
}

static int exp_f32(gs_ctx* ctx, const float* x, float* y, uint32_t n, int32_t location, bool raster) {
    if (!ctx) return GS_ERR_INVALID;
    if ((!x || !y) && n) return fail(ctx, GS_ERR_INVALID, "gs_exp_f32: null buffer");
    if (n == 0) return GS_OK;
    GS_CK(cudaSetDevice(ctx->cfg.device));
    if (location == GS_MEM_DEVICE) {
        launch_exp(x, y, n, ctx->stream, raster);
        GS_CK(cudaGetLastError());
        return GS_OK;
    }
    GS_CK(ctx->aux_f32.reserve((size_t)n * 2));
    float* dx = ctx->aux_f32.p;
    float* dy = dx + n;
    GS_CK(cudaMemcpyAsync(dx, x, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    launch_exp(dx, dy, n, ctx->stream, raster);
    GS_CK(cudaGetLastError());
    GS_CK(cudaMemcpyAsync(y, dy, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    return GS_OK;
}

int gs_exp_f32(gs_ctx* ctx, const float* x, float* y, uint32_t n, int32_t location) {
    return exp_f32(ctx, x, y, n, location, false);
}

int gs_raster_exp_f32(gs_ctx* ctx, const float* x, float* y, uint32_t n, int32_t location) {
    return exp_f32(ctx, x, y, n, location, true);
}

int gs_raster_alpha_f32(gs_ctx* ctx, const float* o, const float* x, float* y, uint32_t n, int32_t location) {
    if (!ctx) return GS_ERR_INVALID;
    if ((!o || !x || !y) && n) return fail(ctx, GS_ERR_INVALID, "gs_raster_alpha_f32: null buffer");
    if (location != GS_MEM_HOST && location != GS_MEM_DEVICE)
        return fail(ctx, GS_ERR_INVALID, "gs_raster_alpha_f32: bad location");
    if (n == 0) return GS_OK;
    GS_CK(cudaSetDevice(ctx->cfg.device));
    if (location == GS_MEM_DEVICE) {
        launch_raster_alpha(o, x, y, n, ctx->stream);
        GS_CK(cudaGetLastError());
        return GS_OK;
    }
    GS_CK(ctx->aux_f32.reserve((size_t)n * 3));
    float* d_o = ctx->aux_f32.p;
    float* d_x = d_o + n;
    float* d_y = d_x + n;
    GS_CK(cudaMemcpyAsync(d_o, o, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    GS_CK(cudaMemcpyAsync(d_x, x, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    launch_raster_alpha(d_o, d_x, d_y, n, ctx->stream);
    GS_CK(cudaGetLastError());
    GS_CK(cudaMemcpyAsync(y, d_y, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    return GS_OK;
}

}  // extern "C"
