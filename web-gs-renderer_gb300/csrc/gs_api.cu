// gs_api.cu -- the C ABI of libwebgs.so (include/gs.h).
//
// Replaces the reference Renderer (src/renderer/renderer.js): the context owns one CUDA stream and
// the per-frame buffers (sized from count * MAX_INSTANCE_FACTOR like renderer.js:531-577, grown on
// demand and kept), and gs_forward sequences the passes of renderer.js:822-932 on that stream,
// replayed from one CUDA graph per (scene, resolution, output set). No pass reads a count back to
// the host: the instance count travels in FrameCtl, which every later kernel reads on the device
// (the reference's indirect dispatch, indirect_arg.wgsl).
#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gs.h"
#include "gs_kernels.h"

using namespace gs;

namespace {

const char* kNoCtxError = "invalid context";

template <class T> struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;  // elements
    cudaError_t reserve(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(n, 1);
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e != cudaSuccess) { p = nullptr; return e; }
        cap = want;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

uint32_t bitlen(uint32_t v) { return v == 0 ? 0u : 32u - (uint32_t)__builtin_clz(v); }

struct GraphKey {
    const void* scene = nullptr;
    uint32_t n = 0, w = 0, h = 0;
    const void* o_rgba = nullptr;
    const void* o_rgb = nullptr;
    const void* o_t = nullptr;
    const void* o_c = nullptr;
    uint64_t alloc_gen = 0;
    bool operator==(const GraphKey& o) const {
        return scene == o.scene && n == o.n && w == o.w && h == o.h && o_rgba == o.o_rgba && o_rgb == o.o_rgb &&
               o_t == o.o_t && o_c == o.o_c && alloc_gen == o.alloc_gen;
    }
};

constexpr int kViewSlots = 16;
enum Pass { kPassPreprocess, kPassScanEmit, kPassSort, kPassRanges, kPassRaster, kPassCount };
const char* kPassLabel[kPassCount] = {"preprocess", "scan+emit", "sort", "tile ranges", "raster"};

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
    std::string err;

    DevBuf<FrameCtl> ctl, aux_ctl;
    FrameCtl* h_ctl = nullptr;  // pinned readback of the counters
    DevBuf<ViewBlock> view;
    DevBuf<float4> rec;
    DevBuf<uint4> meta;
    DevBuf<uint32_t> counts, offsets;
    DevBuf<uint32_t> keys[2], vals[2];
    DevBuf<uint64_t> flags, aux_flags;
    DevBuf<uint32_t> ranges;
    DevBuf<uint32_t> rgba8, n_contrib;
    DevBuf<float> rgb, final_t;
    DevBuf<uint32_t> aux_u32;
    DevBuf<float> aux_f32;
    // backward and loss
    DevBuf<float> grad2d, grows, dl_stage, grad_stage, loss_scratch, loss_io;
    DevBuf<double> loss_sums;

    // last frame
    const gs_scene* last_scene = nullptr;
    uint32_t last_n = 0, width = 0, height = 0, tiles_x = 0, tiles_y = 0, passes = 0, max_instance = 0;
    int sorted_buf = 0;
    bool have_frame = false;

    // graph cache (alloc_gen changes whenever a frame buffer is reallocated)
    uint64_t alloc_gen = 0;
    cudaGraphExec_t exec = nullptr;
    GraphKey key{};

    // pinned ring of view blocks: the H2D copy of a frame's 176-byte view reads from a slot that is
    // not rewritten until that copy has completed (slot_done), so frames never block the host
    ViewBlock* h_views = nullptr;
    cudaEvent_t slot_done[kViewSlots] = {};
    uint32_t next_slot = 0;

    // profiling
    cudaEvent_t ev[kPassCount + 1] = {};
    float pass_ms[kPassCount] = {};
    bool have_timing = false;
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

int status_to_code(gs_ctx* ctx, uint32_t status) {
    if (status & kDevTimeout) return fail(ctx, GS_ERR_TIMEOUT, "a device-side wait hit its iteration limit");
    if (status & kDevOverflow)
        return fail(ctx, GS_ERR_OVERFLOW, "instance count exceeded max_instance; output truncated");
    return GS_OK;
}

bool valid_config(const gs_config& c) {
    const bool tile_ok = c.tile_size == 8 || c.tile_size == 16 || c.tile_size == 32;
    const bool digit_ok = c.digit_bits == 4 || c.digit_bits == 8;
    const bool batch_ok = c.raster_batch == 32 || c.raster_batch == 64 || c.raster_batch == 128 || c.raster_batch == 256;
    return tile_ok && digit_ok && batch_ok && c.max_instance_factor >= 1;
}

// Grows the per-frame buffers for a frame of n Gaussians and `tiles` tiles of w x h pixels.
int ensure_frame_buffers(gs_ctx* ctx, uint32_t n, uint64_t max_instance, uint32_t tiles, uint32_t w, uint32_t h) {
    const uint32_t radix = 1u << ctx->cfg.digit_bits;
    const void* before[] = {ctx->rec.p, ctx->meta.p, ctx->counts.p, ctx->offsets.p, ctx->keys[0].p, ctx->keys[1].p,
                            ctx->vals[0].p, ctx->vals[1].p, ctx->flags.p, ctx->ranges.p, ctx->rgba8.p, ctx->rgb.p,
                            ctx->final_t.p, ctx->n_contrib.p};
    GS_CK(ctx->rec.reserve((size_t)n * kRecFloat4));
    GS_CK(ctx->meta.reserve(n));
    GS_CK(ctx->counts.reserve(((size_t)n + 1 + 7) / 8 * 8));
    GS_CK(ctx->offsets.reserve((size_t)n + 1));
    for (int b = 0; b < 2; ++b) {
        GS_CK(ctx->keys[b].reserve(max_instance));
        GS_CK(ctx->vals[b].reserve(max_instance));
    }
    const size_t sort_parts = (max_instance + kSortPartition - 1) / kSortPartition;
    const size_t scan_parts = ((size_t)n + 1 + kScanPartition - 1) / kScanPartition;
    const size_t words = std::max(sort_parts * radix, scan_parts);
    if (words > ctx->flags.cap || !ctx->flags.p) {
        GS_CK(ctx->flags.reserve(words));
        GS_CK(cudaMemsetAsync(ctx->flags.p, 0, ctx->flags.cap * sizeof(uint64_t), ctx->stream));
    }
    GS_CK(ctx->ranges.reserve((size_t)tiles * 2));
    const size_t pix = (size_t)w * h;
    GS_CK(ctx->rgba8.reserve(pix));
    GS_CK(ctx->rgb.reserve(pix * 3));
    GS_CK(ctx->final_t.reserve(pix));
    GS_CK(ctx->n_contrib.reserve(pix));
    const void* after[] = {ctx->rec.p, ctx->meta.p, ctx->counts.p, ctx->offsets.p, ctx->keys[0].p, ctx->keys[1].p,
                           ctx->vals[0].p, ctx->vals[1].p, ctx->flags.p, ctx->ranges.p, ctx->rgba8.p, ctx->rgb.p,
                           ctx->final_t.p, ctx->n_contrib.p};
    if (std::memcmp(before, after, sizeof(before)) != 0) ++ctx->alloc_gen;
    return GS_OK;
}

struct FrameArgs {
    const gs_scene* scene;
    uint32_t n, w, h, tiles_x, tiles_y, passes, max_instance;
    RasterOut out;
};

// Enqueues one frame (renderer.js:822-932) on the context stream.
void enqueue_frame(gs_ctx* ctx, const FrameArgs& a, bool profile) {
    cudaStream_t s = ctx->stream;
    const uint32_t bits = ctx->cfg.digit_bits, radix = 1u << bits;
    FrameCtl* ctl = ctx->ctl.p;
    if (profile) cudaEventRecord(ctx->ev[0], s);
    launch_frame_begin(ctl, s);
    launch_preprocess(a.scene->rows, a.scene->stride, a.n, ctx->view.p, ctx->cfg.tile_size, ctx->rec.p, ctx->meta.p,
                      ctx->counts.p, ctl, s);
    if (profile) cudaEventRecord(ctx->ev[1], s);
    launch_scan_emit(ctx->counts.p, ctx->meta.p, a.n, a.tiles_x, a.max_instance, bits, a.passes, ctx->offsets.p,
                     ctx->keys[0].p, ctx->vals[0].p, ctl, ctx->flags.p, 0, s);
    if (profile) cudaEventRecord(ctx->ev[2], s);
    int cur = 0;
    for (uint32_t p = 0; p < a.passes; ++p) {
        launch_onesweep(bits, ctx->keys[cur].p, ctx->vals[cur].p, ctx->keys[cur ^ 1].p, ctx->vals[cur ^ 1].p,
                        &ctl->sorted_count, 0, a.max_instance, p * bits, radix - 1u, ctl->hist + p * radix, ctl,
                        ctx->flags.p, 1 + p, 0, s);
        cur ^= 1;
    }
    ctx->sorted_buf = cur;
    if (profile) cudaEventRecord(ctx->ev[3], s);
    cudaMemsetAsync(ctx->ranges.p, 0, (size_t)a.tiles_x * a.tiles_y * 2 * sizeof(uint32_t), s);
    launch_tile_ranges(ctx->keys[cur].p, ctl, a.tiles_x * a.tiles_y, ctx->ranges.p, 0, s);
    if (profile) cudaEventRecord(ctx->ev[4], s);
    launch_raster(ctx->cfg.tile_size, ctx->cfg.raster_batch, ctx->ranges.p, ctx->vals[cur].p, ctx->rec.p, a.n, ctl,
                  a.w, a.h, a.tiles_x, a.tiles_y, a.out, s);
    if (profile) cudaEventRecord(ctx->ev[5], s);
}

}  // namespace

// =====================================================================================================
extern "C" {

const char* gs_version(void) { return "webgs-gb300 0.1 (sm_103a)"; }

void gs_config_default(gs_config* cfg) {
    if (!cfg) return;
    cfg->tile_size = 16;            // TILE_SIZE_X/Y, renderer.js:25-26
    cfg->digit_bits = 8;            // RADIX_DIGITS = 256, renderer.js:67
    cfg->raster_batch = 256;        // TIlE_SIZE batch, raseter.wgsl:217
    cfg->max_instance_factor = 64;  // MAX_INSTANCE_FACTOR, renderer.js:16
    cfg->flags = 0;
    cfg->device = 0;
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
    gs_ctx* ctx = new gs_ctx();
    ctx->cfg = c;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        ctx->ctl.reserve(1) != cudaSuccess || ctx->aux_ctl.reserve(1) != cudaSuccess ||
        ctx->view.reserve(1) != cudaSuccess ||
        cudaMallocHost(&ctx->h_ctl, sizeof(FrameCtl)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_views, sizeof(ViewBlock) * kViewSlots) != cudaSuccess) {
        gs_ctx_destroy(ctx);
        return GS_ERR_OOM;
    }
    cudaMemsetAsync(ctx->ctl.p, 0, sizeof(FrameCtl), ctx->stream);
    cudaMemsetAsync(ctx->aux_ctl.p, 0, sizeof(FrameCtl), ctx->stream);
    for (auto& e : ctx->ev) cudaEventCreate(&e);
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
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : ctx->slot_done)
        if (e) cudaEventDestroy(e);
    if (ctx->h_views) cudaFreeHost(ctx->h_views);
    ctx->ctl.release(); ctx->aux_ctl.release(); ctx->view.release(); ctx->rec.release(); ctx->meta.release();
    ctx->counts.release(); ctx->offsets.release();
    for (int b = 0; b < 2; ++b) { ctx->keys[b].release(); ctx->vals[b].release(); }
    ctx->flags.release(); ctx->aux_flags.release(); ctx->ranges.release(); ctx->rgba8.release();
    ctx->n_contrib.release(); ctx->rgb.release(); ctx->final_t.release(); ctx->aux_u32.release(); ctx->aux_f32.release();
    ctx->grad2d.release(); ctx->grows.release(); ctx->dl_stage.release(); ctx->grad_stage.release();
    ctx->loss_scratch.release(); ctx->loss_io.release(); ctx->loss_sums.release();
    if (ctx->h_ctl) cudaFreeHost(ctx->h_ctl);
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
        if (ctx->key.scene == scene) {
            if (ctx->exec) cudaGraphExecDestroy(ctx->exec);
            ctx->exec = nullptr;
            ctx->key = GraphKey{};
        }
        if (ctx->last_scene == scene) {
            ctx->last_scene = nullptr;
            ctx->have_frame = false;
        }
    }
    if (scene->rows) cudaFree(scene->rows);
    delete scene;
    return GS_OK;
}

uint32_t gs_scene_count(const gs_scene* scene) { return scene ? scene->n : 0u; }

// ---- forward ---------------------------------------------------------------------------------------
int gs_forward(gs_ctx* ctx, const gs_scene* scene, const gs_view* view, const gs_image* out) {
    if (!ctx) return GS_ERR_INVALID;
    if (!scene || scene->ctx != ctx || !view || !out) return fail(ctx, GS_ERR_INVALID, "gs_forward: null argument");
    if (out->location != GS_MEM_HOST && out->location != GS_MEM_DEVICE)
        return fail(ctx, GS_ERR_INVALID, "gs_forward: bad output location");
    const float fw = view->texture_size[0], fh = view->texture_size[1];
    if (!(fw >= 1.0f) || !(fh >= 1.0f) || !(fw <= 65536.0f) || !(fh <= 65536.0f))
        return fail(ctx, GS_ERR_INVALID, "gs_forward: texture size out of range");
    const uint32_t w = (uint32_t)fw, h = (uint32_t)fh, tile = ctx->cfg.tile_size;
    const uint32_t tiles_x = (w + tile - 1) / tile, tiles_y = (h + tile - 1) / tile;
    const uint64_t tiles = (uint64_t)tiles_x * tiles_y;
    if (tiles > 65536u)
        return fail(ctx, GS_ERR_INVALID, "gs_forward: more than 65536 tiles do not fit the key's 16-bit tile field");
    const uint32_t n = scene->n;
    const uint32_t max_instance = n * ctx->cfg.max_instance_factor;
    const uint32_t key_bits = 16u + bitlen((uint32_t)tiles - 1u);
    const uint32_t passes = (key_bits + ctx->cfg.digit_bits - 1) / ctx->cfg.digit_bits;
    GS_CK(cudaSetDevice(ctx->cfg.device));
    int rc = ensure_frame_buffers(ctx, n, max_instance, (uint32_t)tiles, w, h);
    if (rc != GS_OK) return rc;

    const bool dev_out = out->location == GS_MEM_DEVICE;
    // a differentiable context keeps final_t / n_contrib of the last frame in its own buffers for
    // gs_backward; requested device copies of them are made after the frame
    const bool keep_state = (ctx->cfg.flags & GS_FLAG_DIFFERENTIABLE) != 0;
    RasterOut ro;
    ro.rgba8 = out->rgba8 ? (dev_out ? reinterpret_cast<uint32_t*>(out->rgba8) : ctx->rgba8.p) : nullptr;
    ro.rgb = out->rgb ? (dev_out ? out->rgb : ctx->rgb.p) : nullptr;
    if (keep_state) {
        ro.final_t = ctx->final_t.p;
        ro.n_contrib = ctx->n_contrib.p;
    } else {
        ro.final_t = out->final_t ? (dev_out ? out->final_t : ctx->final_t.p) : nullptr;
        ro.n_contrib = out->n_contrib ? (dev_out ? out->n_contrib : ctx->n_contrib.p) : nullptr;
    }

    {
        const uint32_t slot = ctx->next_slot;
        ctx->next_slot = (slot + 1) % kViewSlots;
        GS_CK(cudaEventSynchronize(ctx->slot_done[slot]));
        std::memcpy(&ctx->h_views[slot], view, sizeof(ViewBlock));
        GS_CK(cudaMemcpyAsync(ctx->view.p, &ctx->h_views[slot], sizeof(ViewBlock), cudaMemcpyHostToDevice, ctx->stream));
        GS_CK(cudaEventRecord(ctx->slot_done[slot], ctx->stream));
    }
    FrameArgs fa{scene, n, w, h, tiles_x, tiles_y, passes, max_instance, ro};
    const bool profile = (ctx->cfg.flags & GS_FLAG_PROFILE) != 0;
    const bool use_graph = !profile && (ctx->cfg.flags & GS_FLAG_NO_GRAPH) == 0;
    if (use_graph) {
        GraphKey k{scene, n, w, h, ro.rgba8, ro.rgb, ro.final_t, ro.n_contrib, ctx->alloc_gen};
        if (!ctx->exec || !(k == ctx->key)) {
            if (ctx->exec) cudaGraphExecDestroy(ctx->exec);
            ctx->exec = nullptr;
            cudaGraph_t g = nullptr;
            GS_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            enqueue_frame(ctx, fa, false);
            cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "graph capture");
            e = cudaGraphInstantiate(&ctx->exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { ctx->exec = nullptr; return cuda_fail(ctx, e, "graph instantiate"); }
            ctx->key = k;
        }
        ctx->sorted_buf = (int)(passes & 1u);
        GS_CK(cudaGraphLaunch(ctx->exec, ctx->stream));
    } else {
        enqueue_frame(ctx, fa, profile);
    }
    GS_CK(cudaGetLastError());
    ctx->last_scene = scene;
    ctx->last_n = n;
    ctx->width = w;
    ctx->height = h;
    ctx->tiles_x = tiles_x;
    ctx->tiles_y = tiles_y;
    ctx->passes = passes;
    ctx->max_instance = max_instance;
    ctx->have_frame = true;
    ctx->have_timing = false;
    GS_CK(cudaMemcpyAsync(ctx->h_ctl, ctx->ctl.p, offsetof(FrameCtl, tickets), cudaMemcpyDeviceToHost, ctx->stream));
    if (dev_out && keep_state) {
        const size_t pix = (size_t)w * h;
        if (out->final_t)
            GS_CK(cudaMemcpyAsync(out->final_t, ctx->final_t.p, pix * 4, cudaMemcpyDeviceToDevice, ctx->stream));
        if (out->n_contrib)
            GS_CK(cudaMemcpyAsync(out->n_contrib, ctx->n_contrib.p, pix * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    }

    if (!dev_out) {
        const size_t pix = (size_t)w * h;
        if (out->rgba8) GS_CK(cudaMemcpyAsync(out->rgba8, ctx->rgba8.p, pix * 4, cudaMemcpyDeviceToHost, ctx->stream));
        if (out->rgb) GS_CK(cudaMemcpyAsync(out->rgb, ctx->rgb.p, pix * 12, cudaMemcpyDeviceToHost, ctx->stream));
        if (out->final_t) GS_CK(cudaMemcpyAsync(out->final_t, ctx->final_t.p, pix * 4, cudaMemcpyDeviceToHost, ctx->stream));
        if (out->n_contrib)
            GS_CK(cudaMemcpyAsync(out->n_contrib, ctx->n_contrib.p, pix * 4, cudaMemcpyDeviceToHost, ctx->stream));
        GS_CK(cudaStreamSynchronize(ctx->stream));
        if (profile) {
            for (int p = 0; p < kPassCount; ++p) cudaEventElapsedTime(&ctx->pass_ms[p], ctx->ev[p], ctx->ev[p + 1]);
            ctx->have_timing = true;
        }
        return status_to_code(ctx, ctx->h_ctl->status);
    }
    return GS_OK;
}

int gs_get_frame_info(gs_ctx* ctx, gs_frame_info* info) {
    if (!ctx) return GS_ERR_INVALID;
    if (!info) return fail(ctx, GS_ERR_INVALID, "gs_get_frame_info: null info");
    if (!ctx->have_frame) return fail(ctx, GS_ERR_STATE, "gs_get_frame_info: no frame rendered");
    GS_CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->cfg.flags & GS_FLAG_PROFILE && !ctx->have_timing) {
        for (int p = 0; p < kPassCount; ++p) cudaEventElapsedTime(&ctx->pass_ms[p], ctx->ev[p], ctx->ev[p + 1]);
        ctx->have_timing = true;
    }
    const FrameCtl& c = *ctx->h_ctl;
    info->instance_count = c.instance_count;
    info->sorted_count = c.sorted_count;
    info->max_instance = ctx->max_instance;
    info->visible = c.visible;
    info->near_pass = c.near_pass;
    info->tiles_x = ctx->tiles_x;
    info->tiles_y = ctx->tiles_y;
    info->status = c.status;
    info->sort_passes = ctx->passes;
    return GS_OK;
}

int gs_get_debug(gs_ctx* ctx, const gs_debug* dbg) {
    if (!ctx) return GS_ERR_INVALID;
    if (!dbg) return fail(ctx, GS_ERR_INVALID, "gs_get_debug: null argument");
    if (!ctx->have_frame) return fail(ctx, GS_ERR_STATE, "gs_get_debug: no frame rendered");
    GS_CK(cudaStreamSynchronize(ctx->stream));
    const uint32_t n = ctx->last_n;
    if (dbg->tiles_touched) GS_CK(cudaMemcpy(dbg->tiles_touched, ctx->counts.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
    if (dbg->meta) GS_CK(cudaMemcpy(dbg->meta, ctx->meta.p, (size_t)n * 16, cudaMemcpyDeviceToHost));
    if (dbg->conic_opacity || dbg->pixel || dbg->color) {
        std::vector<float> rec((size_t)n * kRecFloat4 * 4);
        if (n) GS_CK(cudaMemcpy(rec.data(), ctx->rec.p, rec.size() * 4, cudaMemcpyDeviceToHost));
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
    if (dbg->offsets) GS_CK(cudaMemcpy(dbg->offsets, ctx->offsets.p, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost));
    const uint32_t sorted = ctx->h_ctl->sorted_count;
    const size_t kc = std::min<uint64_t>(sorted, dbg->capacity);
    if (dbg->keys && kc) GS_CK(cudaMemcpy(dbg->keys, ctx->keys[ctx->sorted_buf].p, kc * 4, cudaMemcpyDeviceToHost));
    if (dbg->vals && kc) GS_CK(cudaMemcpy(dbg->vals, ctx->vals[ctx->sorted_buf].p, kc * 4, cudaMemcpyDeviceToHost));
    if (dbg->ranges)
        GS_CK(cudaMemcpy(dbg->ranges, ctx->ranges.p, (size_t)ctx->tiles_x * ctx->tiles_y * 8, cudaMemcpyDeviceToHost));
    return GS_OK;
}

int gs_get_timings(gs_ctx* ctx, gs_timing* rows, int32_t max_rows, int32_t* n_rows) {
    if (!ctx) return GS_ERR_INVALID;
    if (!rows || !n_rows || max_rows < 0) return fail(ctx, GS_ERR_INVALID, "gs_get_timings: bad argument");
    if (!(ctx->cfg.flags & GS_FLAG_PROFILE)) return fail(ctx, GS_ERR_STATE, "gs_get_timings: context not profiling");
    if (!ctx->have_frame) return fail(ctx, GS_ERR_STATE, "gs_get_timings: no frame rendered");
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
    *n_rows = k;
    return GS_OK;
}

int gs_backward(gs_ctx* ctx, const gs_scene* scene, const float* dl_drgb, float* grad_packed, int32_t location) {
    if (!ctx) return GS_ERR_INVALID;
    if (!scene || !dl_drgb || !grad_packed || (location != GS_MEM_HOST && location != GS_MEM_DEVICE))
        return fail(ctx, GS_ERR_INVALID, "gs_backward: bad argument");
    if (!(ctx->cfg.flags & GS_FLAG_DIFFERENTIABLE))
        return fail(ctx, GS_ERR_STATE, "gs_backward: context was created without GS_FLAG_DIFFERENTIABLE");
    if (!ctx->have_frame || ctx->last_scene != scene || ctx->last_n != scene->n)
        return fail(ctx, GS_ERR_STATE, "gs_backward: the last gs_forward on this context was not on this scene");
    GS_CK(cudaSetDevice(ctx->cfg.device));
    const uint32_t n = scene->n, w = ctx->width, h = ctx->height;
    const size_t pix = (size_t)w * h;
    GS_CK(ctx->grad2d.reserve((size_t)n * 9));
    GS_CK(ctx->grows.reserve((size_t)scene->stride * kRows));
    const float* dl = dl_drgb;
    if (location == GS_MEM_HOST) {
        GS_CK(ctx->dl_stage.reserve(pix * 3));
        GS_CK(cudaMemcpyAsync(ctx->dl_stage.p, dl_drgb, pix * 12, cudaMemcpyHostToDevice, ctx->stream));
        dl = ctx->dl_stage.p;
    }
    if (n) GS_CK(cudaMemsetAsync(ctx->grad2d.p, 0, (size_t)n * 9 * sizeof(float), ctx->stream));
    launch_raster_backward(ctx->cfg.tile_size, ctx->cfg.raster_batch, ctx->ranges.p, ctx->vals[ctx->sorted_buf].p,
                           ctx->rec.p, n, ctx->ctl.p, w, h, ctx->tiles_x, ctx->tiles_y, ctx->final_t.p,
                           ctx->n_contrib.p, dl, ctx->grad2d.p, ctx->stream);
    launch_preprocess_backward(scene->rows, scene->stride, n, ctx->view.p, ctx->counts.p, ctx->grad2d.p,
                               ctx->grows.p, ctx->stream);
    GS_CK(cudaGetLastError());
    if (location == GS_MEM_DEVICE) {
        launch_rows_to_pack(ctx->grows.p, n, scene->stride, grad_packed, ctx->stream);
        GS_CK(cudaGetLastError());
        return GS_OK;
    }
    GS_CK(ctx->grad_stage.reserve((size_t)n * kRows));
    launch_rows_to_pack(ctx->grows.p, n, scene->stride, ctx->grad_stage.p, ctx->stream);
    GS_CK(cudaGetLastError());
    if (n) GS_CK(cudaMemcpyAsync(grad_packed, ctx->grad_stage.p, (size_t)n * kRows * 4, cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    return GS_OK;
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
    GS_CK(ctx->loss_sums.reserve(2));
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
        const double count = 3.0 * (double)pix;
        if (loss) *loss = sums[1] / count + (double)lambda * (1.0 - sums[0] / count);
    }
    return GS_OK;
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
    const size_t words = ((size_t)n + kSortPartition - 1) / kSortPartition * radix;
    if (words > ctx->aux_flags.cap || !ctx->aux_flags.p) {
        GS_CK(ctx->aux_flags.reserve(words));
        GS_CK(cudaMemsetAsync(ctx->aux_flags.p, 0, ctx->aux_flags.cap * 8, ctx->stream));
    }
    const cudaMemcpyKind kin = location == GS_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    GS_CK(cudaMemcpyAsync(k0, keys, (size_t)n * 4, kin, ctx->stream));
    GS_CK(cudaMemcpyAsync(v0, vals, (size_t)n * 4, kin, ctx->stream));
    FrameCtl* ctl = ctx->aux_ctl.p;
    launch_frame_begin(ctl, ctx->stream);
    launch_digit_hist(k0, n, bits, key_bits, ctl->hist, ctx->stream);
    uint32_t* kb[2] = {k0, k1};
    uint32_t* vb[2] = {v0, v1};
    int cur = 0;
    for (uint32_t p = 0; p < passes; ++p) {
        const uint32_t left = key_bits - p * bits;
        const uint32_t dmask = left >= bits ? radix - 1u : (1u << left) - 1u;
        launch_onesweep(bits, kb[cur], vb[cur], kb[cur ^ 1], vb[cur ^ 1], nullptr, n, n, p * bits, dmask,
                        ctl->hist + p * radix, ctl, ctx->aux_flags.p, 1 + p, 0, ctx->stream);
        cur ^= 1;
    }
    GS_CK(cudaGetLastError());
    const cudaMemcpyKind kout = location == GS_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    GS_CK(cudaMemcpyAsync(keys, kb[cur], (size_t)n * 4, kout, ctx->stream));
    GS_CK(cudaMemcpyAsync(vals, vb[cur], (size_t)n * 4, kout, ctx->stream));
    uint32_t status = 0;
    GS_CK(cudaMemcpyAsync(ctx->h_ctl, ctl, offsetof(FrameCtl, tickets), cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    status = ctx->h_ctl->status;
    ctx->have_frame = false;  // the readback block now holds the sort's counters
    return status_to_code(ctx, status);
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
    launch_frame_begin(ctl, ctx->stream);
    GS_CK(cudaMemsetAsync(d + n, 0, 4, ctx->stream));
    launch_exclusive_scan(d, n, d + n, ctl, ctx->aux_flags.p, 0, ctx->stream);
    GS_CK(cudaGetLastError());
    const cudaMemcpyKind kout = location == GS_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (n) GS_CK(cudaMemcpyAsync(data, d, (size_t)n * 4, kout, ctx->stream));
    uint32_t tot = 0;
    GS_CK(cudaMemcpyAsync(ctx->h_ctl, ctl, offsetof(FrameCtl, tickets), cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaMemcpyAsync(&tot, d + n, 4, cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    if (total) *total = tot;
    ctx->have_frame = false;
    return status_to_code(ctx, ctx->h_ctl->status);
}

int gs_exp_f32(gs_ctx* ctx, const float* x, float* y, uint32_t n, int32_t location) {
    if (!ctx) return GS_ERR_INVALID;
    if ((!x || !y) && n) return fail(ctx, GS_ERR_INVALID, "gs_exp_f32: null buffer");
    if (n == 0) return GS_OK;
    GS_CK(cudaSetDevice(ctx->cfg.device));
    if (location == GS_MEM_DEVICE) {
        launch_exp(x, y, n, ctx->stream);
        GS_CK(cudaGetLastError());
        return GS_OK;
    }
    GS_CK(ctx->aux_f32.reserve((size_t)n * 2));
    float* dx = ctx->aux_f32.p;
    float* dy = dx + n;
    GS_CK(cudaMemcpyAsync(dx, x, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    launch_exp(dx, dy, n, ctx->stream);
    GS_CK(cudaGetLastError());
    GS_CK(cudaMemcpyAsync(y, dy, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    GS_CK(cudaStreamSynchronize(ctx->stream));
    return GS_OK;
}

}  // extern "C"
