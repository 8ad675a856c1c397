/*
 * gs.h -- C ABI of the GB300 splat pipeline (libwebgs.so).
 *
 * Drop-in boundary for the reference's JavaScript Renderer (KoS-Y1/Web-GS-Renderer,
 * src/renderer/renderer.js) and the WebGPU passes it encodes. Every entry point below names the
 * reference interface it replaces. Plain C types only; nothing throws across the ABI; every call
 * returns a status code (GS_OK = 0). One CUDA stream per context; a context is not thread-safe,
 * separate contexts are independent.
 */
#ifndef WEBGS_GS_H
#define WEBGS_GS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference reports through fail() dialogs and device-lost handlers,
 *      src/utils/utils.js:3-47, src/gpu/device.js:30-35) ---------------------------------------- */
#define GS_OK 0
#define GS_ERR_INVALID 1   /* bad argument: null pointer, size out of range, unknown option */
#define GS_ERR_OOM 2       /* device or pinned host allocation failed */
#define GS_ERR_OVERFLOW 3  /* instances exceeded max_instance: output written (a soft error), the
                              instances truncated exactly as emit.wgsl:57-59 truncates them; tile
                              ranges and raster use min(I, max_instance), so the last kept tile
                              renders, where the reference leaves its end unwritten
                              (tile_ranges.wgsl:14,32 bound by the unclamped I) */
#define GS_ERR_TIMEOUT 4   /* a device-side wait hit its iteration limit; results are invalid */
#define GS_ERR_CUDA 5      /* a CUDA runtime call failed; gs_last_error() has the message */
#define GS_ERR_STATE 6     /* call out of order, e.g. backward without a matching forward */
#define GS_ERR_UNSUPPORTED 7
#define GS_ERR_MEMORY 8    /* checked builds only: a store index fell outside its buffer, or a canary
                              pad around a device buffer was overwritten (GS_DEV_BOUNDS / _CANARY) */

/* ---- memory location of caller buffers -------------------------------------------------------- */
#define GS_MEM_HOST 0      /* pageable or pinned host memory; the call is synchronous */
#define GS_MEM_DEVICE 1    /* device memory of the context's GPU; the call is stream-ordered */

/* ---- context flags ---------------------------------------------------------------------------- */
#define GS_FLAG_PROFILE 1u /* record per-pass CUDA events (the reference's GpuProfiler,
                              src/gpu/profiler.js:47-124) */
#define GS_FLAG_NO_GRAPH 2u /* launch kernels one by one instead of replaying a CUDA graph */
#define GS_FLAG_DIFFERENTIABLE 4u /* keep final T and last contributor of the last frame for
                                     gs_backward (8 bytes per pixel of extra writes) */

/* GlobalUniforms (src/shaders/preprocess.wgsl:2-12), packed by renderer.js:773-797: 176 bytes,
 * f32 offsets view@0, viewProj@16, eye@32, count(u32)@35, focal@36, tanFov@38, size@40. */
typedef struct gs_view {
    float view[16];       /* column-major view matrix (camera looks down -z) */
    float view_proj[16];  /* projection * view, clip depth in [0, 1] */
    float camera_pos[3];
    uint32_t count;       /* ignored: the scene's count is used */
    float focal[2];       /* W / (2 tanFovX), H / (2 tanFovY) */
    float tan_fov[2];
    float texture_size[2];/* image width, height in pixels (as floats) */
    uint32_t pad0, pad1;
} gs_view;

/* A camera as the reference's Camera class holds it (src/renderer/camera.js: eye, the point looked at,
 * the world up vector, the vertical field of view, the canvas size, and Z_NEAR / Z_FAR): the input of
 * Camera.getUniform() (camera.js:87-98), 56 bytes. */
typedef struct gs_camera {
    float eye[3];
    float target[3];
    float up[3];
    float fovy_deg;        /* vertical field of view in degrees, in (0, 180) */
    uint32_t width, height;/* image size in pixels */
    float z_near, z_far;   /* 0 < z_near < z_far */
} gs_camera;

/* Tunables. Defaults are the reference's constants (renderer.js:16-26). */
typedef struct gs_config {
    uint32_t tile_size;           /* 16 (reference); 8 and 32 also supported */
    uint32_t digit_bits;          /* radix digit width: 8 (reference) or 4 */
    uint32_t raster_batch;        /* splats staged per raster batch: 32, 64, 128 or 256 */
    uint32_t max_instance_factor; /* instance budget per Gaussian (MAX_INSTANCE_FACTOR = 64) */
    uint32_t flags;               /* GS_FLAG_* */
    int32_t device;               /* CUDA device ordinal */
    uint32_t sort_block;          /* keys per radix-sort block (partition): 4096 (default) or 2048; the
                                     reference sorts in blocks of 256 (radix_parallel.wgsl:20-22) */
} gs_config;

/* Frame outputs. Any pointer may be NULL. All non-NULL pointers live in `location`. */
typedef struct gs_image {
    int32_t location;      /* GS_MEM_HOST or GS_MEM_DEVICE */
    uint8_t* rgba8;        /* W*H*4: rgba8unorm (raseter.wgsl:115), alpha 255 */
    float* rgb;            /* W*H*3: fp32 colour before quantization, pixel-interleaved */
    float* final_t;        /* W*H: transmittance left after the last blended splat */
    uint32_t* n_contrib;   /* W*H: contributor count at the last blended splat (raseter.wgsl:47,102) */
} gs_image;

/* Counters of the last frame (read back on request only; the reference never reads them). */
typedef struct gs_frame_info {
    uint32_t instance_count; /* I: sum of tilesTouched (offset_scan.wgsl:66) */
    uint32_t sorted_count;   /* min(I, max_instance) (indirect_arg.wgsl:16) */
    uint32_t max_instance;
    uint32_t visible;        /* Gaussians with tilesTouched > 0 */
    uint32_t near_pass;      /* Gaussians in front of the near plane (preprocess.wgsl:83) */
    uint32_t tiles_x, tiles_y;
    uint32_t status;         /* device status word: GS_DEV_* bits */
    uint32_t sort_passes;
} gs_frame_info;

#define GS_DEV_OVERFLOW 1u
#define GS_DEV_TIMEOUT 2u
#define GS_DEV_BOUNDS 4u   /* checked builds: a store was skipped because its index was out of bounds */
#define GS_DEV_CANARY 8u   /* checked builds: a canary pad around a device buffer was found overwritten */

/* Intermediate buffers of the last frame, copied to host for parity checks. Any pointer may be
 * NULL. Sizes: N = scene count, T = tiles_x * tiles_y, capacity = entries of keys/vals. */
typedef struct gs_debug {
    uint32_t* tiles_touched; /* N */
    uint32_t* meta;          /* 4N: ((minY<<16)|minX, (maxY<<16)|maxX, depth16, 0) */
    float* conic_opacity;    /* 4N */
    float* pixel;            /* 2N */
    float* color;            /* 4N (vec3f at a 16-byte stride) */
    uint32_t* offsets;       /* N+1 */
    uint32_t* keys;          /* capacity: sorted keys */
    uint32_t* vals;          /* capacity: sorted Gaussian indices */
    uint64_t capacity;
    uint32_t* ranges;        /* 2T */
} gs_debug;

/* Per-pass timing row (the reference's profiler rows {label: {ms}}, profiler.js:113-121). */
typedef struct gs_timing {
    char label[24];
    float ms;
} gs_timing;

typedef struct gs_ctx gs_ctx;
typedef struct gs_scene gs_scene;

/* ---- library --------------------------------------------------------------------------------- */
const char* gs_version(void);
void gs_config_default(gs_config* cfg);

/* Replaces `new Renderer(device, context, format, onProfile)` (renderer.js:160-459) and the
 * WebGPU device request (src/gpu/device.js:3-39). */
int gs_ctx_create(const gs_config* cfg, gs_ctx** out);
int gs_ctx_destroy(gs_ctx* ctx);
/* Message of the last failed call on this context (static string on NULL ctx). */
const char* gs_last_error(const gs_ctx* ctx);
/* Blocks until the context's stream is idle; returns a pending device status (timeout). */
int gs_ctx_synchronize(gs_ctx* ctx);
/* The context's cudaStream_t, for callers that order their own work against it. */
void* gs_ctx_stream(gs_ctx* ctx);

/* Replaces Renderer.uploadGsData(data, name) (renderer.js:468-479): copies `packed` (59*count
 * floats in the layout of preprocess.wgsl:16-24 / loader.js:75-85) to the device. The caller keeps
 * ownership of `packed`; the scene owns its device copy. location: GS_MEM_HOST or GS_MEM_DEVICE. */
int gs_scene_upload(gs_ctx* ctx, const float* packed, uint32_t count, int32_t location, gs_scene** out);
/* Overwrites the attributes of an existing scene (same count), e.g. after an optimizer step. */
int gs_scene_update(gs_ctx* ctx, gs_scene* scene, const float* packed, int32_t location);
int gs_scene_destroy(gs_scene* scene);
uint32_t gs_scene_count(const gs_scene* scene);

/* Replaces Renderer.execute() (renderer.js:481-508) with the passes of renderer.js:822-932:
 * preprocess, offset scan, emit, device-side sizing, radix sort, tile ranges, raster; the blit
 * (blit.wgsl) becomes `out`. Host outputs: returns after the image is on the host; rgba8 and rgb
 * buffers in pinned (page-locked or registered) host memory are written by the raster directly,
 * pageable ones through a staging copy. Device outputs: stream-ordered, returns after launch.
 * Returns GS_ERR_OVERFLOW (outputs written) when the instance count exceeded the budget. */
int gs_forward(gs_ctx* ctx, const gs_scene* scene, const gs_view* view, const gs_image* out);

/* One view of a batch: a scene, its 176-byte view block and its outputs. */
typedef struct gs_batch_view {
    const gs_scene* scene;
    gs_view view;
    gs_image out;
} gs_batch_view;

/* Batched forward (no counterpart in the reference, which renders one view per execute()): all
 * views, of any scenes and resolutions, are captured into one CUDA graph and forked over the
 * context's side streams, so small views share the GPU. Every view's output must use the same
 * location. Same results as gs_forward per view. */
int gs_forward_batch(gs_ctx* ctx, const gs_batch_view* views, uint32_t count);

/* One view of a batch given by its camera: the 176-byte block is built on the device. */
typedef struct gs_batch_camera {
    const gs_scene* scene;
    gs_camera camera;
    gs_image out;
} gs_batch_camera;

/* gs_forward_batch with the view blocks built on the device (no counterpart in the reference, which
 * builds one block per frame on the host, camera.js:87-98 + renderer.js:773-797): the batch uploads
 * its 56-byte cameras, and the graph's first kernel builds every view's block from them, the same
 * bits as gs_camera_view. Results equal gs_forward_batch with those blocks. GS_ERR_INVALID for a
 * camera gs_camera_view would reject. */
int gs_forward_batch_cameras(gs_ctx* ctx, const gs_batch_camera* views, uint32_t count);

/* Camera.getUniform() (camera.js:87-98) for n cameras on the device (no counterpart in the
 * reference): the same bits as gs_camera_view per camera. cams: host memory; out: n blocks in
 * `location` (host: synchronous; device: stream-ordered). */
int gs_camera_views(gs_ctx* ctx, const gs_camera* cams, uint32_t n, gs_view* out, int32_t location);

/* Counters of the last forward (synchronizes). */
int gs_get_frame_info(gs_ctx* ctx, gs_frame_info* info);
/* Counters of view `index` of the last gs_forward_batch (synchronizes). */
int gs_get_batch_frame_info(gs_ctx* ctx, uint32_t index, gs_frame_info* info);
/* Intermediates of the last forward, copied to host (synchronizes). */
int gs_get_debug(gs_ctx* ctx, const gs_debug* dbg);

/* Backward of the last gs_forward on `scene` (no counterpart in the reference, which is
 * forward-only): dL_drgb is W*H*3 floats (gradient w.r.t. the fp32 rgb image); grad receives
 * 59*count floats in the packed input layout. Both in `location`. */
int gs_backward(gs_ctx* ctx, const gs_scene* scene, const float* dl_drgb, float* grad_packed, int32_t location);

/* Backward of views 0..count-1 of the last gs_forward_batch, all of `scene`: dl_drgb[i] is view i's
 * dL/drgb; the gradients of all views are summed into grad_packed (the raster backwards run concurrently,
 * then one pass over the scene per group of up to 16 views adds their attribute gradients). */
int gs_backward_batch(gs_ctx* ctx, const gs_scene* scene, const float* const* dl_drgb, uint32_t count,
                      float* grad_packed, int32_t location);

/* Autotuner (no counterpart in the reference, whose constants are fixed): times gs_forward_batch of
 * `views` over one scene for every tile size {8,16,32} x radix digit width {4,8} x raster batch
 * depth {32,64,128,256} x sort block {2048,4096}, `iters` batches each, re-times the three fastest
 * with 4 x `iters` batches, and returns the fastest of those (other fields from `base`) with its ms
 * per batch. Creates and destroys its own contexts. */
int gs_autotune(const gs_config* base, const float* packed, uint32_t count, const gs_view* views, uint32_t n_views,
                uint32_t iters, gs_config* best, float* best_ms);

/* The same sweep over a batch of several scenes: packed[s] / counts[s] are the scenes (host, packed
 * layout), view i renders scene view_scene[i] (NULL: every view renders scene 0). */
int gs_autotune_scenes(const gs_config* base, const float* const* packed, const uint32_t* counts, uint32_t n_scenes,
                       const gs_view* views, const uint32_t* view_scene, uint32_t n_views, uint32_t iters,
                       gs_config* best, float* best_ms);

/* Loss of the differentiation workload (no counterpart in the reference): L = mean|rgb - target| +
 * lambda * (1 - mean SSIM), SSIM per channel with an 11x11 Gaussian window (sigma 1.5), zero padding,
 * C1 = 0.01^2, C2 = 0.03^2; images H x W x 3. *loss (host, may be NULL) receives L; dl_drgb (may be
 * NULL) receives dL/drgb. Host buffers: synchronous. Device buffers: stream-ordered unless loss is
 * requested. */
int gs_loss_l1_ssim(gs_ctx* ctx, const float* rgb, const float* target, uint32_t width, uint32_t height,
                    float lambda, double* loss, float* dl_drgb, int32_t location);

/* Per-pass timings of the last profiled frame (GS_FLAG_PROFILE); *n_rows receives the count. */
int gs_get_timings(gs_ctx* ctx, gs_timing* rows, int32_t max_rows, int32_t* n_rows);

/* ---- building blocks, exposed for parity tests on arbitrary inputs ---------------------------- */
/* Stable LSD radix sort of (key, value) pairs on the low `key_bits` bits with the context's digit
 * width (radix_parallel.wgsl:26-160). In place; keys/vals in `location`. */
int gs_sort_pairs(gs_ctx* ctx, uint32_t* keys, uint32_t* vals, uint32_t n, uint32_t key_bits, int32_t location);
/* Exclusive scan in place (offset_scan.wgsl:22-67); *total receives the sum (host pointer). */
int gs_exclusive_scan(gs_ctx* ctx, uint32_t* data, uint32_t n, uint32_t* total, int32_t location);
/* Failure-path check (no counterpart in the reference): runs a scan whose lookback waits on a
 * partition that never publishes. The wait gives up after its iteration limit (about a second), the
 * kernel records the timeout in the device status word and returns; the call returns
 * GS_ERR_TIMEOUT and the context stays usable. */
int gs_check_wait_timeout(gs_ctx* ctx);

/* Test hook (no counterpart in the reference): sets the sequence number of every frame control block
 * of ctx -- or, with ctx NULL, of gs_exclusive_scan_static's scratch on the current device. Lookback
 * words carry the low 30 bits of that number, which advances by 16 per frame or scan, so their tags
 * repeat every 2^26 calls; the call on which they start again at zero clears the words first. With
 * this hook a test reaches that call without running 2^26 frames. Synchronous. */
int gs_debug_set_sequence(gs_ctx* ctx, uint32_t seq);

/* 1 for libwebgs_checked.so, 0 for the product library. The checked build (the stand-in for a
 * memory sanitizer, which is not available here) pads every device buffer of a context with canary
 * words that a kernel verifies after each forward, batch and backward, and tests every
 * data-dependent store index against its buffer; a violation sets GS_DEV_BOUNDS / GS_DEV_CANARY and
 * the call returns GS_ERR_MEMORY. */
int gs_checked_build(void);
/* Checked builds: overwrites one canary word after the last frame's sorted-keys buffer (inside the
 * pad the build allocated there), from the host, so a test can see the next frame report it.
 * Product builds: GS_ERR_UNSUPPORTED. */
int gs_debug_damage_canary(gs_ctx* ctx);

/* The pinned fp32 exp of the kernels, evaluated on the device (y = exp(x)). */
int gs_exp_f32(gs_ctx* ctx, const float* x, float* y, uint32_t n, int32_t location);
/* The raster's pinned exp (alpha = o * exp(power), raseter.wgsl:89), defined for x in [-5.6, 0], on
 * the device: for parity tests against the oracle. */
int gs_raster_exp_f32(gs_ctx* ctx, const float* x, float* y, uint32_t n, int32_t location);
/* y = o * exp(x) before the 0.99 clamp, formed on the device as the raster forms it (raseter.wgsl:89),
 * for x at or above o's cut-off ln((1/255)/o) - 1e-3 (the only arguments the raster evaluates): for
 * parity tests against the oracle's o * raster_expf(x). o, x and y hold n floats each. */
int gs_raster_alpha_f32(gs_ctx* ctx, const float* o, const float* x, float* y, uint32_t n, int32_t location);

/* Exclusive scan for callers that must not allocate device memory (no counterpart in the
 * reference). Same result as gs_exclusive_scan, but it needs no context and calls no cudaMalloc,
 * cudaFree or other allocating routine: cudaMalloc/cudaFree can synchronize the whole device, which
 * a real-time frame loop cannot afford, and hosts that own device memory through their own arenas
 * forbid a library from allocating behind them. d_in, d_out (n entries; may be the same buffer) and
 * d_total (one entry, or NULL) are device buffers of the current device; work is ordered on
 * `stream` (a cudaStream_t) and the call returns once it has finished. Scratch is a fixed device
 * array of about 74 KB per GPU, zero-filled when the library's device code loads and held until the
 * process exits; n above 2^24 (16,777,216) returns GS_ERR_INVALID. Every call looks up the array's
 * device address (no allocation); the first call on a device also loads the library's device code,
 * so make it before any stream capture. All calls share the array: calls that overlap on the GPU
 * (other threads, other streams) race and must be serialised by the caller. */
int gs_exclusive_scan_static(const uint32_t* d_in, uint32_t* d_out, uint32_t n, uint32_t* d_total, void* stream);

/* ---- host utilities (no GPU needed) ----------------------------------------------------------- */
/* Camera.getUniform() (src/renderer/camera.js:87-98) with wgpu-matrix lookAt / perspective
 * (camera.js:135-142, 0..1 clip depth) restated: fills the 176-byte block for a camera at `eye`
 * looking at `target`, vertical field of view fovy_deg, image width x height. */
int gs_camera_view(const float eye[3], const float target[3], const float up[3], float fovy_deg,
                   uint32_t width, uint32_t height, float z_near, float z_far, gs_view* out);

/* Seeded synthetic scene in the packed layout (59*count floats). kind 0: one isotropic cluster
 * N(0,1)^3; kind 1: mixture of `clusters` anisotropic clusters in a box of edge `box`. Other
 * attributes: log-scale N(-4, 0.5^2), quaternion N(0,1)^4 normalised, opacity logit N(0, 1.5^2),
 * DC N(0, 0.5^2), rest N(0, 0.05^2). Bit-identical on every host. */
int gs_synth_scene(uint32_t kind, uint32_t count, uint64_t seed, uint32_t clusters, float box, float* packed);

/* Parses a binary little-endian .ply scene, as loadPly does (src/loader/loader.js:56-213): the header
 * up to "end_header" (+ optional CR, LF), a vertex element whose scalar properties of any PLY type
 * include x y z, scale_0..2, rot_0..3, opacity, f_dc_0..2 and f_rest_0..44 (others are skipped),
 * vertex records starting right after the header. Writes *count and, when packed is not NULL,
 * 59*count floats in the packed layout gs_scene_upload takes. Returns GS_ERR_INVALID with the
 * reference's message in err (may be NULL) for a malformed file. */
int gs_ply_parse(const uint8_t* bytes, size_t size, uint32_t* count, float* packed, char* err, size_t err_len);

/* Perturbs a packed scene in place: means += N(0, sigma_mean^2), SH (DC and rest) += N(0, sigma_sh^2). */
int gs_perturb_scene(float* packed, uint32_t count, uint64_t seed, float sigma_mean, float sigma_sh);

/* The present step without a canvas (blit.wgsl / context.js replaced by a file): writes a host rgba8
 * image (width x height x 4, row 0 at the top, as the raster writes it) as a binary PPM (P6, alpha
 * dropped) to `path`. GS_ERR_INVALID for bad arguments or a file that cannot be written. */
int gs_write_ppm(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height);

#ifdef __cplusplus
}
#endif
#endif /* WEBGS_GS_H */
