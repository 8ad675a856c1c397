/*
 * gs_oracle.h -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * CPU restatement of the reference splat pipeline of KoS-Y1/Web-GS-Renderer:
 *   preprocess   src/shaders/preprocess.wgsl:58-284
 *   offset scan  src/shaders/offset_scan.wgsl:22-67
 *   emit         src/shaders/emit.wgsl:28-66
 *   indirect arg src/shaders/indirect_arg.wgsl:14-27
 *   radix sort   src/shaders/radix_parallel.wgsl:26-160 (driven as src/renderer/renderer.js:799-811, 870-917)
 *   tile ranges  src/shaders/tile_ranges.wgsl:7-34
 *   raster       src/shaders/raseter.wgsl:35-117
 * sequenced as src/renderer/renderer.js:822-932.
 *
 * PARITY UNPINNED: the reference ships no tests, fixtures or golden vectors for this path and its
 * WGSL runs only on a WebGPU adapter, which is unavailable on this machine. This restatement is
 * checked against project-written known-answer tests and committed regression fixtures only.
 *
 * fp32 semantics (WGSL leaves contraction and exp precision to the implementation, so they are
 * pinned here and followed bit for bit by the CUDA kernels):
 *   1. IEEE binary32, round to nearest even, subnormals kept (no flush to zero).
 *   2. No contraction: every + - * / rounds on its own, in WGSL source order (left-assoc),
 *      except the two explicit fused forms of rule 5.
 *   3. sqrt and division correctly rounded; floor/ceil exact; normalize(v) = v / sqrt(dot(v,v))
 *      with dot summed in component order.
 *   4. exp(x) = the pinned exp of oracle_expf() (Cody-Waite reduction by ln 2 and a degree-7
 *      Taylor polynomial in Horner form with fma), sigmoid(x) = 1 / (1 + exp(-x)).
 *   4b. the raster's alpha (raseter.wgsl:89) uses the raster exp of oracle_raster_expf_array():
 *      arguments in [-5.6, 0] only, one-fma reduction by ln 2 and a degree-6 minimax polynomial
 *      (under 2 ulp from exp; WGSL allows 3 + 2|x| ulp).
 *   5. raster: power = fma(-0.5, fma(a*dx, dx, (c*dy)*dy), -((b*dx)*dy));
 *              color_k = fma(color_k_splat * alpha, T, color_k).
 *   6. mat*vec and mat*mat: each element is a dot product summed in index order.
 *   7. f32 -> u32 after clamp/saturate: truncation.
 *   8. rgba8unorm store: u8 = floor(clamp(c, 0, 1) * 255 + 0.5), alpha = 255.
 * The FP64 twin runs the same code with double and libm exp/fma to report error against FP64.
 */
#ifndef GS_ORACLE_H
#define GS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-frame results of the fp32 restatement. Every pointer is caller-allocated and may be NULL. */
typedef struct oracle_fwd_out {
    uint32_t* tiles_touched;   /* N: tilesTouched, 0 where culled (offsets buffer before the scan) */
    uint32_t* meta;            /* 4N: ((minY<<16)|minX, (maxY<<16)|maxX, depth16, 0); 0 where culled */
    float* conic_opacity;      /* 4N */
    float* pixel;              /* 2N */
    float* color;              /* 4N: vec3f at a 16-byte stride, .w = 0 */
    uint32_t* offsets;         /* N+1: exclusive scan of tiles_touched */
    uint32_t* keys;            /* keys_capacity: sorted keys (first sorted_count valid) */
    uint32_t* vals;            /* keys_capacity: sorted Gaussian indices */
    uint64_t keys_capacity;
    uint32_t* ranges;          /* 2T: [start, end) per tile, (0,0) when empty */
    float* rgb;                /* W*H*3 fp32 before quantization */
    float* final_t;            /* W*H */
    uint32_t* n_contrib;       /* W*H: contributor count at the last blended splat */
    uint8_t* rgba8;            /* W*H*4 */
    /* outputs */
    uint32_t instance_count;   /* I: total of tiles_touched (renderer.js instanceCountBuffer) */
    uint32_t sorted_count;     /* min(I, max_instance) */
    uint32_t max_instance;     /* factor * N */
    uint32_t tiles_x, tiles_y;
} oracle_fwd_out;

/* fp32 restatement. uniforms: the 176-byte GlobalUniforms block (preprocess.wgsl:2-12).
 * packed: the reference's flat attribute array (preprocess.wgsl:16-24), 59*n floats.
 * tile: tile edge in pixels (16 in the reference). Returns 0 on success. */
int oracle_forward_f32(const void* uniforms, const float* packed, uint32_t n, uint32_t tile,
                       uint32_t max_instance_factor, oracle_fwd_out* out, int threads);

/* As oracle_forward_f32, also writing per-pass wall times (ms: preprocess, scan, emit, sort, tile
 * ranges, raster) and rasterizing only every row_stride-th tile row (1 = the whole frame; used to
 * bound CPU timing samples). */
int oracle_forward_f32_timed(const void* uniforms, const float* packed, uint32_t n, uint32_t tile,
                             uint32_t max_instance_factor, oracle_fwd_out* out, int threads, double* pass_ms,
                             uint32_t row_stride);

/* FP64 twin: same algorithm in double; writes rgb (W*H*3) and final_t (W*H), may be NULL. */
int oracle_forward_f64(const void* uniforms, const float* packed, uint32_t n, uint32_t tile,
                       uint32_t max_instance_factor, double* rgb, double* final_t,
                       uint32_t* instance_count, int threads);

/* The pinned fp32 exp (rule 4), exposed so tests can compare it with the CUDA kernels. */
float oracle_expf(float x);
void oracle_expf_array(const float* x, float* y, uint64_t n);
/* The raster's exp (rule 4b), defined for x in [-5.6, 0]. */
void oracle_raster_expf_array(const float* x, float* y, uint64_t n);

/* Literal restatement of the reference radix sort (count / scan / reorder over 256-element blocks,
 * radix_parallel.wgsl:26-160) on arbitrary pairs, sorting on `passes` 8-bit digits from bit 0. */
void oracle_radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, uint32_t passes);

/* Exclusive scan in place over n entries with the offset_scan.wgsl:22-67 block structure; returns
 * the total. */
uint32_t oracle_exclusive_scan(uint32_t* data, uint32_t n);

/* tile_ranges.wgsl:7-34 as the reference binds it (renderer.js:612): dispatched over ceil(sorted/256)
 * workgroups of 256 but bounded by the unclamped instance count. keys holds `capacity` sorted keys
 * (the first `sorted` valid); ranges (2T words) must be zeroed first. When instance_count exceeds
 * the capacity the last tile's end stays 0. Returns how many threads would read past the keys
 * buffer (left undefined by WGSL, not restated); 0 whenever sorted is a multiple of 256. */
uint32_t oracle_tile_ranges_reference(const uint32_t* keys, uint32_t capacity, uint32_t sorted,
                                      uint32_t instance_count, uint32_t* ranges);

#ifdef __cplusplus
}
#endif
#endif
