// gs_raster.cu -- front-to-back alpha-blending tile rasterizer (src/shaders/raseter.wgsl:35-117).
//
// One CTA per tile, one thread per pixel; each warp owns an 8x4 block of the tile. The tile's
// sorted range is walked in batches of BATCH splats: the CTA votes to stop once every pixel is done
// (raseter.wgsl:54-68 as one __syncthreads_and) and stages the batch's records in shared memory
// with one gather per splat. Every pixel then blends the batch in order with the pinned fp32
// semantics:
//   power = fma(-0.5, fma(a*dx, dx, (c*dy)*dy), -((b*dx)*dy)); skip if power > 0
//   alpha = min(0.99, o * exp(power));                         skip if alpha < 1/255
//   testT = T * (1 - alpha);                                   done if testT < 1e-4
//   C += colour * alpha * T (one fma per channel); T = testT
//
// Two exact shortcuts remove most of the work without changing a single output bit:
//  * cut-off: a pixel whose power is below the splat's cut-off c_o = ln((1/255)/o) - 1e-3 is
//    rejected without its alpha, since o*exp(power) < 1/255 is certain there (the 1e-3 margin is
//    far beyond the rounding of exp, the product and logf); so alpha is only ever used where the
//    raster's exp is defined (lanes of a hit form it anyway and discard it: no branch in a hit);
//  * warp cull: when staging a splat, the CTA computes an octagon (the bounding box and the
//    45-degree box) around the region of the tile where power >= c_o can hold
//    (gs_raster_common.cuh gives the bound). Every warp tests its 8x4 pixel block against the 32
//    octagons of a group in parallel (one per lane, one ballot) and walks only the splats whose
//    octagon meets its block, in range order. A skipped splat would have been rejected by every
//    pixel of the warp at "power < c_o" (or "power > 0"). Contributor counts are range positions, so
//    skipping does not change them.
//
// Full residency (2048 threads per SM, 32 registers; the few spilled bytes cost less than the lost
// warps did), except for the instantiation that also tracks the contributor count (below).
//
// CTA i renders tile order[i]: the tiles listed by decreasing range length, so the longest tiles
// start first instead of forming the tail of the launch (with tiles in index order the clustered
// scenes left about a third of the launch time to a few long tiles).
#include "gs_kernels.h"
#include "gs_raster_common.cuh"

namespace gs {
namespace {

// Residency: 2048 threads per SM (32 registers); the 16x16 instantiation that also tracks the
// contributor count runs at 1536 (40 registers, no spills): 0.2705 -> 0.2683 ms per 1M / 1080p
// differentiable frame, while the plain frame is fastest at full residency (0.2621 against 0.2683).
template <int TILE, bool LAST>
constexpr int raster_min_blocks() { return LAST && TILE == 16 ? 6 : 2048 / (TILE * TILE); }

template <int TILE, int BATCH, bool LAST>
__global__ void __launch_bounds__(TILE * TILE, raster_min_blocks<TILE, LAST>()) k_raster(const uint32_t* __restrict__ ranges,
                                                        const uint32_t* __restrict__ vals,
                                                        const float4* __restrict__ rec, uint32_t n,
                                                        const FrameCtl* __restrict__ ctl, uint32_t width,
                                                        uint32_t height, uint32_t tiles_x, RasterOut out,
                                                        const uint32_t* __restrict__ order) {
    pdl_wait();
    constexpr int THREADS = TILE * TILE;
    constexpr int WX = TILE / 8;  // warps across the tile
    __shared__ float4 s_a[BATCH];    // (x, y, conic.x, conic.y)
    __shared__ float4 s_b[BATCH];    // (conic.z, opacity, r, g)
    __shared__ float2 s_c[BATCH];    // (b, cut)
    __shared__ float4 s_box[BATCH];  // cull box (x0, x1, y0, y1)
    __shared__ float4 s_diag[BATCH];  // its 45-degree box (u0, u1, v0, v1), u = x + y, v = x - y

    const uint32_t tile = order ? order[blockIdx.x] : blockIdx.x;
    const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t bx0 = tx * TILE + 8u * (warp % WX), by0 = ty * TILE + 4u * (warp / WX);
    const uint32_t x = bx0 + (lane & 7u), y = by0 + (lane >> 3);
    const bool inside = x < width && y < height;
    bool done = !inside;
    const uint2 range = reinterpret_cast<const uint2*>(ranges)[tile];
    // a range past the sorted count can only come from a timed-out sort: clamp it
    const uint32_t end = ctl ? min(range.y, ctl->sorted_count) : range.y;
    const uint32_t start = range.x;
    const float fx = (float)x, fy = (float)y;
    const float rx0 = (float)bx0, rx1 = (float)(bx0 + 7u), ry0 = (float)by0, ry1 = (float)(by0 + 3u);
    const float tx0 = (float)(tx * TILE), tx1 = (float)(tx * TILE + TILE - 1u);
    const float ty0 = (float)(ty * TILE), ty1 = (float)(ty * TILE + TILE - 1u);

    float T = 1.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f;
    uint32_t last = 0;

    for (uint32_t i = start; i < end; i += BATCH) {
        if (__syncthreads_and(done)) break;
        for (uint32_t j = threadIdx.x; j < (uint32_t)BATCH; j += THREADS) {
            if (i + j < end) {
                const uint32_t g = vals[i + j];
                if (g < n) {
                    const float4 r0 = __ldg(rec + (size_t)kRecFloat4 * g);
                    const float4 r1 = __ldg(rec + (size_t)kRecFloat4 * g + 1);
                    const float4 r2 = __ldg(rec + (size_t)kRecFloat4 * g + 2);
                    s_a[j] = r0;
                    s_b[j] = r1;
                    s_c[j] = make_float2(r2.x, r2.y);
                    s_box[j] = cull_box(r0.x, r0.y, r0.z, r0.w, r1.x, r2.y, tx0, tx1, ty0, ty1, s_diag[j]);
                } else {  // only after a timed-out sort: a splat that never blends
                    const float inf = __int_as_float(0x7f800000);
                    s_a[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    s_b[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    s_c[j] = make_float2(0.0f, inf);
                    s_box[j] = make_float4(inf, -inf, inf, -inf);
                    s_diag[j] = s_box[j];
                }
            }
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)BATCH, end - i);
        const uint32_t pos0 = i - start + 1u;  // contributor count of the batch's first splat
        for (uint32_t g0 = 0; g0 < cnt; g0 += 32u) {
            if (__all_sync(0xffffffffu, done)) break;
            bool hit = false;
            if (g0 + lane < cnt)
                hit = box_meets(s_box[g0 + lane], rx0, rx1, ry0, ry1) &&
                      box_meets(s_diag[g0 + lane], rx0 + ry0, rx1 + ry1, rx0 - ry1, rx1 - ry0);
            uint32_t m = __ballot_sync(0xffffffffu, hit);
            while (m) {
                const uint32_t j = g0 + (uint32_t)(__ffs(m) - 1);
                m &= m - 1u;
                // no branch in a hit: every lane forms alpha and the blend, and the rejections (pixel
                // done, power > 0, power below the cut-off, alpha < 1/255, termination) only select
                // what is kept. Nearly every hit has lanes on both sides of them, so the branches
                // only added their divergence and reconvergence (raster of the 1M / 1080p frame
                // 0.2510 -> 0.2417 ms, 0.2580 -> 0.2458 ms with the contributor count; with a branch
                // for the rejections by power and selects after it, slower). A rejected lane's exp
                // may be of any argument; its value is discarded.
                const float4 a = s_a[j];
                const float2 c = s_c[j];
                const float4 b = s_b[j];
                const float dx = a.x - fx, dy = a.y - fy;
                const float power = __fmaf_rn(-0.5f, __fmaf_rn(a.z * dx, dx, (b.x * dy) * dy), -((a.w * dx) * dy));
                const bool in = !(done || power > 0.0f || power < c.y);
                const float alpha = fminf(kAlphaClamp, raster_alpha_unclamped(b.y, power));
                const float testT = T * (1.0f - alpha);
                const bool faint = alpha < kEpsilon;
                const bool stop = in && !faint && testT < kBlendThreshold;
                const bool blend = in && !faint && !stop;
                done = done || stop;
                const float wr = __fmaf_rn(b.z * alpha, T, cr), wg = __fmaf_rn(b.w * alpha, T, cg);
                const float wb = __fmaf_rn(c.x * alpha, T, cb);
                cr = blend ? wr : cr;
                cg = blend ? wg : cg;
                cb = blend ? wb : cb;
                T = blend ? testT : T;
                if (LAST && blend) last = pos0 + j;
            }
        }
    }
    if (!inside) return;
    const size_t p = (size_t)y * width + x;
    if (out.rgb) {
        out.rgb[3 * p + 0] = cr;
        out.rgb[3 * p + 1] = cg;
        out.rgb[3 * p + 2] = cb;
    }
    if (out.final_t) out.final_t[p] = T;
    if (LAST) out.n_contrib[p] = last;
    if (out.rgba8) {
        const uint32_t r8 = (uint32_t)(fminf(fmaxf(cr, 0.0f), 1.0f) * 255.0f + 0.5f);
        const uint32_t g8 = (uint32_t)(fminf(fmaxf(cg, 0.0f), 1.0f) * 255.0f + 0.5f);
        const uint32_t b8 = (uint32_t)(fminf(fmaxf(cb, 0.0f), 1.0f) * 255.0f + 0.5f);
        out.rgba8[p] = r8 | (g8 << 8) | (b8 << 16) | (255u << 24);
    }
}

template <int TILE, int BATCH>
void launch_batch(const uint32_t* ranges, const uint32_t* vals, const float4* rec, uint32_t n, const FrameCtl* ctl,
                  uint32_t width, uint32_t height, uint32_t tiles_x, uint32_t tiles_y, const RasterOut& out,
                  const uint32_t* order, cudaStream_t s) {
    const dim3 grid(tiles_x * tiles_y), block(TILE * TILE);
    // the contributor count is tracked only when it is written (a differentiable forward): the
    // plain frame's raster drops its register and update (0.509 -> 0.499 ms per 1M / 1080p frame)
    if (out.n_contrib)
        launch_pdl(k_raster<TILE, BATCH, true>, grid, block, s, ranges, vals, rec, n, ctl, width, height, tiles_x, out,
                   order);
    else
        launch_pdl(k_raster<TILE, BATCH, false>, grid, block, s, ranges, vals, rec, n, ctl, width, height, tiles_x, out,
                   order);
}

template <int TILE>
void launch_tile(uint32_t batch, const uint32_t* ranges, const uint32_t* vals, const float4* rec, uint32_t n,
                 const FrameCtl* ctl, uint32_t width, uint32_t height, uint32_t tiles_x, uint32_t tiles_y,
                 const RasterOut& out, const uint32_t* order, cudaStream_t s) {
    switch (batch) {
        case 32: launch_batch<TILE, 32>(ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, out, order, s); break;
        case 64: launch_batch<TILE, 64>(ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, out, order, s); break;
        case 128: launch_batch<TILE, 128>(ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, out, order, s); break;
        default: launch_batch<TILE, 256>(ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, out, order, s); break;
    }
}

}  // namespace

void launch_raster(uint32_t tile, uint32_t batch, const uint32_t* ranges, const uint32_t* vals, const float4* rec,
                   uint32_t n, const FrameCtl* ctl, uint32_t width, uint32_t height, uint32_t tiles_x,
                   uint32_t tiles_y, const RasterOut& out, const uint32_t* order, cudaStream_t s) {
    if (tile == 8) launch_tile<8>(batch, ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, out, order, s);
    else if (tile == 32) launch_tile<32>(batch, ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, out, order, s);
    else launch_tile<16>(batch, ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, out, order, s);
}

}  // namespace gs
