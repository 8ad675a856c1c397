// gs_raster.cu -- front-to-back alpha-blending tile rasterizer (src/shaders/raseter.wgsl:35-117).
//
// One CTA per tile, one thread per pixel (TILE x TILE threads). The tile's sorted range is walked
// in batches of BATCH splats: the CTA votes to stop once every pixel is done (raseter.wgsl:54-68 as
// one __syncthreads_and), stages the batch's records (position, conic, opacity, colour and the
// alpha cut-off) in shared memory with one gather per splat, then every pixel blends the batch in
// order. The blend follows the pinned fp32 semantics:
//   power = fma(-0.5, fma(a*dx, dx, (c*dy)*dy), -((b*dx)*dy)); skip if power > 0
//   alpha = min(0.99, o * exp(power));                         skip if alpha < 1/255
//   testT = T * (1 - alpha);                                   done if testT < 1e-4
//   C += colour * alpha * T (one fma per channel); T = testT
// Pixels whose power is below the splat's cut-off skip the exp: for them o*exp(power) < 1/255 is
// certain (the cut-off is ln((1/255)/o) less 1e-3, far beyond the rounding of exp, the product
// and logf), so the skip cannot change a result.
#include "gs_kernels.h"

namespace gs {
namespace {

template <int TILE, int BATCH>
__global__ void __launch_bounds__(TILE * TILE) k_raster(const uint32_t* __restrict__ ranges,
                                                        const uint32_t* __restrict__ vals,
                                                        const float4* __restrict__ rec, uint32_t n,
                                                        const FrameCtl* __restrict__ ctl, uint32_t width,
                                                        uint32_t height, uint32_t tiles_x, RasterOut out) {
    constexpr int THREADS = TILE * TILE;
    __shared__ float4 s_a[BATCH];  // (x, y, conic.x, conic.y)
    __shared__ float4 s_b[BATCH];  // (conic.z, opacity, r, g)
    __shared__ float2 s_c[BATCH];  // (b, cut)

    const uint32_t tile = blockIdx.x;
    const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
    const uint32_t lx = threadIdx.x % TILE, ly = threadIdx.x / TILE;
    const uint32_t x = tx * TILE + lx, y = ty * TILE + ly;
    const bool inside = x < width && y < height;
    bool done = !inside;
    const uint2 range = reinterpret_cast<const uint2*>(ranges)[tile];
    // a range past the sorted count can only come from a timed-out sort: clamp it
    const uint32_t end = ctl ? min(range.y, ctl->sorted_count) : range.y;
    const uint32_t start = range.x;
    const float fx = (float)x, fy = (float)y;

    float T = 1.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f;
    uint32_t contributor = 0, last = 0;

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
                } else {  // only after a timed-out sort: a splat that never blends
                    s_a[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    s_b[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    s_c[j] = make_float2(0.0f, __int_as_float(0x7f800000));
                }
            }
        }
        __syncthreads();
        if (!done) {
            const uint32_t cnt = min((uint32_t)BATCH, end - i);
            for (uint32_t j = 0; j < cnt; ++j) {
                ++contributor;
                const float4 a = s_a[j];
                const float2 c = s_c[j];
                const float dx = a.x - fx, dy = a.y - fy;
                const float s4 = s_b[j].x;
                const float q = __fmaf_rn(a.z * dx, dx, (s4 * dy) * dy);
                const float power = __fmaf_rn(-0.5f, q, -((a.w * dx) * dy));
                if (power > 0.0f) continue;
                if (power < c.y) continue;
                const float4 b = s_b[j];
                const float alpha = fminf(kAlphaClamp, b.y * pinned_expf(power));
                if (alpha < kEpsilon) continue;
                const float testT = T * (1.0f - alpha);
                if (testT < kBlendThreshold) {
                    done = true;
                    break;
                }
                cr = __fmaf_rn(b.z * alpha, T, cr);
                cg = __fmaf_rn(b.w * alpha, T, cg);
                cb = __fmaf_rn(c.x * alpha, T, cb);
                T = testT;
                last = contributor;
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
    if (out.n_contrib) out.n_contrib[p] = last;
    if (out.rgba8) {
        const uint32_t r8 = (uint32_t)(fminf(fmaxf(cr, 0.0f), 1.0f) * 255.0f + 0.5f);
        const uint32_t g8 = (uint32_t)(fminf(fmaxf(cg, 0.0f), 1.0f) * 255.0f + 0.5f);
        const uint32_t b8 = (uint32_t)(fminf(fmaxf(cb, 0.0f), 1.0f) * 255.0f + 0.5f);
        out.rgba8[p] = r8 | (g8 << 8) | (b8 << 16) | (255u << 24);
    }
}

template <int TILE>
void launch_tile(uint32_t batch, const uint32_t* ranges, const uint32_t* vals, const float4* rec, uint32_t n,
                 const FrameCtl* ctl, uint32_t width, uint32_t height, uint32_t tiles_x, uint32_t tiles_y,
                 const RasterOut& out, cudaStream_t s) {
    const uint32_t grid = tiles_x * tiles_y;
    switch (batch) {
        case 32: k_raster<TILE, 32><<<grid, TILE * TILE, 0, s>>>(ranges, vals, rec, n, ctl, width, height, tiles_x, out); break;
        case 64: k_raster<TILE, 64><<<grid, TILE * TILE, 0, s>>>(ranges, vals, rec, n, ctl, width, height, tiles_x, out); break;
        case 128: k_raster<TILE, 128><<<grid, TILE * TILE, 0, s>>>(ranges, vals, rec, n, ctl, width, height, tiles_x, out); break;
        default: k_raster<TILE, 256><<<grid, TILE * TILE, 0, s>>>(ranges, vals, rec, n, ctl, width, height, tiles_x, out); break;
    }
}

}  // namespace

void launch_raster(uint32_t tile, uint32_t batch, const uint32_t* ranges, const uint32_t* vals, const float4* rec,
                   uint32_t n, const FrameCtl* ctl, uint32_t width, uint32_t height, uint32_t tiles_x,
                   uint32_t tiles_y, const RasterOut& out, cudaStream_t s) {
    if (tile == 8) launch_tile<8>(batch, ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, out, s);
    else if (tile == 32) launch_tile<32>(batch, ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, out, s);
    else launch_tile<16>(batch, ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, out, s);
}

}  // namespace gs
