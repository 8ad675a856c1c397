// gs_backward.cu -- the raster half of the gradients of the splat pipeline (no counterpart in the
// reference, which only renders):
//   k_raster_backward     per tile, walks each pixel's blended splats back to front from its last
//                         contributor, recomputing power and alpha bit for bit as the forward did
//                         (same pinned arithmetic, the forward's warp cull octagon), recovering T by
//                         division, and accumulating dL/d(pixel.xy, conic, opacity, colour) per
//                         Gaussian: two pixels per lane, the warp reduces by shuffles, nine lanes
//                         issue the atomics.
// The preprocess half (2D gradients -> the 59 attributes) is in gs_preprocess_backward.cu.
// Conventions: gradients flow through the fp32 RGB before quantization; culled Gaussians, skipped
// pairs and splats after a pixel's termination get none; active clamps (alpha 0.99, colour >= 0)
// pass none; where the frustum guard clamps t.x/t.z (t.y/t.z) no gradient flows through t.x (t.y),
// as in 3DGS.
#include "gs_kernels.h"
#include "gs_raster_common.cuh"

namespace gs {
namespace {

__device__ __forceinline__ float hw_exp2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Warp reduce-scatter of eight values: after it, each lane holds the warp total of value
// (lane >> 2) & 7. Halving stages: xor 16 splits the values 0-3 | 4-7 between the half-warps, xor 8
// splits each half again, xor 4 once more (4 + 2 + 1 shuffles), then xor 2 and xor 1 finish the
// sums: 9 shuffles instead of 40 for eight separate reductions.
__device__ __forceinline__ float warp_reduce_scatter8(const float v[8]) {
    const uint32_t lane = threadIdx.x & 31u;
    const bool b4 = lane & 16u, b3 = lane & 8u, b2 = lane & 4u;
    float w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float send = b4 ? v[k] : v[k + 4];
        const float keep = b4 ? v[k + 4] : v[k];
        w[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
    float u[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float send = b3 ? w[k] : w[k + 2];
        const float keep = b3 ? w[k + 2] : w[k];
        u[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    const float send = b2 ? u[0] : u[1];
    float t = (b2 ? u[1] : u[0]) + __shfl_xor_sync(0xffffffffu, send, 4);
    t += __shfl_xor_sync(0xffffffffu, t, 2);
    t += __shfl_xor_sync(0xffffffffu, t, 1);
    return t;
}

// One pixel's backward state: its last contributor L (1-based position in the tile range), the
// transmittance in front of the splat being visited, its colour gradient dC, and D = dC . S, S being
// the colour the splats behind the visited one added to the pixel (S = sum over them of alpha_j T_j c_j).
struct PixState {
    uint32_t L;
    float fx, fy, T, dr, dg, db;
    float d;
};

__device__ __forceinline__ void pix_load(PixState& p, uint32_t x, uint32_t y, uint32_t width, uint32_t height,
                                         const float* __restrict__ final_t, const uint32_t* __restrict__ n_contrib,
                                         const float* __restrict__ dl_drgb) {
    p.fx = (float)x;
    p.fy = (float)y;
    p.L = 0;
    p.T = 1.0f;
    p.dr = p.dg = p.db = 0.0f;
    p.d = 0.0f;
    if (x < width && y < height) {
        const size_t q = (size_t)y * width + x;
        p.L = n_contrib[q];
        p.T = final_t[q];
        p.dr = dl_drgb[3 * q];
        p.dg = dl_drgb[3 * q + 1];
        p.db = dl_drgb[3 * q + 2];
    }
}

// Visits the splat at 1-based range position pos for one pixel: the same power / exp / alpha
// decisions as the forward (bit for bit), then adds this pixel's share of the splat's gradients to
// g = {d px, d py, d conic.x, d conic.y, d conic.z, d opacity, d r, d g, d b}, the first five without
// their constant factors (-1, -1, -1/2, -1, -1/2, applied after the warp reduction). T is recovered by
// division (the approximate reciprocal, 2 ulp, of 1 - alpha >= 0.01 is accurate enough for a
// gradient). With C = sum_i alpha_i T_i c_i and T_{i+1} = T_i (1 - alpha_i),
// dC/dalpha_i = T_i c_i - S_i / (1 - alpha_i), S_i being the colour added behind splat i, so
// dL/dalpha_i = T_i K_i - D_i / (1 - alpha_i) with K_i = dC . c_i and D_i = dC . S_i, and D grows by
// alpha_i T_i K_i per step: one running sum per pixel instead of three (S_r, S_g, S_b), and six fewer
// instructions per step.
// FIRST: g is written rather than added to (zeros when the pixel does not contribute), so the hit's
// accumulators need no zeroing before the lane's first pixel.
template <bool FIRST>
__device__ __forceinline__ bool pix_step(PixState& p, uint32_t pos, const float4& a, const float4& b,
                                         const float2& c, float g[9]) {
    auto none = [&]() {
        if (FIRST)
#pragma unroll
            for (int k = 0; k < 9; ++k) g[k] = 0.0f;
        return false;
    };
    auto acc = [&](int k, float x, float y) { g[k] = FIRST ? x * y : __fmaf_rn(x, y, g[k]); };
    const float dx = a.x - p.fx, dy = a.y - p.fy;
    const float power = __fmaf_rn(-0.5f, __fmaf_rn(a.z * dx, dx, (b.x * dy) * dy), -((a.w * dx) * dy));
    if (pos > p.L || power > 0.0f || power < c.y) return none();
    // The gradient's value only needs exp to a few ulp: 2^(power log2 e) by the hardware's base-2
    // exponential (one multiply and one MUFU op; its relative error and that of the rounded argument
    // stay under 5e-7 on the raster's range [-5.6, 0], where no result is denormal, so flushing to
    // zero changes nothing). The decisions must be the forward's, bit for bit: alpha >= 1/255 and the
    // 0.99 clamp are taken on o * exp(power), so where that product lies within 1e-5 (relative) of
    // either threshold the pinned raster exp is evaluated and decides.
    float G = hw_exp2(power * 1.44269504f);
    float og = b.y * G;
    if (fabsf(og - kEpsilon) <= 1e-5f * kEpsilon || fabsf(og - kAlphaClamp) <= 1e-5f * kAlphaClamp) {
        G = raster_expf(power);
        og = b.y * G;
    }
    const float alpha = fminf(kAlphaClamp, og);
    if (!(alpha >= kEpsilon)) return none();
    // from here on only gradients are formed: fused multiply-adds are fine (the decisions above
    // follow the forward's pinned arithmetic)
    const float ria = __fdividef(1.0f, 1.0f - alpha);
    const float Tb = p.T * ria;  // transmittance in front of this splat
    const float w = alpha * Tb;
    acc(6, w, p.dr);
    acc(7, w, p.dg);
    acc(8, w, p.db);
    const float k = __fmaf_rn(b.z, p.dr, __fmaf_rn(b.w, p.dg, c.x * p.db));  // dC . c
    const float dalpha = __fmaf_rn(Tb, k, -(p.d * ria));
    {
        // a clamped alpha passes no gradient to power and opacity (a select, not a branch: 0.585 ->
        // 0.580 ms per 1M / 1080p backward); the constant factors of d power / d(px, py, conic)
        // (-1, -1, -1/2, -1, -1/2) are applied once per splat after the warp reduction (kGradSign)
        const float da = og <= kAlphaClamp ? dalpha : 0.0f;
        const float gp = da * og;  // dL/dpower
        const float gpdx = gp * dx, gpdy = gp * dy;
        acc(0, gp, __fmaf_rn(a.z, dx, a.w * dy));
        acc(1, gp, __fmaf_rn(b.x, dy, a.w * dx));
        acc(2, gpdx, dx);
        acc(3, gpdx, dy);
        acc(4, gpdy, dy);
        acc(5, da, G);
    }
    p.d = __fmaf_rn(w, k, p.d);
    p.T = Tb;
    return true;
}

// One CTA per tile with TILE*TILE/2 threads: each warp owns an 8x8 pixel block and each lane two
// pixels of it, (x, y) and (x, y + 4), so the per-splat warp reduction and shared-memory loads are
// shared by two pixels. A warp walks only positions up to the largest last-contributor index of its
// own pixels.
template <int TILE, int BATCH>
__global__ void __launch_bounds__(TILE * TILE / 2) k_raster_backward(const uint32_t* __restrict__ ranges,
                                                                     const uint32_t* __restrict__ vals,
                                                                     const float4* __restrict__ rec, uint32_t n,
                                                                     const FrameCtl* __restrict__ ctl,
                                                                     uint32_t width, uint32_t height,
                                                                     uint32_t tiles_x,
                                                                     const float* __restrict__ final_t,
                                                                     const uint32_t* __restrict__ n_contrib,
                                                                     const float* __restrict__ dl_drgb,
                                                                     float* __restrict__ grad2d,
                                                                     const uint32_t* __restrict__ order) {
    pdl_wait();
    constexpr int WX = TILE / 8;
    constexpr int kThreads = TILE * TILE / 2;
    __shared__ float4 s_a[BATCH];
    __shared__ float4 s_b[BATCH];
    __shared__ float2 s_c[BATCH];
    __shared__ float4 s_box[BATCH];
    __shared__ float4 s_diag[BATCH];
    __shared__ uint32_t s_g[BATCH];
    __shared__ uint32_t s_maxl;

    const uint32_t tile = order ? order[blockIdx.x] : blockIdx.x;
    const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t bx0 = tx * TILE + 8u * (warp % WX), by0 = ty * TILE + 8u * (warp / WX);
    const uint32_t x = bx0 + (lane & 7u), y = by0 + (lane >> 3);
    const uint2 range = reinterpret_cast<const uint2*>(ranges)[tile];
    const uint32_t end = ctl ? min(range.y, ctl->sorted_count) : range.y;
    const uint32_t start = range.x;
    const uint32_t len = end > start ? end - start : 0u;
    const float rx0 = (float)bx0, rx1 = (float)(bx0 + 7u), ry0 = (float)by0, ry1 = (float)(by0 + 7u);
    const float tx0 = (float)(tx * TILE), tx1 = (float)(tx * TILE + TILE - 1u);
    const float ty0 = (float)(ty * TILE), ty1 = (float)(ty * TILE + TILE - 1u);

    // factor of the value this lane ends up holding after warp_reduce_scatter8 (see pix_step)
    const float kGradSign[8] = {-1.0f, -1.0f, -0.5f, -1.0f, -0.5f, 1.0f, 1.0f, 1.0f};
    const float sign = kGradSign[(lane >> 2) & 7u];
    PixState p0, p1;
    pix_load(p0, x, y, width, height, final_t, n_contrib, dl_drgb);
    pix_load(p1, x, y + 4u, width, height, final_t, n_contrib, dl_drgb);
    const uint32_t wmax = min(__reduce_max_sync(0xffffffffu, max(p0.L, p1.L)), len);
    if (threadIdx.x == 0) s_maxl = 0;
    __syncthreads();
    if (lane == 0 && wmax) atomicMax(&s_maxl, wmax);
    __syncthreads();
    const uint32_t maxl = s_maxl;

    // positions are 1-based within the tile range; walk batches (lo, hi] from the top down
    for (uint32_t hi = maxl; hi > 0;) {
        const uint32_t lo = hi > (uint32_t)BATCH ? hi - BATCH : 0u;
        const uint32_t cnt = hi - lo;
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < cnt; j += kThreads) {
            const uint32_t g = vals[start + lo + j];
            if (g < n) {
                const float4 r0 = __ldg(rec + (size_t)kRecFloat4 * g);
                const float4 r1 = __ldg(rec + (size_t)kRecFloat4 * g + 1);
                const float4 r2 = __ldg(rec + (size_t)kRecFloat4 * g + 2);
                s_a[j] = r0;
                s_b[j] = r1;
                s_c[j] = make_float2(r2.x, r2.y);
                s_box[j] = cull_box(r0.x, r0.y, r0.z, r0.w, r1.x, r2.y, tx0, tx1, ty0, ty1, s_diag[j]);
                s_g[j] = g;
            } else {
                const float inf = __int_as_float(0x7f800000);
                s_box[j] = make_float4(inf, -inf, inf, -inf);
                s_diag[j] = s_box[j];
                s_g[j] = 0xFFFFFFFFu;
            }
        }
        __syncthreads();
        if (lo < wmax) {
            // groups of 32 from the warp's top position in this batch down, splats in a group from
            // high to low
            const int top = (int)min(cnt, wmax - lo) - 1;
            for (int gtop = top; gtop >= 0; gtop -= 32) {
                const int gbase = gtop - 31;
                const int jj = gbase + (int)lane;
                const bool hit = jj >= 0 && box_meets(s_box[jj], rx0, rx1, ry0, ry1) &&
                                 box_meets(s_diag[jj], rx0 + ry0, rx1 + ry1, rx0 - ry1, rx1 - ry0);
                uint32_t m = __ballot_sync(0xffffffffu, hit);
                while (m) {
                    const int bit = 31 - __clz(m);
                    m &= ~(1u << bit);
                    const int j = gbase + bit;
                    const uint32_t pos = lo + (uint32_t)j + 1u;
                    const float4 a = s_a[j];
                    const float4 b = s_b[j];
                    const float2 c = s_c[j];
                    float g[9];
                    const bool c0 = pix_step<true>(p0, pos, a, b, c, g);
                    const bool c1 = pix_step<false>(p1, pos, a, b, c, g);
                    const uint32_t who = __ballot_sync(0xffffffffu, c0 || c1);
                    if (__popc(who) > 8) {
                        const float mine = sign * warp_reduce_scatter8(g);  // total of value (lane >> 2) & 7
                        const float blue = warp_sum(g[8]);
                        const uint32_t gi = s_g[j];
                        if (gi < n) {
                            float* dst = grad2d + (size_t)9 * gi;
                            if ((lane & 3u) == 0u) atomicAdd(dst + ((lane >> 2) & 7u), mine);
                            if (lane == 2u) atomicAdd(dst + 8, blue);
                        }
                    } else if (who) {
                        // up to eight contributing lanes: each adds its own nine values (nine atomic
                        // instructions for the warp either way) instead of the warp's reduce-scatter.
                        // Measured at 1M / 1080p: up to 4 lanes 0.554 ms, 8 (or 10) 0.545, 16 0.653 (the
                        // per-lane atomics then load L2 more than the reduce-scatter costs); 0.556 without
                        const uint32_t gi = s_g[j];
                        if ((c0 || c1) && gi < n) {
                            float* dst = grad2d + (size_t)9 * gi;
#pragma unroll
                            for (int k = 0; k < 8; ++k) atomicAdd(dst + k, kGradSign[k] * g[k]);
                            atomicAdd(dst + 8, g[8]);
                        }
                    }
                }
            }
        }
        hi = lo;
    }
}

template <int TILE>
void launch_bwd_tile(uint32_t batch, const uint32_t* ranges, const uint32_t* vals, const float4* rec, uint32_t n,
                     const FrameCtl* ctl, uint32_t width, uint32_t height, uint32_t tiles_x, uint32_t tiles_y,
                     const float* final_t, const uint32_t* n_contrib, const float* dl, float* grad2d,
                     const uint32_t* order, cudaStream_t s) {
    const uint32_t grid = tiles_x * tiles_y;
    constexpr int threads = TILE * TILE / 2;
    switch (batch) {
        case 32: launch_pdl(k_raster_backward<TILE, 32>, dim3(grid), dim3(threads), s, ranges, vals, rec, n, ctl, width, height, tiles_x, final_t, n_contrib, dl, grad2d, order); break;
        case 64: launch_pdl(k_raster_backward<TILE, 64>, dim3(grid), dim3(threads), s, ranges, vals, rec, n, ctl, width, height, tiles_x, final_t, n_contrib, dl, grad2d, order); break;
        case 128: launch_pdl(k_raster_backward<TILE, 128>, dim3(grid), dim3(threads), s, ranges, vals, rec, n, ctl, width, height, tiles_x, final_t, n_contrib, dl, grad2d, order); break;
        default: launch_pdl(k_raster_backward<TILE, 256>, dim3(grid), dim3(threads), s, ranges, vals, rec, n, ctl, width, height, tiles_x, final_t, n_contrib, dl, grad2d, order); break;
    }
}

}  // namespace

void launch_raster_backward(uint32_t tile, uint32_t batch, const uint32_t* ranges, const uint32_t* vals,
                            const float4* rec, uint32_t n, const FrameCtl* ctl, uint32_t width, uint32_t height,
                            uint32_t tiles_x, uint32_t tiles_y, const float* final_t, const uint32_t* n_contrib,
                            const float* dl_drgb, float* grad2d, const uint32_t* order, cudaStream_t s) {
    if (tile == 8)
        launch_bwd_tile<8>(batch, ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, final_t, n_contrib, dl_drgb, grad2d, order, s);
    else if (tile == 32)
        launch_bwd_tile<32>(batch, ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, final_t, n_contrib, dl_drgb, grad2d, order, s);
    else
        launch_bwd_tile<16>(batch, ranges, vals, rec, n, ctl, width, height, tiles_x, tiles_y, final_t, n_contrib, dl_drgb, grad2d, order, s);
}

}  // namespace gs
