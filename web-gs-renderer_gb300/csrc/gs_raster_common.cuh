// gs_raster_common.cuh -- pieces shared by the forward raster and its backward: the pinned exp on
// the raster's argument range and the conservative per-warp cull of staged splats.
//
// Cull. For a splat with conic (a, b, c) and cut-off c_o = ln((1/255)/o) - 1e-3, a pixel can only
// pass "power >= c_o" where Q(d) = a dx^2 + 2b dx dy + c dy^2 <= K', K' = -2 c_o plus the worst
// rounding error of the pinned power formula anywhere in the tile (16 eps times S_max, the sum of
// the absolute terms bounded over the tile). The cull box is the bounding box of {Q <= K'}, with
// det = ac - b^2 taken at its lower rounding bound; its 45-degree box bounds u = x + y and v = x - y
// over the same region (half-extents sqrt(K' (a + c -+ 2b) / det)), and the two together form an
// octagon around the ellipse. A splat whose octagon misses a warp's pixel block would have been
// rejected by every pixel of the block at "power < c_o" (or "power > 0"), so skipping it changes no
// output bit. Splats whose region cannot be bounded safely (non-positive-definite or non-finite
// values) are never culled. Against the box alone the octagon removes 13.5% of the (8x4 block,
// splat) hits of the 1M / 1080p frame and 10.9% of the (8x8 block, splat) hits.
#pragma once
#include "gs_common.cuh"

namespace gs {

// The raster's exp (alpha = o * exp(power), raseter.wgsl:89), pinned like the oracle's raster_expf.
// For an opacity o in (0, 1] the cut-off is at least ln(1/255) - 1e-3 > -5.6, so every argument lies in
// [-5.6, 0] and no range checks are needed. n = rint(x log2 e) comes from one fma with the 1.5 * 2^23
// shift (the sum rounds to an integer, to nearest even, and its low mantissa bits are n, which also
// give 2^n without a float-to-int conversion); r = x - n ln2 is one fma with the f32 ln2 (|n| <= 8, so
// r stays within 1.6e-8 of the exact reduction); e^r is a degree-6 polynomial with c0 = c1 = 1 and
// c2..c6 from the project's relative-error minimax fit on [-ln2/2, ln2/2]. Under 0.9 ulp from exp on
// the range (the tests check it against the FP64 exp and bit for bit against the oracle). 11
// instructions, against 15 for the degree-7 Taylor form of the general pinned exp.
// o = 0 (cut-off +inf) never gets here; for a NaN opacity the product o * exp(.) is NaN whatever this
// returns, as with pinned_expf.
// raster_exp_poly gives the two parts: it returns the polynomial p = e^r and sets t, whose low
// mantissa bits hold n (e^x = p 2^n).
__device__ __forceinline__ float raster_exp_poly(float x, float& t) {
    t = __fmaf_rn(x, 0x1.715476p+0f, 12582912.0f);
    const float n = __fadd_rn(t, -12582912.0f);
    const float r = __fmaf_rn(-n, 0x1.62e43p-1f, x);
    float p = 0x1.6c350cp-10f;
    p = __fmaf_rn(p, r, 0x1.1246dap-7f);
    p = __fmaf_rn(p, r, 0x1.555638p-5f);
    p = __fmaf_rn(p, r, 0x1.55547ep-3f);
    p = __fmaf_rn(p, r, 0x1.fffffep-2f);
    p = __fmaf_rn(p, r, 1.0f);
    return __fmaf_rn(p, r, 1.0f);
}

__device__ __forceinline__ float raster_expf(float x) {
    float t;
    const float p = raster_exp_poly(x, t);
    return __fmul_rn(p, __int_as_float((__float_as_int(t) + 127) << 23));
}

// o * raster_expf(x), bit for bit, for an argument at or above o's cut-off (x >= ln((1/255)/o) - 1e-3,
// the only arguments the raster evaluates): raster_expf multiplies p by 2^n exactly, so o * (p 2^n)
// rounds once, like (o p) 2^n, and scaling by 2^n commutes with rounding while nothing under- or
// overflows. Above the cut-off o p 2^n is at least about 1/255 and o p at most about 1, all normal,
// so 2^n is applied by adding n to the exponent field of o p: one integer op (the low bits of t hold
// n; shifted up by 23 the rest of t falls off) instead of building 2^n and a second multiply (raster
// of the 1M / 1080p frame 0.2621 -> 0.2583 ms). Where o p is NaN (a NaN argument or opacity) it is
// the GPU's positive canonical NaN, which the add leaves a NaN or turns into a large positive finite
// value; min(0.99, .) makes 0.99 of either, as it does of the NaN of o * raster_expf.
__device__ __forceinline__ float raster_alpha_unclamped(float o, float x) {
    float t;
    const float p = raster_exp_poly(x, t);
    return __int_as_float(__float_as_int(__fmul_rn(o, p)) + (__float_as_int(t) << 23));
}

__device__ __forceinline__ bool finite_f(float v) { return fabsf(v) <= 3.0e38f; }

// Conservative box (x0, x1, y0, y1) for the tile [tx0,tx1] x [ty0,ty1], and in diag its 45-degree
// box (u0, u1, v0, v1): (+inf, -inf, +inf, -inf) when no pixel can pass, (-inf, +inf, -inf, +inf)
// when no safe bound exists. A warp block [rx0, rx1] x [ry0, ry1] spans u in [rx0 + ry0, rx1 + ry1]
// and v in [rx0 - ry1, rx1 - ry0] (exact: integer coordinates).
__device__ __forceinline__ float4 cull_box(float x, float y, float a, float b, float c, float cut, float tx0,
                                           float tx1, float ty0, float ty1, float4& diag) {
    const float inf = __int_as_float(0x7f800000);
    const float4 keep_all = make_float4(-inf, inf, -inf, inf);
    diag = keep_all;
    if (!(finite_f(x) && finite_f(y) && finite_f(a) && finite_f(b) && finite_f(c)) || cut != cut) return keep_all;
    if (!(a > 0.0f) || !(c > 0.0f)) return keep_all;
    const float dxm = fmaxf(fabsf(x - tx0), fabsf(x - tx1));
    const float dym = fmaxf(fabsf(y - ty0), fabsf(y - ty1));
    const float smax = (a * dxm * dxm + c * dym * dym + 2.0f * fabsf(b) * dxm * dym) * 1.01f;
    if (!finite_f(smax)) return keep_all;
    if (cut > 0.0f) {  // power <= 0 < cut everywhere
        diag = make_float4(inf, -inf, inf, -inf);
        return diag;
    }
    const float ac = a * c, bb = b * b;
    const float det_lo = (ac - bb) - 4.0f * 0x1p-24f * (ac + bb);
    if (!(det_lo > 0.0f)) return keep_all;
    const float k = (-2.0f * cut + 0x1p-20f * smax) * 1.000001f;
    // approximate divide and square root (a few ulp), far inside the 1e-5 relative margin
    const float vx = __fdividef(k * c, det_lo), vy = __fdividef(k * a, det_lo);
    const float hx = vx * rsqrtf(vx) * 1.00001f + 1.0e-3f + fabsf(x) * 0x1p-22f;
    const float hy = vy * rsqrtf(vy) * 1.00001f + 1.0e-3f + fabsf(y) * 0x1p-22f;
    if (!finite_f(hx) || !finite_f(hy)) return keep_all;
    // the same region's extent along u = x + y and v = x - y: sqrt(K' (a + c -+ 2b) / det), the
    // quadratic forms bounded above (they are positive: a, c > 0 and det > 0)
    const float apc = a + c, b2 = 2.0f * b;
    const float su = (apc - b2) + 4.0f * 0x1p-24f * (apc + fabsf(b2));
    const float sv = (apc + b2) + 4.0f * 0x1p-24f * (apc + fabsf(b2));
    const float wu = __fdividef(k * su, det_lo), wv = __fdividef(k * sv, det_lo);
    const float u = x + y, v = x - y;
    const float hu = wu * rsqrtf(wu) * 1.00001f + 1.0e-3f + fabsf(u) * 0x1p-22f;
    const float hv = wv * rsqrtf(wv) * 1.00001f + 1.0e-3f + fabsf(v) * 0x1p-22f;
    if (finite_f(hu) && finite_f(hv) && su > 0.0f && sv > 0.0f) diag = make_float4(u - hu, u + hu, v - hv, v + hv);
    return make_float4(x - hx, x + hx, y - hy, y + hy);
}

// Whether the box meets the pixel block [rx0,rx1] x [ry0,ry1].
__device__ __forceinline__ bool box_meets(const float4& box, float rx0, float rx1, float ry0, float ry1) {
    return box.y >= rx0 && box.x <= rx1 && box.w >= ry0 && box.z <= ry1;
}

}  // namespace gs
