// gs_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
//
// CPU restatement of the reference splat pipeline, one function per WGSL pass, each citing the
// reference file:line it follows. fp32 semantics are the ones pinned in gs_oracle.h; build with
// -ffp-contract=off so that only the explicit fma calls fuse. PARITY UNPINNED (see gs_oracle.h).
#include "gs_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// GlobalUniforms, preprocess.wgsl:2-12; packed at renderer.js:773-797 (176 bytes).
struct Uniforms {
    float view[16];      // column-major mat4x4f
    float viewProj[16];
    float cameraPos[3];
    uint32_t count;
    float focal[2];
    float tanFov[2];
    float textureSize[2];
    uint32_t pad0, pad1;
};
static_assert(sizeof(Uniforms) == 176, "GlobalUniforms is 176 bytes");

// ---- pinned exp (rule 4) ------------------------------------------------------------------------
// exp(x) = 2^n * e^r with n = rint(x*log2(e)), r = x - n*ln2 (ln2 split in two f32 parts, each
// subtraction one fma), e^r by the Taylor series to degree 7 in Horner form (|r| <= ln2/2, so the
// truncation error is below 6e-9 relative). 2^n is applied as two exact power-of-two factors so
// that subnormal results round once.
float pinned_expf(float x) {
    if (x != x) return x;
    if (x > 89.0f) return INFINITY;
    if (x < -104.0f) return 0.0f;
    const float kLog2e = 0x1.715476p+0f;
    const float kLn2Hi = 0x1.62e43p-1f;
    const float kLn2Lo = -0x1.05c61p-29f;
    float n = std::rint(x * kLog2e);
    float r = std::fmaf(-n, kLn2Hi, x);
    r = std::fmaf(-n, kLn2Lo, r);
    float p = 0x1.a01a02p-13f;            // 1/7!
    p = std::fmaf(p, r, 0x1.6c16c2p-10f); // 1/6!
    p = std::fmaf(p, r, 0x1.111112p-7f);  // 1/5!
    p = std::fmaf(p, r, 0x1.555556p-5f);  // 1/4!
    p = std::fmaf(p, r, 0x1.555556p-3f);  // 1/3!
    p = std::fmaf(p, r, 0.5f);
    p = std::fmaf(p, r, 1.0f);
    p = std::fmaf(p, r, 1.0f);
    int k = (int)n;
    int k1 = k / 2;
    int k2 = k - k1;
    uint32_t b1 = (uint32_t)(k1 + 127) << 23, b2 = (uint32_t)(k2 + 127) << 23;
    float s1, s2;
    std::memcpy(&s1, &b1, 4);
    std::memcpy(&s2, &b2, 4);
    return (p * s1) * s2;
}

// The raster's exp (rule 4b): the alpha of raseter.wgsl:89 evaluates exp only between a splat's
// cut-off (>= ln(1/255) - 1e-3 > -5.6) and 0, so no range checks are needed there. n = rint(x log2 e)
// by one fma with the 1.5 * 2^23 shift (the sum's low mantissa bits are n), r = x - n ln2 by one fma
// (|n| <= 8 here, so the f32 ln2 alone keeps r within 1.6e-8 of x - n ln2), e^r by a degree-6
// polynomial with c0 = c1 = 1 whose c2..c6 are the project's relative-error minimax fit on
// [-ln2/2, ln2/2] (Remez exchange; 4.3e-9 relative before rounding), and 2^n from the shift's bits.
// Every step is an IEEE-754 operation.
float raster_expf(float x) {
    const float t = std::fmaf(x, 0x1.715476p+0f, 12582912.0f);
    const float n = t - 12582912.0f;
    const float r = std::fmaf(-n, 0x1.62e43p-1f, x);
    float p = 0x1.6c350cp-10f;
    p = std::fmaf(p, r, 0x1.1246dap-7f);
    p = std::fmaf(p, r, 0x1.555638p-5f);
    p = std::fmaf(p, r, 0x1.55547ep-3f);
    p = std::fmaf(p, r, 0x1.fffffep-2f);
    p = std::fmaf(p, r, 1.0f);
    p = std::fmaf(p, r, 1.0f);
    uint32_t tb;
    std::memcpy(&tb, &t, 4);
    const uint32_t sb = (tb + 127u) << 23;  // (n + 127) << 23: the shift's own exponent bits drop out
    float scale;
    std::memcpy(&scale, &sb, 4);
    return p * scale;
}

// The raster's alpha exp over every argument the WGSL evaluates it at (power <= 0). The CUDA raster
// uses it only from the splat's cut-off up (power >= ln((1/255)/o) - 1e-3 > -5.6 for any o in
// [0, 1]; a pixel below skips, its alpha being below 1/255 for sure); here raster_expf covers
// [-5.6, 0] and the general pinned exp the arguments below, where any value keeps alpha below 1/255
// and so gives the same skip. (A NaN opacity makes alpha 0.99 whatever exp returns, in both.)
float alpha_expf(float x) { return x >= -5.6f ? raster_expf(x) : pinned_expf(x); }

template <class T> struct Num;
template <> struct Num<float> {
    static float ex(float x) { return pinned_expf(x); }
    static float ex_raster(float x) { return alpha_expf(x); }
    static float fma(float a, float b, float c) { return std::fmaf(a, b, c); }
};
template <> struct Num<double> {
    static double ex(double x) { return std::exp(x); }
    static double ex_raster(double x) { return std::exp(x); }
    static double fma(double a, double b, double c) { return std::fma(a, b, c); }
};

// ---- constants (preprocess.wgsl:32-54, raseter.wgsl:19-21), always the f32 literals ----------
const float kSmallValue = 0.0000001f;
const float kZNearView = 0.2f;
const float kFrustumExtended = 1.3f;
const float kShC0 = 0.28209479177387814f;
const float kShC1 = 0.4886025119029199f;
const float kShC2_0 = 1.0925484305920792f;
const float kShC2_1 = -1.0925484305920792f;
const float kShC2_2 = 0.31539156525252005f;
const float kShC2_3 = -1.0925484305920792f;
const float kShC2_4 = 0.5462742152960396f;
const float kShC3_0 = -0.5900435899266435f;
const float kShC3_1 = 2.890611442640554f;
const float kShC3_2 = -0.4570457994644658f;
const float kShC3_3 = 0.3731763325901154f;
const float kShC3_4 = -0.4570457994644658f;
const float kShC3_5 = 1.445305721320277f;
const float kShC3_6 = -0.5900435899266435f;
const float kAlphaClamp = 0.99f;
const float kEpsilon = 0x1.010102p-8f;  // 1.0f / 255.0f
const float kBlendThreshold = 0.0001f;

// Column-major 3x3 (m[col][row]) and 3-column x 2-row matrices, as WGSL mat3x3f / mat3x2f.
template <class T> struct Mat3 { T m[3][3]; };
template <class T> struct Mat3x2 { T m[3][2]; };
template <class T> struct Mat2 { T m[2][2]; };

// A*B for column-major matrices, each element a dot product in index order (rule 6).
template <class T> Mat3<T> mul33(const Mat3<T>& a, const Mat3<T>& b) {
    Mat3<T> c;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
            T s = a.m[0][i] * b.m[j][0];
            s = s + a.m[1][i] * b.m[j][1];
            s = s + a.m[2][i] * b.m[j][2];
            c.m[j][i] = s;
        }
    return c;
}
template <class T> Mat3<T> transpose33(const Mat3<T>& a) {
    Mat3<T> t;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) t.m[j][i] = a.m[i][j];
    return t;
}
// mat3x2 * mat3x3 -> mat3x2
template <class T> Mat3x2<T> mul32_33(const Mat3x2<T>& a, const Mat3<T>& b) {
    Mat3x2<T> c;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 2; ++i) {
            T s = a.m[0][i] * b.m[j][0];
            s = s + a.m[1][i] * b.m[j][1];
            s = s + a.m[2][i] * b.m[j][2];
            c.m[j][i] = s;
        }
    return c;
}
// mat3x2 * transpose(mat3x2) (a mat2x3) -> mat2x2
template <class T> Mat2<T> mul32_23t(const Mat3x2<T>& a, const Mat3x2<T>& j) {
    Mat2<T> c;
    for (int col = 0; col < 2; ++col)
        for (int i = 0; i < 2; ++i) {
            // transpose(J)[col][k] = J[k][col]
            T s = a.m[0][i] * j.m[0][col];
            s = s + a.m[1][i] * j.m[1][col];
            s = s + a.m[2][i] * j.m[2][col];
            c.m[col][i] = s;
        }
    return c;
}

// mat4 * vec4(p, 1), column-major (rule 6).
template <class T> void mat4_mul_point(const float* m, T x, T y, T z, T out[4]) {
    for (int i = 0; i < 4; ++i) {
        T s = (T)m[0 * 4 + i] * x;
        s = s + (T)m[1 * 4 + i] * y;
        s = s + (T)m[2 * 4 + i] * z;
        s = s + (T)m[3 * 4 + i] * (T)1;
        out[i] = s;
    }
}

template <class T> inline T tmin(T a, T b) { return std::fmin(a, b); }
template <class T> inline T tmax(T a, T b) { return std::fmax(a, b); }

// Per-Gaussian preprocess outputs (preprocess.wgsl:26-30).
template <class T> struct Pre {
    std::vector<uint32_t> tiles_touched;  // N (0 = culled)
    std::vector<uint32_t> meta;           // 4N
    std::vector<T> conic_opacity;         // 4N
    std::vector<T> pixel;                 // 2N
    std::vector<T> color;                 // 4N
};

// preprocess.wgsl:58-144 (helpers :146-284).
template <class T>
void preprocess(const Uniforms& u, const float* params, uint32_t count, uint32_t tile, Pre<T>& out,
                int threads) {
    const uint64_t n = count;
    out.tiles_touched.assign(n, 0u);
    out.meta.assign(4 * n, 0u);
    out.conic_opacity.assign(4 * n, (T)0);
    out.pixel.assign(2 * n, (T)0);
    out.color.assign(4 * n, (T)0);
    const uint64_t positionOffset = 0;
    const uint64_t scaleOffset = positionOffset + n * 3;
    const uint64_t quaternionOffset = scaleOffset + n * 3;
    const uint64_t colorOffset = quaternionOffset + n * 4;
    const uint64_t opacityOffset = colorOffset + n * 3;
    const uint64_t shOffset = opacityOffset + n;
    const T W = (T)u.textureSize[0], H = (T)u.textureSize[1];

#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t gi = 0; gi < (int64_t)n; ++gi) {
        const uint64_t g = (uint64_t)gi;
        const T px = params[positionOffset + g * 3], py = params[positionOffset + g * 3 + 1],
                pz = params[positionOffset + g * 3 + 2];
        T pv[4];
        mat4_mul_point<T>(u.view, px, py, pz, pv);
        // :83 near culling (view space is -z forward)
        if (pv[2] >= -(T)kZNearView) continue;
        T clip[4];
        mat4_mul_point<T>(u.viewProj, px, py, pz, clip);
        const T wden = clip[3] + (T)kSmallValue;
        const T ndcx = clip[0] / wden, ndcy = clip[1] / wden, ndcz = clip[2] / wden;
        // ndcToPixel :207-209
        const T pixx = ((ndcx + (T)1) * W - (T)1) * (T)0.5f;
        const T pixy = ((ndcy + (T)1) * H - (T)1) * (T)0.5f;
        out.pixel[2 * g] = pixx;
        out.pixel[2 * g + 1] = pixy;

        // :95-100 3D covariance
        const T sx = Num<T>::ex((T)params[scaleOffset + g * 3]);
        const T sy = Num<T>::ex((T)params[scaleOffset + g * 3 + 1]);
        const T sz = Num<T>::ex((T)params[scaleOffset + g * 3 + 2]);
        const T q0 = params[quaternionOffset + g * 4], q1 = params[quaternionOffset + g * 4 + 1],
                q2 = params[quaternionOffset + g * 4 + 2], q3 = params[quaternionOffset + g * 4 + 3];
        // normalize(vec4f(q.y, q.z, q.w, q.x))
        const T qlen = std::sqrt(((q1 * q1 + q2 * q2) + q3 * q3) + q0 * q0);
        const T qx = q1 / qlen, qy = q2 / qlen, qz = q3 / qlen, qw = q0 / qlen;
        // quantToMat3 :181-201
        const T x2 = qx + qx, y2 = qy + qy, z2 = qz + qz;
        const T xx = qx * x2, xy = qx * y2, xz = qx * z2;
        const T yy = qy * y2, yz = qy * z2, zz = qz * z2;
        const T wx = qw * x2, wy = qw * y2, wz = qw * z2;
        Mat3<T> R;
        R.m[0][0] = (T)1 - (yy + zz); R.m[0][1] = xy + wz;            R.m[0][2] = xz - wy;
        R.m[1][0] = xy - wz;            R.m[1][1] = (T)1 - (xx + zz); R.m[1][2] = yz + wx;
        R.m[2][0] = xz + wy;            R.m[2][1] = yz - wx;            R.m[2][2] = (T)1 - (xx + yy);
        Mat3<T> S{};
        S.m[0][0] = sx; S.m[1][1] = sy; S.m[2][2] = sz;
        const Mat3<T> cov = mul33(mul33(mul33(R, S), transpose33(S)), transpose33(R));

        // calculateCovariance2D :251-269
        const T limx = (T)kFrustumExtended * (T)u.tanFov[0];
        const T limy = (T)kFrustumExtended * (T)u.tanFov[1];
        T tx = pv[0], ty = pv[1];
        const T tz = pv[2];
        tx = tmin(limx, tmax(-limx, tx / tz)) * tz;
        ty = tmin(limy, tmax(-limy, ty / tz)) * tz;
        // calculateJocabian :211-217
        Mat3x2<T> J;
        const T fx = (T)u.focal[0], fy = (T)u.focal[1];
        J.m[0][0] = fx / tz;             J.m[0][1] = (T)0;
        J.m[1][0] = (T)0;                J.m[1][1] = fy / tz;
        J.m[2][0] = (-fx * tx) / (tz * tz);
        J.m[2][1] = (-fy * ty) / (tz * tz);
        Mat3<T> Wm;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) Wm.m[c][r] = (T)u.view[c * 4 + r];
        const Mat3x2<T> jw = mul32_33(J, Wm);
        const Mat3x2<T> jwc = mul32_33(jw, cov);
        const Mat3x2<T> jwcw = mul32_33(jwc, transpose33(Wm));
        const Mat2<T> c2 = mul32_23t(jwcw, J);
        const T ca = c2.m[0][0] + (T)0.3f, cb = c2.m[0][1], cc = c2.m[1][1] + (T)0.3f;

        // :103-104 det and calculateRadius :271-275
        const T det = ca * cc - cb * cb;
        const T mid = (T)0.5f * (ca + cc);
        const T lambda = mid + std::sqrt(tmax((T)0.1f, mid * mid - det));
        const T radius = std::ceil((T)3.0f * std::sqrt(lambda));

        // :106-112 conic and sigmoid opacity (:203-205)
        const T opacity = (T)1 / ((T)1 + Num<T>::ex(-(T)params[opacityOffset + g]));
        out.conic_opacity[4 * g + 0] = cc / det;
        out.conic_opacity[4 * g + 1] = -cb / det;
        out.conic_opacity[4 * g + 2] = ca / det;
        out.conic_opacity[4 * g + 3] = opacity;

        // :114-115 view direction and calculateColor :219-249
        const T dx = px - (T)u.cameraPos[0], dy = py - (T)u.cameraPos[1], dz = pz - (T)u.cameraPos[2];
        const T dlen = std::sqrt((dx * dx + dy * dy) + dz * dz);
        const T x = dx / dlen, y = dy / dlen, z = dz / dlen;
        const T sxx = x * x, syy = y * y, szz = z * z;
        const T sxy = x * y, syz = y * z, sxz = x * z;
        const T w1 = (T)kShC1 * y;
        const T w2 = (T)kShC1 * z;
        const T w3 = (T)kShC1 * x;
        const T w4 = (T)kShC2_0 * sxy;
        const T w5 = (T)kShC2_1 * syz;
        const T w6 = (T)kShC2_2 * (((T)2.0f * szz - sxx) - syy);
        const T w7 = (T)kShC2_3 * sxz;
        const T w8 = (T)kShC2_4 * (sxx - syy);
        const T w9 = ((T)kShC3_0 * y) * ((T)3.0f * sxx - syy);
        const T w10 = ((T)kShC3_1 * sxy) * z;
        const T w11 = ((T)kShC3_2 * y) * (((T)4.0f * szz - sxx) - syy);
        const T w12 = ((T)kShC3_3 * z) * (((T)2.0f * szz - (T)3.0f * sxx) - (T)3.0f * syy);
        const T w13 = ((T)kShC3_4 * x) * (((T)4.0f * szz - sxx) - syy);
        const T w14 = ((T)kShC3_5 * z) * (sxx - syy);
        const T w15 = ((T)kShC3_6 * x) * (sxx - (T)3.0f * syy);
        for (int ch = 0; ch < 3; ++ch) {
            // getShRest :159-162 -- channel-major: f_rest index g*45 + c + 15*channel
            const float* rest = params + shOffset + g * 45 + 15 * ch;
            T r = (T)kShC0 * (T)params[colorOffset + g * 3 + ch];
            r = r - w1 * (T)rest[0];
            r = r + w2 * (T)rest[1];
            r = r - w3 * (T)rest[2];
            r = r + w4 * (T)rest[3];
            r = r + w5 * (T)rest[4];
            r = r + w6 * (T)rest[5];
            r = r + w7 * (T)rest[6];
            r = r + w8 * (T)rest[7];
            r = r + w9 * (T)rest[8];
            r = r + w10 * (T)rest[9];
            r = r + w11 * (T)rest[10];
            r = r + w12 * (T)rest[11];
            r = r + w13 * (T)rest[12];
            r = r + w14 * (T)rest[13];
            r = r + w15 * (T)rest[14];
            r = r + (T)0.5f;
            out.color[4 * g + ch] = tmax(r, (T)0);
        }

        // :117-120 frustum culling (isInFrustum :277-284)
        if (pixx + radius < (T)0 || pixx - radius > W || pixy + radius < (T)0 || pixy - radius > H) continue;

        // :122-143 tile AABB, depth16, tilesTouched, meta
        const T bminx = pixx - radius, bminy = pixy - radius;
        const T bmaxx = pixx + radius, bmaxy = pixy + radius;
        const uint32_t tilesPerRow = ((uint32_t)u.textureSize[0] + tile - 1u) / tile;
        const uint32_t tilesPerColumn = ((uint32_t)u.textureSize[1] + tile - 1u) / tile;
        const T ft = (T)(float)tile;
        auto tclamp = [](T v, T hi) { return tmin(tmax(v, (T)0), hi); };
        const uint32_t minTileX = (uint32_t)tclamp(std::floor(bminx / ft), (T)(float)(tilesPerRow - 1u));
        const uint32_t minTileY = (uint32_t)tclamp(std::floor(bminy / ft), (T)(float)(tilesPerColumn - 1u));
        const uint32_t maxTileX = (uint32_t)tclamp(std::floor(bmaxx / ft), (T)(float)(tilesPerRow - 1u));
        const uint32_t maxTileY = (uint32_t)tclamp(std::floor(bmaxy / ft), (T)(float)(tilesPerColumn - 1u));
        const uint32_t depthU16 = (uint32_t)(tmin(tmax(ndcz, (T)0), (T)1) * (T)65535.0f);
        out.tiles_touched[g] = (maxTileX - minTileX + 1u) * (maxTileY - minTileY + 1u);
        out.meta[4 * g + 0] = (minTileY << 16u) | minTileX;
        out.meta[4 * g + 1] = (maxTileY << 16u) | maxTileX;
        out.meta[4 * g + 2] = depthU16;
        out.meta[4 * g + 3] = 0u;
    }
}

// offset_scan.wgsl:22-67: one workgroup of 256 walks the N+1 entries block by block, scanning
// each block (Hillis-Steele) and adding the running carry. u32 addition wraps mod 2^32 and is
// associative, so the block walk equals this sequential exclusive scan.
uint32_t exclusive_scan(uint32_t* data, uint64_t n) {
    uint32_t carry = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const uint32_t c = data[i];
        data[i] = carry;
        carry += c;
    }
    return carry;
}

// emit.wgsl:28-66.
void emit(const uint32_t* offsets, const uint32_t* meta, uint32_t count, uint32_t tilesPerRow,
          uint32_t maxInstanceCount, uint32_t* keys, uint32_t* vals, int threads) {
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads)
    for (int64_t gi = 0; gi < (int64_t)count; ++gi) {
        const uint32_t g = (uint32_t)gi;
        const uint32_t base = offsets[g];
        const uint32_t n = offsets[g + 1] - base;
        if (n == 0u) continue;
        const uint32_t minTileX = meta[4 * g] & 0xFFFFu, minTileY = meta[4 * g] >> 16u;
        const uint32_t maxTileX = meta[4 * g + 1] & 0xFFFFu, maxTileY = meta[4 * g + 1] >> 16u;
        const uint32_t depth16 = meta[4 * g + 2] & 0xFFFFu;
        uint32_t slot = base;
        bool stop = false;
        for (uint32_t ty = minTileY; ty <= maxTileY && !stop; ++ty)
            for (uint32_t tx = minTileX; tx <= maxTileX; ++tx) {
                if (slot >= maxInstanceCount) { stop = true; break; }
                const uint32_t tileId = ty * tilesPerRow + tx;
                keys[slot] = (tileId << 16u) | depth16;
                vals[slot] = g;
                ++slot;
            }
    }
}

// radix_parallel.wgsl:26-160 for one pass: countMain (per-256-block digit histogram stored
// digit-major), scanLocal/BlockSums/AddOffset (= exclusive scan of the whole digit-major table),
// reorderMain (rank = equal digits in lower lanes of the block). The reference sizes the table by
// blockCountMax = ceil(64N/256); blocks past ceil(n/256) hold zeros and do not change the scan.
void radix_pass(const uint32_t* keys, const uint32_t* vals, uint32_t* okeys, uint32_t* ovals, uint32_t n,
                uint32_t shift) {
    const uint32_t kBlock = 256u;
    const uint32_t blocks = (n + kBlock - 1u) / kBlock;
    std::vector<uint32_t> counts((size_t)256 * blocks, 0u);
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t d = (keys[i] >> shift) & 0xFFu;
        counts[(size_t)d * blocks + i / kBlock] += 1u;
    }
    exclusive_scan(counts.data(), counts.size());
    uint32_t rank[256];
    for (uint32_t b = 0; b < blocks; ++b) {
        std::memset(rank, 0, sizeof(rank));
        const uint32_t lo = b * kBlock, hi = std::min(n, lo + kBlock);
        for (uint32_t i = lo; i < hi; ++i) {
            const uint32_t d = (keys[i] >> shift) & 0xFFu;
            const uint32_t pos = counts[(size_t)d * blocks + b] + rank[d]++;
            okeys[pos] = keys[i];
            ovals[pos] = vals[i];
        }
    }
}

// tile_ranges.wgsl:7-34, over the sorted prefix of n instances (ranges cleared beforehand,
// renderer.js:919).
void tile_ranges(const uint32_t* keys, uint32_t n, uint32_t* ranges) {
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t tileIndex = keys[i] >> 16u;
        if (i == 0u) {
            ranges[tileIndex * 2] = 0u;
        } else {
            const uint32_t prev = keys[i - 1] >> 16u;
            if (tileIndex > prev) {
                ranges[prev * 2 + 1] = i;
                ranges[tileIndex * 2] = i;
            }
        }
        if (i == n - 1u) ranges[tileIndex * 2 + 1] = n;
    }
}

// tile_ranges.wgsl:7-34 exactly as the reference binds it, for the overflow contract: the pass is
// dispatched with the sort's indirect grid, ceil(min(I, capacity) / 256) workgroups of 256
// (indirect_arg.wgsl:16-21), but its bound and its last-instance test use the unclamped instance
// count I (renderer.js:612 binds instanceCountBuffer, tile_ranges.wgsl:14,32). With I > capacity the
// last tile's end is never written (it keeps the 0 of renderer.js:919), and threads at or past the
// capacity would read beyond the keys buffer, which WGSL leaves to the implementation (robust buffer
// access); they are not restated, only counted (the return value).
uint32_t tile_ranges_as_bound(const uint32_t* keys, uint32_t capacity, uint32_t sorted, uint32_t instanceCount,
                              uint32_t* ranges) {
    const uint64_t threads = ((uint64_t)sorted + 255u) / 256u * 256u;
    uint32_t beyond = 0;
    for (uint64_t g = 0; g < threads; ++g) {
        const uint32_t gindex = (uint32_t)g;
        if (gindex >= instanceCount) continue;
        if (gindex >= capacity) {
            ++beyond;
            continue;
        }
        const uint32_t tileIndex = keys[gindex] >> 16u;
        if (gindex == 0u) {
            ranges[tileIndex * 2] = 0u;
        } else {
            const uint32_t prev = keys[gindex - 1] >> 16u;
            if (tileIndex > prev) {
                ranges[prev * 2 + 1] = gindex;
                ranges[tileIndex * 2] = gindex;
            }
        }
        if (gindex == instanceCount - 1u) ranges[tileIndex * 2 + 1] = instanceCount;
    }
    return beyond;
}

// raseter.wgsl:35-117. One pixel walks its tile's range front to back. The reference's batches of
// 256 and its all-done vote only skip work for pixels that are already done, so a per-pixel walk
// gives the same result.
template <class T>
void raster(const Uniforms& u, uint32_t tile, const uint32_t* ranges, const uint32_t* vals, const Pre<T>& pre,
            T* rgb, T* final_t, uint32_t* n_contrib, uint8_t* rgba8, int threads, uint32_t row_stride = 1) {
    const uint32_t W = (uint32_t)u.textureSize[0], H = (uint32_t)u.textureSize[1];
    const uint32_t tilesPerRow = (W + tile - 1u) / tile;
    const uint32_t tilesPerCol = (H + tile - 1u) / tile;
    const int64_t ntiles = (int64_t)tilesPerRow * tilesPerCol;
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (int64_t t = 0; t < ntiles; ++t) {
        const uint32_t tileX = (uint32_t)(t % tilesPerRow), tileY = (uint32_t)(t / tilesPerRow);
        if (tileY % row_stride != 0u) continue;  // timing samples render every row_stride-th tile row
        const uint32_t start = ranges[t * 2], end = ranges[t * 2 + 1];
        for (uint32_t ly = 0; ly < tile; ++ly)
            for (uint32_t lx = 0; lx < tile; ++lx) {
                const uint32_t x = tileX * tile + lx, y = tileY * tile + ly;
                if (x >= W || y >= H) continue;
                const T fpx = (T)(float)x, fpy = (T)(float)y;
                T Tr = (T)1;
                T c[3] = {(T)0, (T)0, (T)0};
                uint32_t contributor = 0, last = 0;
                for (uint32_t i = start; i < end; ++i) {
                    ++contributor;
                    const uint32_t g = vals[i];
                    const T a = pre.conic_opacity[4 * (size_t)g], b = pre.conic_opacity[4 * (size_t)g + 1],
                            cc = pre.conic_opacity[4 * (size_t)g + 2], o = pre.conic_opacity[4 * (size_t)g + 3];
                    const T dx = pre.pixel[2 * (size_t)g] - fpx;
                    const T dy = pre.pixel[2 * (size_t)g + 1] - fpy;
                    // calculatePower raseter.wgsl:112-116, contracted as pinned (rule 5)
                    const T q = Num<T>::fma(a * dx, dx, (cc * dy) * dy);
                    const T power = Num<T>::fma((T)-0.5f, q, -((b * dx) * dy));
                    if (power > (T)0) continue;
                    const T alpha = tmin((T)kAlphaClamp, o * Num<T>::ex_raster(power));
                    if (alpha < (T)kEpsilon) continue;
                    const T testT = Tr * ((T)1 - alpha);
                    if (testT < (T)kBlendThreshold) break;  // done = true; the loop ends
                    for (int k = 0; k < 3; ++k)
                        c[k] = Num<T>::fma(pre.color[4 * (size_t)g + k] * alpha, Tr, c[k]);
                    Tr = testT;
                    last = contributor;
                }
                const size_t p = (size_t)y * W + x;
                if (rgb) {
                    rgb[3 * p] = c[0];
                    rgb[3 * p + 1] = c[1];
                    rgb[3 * p + 2] = c[2];
                }
                if (final_t) final_t[p] = Tr;
                if (n_contrib) n_contrib[p] = last;
                if (rgba8) {
                    for (int k = 0; k < 3; ++k) {
                        const float v = std::fmin(std::fmax((float)c[k], 0.0f), 1.0f);
                        rgba8[4 * p + k] = (uint8_t)(uint32_t)(v * 255.0f + 0.5f);
                    }
                    rgba8[4 * p + 3] = 255u;
                }
            }
    }
}

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// renderer.js:822-932 for one frame: clear offsets, preprocess, offset scan, emit, indirect arg,
// 4 radix passes, clear + tile ranges, raster.
template <class T>
int forward(const void* uniforms, const float* packed, uint32_t n, uint32_t tile, uint32_t factor,
            oracle_fwd_out* out, T* rgb, T* final_t, uint32_t* instance_count_out, int threads,
            double* pass_ms, uint32_t row_stride = 1) {
    if (!uniforms || (!packed && n) || tile == 0u || factor == 0u) return 1;
    Uniforms u;
    std::memcpy(&u, uniforms, sizeof(u));
    if (threads <= 0) threads = 1;
    const uint32_t W = (uint32_t)u.textureSize[0], H = (uint32_t)u.textureSize[1];
    const uint32_t tilesPerRow = (W + tile - 1u) / tile, tilesPerCol = (H + tile - 1u) / tile;
    const uint64_t T_ = (uint64_t)tilesPerRow * tilesPerCol;
    const uint64_t maxInstance64 = (uint64_t)n * factor;
    if (maxInstance64 > 0xFFFFFFFFull) return 1;
    const uint32_t maxInstance = (uint32_t)maxInstance64;

    auto t0 = std::chrono::steady_clock::now();
    Pre<T> pre;
    preprocess<T>(u, packed, n, tile, pre, threads);
    if (pass_ms) pass_ms[0] = ms_since(t0);

    t0 = std::chrono::steady_clock::now();
    std::vector<uint32_t> offsets((size_t)n + 1, 0u);
    std::copy(pre.tiles_touched.begin(), pre.tiles_touched.end(), offsets.begin());
    const uint32_t instanceCount = exclusive_scan(offsets.data(), offsets.size());
    if (pass_ms) pass_ms[1] = ms_since(t0);

    t0 = std::chrono::steady_clock::now();
    const uint32_t sorted = std::min(instanceCount, maxInstance);  // indirect_arg.wgsl:16
    std::vector<uint32_t> keys(sorted), vals(sorted), k2(sorted), v2(sorted);
    emit(offsets.data(), pre.meta.data(), n, tilesPerRow, maxInstance, keys.data(), vals.data(), threads);
    if (pass_ms) pass_ms[2] = ms_since(t0);

    t0 = std::chrono::steady_clock::now();
    for (uint32_t pass = 0; pass < 4; ++pass) {  // renderer.js:874-917, ping-pong by parity
        radix_pass(keys.data(), vals.data(), k2.data(), v2.data(), sorted, pass * 8u);
        keys.swap(k2);
        vals.swap(v2);
    }
    if (pass_ms) pass_ms[3] = ms_since(t0);

    t0 = std::chrono::steady_clock::now();
    std::vector<uint32_t> ranges(2 * T_, 0u);
    tile_ranges(keys.data(), sorted, ranges.data());
    if (pass_ms) pass_ms[4] = ms_since(t0);

    t0 = std::chrono::steady_clock::now();
    raster<T>(u, tile, ranges.data(), vals.data(), pre, rgb, final_t, out ? out->n_contrib : nullptr,
              out ? out->rgba8 : nullptr, threads, row_stride == 0 ? 1u : row_stride);
    if (pass_ms) pass_ms[5] = ms_since(t0);

    if (instance_count_out) *instance_count_out = instanceCount;
    if (out) {
        if (out->tiles_touched) std::copy(pre.tiles_touched.begin(), pre.tiles_touched.end(), out->tiles_touched);
        if (out->meta) std::copy(pre.meta.begin(), pre.meta.end(), out->meta);
        if constexpr (sizeof(T) == sizeof(float)) {
            if (out->conic_opacity) std::copy(pre.conic_opacity.begin(), pre.conic_opacity.end(), out->conic_opacity);
            if (out->pixel) std::copy(pre.pixel.begin(), pre.pixel.end(), out->pixel);
            if (out->color) std::copy(pre.color.begin(), pre.color.end(), out->color);
        }
        if (out->offsets) std::copy(offsets.begin(), offsets.end(), out->offsets);
        const uint64_t kc = std::min<uint64_t>(sorted, out->keys_capacity);
        if (out->keys) std::copy(keys.begin(), keys.begin() + kc, out->keys);
        if (out->vals) std::copy(vals.begin(), vals.begin() + kc, out->vals);
        if (out->ranges) std::copy(ranges.begin(), ranges.end(), out->ranges);
        out->instance_count = instanceCount;
        out->sorted_count = sorted;
        out->max_instance = maxInstance;
        out->tiles_x = tilesPerRow;
        out->tiles_y = tilesPerCol;
    }
    return 0;
}

}  // namespace

extern "C" {

float oracle_expf(float x) { return pinned_expf(x); }

void oracle_raster_expf_array(const float* x, float* y, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) y[i] = raster_expf(x[i]);
}

void oracle_expf_array(const float* x, float* y, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) y[i] = pinned_expf(x[i]);
}

int oracle_forward_f32(const void* uniforms, const float* packed, uint32_t n, uint32_t tile,
                       uint32_t max_instance_factor, oracle_fwd_out* out, int threads) {
    return forward<float>(uniforms, packed, n, tile, max_instance_factor, out, out ? out->rgb : nullptr,
                          out ? out->final_t : nullptr, nullptr, threads, nullptr);
}

int oracle_forward_f32_timed(const void* uniforms, const float* packed, uint32_t n, uint32_t tile,
                             uint32_t max_instance_factor, oracle_fwd_out* out, int threads, double* pass_ms,
                             uint32_t row_stride) {
    return forward<float>(uniforms, packed, n, tile, max_instance_factor, out, out ? out->rgb : nullptr,
                          out ? out->final_t : nullptr, nullptr, threads, pass_ms, row_stride);
}

int oracle_forward_f64(const void* uniforms, const float* packed, uint32_t n, uint32_t tile,
                       uint32_t max_instance_factor, double* rgb, double* final_t, uint32_t* instance_count,
                       int threads) {
    return forward<double>(uniforms, packed, n, tile, max_instance_factor, nullptr, rgb, final_t, instance_count,
                           threads, nullptr);
}

void oracle_radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, uint32_t passes) {
    std::vector<uint32_t> k2(n), v2(n);
    for (uint32_t p = 0; p < passes; ++p) {
        radix_pass(keys, vals, k2.data(), v2.data(), n, 8u * p);
        std::memcpy(keys, k2.data(), (size_t)n * 4);
        std::memcpy(vals, v2.data(), (size_t)n * 4);
    }
}

uint32_t oracle_exclusive_scan(uint32_t* data, uint32_t n) { return exclusive_scan(data, n); }

uint32_t oracle_tile_ranges_reference(const uint32_t* keys, uint32_t capacity, uint32_t sorted,
                                      uint32_t instance_count, uint32_t* ranges) {
    return tile_ranges_as_bound(keys, capacity, sorted, instance_count, ranges);
}

}  // extern "C"

// =====================================================================================================
// Backward (no counterpart in the reference, which is forward-only): the FP64 adjoint of the pipeline
// above, used to check the CUDA backward, plus the L1 + SSIM loss of the differentiation workload.
// Conventions, stated once:
//   * gradients flow through the fp32-before-quantization RGB; rgba8 has none;
//   * culled Gaussians (near plane, frustum), skipped pairs (power > 0, alpha < 1/255) and splats after
//     a pixel's termination get zero gradient; the 0.99 alpha clamp and the max(colour, 0) clamp have
//     zero derivative where active;
//   * the frustum-guard clamp of t.xy (preprocess.wgsl:254-255) is masked as in 3DGS: where t.x/t.z
//     (t.y/t.z) is clamped, no gradient flows through t.x (t.y); t.z keeps its path through J;
//   * tile rects, depth16 and sort order are piecewise constant: no gradient.
// =====================================================================================================
namespace {

template <class T> struct Mat3T { T m[3][3]; };  // [row][col] (plain math layout, unlike Mat3)

// Per-Gaussian forward quantities of preprocess.wgsl:58-144, recomputed for the backward.
template <class T> struct GaussState {
    bool near_ok = false;
    T p[3], pv[4], clip[4], wden;
    T s[3], q[4], qlen, qraw[4];  // q = normalized (x, y, z, w)
    T R[3][3];                    // [row][col]
    T Sigma[3][3];
    T tx, ty, tz;
    bool clampx, clampy;
    T J[2][3];
    T Wr[3][3];                   // upper-left 3x3 of the view matrix, [row][col]
    T M[2][3];                    // J * Wr
    T a, b, c, det;
    T opacity;
    T v[3], vlen, dir[3];
    T Y[16];
    T raw[3];                     // SH sum + 0.5 before max(., 0)
};

template <class T> T sh_basis(const T d[3], T Y[16]) {
    const T x = d[0], y = d[1], z = d[2];
    const T xx = x * x, yy = y * y, zz = z * z;
    Y[0] = (T)kShC0;
    Y[1] = -(T)kShC1 * y;
    Y[2] = (T)kShC1 * z;
    Y[3] = -(T)kShC1 * x;
    Y[4] = (T)kShC2_0 * x * y;
    Y[5] = (T)kShC2_1 * y * z;
    Y[6] = (T)kShC2_2 * (2 * zz - xx - yy);
    Y[7] = (T)kShC2_3 * x * z;
    Y[8] = (T)kShC2_4 * (xx - yy);
    Y[9] = (T)kShC3_0 * y * (3 * xx - yy);
    Y[10] = (T)kShC3_1 * x * y * z;
    Y[11] = (T)kShC3_2 * y * (4 * zz - xx - yy);
    Y[12] = (T)kShC3_3 * z * (2 * zz - 3 * xx - 3 * yy);
    Y[13] = (T)kShC3_4 * x * (4 * zz - xx - yy);
    Y[14] = (T)kShC3_5 * z * (xx - yy);
    Y[15] = (T)kShC3_6 * x * (xx - 3 * yy);
    return Y[0];
}

// d(sum_k Y_k w_k)/d(x, y, z) for weights w_k.
template <class T> void sh_basis_grad(const T d[3], const T w[16], T out[3]) {
    const T x = d[0], y = d[1], z = d[2];
    const T xx = x * x, yy = y * y, zz = z * z;
    T gx = 0, gy = 0, gz = 0;
    gy += -(T)kShC1 * w[1];
    gz += (T)kShC1 * w[2];
    gx += -(T)kShC1 * w[3];
    gx += (T)kShC2_0 * y * w[4];          gy += (T)kShC2_0 * x * w[4];
    gy += (T)kShC2_1 * z * w[5];          gz += (T)kShC2_1 * y * w[5];
    gx += -2 * (T)kShC2_2 * x * w[6];     gy += -2 * (T)kShC2_2 * y * w[6];     gz += 4 * (T)kShC2_2 * z * w[6];
    gx += (T)kShC2_3 * z * w[7];          gz += (T)kShC2_3 * x * w[7];
    gx += 2 * (T)kShC2_4 * x * w[8];      gy += -2 * (T)kShC2_4 * y * w[8];
    gx += 6 * (T)kShC3_0 * x * y * w[9];  gy += (T)kShC3_0 * (3 * xx - 3 * yy) * w[9];
    gx += (T)kShC3_1 * y * z * w[10];     gy += (T)kShC3_1 * x * z * w[10];     gz += (T)kShC3_1 * x * y * w[10];
    gx += -2 * (T)kShC3_2 * x * y * w[11]; gy += (T)kShC3_2 * (4 * zz - xx - 3 * yy) * w[11]; gz += 8 * (T)kShC3_2 * y * z * w[11];
    gx += -6 * (T)kShC3_3 * x * z * w[12]; gy += -6 * (T)kShC3_3 * y * z * w[12]; gz += (T)kShC3_3 * (6 * zz - 3 * xx - 3 * yy) * w[12];
    gx += (T)kShC3_4 * (4 * zz - 3 * xx - yy) * w[13]; gy += -2 * (T)kShC3_4 * x * y * w[13]; gz += 8 * (T)kShC3_4 * x * z * w[13];
    gx += 2 * (T)kShC3_5 * x * z * w[14]; gy += -2 * (T)kShC3_5 * y * z * w[14]; gz += (T)kShC3_5 * (xx - yy) * w[14];
    gx += (T)kShC3_6 * (3 * xx - 3 * yy) * w[15]; gy += -6 * (T)kShC3_6 * x * y * w[15];
    out[0] = gx; out[1] = gy; out[2] = gz;
}

template <class T>
GaussState<T> gauss_forward(const Uniforms& u, const float* params, uint64_t n, uint64_t g) {
    GaussState<T> st;
    const float* P = params;
    for (int i = 0; i < 3; ++i) st.p[i] = P[g * 3 + i];
    for (int i = 0; i < 4; ++i) {
        st.pv[i] = (T)u.view[0 * 4 + i] * st.p[0] + (T)u.view[1 * 4 + i] * st.p[1] + (T)u.view[2 * 4 + i] * st.p[2] +
                   (T)u.view[3 * 4 + i];
        st.clip[i] = (T)u.viewProj[0 * 4 + i] * st.p[0] + (T)u.viewProj[1 * 4 + i] * st.p[1] +
                     (T)u.viewProj[2 * 4 + i] * st.p[2] + (T)u.viewProj[3 * 4 + i];
    }
    st.near_ok = !(st.pv[2] >= -(T)kZNearView);
    if (!st.near_ok) return st;
    st.wden = st.clip[3] + (T)kSmallValue;
    const float* sc = P + 3 * n + g * 3;
    const float* qs = P + 6 * n + g * 4;
    for (int i = 0; i < 3; ++i) st.s[i] = std::exp((T)sc[i]);
    st.qraw[0] = qs[1]; st.qraw[1] = qs[2]; st.qraw[2] = qs[3]; st.qraw[3] = qs[0];
    st.qlen = std::sqrt(st.qraw[0] * st.qraw[0] + st.qraw[1] * st.qraw[1] + st.qraw[2] * st.qraw[2] + st.qraw[3] * st.qraw[3]);
    for (int i = 0; i < 4; ++i) st.q[i] = st.qraw[i] / st.qlen;
    const T x = st.q[0], y = st.q[1], z = st.q[2], w = st.q[3];
    st.R[0][0] = 1 - 2 * (y * y + z * z); st.R[0][1] = 2 * (x * y - w * z);     st.R[0][2] = 2 * (x * z + w * y);
    st.R[1][0] = 2 * (x * y + w * z);     st.R[1][1] = 1 - 2 * (x * x + z * z); st.R[1][2] = 2 * (y * z - w * x);
    st.R[2][0] = 2 * (x * z - w * y);     st.R[2][1] = 2 * (y * z + w * x);     st.R[2][2] = 1 - 2 * (x * x + y * y);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            T acc = 0;
            for (int k = 0; k < 3; ++k) acc += st.R[i][k] * st.s[k] * st.s[k] * st.R[j][k];
            st.Sigma[i][j] = acc;
        }
    const T limx = (T)kFrustumExtended * (T)u.tanFov[0], limy = (T)kFrustumExtended * (T)u.tanFov[1];
    st.tz = st.pv[2];
    const T rx = st.pv[0] / st.tz, ry = st.pv[1] / st.tz;
    st.clampx = rx < -limx || rx > limx;
    st.clampy = ry < -limy || ry > limy;
    st.tx = tmin(limx, tmax(-limx, rx)) * st.tz;
    st.ty = tmin(limy, tmax(-limy, ry)) * st.tz;
    const T fx = (T)u.focal[0], fy = (T)u.focal[1];
    st.J[0][0] = fx / st.tz; st.J[0][1] = 0; st.J[0][2] = -fx * st.tx / (st.tz * st.tz);
    st.J[1][0] = 0; st.J[1][1] = fy / st.tz; st.J[1][2] = -fy * st.ty / (st.tz * st.tz);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) st.Wr[r][c] = (T)u.view[c * 4 + r];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 3; ++c) {
            T acc = 0;
            for (int k = 0; k < 3; ++k) acc += st.J[r][k] * st.Wr[k][c];
            st.M[r][c] = acc;
        }
    T cov2[2][2];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
            T acc = 0;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) acc += st.M[r][i] * st.Sigma[i][j] * st.M[c][j];
            cov2[r][c] = acc;
        }
    st.a = cov2[0][0] + (T)0.3f;
    st.b = cov2[0][1];
    st.c = cov2[1][1] + (T)0.3f;
    st.det = st.a * st.c - st.b * st.b;
    st.opacity = (T)1 / ((T)1 + std::exp(-(T)P[13 * n + g]));
    for (int i = 0; i < 3; ++i) st.v[i] = st.p[i] - (T)u.cameraPos[i];
    st.vlen = std::sqrt(st.v[0] * st.v[0] + st.v[1] * st.v[1] + st.v[2] * st.v[2]);
    for (int i = 0; i < 3; ++i) st.dir[i] = st.v[i] / st.vlen;
    sh_basis<T>(st.dir, st.Y);
    for (int ch = 0; ch < 3; ++ch) {
        T r = st.Y[0] * (T)P[10 * n + g * 3 + ch];
        for (int k = 1; k < 16; ++k) r += st.Y[k] * (T)P[14 * n + g * 45 + (k - 1) + 15 * ch];
        st.raw[ch] = r + (T)0.5f;
    }
    return st;
}

// dL/d(pixel.xy, conic.xyz, opacity, colour.rgb) of one Gaussian -> dL/d(packed attributes).
template <class T>
void gauss_backward(const Uniforms& u, const float* P, uint64_t n, uint64_t g, const T* d2, T* grad) {
    const GaussState<T> st = gauss_forward<T>(u, P, n, g);
    if (!st.near_ok) return;
    T gp[3] = {0, 0, 0};
    // colour (SH): dL/dcoef and dL/ddir
    T gcol[3];
    for (int ch = 0; ch < 3; ++ch) gcol[ch] = st.raw[ch] < 0 ? (T)0 : d2[6 + ch];
    T wsh[16];
    for (int k = 0; k < 16; ++k) {
        T acc = 0;
        for (int ch = 0; ch < 3; ++ch) {
            const T coef = k == 0 ? (T)P[10 * n + g * 3 + ch] : (T)P[14 * n + g * 45 + (k - 1) + 15 * ch];
            acc += coef * gcol[ch];
            const T gk = st.Y[k] * gcol[ch];
            if (k == 0) grad[10 * n + g * 3 + ch] += gk;
            else grad[14 * n + g * 45 + (k - 1) + 15 * ch] += gk;
        }
        wsh[k] = acc;
    }
    T gdir[3];
    sh_basis_grad<T>(st.dir, wsh, gdir);
    const T dd = gdir[0] * st.dir[0] + gdir[1] * st.dir[1] + gdir[2] * st.dir[2];
    for (int i = 0; i < 3; ++i) gp[i] += (gdir[i] - st.dir[i] * dd) / st.vlen;
    // opacity
    grad[13 * n + g] += d2[5] * st.opacity * ((T)1 - st.opacity);
    // conic -> cov2' (a, b, c)
    const T gA = d2[2], gB = d2[3], gC = d2[4];
    const T det2 = st.det * st.det;
    const T ga = gA * (-st.c * st.c / det2) + gB * (st.b * st.c / det2) + gC * (-st.b * st.b / det2);
    const T gb = gA * (2 * st.b * st.c / det2) + gB * (-(st.a * st.c + st.b * st.b) / det2) + gC * (2 * st.a * st.b / det2);
    const T gc = gA * (-st.b * st.b / det2) + gB * (st.b * st.a / det2) + gC * (-st.a * st.a / det2);
    const T G2[2][2] = {{ga, gb / 2}, {gb / 2, gc}};
    // cov2 = M Sigma M^T: dL/dSigma = M^T G2 M, dL/dM = 2 G2 M Sigma
    T gSigma[3][3], gM[2][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            T acc = 0;
            for (int r = 0; r < 2; ++r)
                for (int c = 0; c < 2; ++c) acc += st.M[r][i] * G2[r][c] * st.M[c][j];
            gSigma[i][j] = acc;
        }
    for (int r = 0; r < 2; ++r)
        for (int j = 0; j < 3; ++j) {
            T acc = 0;
            for (int c = 0; c < 2; ++c)
                for (int k = 0; k < 3; ++k) acc += G2[r][c] * st.M[c][k] * st.Sigma[k][j];
            gM[r][j] = 2 * acc;
        }
    // M = J Wr: dL/dJ = dL/dM Wr^T
    T gJ[2][3];
    for (int r = 0; r < 2; ++r)
        for (int k = 0; k < 3; ++k) {
            T acc = 0;
            for (int c = 0; c < 3; ++c) acc += gM[r][c] * st.Wr[k][c];
            gJ[r][k] = acc;
        }
    const T fx = (T)u.focal[0], fy = (T)u.focal[1], tz = st.tz, tz2 = tz * tz, tz3 = tz2 * tz;
    T gpv[3];
    gpv[0] = st.clampx ? (T)0 : gJ[0][2] * (-fx / tz2);
    gpv[1] = st.clampy ? (T)0 : gJ[1][2] * (-fy / tz2);
    gpv[2] = gJ[0][0] * (-fx / tz2) + gJ[0][2] * (2 * fx * st.tx / tz3) + gJ[1][1] * (-fy / tz2) +
             gJ[1][2] * (2 * fy * st.ty / tz3);
    for (int i = 0; i < 3; ++i) gp[i] += st.Wr[0][i] * gpv[0] + st.Wr[1][i] * gpv[1] + st.Wr[2][i] * gpv[2];
    // pixel position -> ndc -> clip -> p
    const T gndx = d2[0] * (T)u.textureSize[0] * (T)0.5, gndy = d2[1] * (T)u.textureSize[1] * (T)0.5;
    const T gcx = gndx / st.wden, gcy = gndy / st.wden;
    const T gcw = -(gndx * st.clip[0] + gndy * st.clip[1]) / (st.wden * st.wden);
    for (int i = 0; i < 3; ++i)
        gp[i] += (T)u.viewProj[i * 4 + 0] * gcx + (T)u.viewProj[i * 4 + 1] * gcy + (T)u.viewProj[i * 4 + 3] * gcw;
    for (int i = 0; i < 3; ++i) grad[g * 3 + i] += gp[i];
    // Sigma = A A^T, A = R diag(s)
    T A[3][3], gAm[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = st.R[i][j] * st.s[j];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            T acc = 0;
            for (int k = 0; k < 3; ++k) acc += (gSigma[i][k] + gSigma[k][i]) * A[k][j];
            gAm[i][j] = acc;
        }
    T gR[3][3];
    for (int j = 0; j < 3; ++j) {
        T gs = 0;
        for (int i = 0; i < 3; ++i) {
            gs += gAm[i][j] * st.R[i][j];
            gR[i][j] = gAm[i][j] * st.s[j];
        }
        grad[3 * n + g * 3 + j] += gs * st.s[j];  // d s / d logscale = s
    }
    const T x = st.q[0], y = st.q[1], z = st.q[2], w = st.q[3];
    T gq[4];
    gq[0] = gR[1][0] * 2 * y + gR[2][0] * 2 * z + gR[0][1] * 2 * y + gR[1][1] * -4 * x + gR[2][1] * 2 * w +
            gR[0][2] * 2 * z + gR[1][2] * -2 * w + gR[2][2] * -4 * x;
    gq[1] = gR[0][0] * -4 * y + gR[1][0] * 2 * x + gR[2][0] * -2 * w + gR[0][1] * 2 * x + gR[2][1] * 2 * z +
            gR[0][2] * 2 * w + gR[1][2] * 2 * z + gR[2][2] * -4 * y;
    gq[2] = gR[0][0] * -4 * z + gR[1][0] * 2 * w + gR[2][0] * 2 * x + gR[0][1] * -2 * w + gR[1][1] * -4 * z +
            gR[2][1] * 2 * y + gR[0][2] * 2 * x + gR[1][2] * 2 * y;
    gq[3] = gR[1][0] * 2 * z + gR[2][0] * -2 * y + gR[0][1] * -2 * z + gR[2][1] * 2 * x + gR[0][2] * 2 * y +
            gR[1][2] * -2 * x;
    const T qd = gq[0] * st.q[0] + gq[1] * st.q[1] + gq[2] * st.q[2] + gq[3] * st.q[3];
    T gqr[4];
    for (int i = 0; i < 4; ++i) gqr[i] = (gq[i] - st.q[i] * qd) / st.qlen;
    // stored (rot_0..3) = (w, x, y, z)
    grad[6 * n + g * 4 + 0] += gqr[3];
    grad[6 * n + g * 4 + 1] += gqr[0];
    grad[6 * n + g * 4 + 2] += gqr[1];
    grad[6 * n + g * 4 + 3] += gqr[2];
}

// FP64 frame with the state the adjoint needs: per-Gaussian records and the sorted binning.
template <class T>
void backward_frame(const Uniforms& u, const float* packed, uint32_t n, uint32_t tile, uint32_t factor,
                    const T* dl_drgb, T* grad, T* rgb_out, int threads) {
    Pre<T> pre;
    preprocess<T>(u, packed, n, tile, pre, threads);
    std::vector<uint32_t> offsets((size_t)n + 1, 0u);
    std::copy(pre.tiles_touched.begin(), pre.tiles_touched.end(), offsets.begin());
    const uint32_t I = exclusive_scan(offsets.data(), offsets.size());
    const uint32_t W = (uint32_t)u.textureSize[0], H = (uint32_t)u.textureSize[1];
    const uint32_t tpr = (W + tile - 1) / tile, tpc = (H + tile - 1) / tile;
    const uint32_t maxI = n * factor, S = std::min(I, maxI);
    std::vector<uint32_t> keys(S), vals(S), k2(S), v2(S);
    emit(offsets.data(), pre.meta.data(), n, tpr, maxI, keys.data(), vals.data(), threads);
    for (uint32_t p = 0; p < 4; ++p) {
        radix_pass(keys.data(), vals.data(), k2.data(), v2.data(), S, 8 * p);
        keys.swap(k2);
        vals.swap(v2);
    }
    std::vector<uint32_t> ranges((size_t)tpr * tpc * 2, 0u);
    tile_ranges(keys.data(), S, ranges.data());
    std::vector<T> inst(9 * (size_t)S, (T)0);  // per-instance 2D gradients (each instance is in one tile)
    const int64_t ntiles = (int64_t)tpr * tpc;
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (int64_t t = 0; t < ntiles; ++t) {
        const uint32_t start = ranges[t * 2], end = ranges[t * 2 + 1];
        const uint32_t tX = (uint32_t)(t % tpr), tY = (uint32_t)(t / tpr);
        std::vector<uint32_t> list;
        std::vector<T> alist, glist, tlist;
        for (uint32_t ly = 0; ly < tile; ++ly)
            for (uint32_t lx = 0; lx < tile; ++lx) {
                const uint32_t x = tX * tile + lx, y = tY * tile + ly;
                if (x >= W || y >= H) continue;
                const T fpx = (T)(float)x, fpy = (T)(float)y;
                list.clear(); alist.clear(); glist.clear(); tlist.clear();
                T Tr = 1, c[3] = {0, 0, 0};
                for (uint32_t i = start; i < end; ++i) {
                    const uint32_t g = vals[i];
                    const T A = pre.conic_opacity[4 * (size_t)g], B = pre.conic_opacity[4 * (size_t)g + 1],
                            C = pre.conic_opacity[4 * (size_t)g + 2], o = pre.conic_opacity[4 * (size_t)g + 3];
                    const T dx = pre.pixel[2 * (size_t)g] - fpx, dy = pre.pixel[2 * (size_t)g + 1] - fpy;
                    const T power = std::fma((T)-0.5, std::fma(A * dx, dx, (C * dy) * dy), -((B * dx) * dy));
                    if (power > 0) continue;
                    const T G = std::exp(power);
                    const T alpha = tmin((T)kAlphaClamp, o * G);
                    if (alpha < (T)kEpsilon) continue;
                    const T testT = Tr * (1 - alpha);
                    if (testT < (T)kBlendThreshold) break;
                    for (int k = 0; k < 3; ++k) c[k] += pre.color[4 * (size_t)g + k] * alpha * Tr;
                    list.push_back(i); alist.push_back(alpha); glist.push_back(G); tlist.push_back(Tr);
                    Tr = testT;
                }
                const size_t pidx = (size_t)y * W + x;
                if (rgb_out)
                    for (int k = 0; k < 3; ++k) rgb_out[3 * pidx + k] = c[k];
                const T* dl = dl_drgb + 3 * pidx;
                T acc[3] = {0, 0, 0}, lastA = 0, lastC[3] = {0, 0, 0};
                for (size_t k = list.size(); k-- > 0;) {
                    const uint32_t i = list[k];
                    const uint32_t g = vals[i];
                    const T alpha = alist[k], G = glist[k], Tk = tlist[k];
                    const T* col = &pre.color[4 * (size_t)g];
                    for (int ch = 0; ch < 3; ++ch) acc[ch] = lastA * lastC[ch] + (1 - lastA) * acc[ch];
                    T dalpha = 0;
                    for (int ch = 0; ch < 3; ++ch) dalpha += (col[ch] - acc[ch]) * dl[ch];
                    dalpha *= Tk;
                    T* ig = &inst[9 * (size_t)i];
                    for (int ch = 0; ch < 3; ++ch) ig[6 + ch] += alpha * Tk * dl[ch];
                    const T o = pre.conic_opacity[4 * (size_t)g + 3];
                    if (o * G <= (T)kAlphaClamp) {  // unclamped alpha = o * G
                        const T A = pre.conic_opacity[4 * (size_t)g], B = pre.conic_opacity[4 * (size_t)g + 1],
                                C = pre.conic_opacity[4 * (size_t)g + 2];
                        const T dx = pre.pixel[2 * (size_t)g] - fpx, dy = pre.pixel[2 * (size_t)g + 1] - fpy;
                        const T gpow = dalpha * o * G;
                        ig[0] += gpow * (-A * dx - B * dy);
                        ig[1] += gpow * (-C * dy - B * dx);
                        ig[2] += gpow * (T)-0.5 * dx * dx;
                        ig[3] += gpow * -dx * dy;
                        ig[4] += gpow * (T)-0.5 * dy * dy;
                        ig[5] += dalpha * G;
                    }
                    lastA = alpha;
                    for (int ch = 0; ch < 3; ++ch) lastC[ch] = col[ch];
                }
            }
    }
    std::vector<T> d2((size_t)n * 9, (T)0);
    for (uint32_t i = 0; i < S; ++i)
        for (int k = 0; k < 9; ++k) d2[9 * (size_t)vals[i] + k] += inst[9 * (size_t)i + k];
    std::fill(grad, grad + (size_t)n * 59, (T)0);
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t gi = 0; gi < (int64_t)n; ++gi) {
        if (pre.tiles_touched[gi] == 0) continue;
        gauss_backward<T>(u, packed, n, (uint64_t)gi, &d2[9 * (size_t)gi], grad);
    }
}

// L = mean|x - y| + lambda * (1 - mean SSIM), SSIM per channel with an 11x11 Gaussian window
// (sigma 1.5, normalised), zero padding, C1 = 0.01^2, C2 = 0.03^2. Images are H x W x 3.
struct SsimWindow {
    double w[11];
    SsimWindow() {
        double s = 0;
        for (int i = 0; i < 11; ++i) { w[i] = std::exp(-(double)((i - 5) * (i - 5)) / (2.0 * 1.5 * 1.5)); s += w[i]; }
        for (double& v : w) v /= s;
    }
};
// separable correlation with zero padding, one channel plane (H x W)
// Rows (then columns) are independent, so the loops run on all host cores; every output element is
// the same sum in the same order as on one core.
void blur(const std::vector<double>& in, std::vector<double>& out, uint32_t W, uint32_t H, const SsimWindow& k) {
    std::vector<double> tmp((size_t)W * H, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t yi = 0; yi < (int64_t)H; ++yi)
        for (uint32_t x = 0, y = (uint32_t)yi; x < W; ++x) {
            double s = 0;
            for (int i = -5; i <= 5; ++i) {
                const int xx = (int)x + i;
                if (xx >= 0 && xx < (int)W) s += k.w[i + 5] * in[(size_t)y * W + xx];
            }
            tmp[(size_t)y * W + x] = s;
        }
    out.assign((size_t)W * H, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t yi = 0; yi < (int64_t)H; ++yi)
        for (uint32_t x = 0, y = (uint32_t)yi; x < W; ++x) {
            double s = 0;
            for (int i = -5; i <= 5; ++i) {
                const int yy = (int)y + i;
                if (yy >= 0 && yy < (int)H) s += k.w[i + 5] * tmp[(size_t)yy * W + x];
            }
            out[(size_t)y * W + x] = s;
        }
}

double loss_l1_ssim(const double* X, const double* Yi, uint32_t W, uint32_t H, double lambda, double* grad) {
    const size_t P = (size_t)W * H;
    const double C1 = 0.01 * 0.01, C2 = 0.03 * 0.03;
    const SsimWindow k;
    double l1 = 0, ssim_sum = 0;
    for (size_t i = 0; i < 3 * P; ++i) {
        const double d = X[i] - Yi[i];
        l1 += std::fabs(d);
        if (grad) grad[i] = (d > 0 ? 1.0 : (d < 0 ? -1.0 : 0.0)) / (double)(3 * P);
    }
    l1 /= (double)(3 * P);
    for (int ch = 0; ch < 3; ++ch) {
        std::vector<double> x(P), y(P), xx(P), yy(P), xy(P);
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)P; ++ii) {
            const size_t i = (size_t)ii;
            x[i] = X[3 * i + ch]; y[i] = Yi[3 * i + ch];
            xx[i] = x[i] * x[i]; yy[i] = y[i] * y[i]; xy[i] = x[i] * y[i];
        }
        std::vector<double> mx, my, mxx, myy, mxy;
        blur(x, mx, W, H, k); blur(y, my, W, H, k); blur(xx, mxx, W, H, k); blur(yy, myy, W, H, k); blur(xy, mxy, W, H, k);
        std::vector<double> d1(P), d2(P), d3(P);  // dS/dm1, dS/dm2(=dS/dsxx), dS/dmxy(=dS/dsxy)
        std::vector<double> smap(P);
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)P; ++ii) {
            const size_t i = (size_t)ii;
            const double sxx = mxx[i] - mx[i] * mx[i], syy = myy[i] - my[i] * my[i], sxy = mxy[i] - mx[i] * my[i];
            const double A1 = 2 * mx[i] * my[i] + C1, A2 = 2 * sxy + C2;
            const double B1 = mx[i] * mx[i] + my[i] * my[i] + C1, B2 = sxx + syy + C2;
            const double s = A1 * A2 / (B1 * B2);
            smap[i] = s;
            const double ds_dmx = (2 * my[i] * A2) / (B1 * B2) - s * (2 * mx[i]) / B1;
            const double ds_dsxx = -s / B2;
            const double ds_dsxy = 2 * A1 / (B1 * B2);
            d1[i] = ds_dmx + ds_dsxx * (-2 * mx[i]) + ds_dsxy * (-my[i]);
            d2[i] = ds_dsxx;
            d3[i] = ds_dsxy;
        }
        for (size_t i = 0; i < P; ++i) ssim_sum += smap[i];  // in index order, as on one core
        if (grad) {
            std::vector<double> b1, b2, b3;
            blur(d1, b1, W, H, k); blur(d2, b2, W, H, k); blur(d3, b3, W, H, k);
            const double scale = -lambda / (double)(3 * P);
#pragma omp parallel for schedule(static)
            for (int64_t ii = 0; ii < (int64_t)P; ++ii) {
                const size_t i = (size_t)ii;
                grad[3 * i + ch] += scale * (b1[i] + 2 * x[i] * b2[i] + y[i] * b3[i]);
            }
        }
    }
    return l1 + lambda * (1.0 - ssim_sum / (double)(3 * P));
}

}  // namespace

extern "C" {

int oracle_backward_f64(const void* uniforms, const float* packed, uint32_t n, uint32_t tile, uint32_t factor,
                        const double* dl_drgb, double* grad_packed, double* rgb_out, int threads) {
    if (!uniforms || !dl_drgb || !grad_packed || (!packed && n) || tile == 0 || factor == 0) return 1;
    Uniforms u;
    std::memcpy(&u, uniforms, sizeof(u));
    backward_frame<double>(u, packed, n, tile, factor, dl_drgb, grad_packed, rgb_out, threads <= 0 ? 1 : threads);
    return 0;
}

double oracle_loss_l1_ssim(const double* x, const double* y, uint32_t w, uint32_t h, double lambda, double* dl_dx) {
    return loss_l1_ssim(x, y, w, h, lambda, dl_dx);
}

}  // extern "C"
