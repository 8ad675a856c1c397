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

template <class T> struct Num;
template <> struct Num<float> {
    static float ex(float x) { return pinned_expf(x); }
    static float fma(float a, float b, float c) { return std::fmaf(a, b, c); }
};
template <> struct Num<double> {
    static double ex(double x) { return std::exp(x); }
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

// emit.wgsl:95-133.
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
                    // calculatePower :307-311, contracted as pinned (rule 5)
                    const T q = Num<T>::fma(a * dx, dx, (cc * dy) * dy);
                    const T power = Num<T>::fma((T)-0.5f, q, -((b * dx) * dy));
                    if (power > (T)0) continue;
                    const T alpha = tmin((T)kAlphaClamp, o * Num<T>::ex(power));
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

}  // extern "C"
