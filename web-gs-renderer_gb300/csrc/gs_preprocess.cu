// gs_preprocess.cu -- per-Gaussian preprocess (src/shaders/preprocess.wgsl:58-284) and the scene
// layout conversions.
//
// One thread per Gaussian over the structure-of-arrays scene rows. Each CTA stages its 128-Gaussian
// slice of the 59 rows in shared memory with bulk copies (TMA, two mbarriers), so the whole 30 KB is
// in flight before any arithmetic starts and the kernel streams the scene at HBM rate. The
// arithmetic follows the WGSL source order with no contraction (the file is built with -fmad=false)
// so that every output bit equals the reference restatement.
#include "gs_kernels.h"
#include "gs_raster_common.cuh"

namespace gs {
namespace {

struct M3 { float m[3][3]; };  // column-major, m[col][row] as WGSL mat3x3f

__device__ __forceinline__ M3 mul33(const M3& a, const M3& b) {
    M3 c;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float s = a.m[0][i] * b.m[j][0];
            s = s + a.m[1][i] * b.m[j][1];
            s = s + a.m[2][i] * b.m[j][2];
            c.m[j][i] = s;
        }
    return c;
}
__device__ __forceinline__ M3 tr33(const M3& a) {
    M3 t;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i) t.m[j][i] = a.m[i][j];
    return t;
}

constexpr uint32_t kPreGroup = 128;  // Gaussians (threads) per preprocess CTA

// The CTA's 128-Gaussian slice of all 59 attribute rows is staged in shared memory by bulk copies
// (cp.async.bulk, 59 x 512 bytes issued by one thread), so every CTA has its whole 30 KB in flight
// at once; threads then read their attributes from shared memory. The 14 geometry rows (position,
// log-scale, rotation, f_dc, opacity) complete on one mbarrier and the 45 f_rest rows on another,
// so the projection and covariance work overlaps the arrival of the SH coefficients.

// Bounded wait on a bulk-copy barrier: on expiry the timeout is recorded and the kernel goes on
// with what has arrived.
__device__ __forceinline__ void wait_staged(uint64_t* bar, FrameCtl* ctl) {
    uint32_t spins = 0;
    while (!mbar_try_wait(bar, 0)) {
        if (++spins > kSpinLimit) {
            if (threadIdx.x == 0) atomicOr(&ctl->status, kDevTimeout);
            break;
        }
    }
}
// One Gaussian g of one view (preprocess.wgsl:58-143): writes its raster record, rect/depth16 and
// tile count, or a zero count when it is culled. attr(row) reads a staged attribute; sh_ready() is
// called before the first f_rest read. Returns whether the Gaussian passed the near plane.
template <class AF, class SF>
__device__ __forceinline__ bool preprocess_gaussian(uint32_t g, const ViewBlock& sv, uint32_t tile, AF attr,
                                                    SF sh_ready, float4* __restrict__ rec, uint4* __restrict__ meta,
                                                    uint32_t* __restrict__ counts) {
    const float px = attr(kRowPos + 0);
    const float py = attr(kRowPos + 1);
    const float pz = attr(kRowPos + 2);

    // uniforms.view * vec4f(position, 1.0f)  (:79)
    float pv[4], clip[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float s = sv.view[0 * 4 + i] * px;
        s = s + sv.view[1 * 4 + i] * py;
        s = s + sv.view[2 * 4 + i] * pz;
        s = s + sv.view[3 * 4 + i] * 1.0f;
        pv[i] = s;
    }
    // near culling (:83)
    if (pv[2] >= -kZNearView) {
        counts[g] = 0u;
        return false;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float s = sv.viewProj[0 * 4 + i] * px;
        s = s + sv.viewProj[1 * 4 + i] * py;
        s = s + sv.viewProj[2 * 4 + i] * pz;
        s = s + sv.viewProj[3 * 4 + i] * 1.0f;
        clip[i] = s;
    }
    const float W = sv.textureSize[0], H = sv.textureSize[1];
    const float wden = clip[3] + kSmallValue;
    const float ndcx = clip[0] / wden, ndcy = clip[1] / wden, ndcz = clip[2] / wden;
    const float pixx = ((ndcx + 1.0f) * W - 1.0f) * 0.5f;
    const float pixy = ((ndcy + 1.0f) * H - 1.0f) * 0.5f;

    // 3D covariance (:95-100): R * S * transpose(S) * transpose(R)
    const float sx = pinned_expf(attr(kRowScale + 0));
    const float sy = pinned_expf(attr(kRowScale + 1));
    const float sz = pinned_expf(attr(kRowScale + 2));
    const float q0 = attr(kRowQuat + 0);
    const float q1 = attr(kRowQuat + 1);
    const float q2 = attr(kRowQuat + 2);
    const float q3 = attr(kRowQuat + 3);
    const float qlen = sqrtf(((q1 * q1 + q2 * q2) + q3 * q3) + q0 * q0);
    const float qx = q1 / qlen, qy = q2 / qlen, qz = q3 / qlen, qw = q0 / qlen;
    const float x2 = qx + qx, y2 = qy + qy, z2 = qz + qz;
    const float xx = qx * x2, xy = qx * y2, xz = qx * z2;
    const float yy = qy * y2, yz = qy * z2, zz = qz * z2;
    const float wx = qw * x2, wy = qw * y2, wz = qw * z2;
    M3 R;
    R.m[0][0] = 1.0f - (yy + zz); R.m[0][1] = xy + wz;          R.m[0][2] = xz - wy;
    R.m[1][0] = xy - wz;          R.m[1][1] = 1.0f - (xx + zz); R.m[1][2] = yz + wx;
    R.m[2][0] = xz + wy;          R.m[2][1] = yz - wx;          R.m[2][2] = 1.0f - (xx + yy);
    M3 S;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i) S.m[j][i] = 0.0f;
    S.m[0][0] = sx; S.m[1][1] = sy; S.m[2][2] = sz;
    const M3 cov = mul33(mul33(mul33(R, S), tr33(S)), tr33(R));

    // calculateCovariance2D (:251-269)
    const float limx = kFrustumExtended * sv.tanFov[0];
    const float limy = kFrustumExtended * sv.tanFov[1];
    const float tz = pv[2];
    const float tx = fminf(limx, fmaxf(-limx, pv[0] / tz)) * tz;
    const float ty = fminf(limy, fmaxf(-limy, pv[1] / tz)) * tz;
    const float fx = sv.focal[0], fy = sv.focal[1];
    // J: mat3x2 columns (fx/z, 0), (0, fy/z), (-fx*x/z^2, -fy*y/z^2)
    float J[3][2];
    J[0][0] = fx / tz; J[0][1] = 0.0f;
    J[1][0] = 0.0f;    J[1][1] = fy / tz;
    J[2][0] = (-fx * tx) / (tz * tz);
    J[2][1] = (-fy * ty) / (tz * tz);
    M3 Wm;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) Wm.m[c][r] = sv.view[c * 4 + r];
    const M3 Wt = tr33(Wm);
    float A[3][2], B[3][2];
    // J * W
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            float s = J[0][i] * Wm.m[j][0];
            s = s + J[1][i] * Wm.m[j][1];
            s = s + J[2][i] * Wm.m[j][2];
            A[j][i] = s;
        }
    // * covariance
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            float s = A[0][i] * cov.m[j][0];
            s = s + A[1][i] * cov.m[j][1];
            s = s + A[2][i] * cov.m[j][2];
            B[j][i] = s;
        }
    // * transpose(W)
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            float s = B[0][i] * Wt.m[j][0];
            s = s + B[1][i] * Wt.m[j][1];
            s = s + B[2][i] * Wt.m[j][2];
            A[j][i] = s;
        }
    // * transpose(J)
    float C[2][2];
#pragma unroll
    for (int col = 0; col < 2; ++col)
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            float s = A[0][i] * J[0][col];
            s = s + A[1][i] * J[1][col];
            s = s + A[2][i] * J[2][col];
            C[col][i] = s;
        }
    const float ca = C[0][0] + 0.3f, cb = C[0][1], cc = C[1][1] + 0.3f;

    // det, calculateRadius (:103-104, :271-275)
    const float det = ca * cc - cb * cb;
    const float mid = 0.5f * (ca + cc);
    const float lambda = mid + sqrtf(fmaxf(0.1f, mid * mid - det));
    const float radius = ceilf(3.0f * sqrtf(lambda));

    // conic and sigmoid opacity (:106-112, :203-205)
    const float op_logit = attr(kRowOpacity);
    const float opacity = 1.0f / (1.0f + pinned_expf(-op_logit));
    const float conx = cc / det, cony = -cb / det, conz = ca / det;

    // view direction and degree-3 SH colour (:114-115, :219-249)
    const float dx = px - sv.cameraPos[0], dy = py - sv.cameraPos[1], dz = pz - sv.cameraPos[2];
    const float dlen = sqrtf((dx * dx + dy * dy) + dz * dz);
    const float x = dx / dlen, y = dy / dlen, z = dz / dlen;
    const float sxx = x * x, syy = y * y, szz = z * z;
    const float sxy = x * y, syz = y * z, sxz = x * z;
    float w[16];
    w[1] = kShC1 * y;
    w[2] = kShC1 * z;
    w[3] = kShC1 * x;
    w[4] = kShC2_0 * sxy;
    w[5] = kShC2_1 * syz;
    w[6] = kShC2_2 * ((2.0f * szz - sxx) - syy);
    w[7] = kShC2_3 * sxz;
    w[8] = kShC2_4 * (sxx - syy);
    w[9] = (kShC3_0 * y) * (3.0f * sxx - syy);
    w[10] = (kShC3_1 * sxy) * z;
    w[11] = (kShC3_2 * y) * ((4.0f * szz - sxx) - syy);
    w[12] = (kShC3_3 * z) * ((2.0f * szz - 3.0f * sxx) - 3.0f * syy);
    w[13] = (kShC3_4 * x) * ((4.0f * szz - sxx) - syy);
    w[14] = (kShC3_5 * z) * (sxx - syy);
    w[15] = (kShC3_6 * x) * (sxx - 3.0f * syy);
    sh_ready();  // the f_rest rows may arrive after the geometry rows
    float col[3];
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const int rest = kRowRest + 15 * ch;
        float r = kShC0 * attr(kRowDc + ch);
        r = r - w[1] * attr(rest + 0);
        r = r + w[2] * attr(rest + 1);
        r = r - w[3] * attr(rest + 2);
#pragma unroll
        for (int k = 3; k < 15; ++k) r = r + w[k + 1] * attr(rest + k);
        r = r + 0.5f;
        col[ch] = fmaxf(r, 0.0f);
    }
    // power below which o * exp(power) < 1/255 for certain: ln(eps / o) less a margin far above the
    // combined rounding error of the exp, the product and logf (see raster).
    const float cut = logf(kEpsilon / opacity) - 1.0e-3f;
    rec[(size_t)kRecFloat4 * g + 0] = make_float4(pixx, pixy, conx, cony);
    rec[(size_t)kRecFloat4 * g + 1] = make_float4(conz, opacity, col[0], col[1]);
    rec[(size_t)kRecFloat4 * g + 2] = make_float4(col[2], cut, 0.0f, 0.0f);

    // frustum culling (:117-120)
    if (pixx + radius < 0.0f || pixx - radius > W || pixy + radius < 0.0f || pixy - radius > H) {
        counts[g] = 0u;
        return true;
    }
    // tile AABB, depth16, tilesTouched (:122-143)
    const float bminx = pixx - radius, bminy = pixy - radius;
    const float bmaxx = pixx + radius, bmaxy = pixy + radius;
    const uint32_t tilesPerRow = ((uint32_t)W + tile - 1u) / tile;
    const uint32_t tilesPerColumn = ((uint32_t)H + tile - 1u) / tile;
    const float ft = (float)tile;
    const float hx = (float)(tilesPerRow - 1u), hy = (float)(tilesPerColumn - 1u);
    const uint32_t minTileX = (uint32_t)fminf(fmaxf(floorf(bminx / ft), 0.0f), hx);
    const uint32_t minTileY = (uint32_t)fminf(fmaxf(floorf(bminy / ft), 0.0f), hy);
    const uint32_t maxTileX = (uint32_t)fminf(fmaxf(floorf(bmaxx / ft), 0.0f), hx);
    const uint32_t maxTileY = (uint32_t)fminf(fmaxf(floorf(bmaxy / ft), 0.0f), hy);
    const uint32_t depthU16 = (uint32_t)(fminf(fmaxf(ndcz, 0.0f), 1.0f) * 65535.0f);
    counts[g] = (maxTileX - minTileX + 1u) * (maxTileY - minTileY + 1u);
    meta[g] = make_uint4((minTileY << 16u) | minTileX, (maxTileY << 16u) | maxTileX, depthU16, 0u);
    return true;
}

__global__ void __launch_bounds__(kPreGroup) k_preprocess(const float* __restrict__ rows, uint32_t stride, uint32_t n,
                                                          const ViewBlock* __restrict__ vb, uint32_t tile,
                                                          float4* __restrict__ rec, uint4* __restrict__ meta,
                                                          uint32_t* __restrict__ counts, FrameCtl* ctl) {
    pdl_wait();
    __shared__ __align__(128) float s_rows[kRows][kPreGroup];
    __shared__ __align__(8) uint64_t s_bar[2];  // [0]: geometry rows, [1]: f_rest rows
    __shared__ ViewBlock sv;
    const uint32_t lt = threadIdx.x;
    const uint32_t g0 = blockIdx.x * kPreGroup;
    if (lt == 0) {
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
    }
    if (lt < 44) reinterpret_cast<uint32_t*>(&sv)[lt] = reinterpret_cast<const uint32_t*>(vb)[lt];
    __syncthreads();
    const bool staged = g0 < stride;
    if (lt == 0 && staged) {
        // stride and g0 are multiples of 64: every row slice starts 256-byte aligned and spans a
        // multiple of 256 bytes
        const uint32_t cols = min(kPreGroup, stride - g0);
        mbar_expect_tx(&s_bar[0], kRowRest * cols * 4u);
        for (int r = 0; r < kRowRest; ++r) bulk_g2s(&s_rows[r][0], rows + (size_t)r * stride + g0, cols * 4u, &s_bar[0]);
        mbar_expect_tx(&s_bar[1], (kRows - kRowRest) * cols * 4u);
        for (int r = kRowRest; r < kRows; ++r)
            bulk_g2s(&s_rows[r][0], rows + (size_t)r * stride + g0, cols * 4u, &s_bar[1]);
    }
    if (staged) wait_staged(&s_bar[0], ctl);
    auto attr = [&](int row) { return s_rows[row][lt]; };
    const uint32_t g = g0 + lt;
    if (g == 0) counts[n] = 0u;  // the N+1-th scan entry (cleared by renderer.js:826)
    bool near_ok = false;
    if (g < n)
        near_ok = preprocess_gaussian(g, sv, tile, attr, [&]() { if (staged) wait_staged(&s_bar[1], ctl); }, rec, meta,
                                      counts);
    // every thread waits for the f_rest copies (those that evaluated SH already have): the CTA's
    // shared memory must not be released while a bulk copy still writes into it
    if (staged) wait_staged(&s_bar[1], ctl);
    const int block_near = __syncthreads_count(near_ok);  // survivors of the near plane, for the statistics
    if (lt == 0 && block_near) atomicAdd(&ctl->near_pass, (uint32_t)block_near);
}

// Several views of one scene: the CTA stages its slice of the attribute rows once and preprocesses
// every view from shared memory, so the scene is read once per group of views.
__global__ void __launch_bounds__(kPreGroup) k_preprocess_multi(const float* __restrict__ rows, uint32_t stride,
                                                                uint32_t n, uint32_t tile, MultiViewFrames mv) {
    __shared__ __align__(128) float s_rows[kRows][kPreGroup];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ ViewBlock sv;
    const uint32_t lt = threadIdx.x;
    const uint32_t g0 = blockIdx.x * kPreGroup;
    const uint32_t g = g0 + lt;
    if (lt == 0) mbar_init(&s_bar, 1);
    __syncthreads();
    if (lt == 0) {
        // g0 < stride (g0 < n <= stride, or g0 = 0 for an empty scene, whose stride is 64); stride and g0
        // are multiples of 64: 256-byte aligned slices
        const uint32_t cols = min(kPreGroup, stride - g0);
        mbar_expect_tx(&s_bar, kRows * cols * 4u);
        for (int r = 0; r < kRows; ++r) bulk_g2s(&s_rows[r][0], rows + (size_t)r * stride + g0, cols * 4u, &s_bar);
    }
    {
        uint32_t spins = 0;
        while (!mbar_try_wait(&s_bar, 0)) {
            if (++spins > kSpinLimit) {
                if (lt == 0)
                    for (uint32_t v = 0; v < mv.count; ++v) atomicOr(&mv.ctl[v]->status, kDevTimeout);
                break;
            }
        }
    }
    auto attr = [&](int row) { return s_rows[row][lt]; };
    for (uint32_t v = 0; v < mv.count; ++v) {
        __syncthreads();  // sv is rewritten per view
        if (lt < 44) reinterpret_cast<uint32_t*>(&sv)[lt] = reinterpret_cast<const uint32_t*>(mv.view[v])[lt];
        __syncthreads();
        if (g == 0) mv.counts[v][n] = 0u;
        bool near_ok = false;
        if (g < n) near_ok = preprocess_gaussian(g, sv, tile, attr, []() {}, mv.rec[v], mv.meta[v], mv.counts[v]);
        const int block_near = __syncthreads_count(near_ok);
        if (lt == 0 && block_near) atomicAdd(&mv.ctl[v]->near_pass, (uint32_t)block_near);
    }
}

// Attribute blocks of the packed layout (preprocess.wgsl:16-24): first row, floats per Gaussian, and
// the block's offset in units of n floats.
__device__ __forceinline__ void attr_block(uint32_t b, uint32_t& row0, uint32_t& width, uint32_t& off) {
    switch (b) {
        case 0: row0 = 0; width = 3; off = 0; break;     // positions
        case 1: row0 = 3; width = 3; off = 3; break;     // log-scales
        case 2: row0 = 6; width = 4; off = 6; break;     // rotations
        case 3: row0 = 10; width = 3; off = 10; break;   // f_dc
        case 4: row0 = 13; width = 1; off = 13; break;   // opacity
        default: row0 = 14; width = 45; off = 14; break; // f_rest
    }
}
constexpr uint32_t kTransposeGroup = 128;  // Gaussians per CTA of the layout transpose

// packed -> rows. A CTA moves kTransposeGroup Gaussians of one attribute block: one coalesced read
// of the block's contiguous chunk into shared memory, then one coalesced write per row. Padding
// columns (n <= g < stride) are zeroed.
__global__ void __launch_bounds__(256) k_pack_to_rows(const float* __restrict__ packed, uint32_t n, uint32_t stride,
                                                      float* __restrict__ rows) {
    __shared__ float s[kTransposeGroup * 45];
    uint32_t row0, width, off;
    attr_block(blockIdx.y, row0, width, off);
    const uint32_t g0 = blockIdx.x * kTransposeGroup;
    const uint32_t cnt = g0 < n ? min(kTransposeGroup, n - g0) : 0u;
    const float* src = packed + (uint64_t)off * n + (uint64_t)g0 * width;
    for (uint32_t i = threadIdx.x; i < cnt * width; i += blockDim.x) s[i] = src[i];
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < width * kTransposeGroup; i += blockDim.x) {
        const uint32_t c = i / kTransposeGroup, lg = i % kTransposeGroup, g = g0 + lg;
        if (g < stride) rows[(size_t)(row0 + c) * stride + g] = lg < cnt ? s[lg * width + c] : 0.0f;
    }
}

template <bool RASTER>
__global__ void k_exp(const float* __restrict__ x, float* __restrict__ y, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = RASTER ? raster_expf(x[i]) : pinned_expf(x[i]);
}

__global__ void k_raster_alpha(const float* __restrict__ o, const float* __restrict__ x, float* __restrict__ y,
                               uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = raster_alpha_unclamped(o[i], x[i]);
}

}  // namespace

void launch_preprocess(const float* rows, uint32_t stride, uint32_t n, const ViewBlock* view, uint32_t tile,
                       float4* rec, uint4* meta, uint32_t* counts, FrameCtl* ctl, cudaStream_t s) {
    const uint32_t blocks = (n + kPreGroup - 1u) / kPreGroup;
    launch_pdl(k_preprocess, dim3(blocks > 0 ? blocks : 1u), dim3(kPreGroup), s, rows, stride, n, view, tile, rec, meta,
               counts, ctl);
}

void launch_preprocess_multi(const float* rows, uint32_t stride, uint32_t n, uint32_t tile, const MultiViewFrames& mv,
                             cudaStream_t s) {
    if (mv.count == 0) return;
    // at least one CTA: with an empty scene it still writes each view's scan entry counts[n] = 0
    const uint32_t blocks = n ? (n + kPreGroup - 1u) / kPreGroup : 1u;
    k_preprocess_multi<<<blocks, kPreGroup, 0, s>>>(rows, stride, n, tile, mv);
}

void launch_pack_to_rows(const float* packed, uint32_t n, uint32_t stride, float* rows, cudaStream_t s) {
    dim3 grid((stride + kTransposeGroup - 1u) / kTransposeGroup, 6);
    k_pack_to_rows<<<grid, 256, 0, s>>>(packed, n, stride, rows);
}

void launch_raster_alpha(const float* o, const float* x, float* y, uint32_t n, cudaStream_t s) {
    if (n == 0) return;
    k_raster_alpha<<<(n + 255u) / 256u, 256, 0, s>>>(o, x, y, n);
}

void launch_exp(const float* x, float* y, uint32_t n, cudaStream_t s, bool raster) {
    if (n == 0) return;
    if (raster) k_exp<true><<<(n + 255u) / 256u, 256, 0, s>>>(x, y, n);
    else k_exp<false><<<(n + 255u) / 256u, 256, 0, s>>>(x, y, n);
}

}  // namespace gs
