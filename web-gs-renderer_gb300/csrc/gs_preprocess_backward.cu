// gs_preprocess_backward.cu -- the preprocess half of the gradients: from the per-Gaussian 2D
// gradients the raster backward accumulates (dL/d pixel position, conic, opacity, colour) to the 59
// packed attributes, for one view or for several views of one scene.
//
// This file is built with multiply-add contraction and the approximate division and square root, and
// it recomputes exp with the hardware approximation (__expf): it only forms gradients, and no bit of
// its output has to match the forward's pinned arithmetic.
#include "gs_kernels.h"

namespace gs {
namespace {

// ---- preprocess backward ---------------------------------------------------------------------------
constexpr uint32_t kBwdGroup = 128;  // Gaussians (threads) per preprocess-backward CTA
// Floats per staged attribute row: rows start 16-byte aligned (bulk-copy destinations) and the
// packed write-out reads them with at most 4-way bank conflicts.
constexpr uint32_t kBwdPitch = 132;

// Chain rule of one visible Gaussian from its 2D gradients d2 = dL/d(pixel.xy, conic, opacity, rgb)
// back to its 59 attributes. R_(row) reads an attribute, W_(row, v) emits its gradient; every W_ of a
// row comes after the last R_ of that row, so W_ may overwrite the staged attribute in place.
template <class RF, class WF, class SF>
__device__ __forceinline__ void backward_gaussian(const ViewBlock& sv, const float* __restrict__ d2, RF R_, WF W_,
                                                  SF sh_ready) {
    const float gpx = d2[0], gpy = d2[1], gA = d2[2], gB = d2[3], gC = d2[4], go = d2[5];
    const float p[3] = {R_(0), R_(1), R_(2)};
    float pv[4], clip[4];
    for (int i = 0; i < 4; ++i) {
        pv[i] = sv.view[i] * p[0] + sv.view[4 + i] * p[1] + sv.view[8 + i] * p[2] + sv.view[12 + i];
        clip[i] = sv.viewProj[i] * p[0] + sv.viewProj[4 + i] * p[1] + sv.viewProj[8 + i] * p[2] + sv.viewProj[12 + i];
    }
    const float wden = clip[3] + kSmallValue;
    // rotation and scale
    float s[3];
    for (int i = 0; i < 3; ++i) s[i] = __expf(R_(kRowScale + i));
    const float qr[4] = {R_(kRowQuat + 1), R_(kRowQuat + 2), R_(kRowQuat + 3), R_(kRowQuat + 0)};  // (x, y, z, w)
    const float qlen = sqrtf(qr[0] * qr[0] + qr[1] * qr[1] + qr[2] * qr[2] + qr[3] * qr[3]);
    const float q[4] = {qr[0] / qlen, qr[1] / qlen, qr[2] / qlen, qr[3] / qlen};
    const float x = q[0], y = q[1], z = q[2], w = q[3];
    float R[3][3];  // [row][col]
    R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - w * z);     R[0][2] = 2 * (x * z + w * y);
    R[1][0] = 2 * (x * y + w * z);     R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - w * x);
    R[2][0] = 2 * (x * z - w * y);     R[2][1] = 2 * (y * z + w * x);     R[2][2] = 1 - 2 * (x * x + y * y);
    float A[3][3], Sg[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = R[i][j] * s[j];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Sg[i][j] = A[i][0] * A[j][0] + A[i][1] * A[j][1] + A[i][2] * A[j][2];
    // 2D covariance
    const float limx = kFrustumExtended * sv.tanFov[0], limy = kFrustumExtended * sv.tanFov[1];
    const float tz = pv[2];
    const float rxr = pv[0] / tz, ryr = pv[1] / tz;
    const bool clampx = rxr < -limx || rxr > limx, clampy = ryr < -limy || ryr > limy;
    const float tx = fminf(limx, fmaxf(-limx, rxr)) * tz, ty = fminf(limy, fmaxf(-limy, ryr)) * tz;
    const float fxl = sv.focal[0], fyl = sv.focal[1];
    const float J[2][3] = {{fxl / tz, 0.0f, -fxl * tx / (tz * tz)}, {0.0f, fyl / tz, -fyl * ty / (tz * tz)}};
    float Wr[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Wr[r][c] = sv.view[c * 4 + r];
    float M[2][3];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 3; ++c) M[r][c] = J[r][0] * Wr[0][c] + J[r][1] * Wr[1][c] + J[r][2] * Wr[2][c];
    float MS[2][3];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 3; ++c) MS[r][c] = M[r][0] * Sg[0][c] + M[r][1] * Sg[1][c] + M[r][2] * Sg[2][c];
    const float ca = MS[0][0] * M[0][0] + MS[0][1] * M[0][1] + MS[0][2] * M[0][2] + 0.3f;
    const float cb = MS[0][0] * M[1][0] + MS[0][1] * M[1][1] + MS[0][2] * M[1][2];
    const float cc = MS[1][0] * M[1][0] + MS[1][1] * M[1][1] + MS[1][2] * M[1][2] + 0.3f;
    const float det = ca * cc - cb * cb, det2 = det * det;
    // conic -> (a, b, c)
    const float ga = gA * (-cc * cc / det2) + gB * (cb * cc / det2) + gC * (-cb * cb / det2);
    const float gb = gA * (2 * cb * cc / det2) + gB * (-(ca * cc + cb * cb) / det2) + gC * (2 * ca * cb / det2);
    const float gc = gA * (-cb * cb / det2) + gB * (cb * ca / det2) + gC * (-ca * ca / det2);
    const float G2[2][2] = {{ga, 0.5f * gb}, {0.5f * gb, gc}};
    // dL/dSigma = M^T G2 M ; dL/dM = 2 G2 M Sigma
    float GM[2][3];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 3; ++c) GM[r][c] = G2[r][0] * M[0][c] + G2[r][1] * M[1][c];
    float gS[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) gS[i][j] = M[0][i] * GM[0][j] + M[1][i] * GM[1][j];
    float gM[2][3];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 3; ++c) gM[r][c] = 2.0f * (G2[r][0] * MS[0][c] + G2[r][1] * MS[1][c]);
    // dL/dJ = dL/dM Wr^T
    float gJ[2][3];
    for (int r = 0; r < 2; ++r)
        for (int k = 0; k < 3; ++k) gJ[r][k] = gM[r][0] * Wr[k][0] + gM[r][1] * Wr[k][1] + gM[r][2] * Wr[k][2];
    const float tz2 = tz * tz, tz3 = tz2 * tz;
    float gpv[3];
    gpv[0] = clampx ? 0.0f : gJ[0][2] * (-fxl / tz2);
    gpv[1] = clampy ? 0.0f : gJ[1][2] * (-fyl / tz2);
    gpv[2] = gJ[0][0] * (-fxl / tz2) + gJ[0][2] * (2.0f * fxl * tx / tz3) + gJ[1][1] * (-fyl / tz2) +
             gJ[1][2] * (2.0f * fyl * ty / tz3);
    float gp[3];
    for (int i = 0; i < 3; ++i) gp[i] = Wr[0][i] * gpv[0] + Wr[1][i] * gpv[1] + Wr[2][i] * gpv[2];
    // pixel position -> clip -> p
    const float gndx = gpx * sv.textureSize[0] * 0.5f, gndy = gpy * sv.textureSize[1] * 0.5f;
    const float gcx = gndx / wden, gcy = gndy / wden, gcw = -(gndx * clip[0] + gndy * clip[1]) / (wden * wden);
    for (int i = 0; i < 3; ++i) gp[i] += sv.viewProj[i * 4 + 0] * gcx + sv.viewProj[i * 4 + 1] * gcy + sv.viewProj[i * 4 + 3] * gcw;
    // colour (SH)
    float v[3] = {p[0] - sv.cameraPos[0], p[1] - sv.cameraPos[1], p[2] - sv.cameraPos[2]};
    const float vlen = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const float dx_ = v[0] / vlen, dy_ = v[1] / vlen, dz_ = v[2] / vlen;
    const float xx = dx_ * dx_, yy = dy_ * dy_, zz = dz_ * dz_;
    float Y[16];
    Y[0] = kShC0;
    Y[1] = -kShC1 * dy_;
    Y[2] = kShC1 * dz_;
    Y[3] = -kShC1 * dx_;
    Y[4] = kShC2_0 * dx_ * dy_;
    Y[5] = kShC2_1 * dy_ * dz_;
    Y[6] = kShC2_2 * (2 * zz - xx - yy);
    Y[7] = kShC2_3 * dx_ * dz_;
    Y[8] = kShC2_4 * (xx - yy);
    Y[9] = kShC3_0 * dy_ * (3 * xx - yy);
    Y[10] = kShC3_1 * dx_ * dy_ * dz_;
    Y[11] = kShC3_2 * dy_ * (4 * zz - xx - yy);
    Y[12] = kShC3_3 * dz_ * (2 * zz - 3 * xx - 3 * yy);
    Y[13] = kShC3_4 * dx_ * (4 * zz - xx - yy);
    Y[14] = kShC3_5 * dz_ * (xx - yy);
    Y[15] = kShC3_6 * dx_ * (xx - 3 * yy);
    sh_ready();  // the f_rest rows arrive on their own barrier
    float gcol[3];
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        float raw = Y[0] * R_(kRowDc + ch);
#pragma unroll
        for (int k = 1; k < 16; ++k) raw += Y[k] * R_(kRowRest + (k - 1) + 15 * ch);
        raw += 0.5f;
        gcol[ch] = raw < 0.0f ? 0.0f : d2[6 + ch];
    }
    float wsh[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        float acc = 0.0f;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            const int row = k == 0 ? kRowDc + ch : kRowRest + (k - 1) + 15 * ch;
            acc += R_(row) * gcol[ch];
            W_(row, Y[k] * gcol[ch]);
        }
        wsh[k] = acc;
    }
    float gdx = 0, gdy = 0, gdz = 0;
    gdy += -kShC1 * wsh[1];
    gdz += kShC1 * wsh[2];
    gdx += -kShC1 * wsh[3];
    gdx += kShC2_0 * dy_ * wsh[4];           gdy += kShC2_0 * dx_ * wsh[4];
    gdy += kShC2_1 * dz_ * wsh[5];           gdz += kShC2_1 * dy_ * wsh[5];
    gdx += -2 * kShC2_2 * dx_ * wsh[6];      gdy += -2 * kShC2_2 * dy_ * wsh[6];      gdz += 4 * kShC2_2 * dz_ * wsh[6];
    gdx += kShC2_3 * dz_ * wsh[7];           gdz += kShC2_3 * dx_ * wsh[7];
    gdx += 2 * kShC2_4 * dx_ * wsh[8];       gdy += -2 * kShC2_4 * dy_ * wsh[8];
    gdx += 6 * kShC3_0 * dx_ * dy_ * wsh[9]; gdy += kShC3_0 * (3 * xx - 3 * yy) * wsh[9];
    gdx += kShC3_1 * dy_ * dz_ * wsh[10];    gdy += kShC3_1 * dx_ * dz_ * wsh[10];    gdz += kShC3_1 * dx_ * dy_ * wsh[10];
    gdx += -2 * kShC3_2 * dx_ * dy_ * wsh[11]; gdy += kShC3_2 * (4 * zz - xx - 3 * yy) * wsh[11]; gdz += 8 * kShC3_2 * dy_ * dz_ * wsh[11];
    gdx += -6 * kShC3_3 * dx_ * dz_ * wsh[12]; gdy += -6 * kShC3_3 * dy_ * dz_ * wsh[12]; gdz += kShC3_3 * (6 * zz - 3 * xx - 3 * yy) * wsh[12];
    gdx += kShC3_4 * (4 * zz - 3 * xx - yy) * wsh[13]; gdy += -2 * kShC3_4 * dx_ * dy_ * wsh[13]; gdz += 8 * kShC3_4 * dx_ * dz_ * wsh[13];
    gdx += 2 * kShC3_5 * dx_ * dz_ * wsh[14]; gdy += -2 * kShC3_5 * dy_ * dz_ * wsh[14]; gdz += kShC3_5 * (xx - yy) * wsh[14];
    gdx += kShC3_6 * (3 * xx - 3 * yy) * wsh[15]; gdy += -6 * kShC3_6 * dx_ * dy_ * wsh[15];
    const float ddot = gdx * dx_ + gdy * dy_ + gdz * dz_;
    gp[0] += (gdx - dx_ * ddot) / vlen;
    gp[1] += (gdy - dy_ * ddot) / vlen;
    gp[2] += (gdz - dz_ * ddot) / vlen;
    for (int i = 0; i < 3; ++i) W_(kRowPos + i, gp[i]);
    // opacity logit
    const float op = 1.0f / (1.0f + __expf(-R_(kRowOpacity)));
    W_(kRowOpacity, go * op * (1.0f - op));
    // Sigma = A A^T -> A -> (R, s) -> (quaternion, log-scale)
    float gAm[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            gAm[i][j] = (gS[i][0] + gS[0][i]) * A[0][j] + (gS[i][1] + gS[1][i]) * A[1][j] + (gS[i][2] + gS[2][i]) * A[2][j];
    float gR[3][3];
    for (int j = 0; j < 3; ++j) {
        float gs = 0.0f;
        for (int i = 0; i < 3; ++i) {
            gs += gAm[i][j] * R[i][j];
            gR[i][j] = gAm[i][j] * s[j];
        }
        W_(kRowScale + j, gs * s[j]);
    }
    float gq[4];
    gq[0] = gR[1][0] * 2 * y + gR[2][0] * 2 * z + gR[0][1] * 2 * y + gR[1][1] * -4 * x + gR[2][1] * 2 * w +
            gR[0][2] * 2 * z + gR[1][2] * -2 * w + gR[2][2] * -4 * x;
    gq[1] = gR[0][0] * -4 * y + gR[1][0] * 2 * x + gR[2][0] * -2 * w + gR[0][1] * 2 * x + gR[2][1] * 2 * z +
            gR[0][2] * 2 * w + gR[1][2] * 2 * z + gR[2][2] * -4 * y;
    gq[2] = gR[0][0] * -4 * z + gR[1][0] * 2 * w + gR[2][0] * 2 * x + gR[0][1] * -2 * w + gR[1][1] * -4 * z +
            gR[2][1] * 2 * y + gR[0][2] * 2 * x + gR[1][2] * 2 * y;
    gq[3] = gR[1][0] * 2 * z + gR[2][0] * -2 * y + gR[0][1] * -2 * z + gR[2][1] * 2 * x + gR[0][2] * 2 * y +
            gR[1][2] * -2 * x;
    const float qd = gq[0] * q[0] + gq[1] * q[1] + gq[2] * q[2] + gq[3] * q[3];
    W_(kRowQuat + 0, (gq[3] - q[3] * qd) / qlen);  // stored rot_0 = w
    W_(kRowQuat + 1, (gq[0] - q[0] * qd) / qlen);
    W_(kRowQuat + 2, (gq[1] - q[1] * qd) / qlen);
    W_(kRowQuat + 3, (gq[2] - q[2] * qd) / qlen);
}

// Writes the CTA's gradient tile (one column per Gaussian, rows as the scene layout) to its slice of
// the packed layout: the Gaussians [g0, g0 + cnt) occupy one contiguous range of each attribute
// block, so every block is one coalesced run. zero: write zeros; add: add to what `out` holds.
// The narrow blocks (1 to 4 values per Gaussian) walk the run one element per lane. The 45-value
// f_rest block maps lanes to attribute rows instead: a lane reads four consecutive Gaussians of its
// row with one 16-byte load (eight lanes of a phase hit eight distinct 4-bank groups: no conflict,
// where a column read down the rows is 4-way) and makes four stores, each of which the warp's 32
// lanes (32 consecutive rows) complete as one contiguous 128-byte run.
__device__ __forceinline__ void write_packed(const float (*tile)[kBwdPitch], float* __restrict__ out, uint32_t n,
                                             uint32_t g0, uint32_t cnt, bool zero, bool add) {
    struct Block { uint32_t row, width, base; };
    const Block blocks[5] = {{kRowPos, 3, 0}, {kRowScale, 3, 3}, {kRowQuat, 4, 6}, {kRowDc, 3, 10}, {kRowOpacity, 1, 13}};
#pragma unroll
    for (int bi = 0; bi < 5; ++bi) {
        const Block bk = blocks[bi];
        float* dst = out + (size_t)bk.base * n + (size_t)bk.width * g0;
        const uint32_t total = bk.width * cnt;
        for (uint32_t i = threadIdx.x; i < total; i += kBwdGroup) {
            const float v = zero ? 0.0f : tile[bk.row + i % bk.width][i / bk.width];
            dst[i] = add ? dst[i] + v : v;
        }
    }
    constexpr uint32_t kRest = kRows - kRowRest;  // 45
    static_assert(kRest > 32 && kRest <= 64, "two row passes cover f_rest");
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    float* dst = out + (size_t)14 * n + (size_t)kRest * g0;
    for (uint32_t task = warp; task < 2u * (kBwdGroup / 4u); task += kBwdGroup / 32u) {
        const uint32_t r = (task & 1u) * 32u + lane;  // f_rest row
        const uint32_t c0 = (task >> 1) * 4u;          // first of four Gaussians (column)
        if (r >= kRest || c0 >= cnt) continue;
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (!zero) v = *reinterpret_cast<const float4*>(&tile[kRowRest + r][c0]);
        const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (uint32_t k = 0; k < 4u; ++k) {
            if (c0 + k >= cnt) break;
            float* p = dst + (size_t)(c0 + k) * kRest + r;
            *p = add ? *p + vv[k] : vv[k];
        }
    }
}

// One thread per Gaussian, six CTAs per SM (80 registers: the few spills cost less than the lost
// residency). Everything a CTA reads comes in by bulk copies into shared memory, all issued at once
// on two mbarriers: the view block, the slice's tilesTouched counts and 2D gradients and its 14
// geometry attribute rows on the first; its 45 f_rest rows on the second, whose arrival overlaps the
// geometric part of the chain rule (a slice with no visible Gaussian only waits for them and writes
// zeros). The gradients replace the staged attributes in shared memory and the CTA
// writes its slice of the packed layout (pos | log-scale | rot | f_dc | opacity | f_rest blocks, the
// layout gs_scene_upload takes) with coalesced stores; invisible Gaussians get zeros.
// Reads past the slice: counts are read in whole 16-byte units (the buffer holds roundup(N + 1, 8)
// entries) and grad2d likewise (it holds 9N + 4 floats).
__global__ void __launch_bounds__(kBwdGroup, 6) k_preprocess_backward(const float* __restrict__ rows, uint32_t stride,
                                                                   uint32_t n, const ViewBlock* __restrict__ vb,
                                                                   const uint32_t* __restrict__ counts,
                                                                   float* __restrict__ grad2d,
                                                                   float* __restrict__ out, uint32_t* status) {
    pdl_wait();
    static_assert(sizeof(ViewBlock) % 16 == 0, "the view block is copied in 16-byte units");
    __shared__ __align__(128) float s_rows[kRows][kBwdPitch];
    __shared__ __align__(16) float s_d2[kBwdGroup * 9];
    __shared__ __align__(16) uint32_t s_cnt[kBwdGroup];
    __shared__ __align__(16) ViewBlock sv;
    __shared__ __align__(8) uint64_t s_bar[2];  // [0]: view, counts, 2D gradients, geometry rows; [1]: f_rest rows
    const uint32_t lt = threadIdx.x;
    const uint32_t g0 = blockIdx.x * kBwdGroup;
    const uint32_t cnt = min(kBwdGroup, n - g0);  // Gaussians of this CTA (g0 < n)
    // stride and g0 are multiples of 64 floats: every row slice starts 256-byte aligned and spans a
    // multiple of 256 bytes (g0 < n <= stride)
    const uint32_t cols = min(kBwdGroup, stride - g0);
    if (lt == 0) {
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
    }
    __syncthreads();
    // bounded wait: on expiry the timeout is recorded and the kernel goes on with what is there
    auto wait_bar = [&](uint64_t* bar) {
        uint32_t spins = 0;
        while (!mbar_try_wait(bar, 0)) {
            if (++spins > kSpinLimit) {
                if (lt == 0 && status) atomicOr(status, kDevTimeout);
                break;
            }
        }
    };
    if (lt == 0) {
        const uint32_t cnt_bytes = ((cnt + 3u) & ~3u) * 4u;
        const uint32_t d2_bytes = (cnt * 36u + 15u) & ~15u;
        mbar_expect_tx(&s_bar[0], (uint32_t)sizeof(ViewBlock) + cnt_bytes + d2_bytes + kRowRest * cols * 4u);
        bulk_g2s(&sv, vb, (uint32_t)sizeof(ViewBlock), &s_bar[0]);
        bulk_g2s(s_cnt, counts + g0, cnt_bytes, &s_bar[0]);
        bulk_g2s(s_d2, grad2d + (size_t)9 * g0, d2_bytes, &s_bar[0]);
        for (int r = 0; r < kRowRest; ++r)
            bulk_g2s(&s_rows[r][0], rows + (size_t)r * stride + g0, cols * 4u, &s_bar[0]);
        // the f_rest rows too, at once: with the Gaussians in scene order almost every slice holds a
        // visible one, and waiting for the counts before asking for them costs a round trip per CTA
        mbar_expect_tx(&s_bar[1], (kRows - kRowRest) * cols * 4u);
        for (int r = kRowRest; r < kRows; ++r)
            bulk_g2s(&s_rows[r][0], rows + (size_t)r * stride + g0, cols * 4u, &s_bar[1]);
    }
    wait_bar(&s_bar[0]);
    const bool vis = lt < cnt && s_cnt[lt] != 0u;
    const int any = __syncthreads_or(vis);
    if (!any) wait_bar(&s_bar[1]);  // no bulk copy may still write into shared memory when the CTA leaves
    if (any) {
        // the slice's 2D gradients are in shared memory now (every thread passed the copy's barrier):
        // clear them in global memory for the next raster backward, which only accumulates
        for (uint32_t i = lt; i < 9u * cnt; i += kBwdGroup) grad2d[(size_t)9 * g0 + i] = 0.0f;
        if (vis) {
            auto R_ = [&](int row) { return s_rows[row][lt]; };
            auto W_ = [&](int row, float v) { s_rows[row][lt] = v; };
            backward_gaussian(sv, s_d2 + 9 * lt, R_, W_, [&]() { wait_bar(&s_bar[1]); });
        } else {
            // every thread waits for the f_rest copies before it overwrites its column or leaves: no
            // bulk copy may still write into shared memory that is reused or released
            wait_bar(&s_bar[1]);
            for (int r = 0; r < kRows; ++r) s_rows[r][lt] = 0.0f;
        }
    }
    __syncthreads();
    write_packed(s_rows, out, n, g0, cnt, !any, false);
}

// Several views of one scene: one thread per Gaussian stages the 59 attribute rows once (bulk copies)
// and runs the chain rule for every view that sees the Gaussian, summing the views' gradients in a
// shared-memory tile of its own column; the CTA then writes its slice of the packed layout with
// coalesced stores (stored, or added to what an earlier group of views wrote). The scene is read
// once per batch instead of once per view, and no atomics, clearing or transpose pass are needed.
__global__ void __launch_bounds__(kBwdGroup) k_preprocess_backward_multi(const float* __restrict__ rows,
                                                                         uint32_t stride, uint32_t n,
                                                                         MultiViewGrads mv, float* __restrict__ out,
                                                                         int add, uint32_t* status) {
    extern __shared__ __align__(128) float s_dyn[];
    float(*s_rows)[kBwdPitch] = reinterpret_cast<float(*)[kBwdPitch]>(s_dyn);
    float(*s_grad)[kBwdPitch] = reinterpret_cast<float(*)[kBwdPitch]>(s_dyn + kRows * kBwdPitch);
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ ViewBlock sv;
    const uint32_t lt = threadIdx.x;
    const uint32_t g0 = blockIdx.x * kBwdGroup;
    const uint32_t g = g0 + lt;
    const uint32_t cnt = min(kBwdGroup, n - g0);  // Gaussians of this CTA (g0 < n)
    uint32_t seen = 0u;                           // views that see this Gaussian (bit per view)
    for (uint32_t v = 0; v < mv.count; ++v)
        if (g < n && mv.counts[v][g] != 0u) seen |= 1u << v;
    if (lt == 0) mbar_init(&s_bar, 1);
    for (int r = 0; r < kRows; ++r) s_grad[r][lt] = 0.0f;
    const int any = __syncthreads_or(seen != 0u);
    if (any) {
        if (lt == 0) {
            // stride and g0 are multiples of 64 floats: 256-byte aligned slices of 256-byte multiples
            const uint32_t cols = min(kBwdGroup, stride - g0);
            mbar_expect_tx(&s_bar, kRows * cols * 4u);
            for (int r = 0; r < kRows; ++r) bulk_g2s(&s_rows[r][0], rows + (size_t)r * stride + g0, cols * 4u, &s_bar);
        }
        uint32_t spins = 0;
        while (!mbar_try_wait(&s_bar, 0)) {  // every thread waits: no copy may outlive the CTA
            if (++spins > kSpinLimit) {
                if (lt == 0 && status) atomicOr(status, kDevTimeout);
                break;
            }
        }
        auto R_ = [&](int row) { return s_rows[row][lt]; };
        auto W_ = [&](int row, float val) { s_grad[row][lt] += val; };
        for (uint32_t v = 0; v < mv.count; ++v) {
            __syncthreads();  // sv is rewritten per view
            if (lt < 44) reinterpret_cast<uint32_t*>(&sv)[lt] = reinterpret_cast<const uint32_t*>(mv.view[v])[lt];
            __syncthreads();
            if (seen & (1u << v)) {
                float* d2 = mv.grad2d[v] + (size_t)9 * g;
                backward_gaussian(sv, d2, R_, W_, []() {});
                // cleared for the next raster backward, which only accumulates
#pragma unroll
                for (int k = 0; k < 9; ++k) d2[k] = 0.0f;
            }
        }
    }
    __syncthreads();
    write_packed(s_grad, out, n, g0, cnt, false, add != 0);
}

}  // namespace

size_t preprocess_backward_multi_smem() { return (size_t)2 * kRows * kBwdPitch * sizeof(float); }

void configure_backward_kernels() {
    cudaFuncSetAttribute(k_preprocess_backward_multi, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)preprocess_backward_multi_smem());
}

void launch_preprocess_backward_multi(const float* rows, uint32_t stride, uint32_t n, const MultiViewGrads& mv,
                                      float* out, bool add, uint32_t* status, cudaStream_t s) {
    if (n == 0 || mv.count == 0) return;
    k_preprocess_backward_multi<<<(n + kBwdGroup - 1u) / kBwdGroup, kBwdGroup, preprocess_backward_multi_smem(), s>>>(
        rows, stride, n, mv, out, add ? 1 : 0, status);
}

void launch_preprocess_backward(const float* rows, uint32_t stride, uint32_t n, const ViewBlock* view,
                                const uint32_t* counts, float* grad2d, float* out, uint32_t* status,
                                cudaStream_t s) {
    if (n == 0) return;
    launch_pdl(k_preprocess_backward, dim3((n + kBwdGroup - 1u) / kBwdGroup), dim3(kBwdGroup), s, rows, stride, n, view,
               counts, grad2d, out, status);
}

}  // namespace gs
