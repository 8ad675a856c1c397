// gs_loss.cu -- L = mean|x - y| + lambda * (1 - mean SSIM) and dL/dx on the device, for the
// differentiation workload (no counterpart in the reference). SSIM is per channel with an 11x11
// Gaussian window (sigma 1.5, normalised, separable), zero padding, C1 = 0.01^2, C2 = 0.03^2. With
// the filtered moments m1 = G*x, m2 = G*x^2, mxy = G*(xy) the gradient is
//   dSSIM/dx = G*(dS/dm1) + 2x G*(dS/dm2) + y G*(dS/dmxy)
// (the window is symmetric). Two kernels, each on 32x16 output tiles of one channel with a 5-pixel
// halo staged in shared memory (both separable passes happen there):
//   k_ssim_fwd  moments -> SSIM map -> its three partials (to global) + per-block SSIM and L1 sums;
//   k_ssim_bwd  blurred partials + the L1 term -> dL/dx.
// Images are H x W x 3 (pixel-interleaved). The loss is not bit-pinned: this file is built with
// multiply-add contraction and the approximate division, and its filters use fused multiply-adds.
#include <cmath>

#include "gs_kernels.h"

namespace gs {
namespace {

struct Window {
    float w[11];
};

constexpr int kT = 32;              // output tile (kT x kT pixels of one channel)
constexpr int kR = 5;               // window radius
constexpr int kH = kT + 2 * kR;     // haloed tile edge (42)
constexpr int kPitchIn = kH + 1;    // 43: the horizontal pass reads rows conflict-free
constexpr int kPitchH = kT + 1;     // 33
constexpr int kThreads = 256;
constexpr int kRunH = 8;            // horizontal pass: 8 consecutive outputs of one row per thread
constexpr int kItemsH = kH * (kT / kRunH);  // 168 row runs
constexpr int kRunV = 4;            // vertical pass: 4 consecutive outputs of one column per thread
static_assert(kT * (kT / kRunV) == kThreads, "one vertical run per thread");

// Stages rows [ty0, ty0 + kH) x cols [tx0, tx0 + kH) of channel ch of an H x W x 3 image (zeros
// outside) into dst (pitch kPitchIn).
__device__ __forceinline__ void stage_channel(const float* __restrict__ img, uint32_t W, uint32_t H, int tx0,
                                              int ty0, int ch, float* dst) {
    // a fixed trip count, so that all of a thread's loads are in flight before the first store
    constexpr int kIters = (kH * kH + kThreads - 1) / kThreads;
    float v[kIters];
#pragma unroll
    for (int it = 0; it < kIters; ++it) {
        const int i = threadIdx.x + it * kThreads;
        const int ly = i / kH, lx = i - ly * kH, gx = tx0 + lx, gy = ty0 + ly;
        v[it] = 0.0f;
        if (i < kH * kH && gx >= 0 && gx < (int)W && gy >= 0 && gy < (int)H) v[it] = img[((size_t)gy * W + gx) * 3 + ch];
    }
#pragma unroll
    for (int it = 0; it < kIters; ++it) {
        const int i = threadIdx.x + it * kThreads;
        if (i < kH * kH) dst[(i / kH) * kPitchIn + i % kH] = v[it];
    }
}

// Moments of x and y over the window, the SSIM map, its partials with respect to the moments, and
// per-block sums of SSIM and |x - y|. Each thread filters a run of 8 outputs of one row (the 18 inputs
// it needs stay in registers), then a run of 4 outputs of one column.
__global__ void __launch_bounds__(kThreads) k_ssim_fwd(const float* __restrict__ x, const float* __restrict__ y,
                                                       uint32_t W, uint32_t H, Window win,
                                                       float* __restrict__ partial /* 9 planes */,
                                                       double* __restrict__ block_sums) {
    pdl_wait();
    __shared__ float sx[kH * kPitchIn], sy[kH * kPitchIn];
    __shared__ float hm[5][kH * kPitchH];
    __shared__ float red[2][kThreads / 32];
    const int ch = blockIdx.z;
    const int tx0 = blockIdx.x * kT - kR, ty0 = blockIdx.y * kT - kR;
    const int tid = threadIdx.x;
    stage_channel(x, W, H, tx0, ty0, ch, sx);
    stage_channel(y, W, H, tx0, ty0, ch, sy);
    __syncthreads();
    if (tid < kItemsH) {
        const int r = tid / (kT / kRunH), c0 = (tid % (kT / kRunH)) * kRunH;
        constexpr int kIn = kRunH + 2 * kR;
        float a[kIn], b[kIn];
#pragma unroll
        for (int j = 0; j < kIn; ++j) {
            a[j] = sx[r * kPitchIn + c0 + j];
            b[j] = sy[r * kPitchIn + c0 + j];
        }
        // one quantity at a time (x, y, x^2, y^2, xy): its inputs formed once, then one fused
        // multiply-add per tap and output
#pragma unroll
        for (int qn = 0; qn < 5; ++qn) {
            float v[kIn];
#pragma unroll
            for (int j = 0; j < kIn; ++j)
                v[j] = qn == 0 ? a[j] : qn == 1 ? b[j] : qn == 2 ? a[j] * a[j] : qn == 3 ? b[j] * b[j] : a[j] * b[j];
#pragma unroll
            for (int o = 0; o < kRunH; ++o) {
                float acc = 0.0f;
#pragma unroll
                for (int k = 0; k < 2 * kR + 1; ++k) acc = fmaf(win.w[k], v[o + k], acc);
                hm[qn][r * kPitchH + c0 + o] = acc;
            }
        }
    }
    __syncthreads();
    const int c = tid % kT, r0 = (tid / kT) * kRunV;
    const int gx = blockIdx.x * kT + c;
    float m[kRunV][5];
#pragma unroll
    for (int o = 0; o < kRunV; ++o)
#pragma unroll
        for (int q = 0; q < 5; ++q) m[o][q] = 0.0f;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        float v[kRunV + 2 * kR];
#pragma unroll
        for (int j = 0; j < kRunV + 2 * kR; ++j) v[j] = hm[q][(r0 + j) * kPitchH + c];
#pragma unroll
        for (int o = 0; o < kRunV; ++o)
#pragma unroll
            for (int k = 0; k < 2 * kR + 1; ++k) m[o][q] = fmaf(win.w[k], v[o + k], m[o][q]);
    }
    const size_t P = (size_t)W * H;
    float ssim = 0.0f, l1 = 0.0f;
#pragma unroll
    for (int o = 0; o < kRunV; ++o) {
        const int gy = blockIdx.y * kT + r0 + o;
        if (gx >= (int)W || gy >= (int)H) continue;
        const float C1 = 0.01f * 0.01f, C2 = 0.03f * 0.03f;
        const float mx = m[o][0], my = m[o][1];
        const float sxx = m[o][2] - mx * mx, syy = m[o][3] - my * my, sxy = m[o][4] - mx * my;
        const float A1 = 2.0f * mx * my + C1, A2 = 2.0f * sxy + C2;
        const float B1 = mx * mx + my * my + C1, B2 = sxx + syy + C2;
        const float inv_b = 1.0f / (B1 * B2);  // 1/B1 = B2 inv_b, 1/B2 = B1 inv_b
        const float sv = A1 * A2 * inv_b;
        const float ds_dmx = (2.0f * my * A2) * inv_b - sv * (2.0f * mx) * (B2 * inv_b);
        const float ds_dsxx = -sv * (B1 * inv_b);
        const float ds_dsxy = 2.0f * A1 * inv_b;
        const size_t po = (size_t)gy * W + gx;
        partial[(ch * 3 + 0) * P + po] = ds_dmx + ds_dsxx * (-2.0f * mx) + ds_dsxy * (-my);
        partial[(ch * 3 + 1) * P + po] = ds_dsxx;
        partial[(ch * 3 + 2) * P + po] = ds_dsxy;
        ssim += sv;
        l1 += fabsf(sx[(r0 + o + kR) * kPitchIn + c + kR] - sy[(r0 + o + kR) * kPitchIn + c + kR]);
    }
    for (int k = 16; k > 0; k >>= 1) {
        ssim += __shfl_xor_sync(0xffffffffu, ssim, k);
        l1 += __shfl_xor_sync(0xffffffffu, l1, k);
    }
    const int lane = tid & 31, warp = tid >> 5;
    if (lane == 0) { red[0][warp] = ssim; red[1][warp] = l1; }
    __syncthreads();
    if (warp == 0) {
        constexpr int kWarps = kThreads / 32;
        float s_ = lane < kWarps ? red[0][lane] : 0.0f, l_ = lane < kWarps ? red[1][lane] : 0.0f;
        for (int k = 16; k > 0; k >>= 1) {
            s_ += __shfl_xor_sync(0xffffffffu, s_, k);
            l_ += __shfl_xor_sync(0xffffffffu, l_, k);
        }
        if (lane == 0) {
            const size_t blk = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
            block_sums[2 * blk] = (double)s_;
            block_sums[2 * blk + 1] = (double)l_;
        }
    }
}

// dL/dx from the blurred partials (same tiling and register blocking as k_ssim_fwd).
__device__ void reduce_sums(double* __restrict__ sums, size_t blocks);

// sums (may be null): block 0 also reduces the forward's per-block sums into sums[0..1], while the
// other blocks filter, so the loss value needs no kernel of its own when a gradient is formed.
__global__ void __launch_bounds__(kThreads) k_ssim_bwd(const float* __restrict__ partial, const float* __restrict__ x,
                                                       const float* __restrict__ y, uint32_t W, uint32_t H,
                                                       Window win, float lambda, float* __restrict__ dl,
                                                       double* __restrict__ sums, size_t sum_blocks) {
    pdl_wait();
    if (sums && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) reduce_sums(sums, sum_blocks);
    __shared__ float sp[3][kH * kPitchIn];
    __shared__ float hp[3][kH * kPitchH];
    const int ch = blockIdx.z;
    const int tx0 = blockIdx.x * kT - kR, ty0 = blockIdx.y * kT - kR;
    const int tid = threadIdx.x;
    const size_t P = (size_t)W * H;
    const int c = tid % kT, r0 = (tid / kT) * kRunV;
    const int gx = blockIdx.x * kT + c;
    // this thread's x and y, loaded first so that they arrive during the staging and the filtering
    float xv[kRunV], yv[kRunV];
#pragma unroll
    for (int o = 0; o < kRunV; ++o) {
        const int gy = blockIdx.y * kT + r0 + o;
        const bool in = gx < (int)W && gy < (int)H;
        const size_t q = in ? ((size_t)gy * W + gx) * 3 + ch : 0;
        xv[o] = in ? x[q] : 0.0f;
        yv[o] = in ? y[q] : 0.0f;
    }
    {
        constexpr int kIters = (kH * kH + kThreads - 1) / kThreads;
        float v[kIters][3];
#pragma unroll
        for (int it = 0; it < kIters; ++it) {
            const int i = tid + it * kThreads;
            const int ly = i / kH, lx = i - ly * kH, gx = tx0 + lx, gy = ty0 + ly;
            const bool in = i < kH * kH && gx >= 0 && gx < (int)W && gy >= 0 && gy < (int)H;
            const size_t o = in ? (size_t)gy * W + gx : 0;
#pragma unroll
            for (int q = 0; q < 3; ++q) v[it][q] = in ? partial[(ch * 3 + q) * P + o] : 0.0f;
        }
#pragma unroll
        for (int it = 0; it < kIters; ++it) {
            const int i = tid + it * kThreads;
            if (i < kH * kH)
#pragma unroll
                for (int q = 0; q < 3; ++q) sp[q][(i / kH) * kPitchIn + i % kH] = v[it][q];
        }
    }
    __syncthreads();
    if (tid < kItemsH) {
        const int r = tid / (kT / kRunH), c0 = (tid % (kT / kRunH)) * kRunH;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            float v[kRunH + 2 * kR];
#pragma unroll
            for (int j = 0; j < kRunH + 2 * kR; ++j) v[j] = sp[q][r * kPitchIn + c0 + j];
#pragma unroll
            for (int o = 0; o < kRunH; ++o) {
                float acc = 0.0f;
#pragma unroll
                for (int k = 0; k < 2 * kR + 1; ++k) acc = fmaf(win.w[k], v[o + k], acc);
                hp[q][r * kPitchH + c0 + o] = acc;
            }
        }
    }
    __syncthreads();
    float bl[kRunV][3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        float v[kRunV + 2 * kR];
#pragma unroll
        for (int j = 0; j < kRunV + 2 * kR; ++j) v[j] = hp[q][(r0 + j) * kPitchH + c];
#pragma unroll
        for (int o = 0; o < kRunV; ++o) {
            float acc = 0.0f;
#pragma unroll
            for (int k = 0; k < 2 * kR + 1; ++k) acc = fmaf(win.w[k], v[o + k], acc);
            bl[o][q] = acc;
        }
    }
    const float inv = 1.0f / (float)(3 * P);
#pragma unroll
    for (int o = 0; o < kRunV; ++o) {
        const int gy = blockIdx.y * kT + r0 + o;
        if (gx >= (int)W || gy >= (int)H) continue;
        const size_t q = ((size_t)gy * W + gx) * 3 + ch;
        const float d = xv[o] - yv[o];
        const float g_l1 = (d > 0.0f ? inv : (d < 0.0f ? -inv : 0.0f));
        dl[q] = g_l1 - lambda * inv * (bl[o][0] + 2.0f * xv[o] * bl[o][1] + yv[o] * bl[o][2]);
    }
}

// sums[0..1] = column sums of the per-block partials that follow them, by one CTA in a fixed order
// (the same sum on every call)
__device__ void reduce_sums(double* __restrict__ sums, size_t blocks) {
    __shared__ double red[2][32];
    double a = 0.0, b = 0.0;
    const double* part = sums + 2;
    for (size_t i = threadIdx.x; i < blocks; i += blockDim.x) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    for (int k = 16; k > 0; k >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, k);
        b += __shfl_xor_sync(0xffffffffu, b, k);
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0) { red[0][warp] = a; red[1][warp] = b; }
    __syncthreads();
    if (warp == 0) {
        const uint32_t nw = blockDim.x >> 5;
        a = lane < nw ? red[0][lane] : 0.0;
        b = lane < nw ? red[1][lane] : 0.0;
        for (int k = 16; k > 0; k >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, k);
            b += __shfl_xor_sync(0xffffffffu, b, k);
        }
        if (lane == 0) {
            sums[0] = a;
            sums[1] = b;
        }
    }
}

__global__ void k_reduce_sums(double* __restrict__ sums, size_t blocks) {
    pdl_wait();
    reduce_sums(sums, blocks);
}

Window make_window() {
    Window w;
    double s = 0, v[11];
    for (int i = 0; i < 11; ++i) {
        v[i] = std::exp(-(double)((i - 5) * (i - 5)) / (2.0 * 1.5 * 1.5));
        s += v[i];
    }
    for (int i = 0; i < 11; ++i) w.w[i] = (float)(v[i] / s);
    return w;
}

dim3 loss_grid(uint32_t width, uint32_t height) {
    return dim3((width + kT - 1) / kT, (height + kT - 1) / kT, 3);
}

}  // namespace

size_t loss_scratch_floats(uint32_t width, uint32_t height) { return (size_t)width * height * 9; }

size_t loss_sum_doubles(uint32_t width, uint32_t height) {
    const dim3 g = loss_grid(width, height);
    return 2 + 2 * (size_t)g.x * g.y * g.z;
}

void launch_loss_l1_ssim(const float* x, const float* y, uint32_t width, uint32_t height, float lambda,
                         float* scratch, double* sums, float* dl, cudaStream_t s) {
    const Window win = make_window();
    const dim3 grid = loss_grid(width, height), block(kThreads);
    const size_t blocks = (size_t)grid.x * grid.y * grid.z;
    launch_pdl(k_ssim_fwd, grid, block, s, x, y, width, height, win, scratch, sums + 2);
    if (dl) launch_pdl(k_ssim_bwd, grid, block, s, scratch, x, y, width, height, win, lambda, dl, sums, blocks);
    else launch_pdl(k_reduce_sums, dim3(1), dim3(1024), s, sums, blocks);
}

}  // namespace gs
