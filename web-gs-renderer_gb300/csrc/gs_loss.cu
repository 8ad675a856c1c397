// gs_loss.cu -- L = mean|x - y| + lambda * (1 - mean SSIM) and dL/dx on the device, for the
// differentiation workload (no counterpart in the reference). SSIM is per channel with an 11x11
// Gaussian window (sigma 1.5, normalised, separable), zero padding, C1 = 0.01^2, C2 = 0.03^2. With
// the filtered moments m1 = G*x, m2 = G*x^2, mxy = G*(xy) the gradient is
//   dSSIM/dx = G*(dS/dm1) + 2x G*(dS/dm2) + y G*(dS/dmxy)
// (the window is symmetric). Two kernels, each on 32x16 output tiles of one channel with a 5-pixel
// halo staged in shared memory (both separable passes happen there):
//   k_ssim_fwd  moments -> SSIM map -> its three partials (to global) + per-block SSIM and L1 sums;
//   k_ssim_bwd  blurred partials + the L1 term -> dL/dx.
// Images are H x W x 3 (pixel-interleaved).
#include <cmath>

#include "gs_kernels.h"

namespace gs {
namespace {

struct Window {
    float w[11];
};

constexpr int kTX = 32, kTY = 16, kR = 5;
constexpr int kHX = kTX + 2 * kR, kHY = kTY + 2 * kR;  // haloed tile

__global__ void __launch_bounds__(kTX * kTY) k_ssim_fwd(const float* __restrict__ x, const float* __restrict__ y,
                                                        uint32_t W, uint32_t H, Window win,
                                                        float* __restrict__ partial /* 9 planes */,
                                                        double* __restrict__ block_sums) {
    __shared__ float sx[kHY][kHX], sy[kHY][kHX];
    __shared__ float hm[5][kHY][kTX];
    __shared__ float red[2][kTX * kTY / 32];
    const int ch = blockIdx.z;
    const int tx0 = blockIdx.x * kTX - kR, ty0 = blockIdx.y * kTY - kR;
    const int tid = threadIdx.y * kTX + threadIdx.x;
    for (int i = tid; i < kHX * kHY; i += kTX * kTY) {
        const int lx = i % kHX, ly = i / kHX, gx = tx0 + lx, gy = ty0 + ly;
        float a = 0.0f, b = 0.0f;
        if (gx >= 0 && gx < (int)W && gy >= 0 && gy < (int)H) {
            const size_t q = ((size_t)gy * W + gx) * 3 + ch;
            a = x[q];
            b = y[q];
        }
        sx[ly][lx] = a;
        sy[ly][lx] = b;
    }
    __syncthreads();
    for (int i = tid; i < kTX * kHY; i += kTX * kTY) {  // horizontal pass over every haloed row
        const int c = i % kTX, r = i / kTX;
        float s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0;
#pragma unroll
        for (int k = 0; k < 11; ++k) {
            const float a = sx[r][c + k], b = sy[r][c + k], w = win.w[k];
            s0 += w * a;
            s1 += w * b;
            s2 += w * a * a;
            s3 += w * b * b;
            s4 += w * a * b;
        }
        hm[0][r][c] = s0; hm[1][r][c] = s1; hm[2][r][c] = s2; hm[3][r][c] = s3; hm[4][r][c] = s4;
    }
    __syncthreads();
    const int c = threadIdx.x, r = threadIdx.y;
    const int gx = blockIdx.x * kTX + c, gy = blockIdx.y * kTY + r;
    float ssim = 0.0f, l1 = 0.0f;
    if (gx < (int)W && gy < (int)H) {
        float m[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int k = 0; k < 11; ++k) {
            const float w = win.w[k];
#pragma unroll
            for (int q = 0; q < 5; ++q) m[q] += w * hm[q][r + k][c];
        }
        const float C1 = 0.01f * 0.01f, C2 = 0.03f * 0.03f;
        const float mx = m[0], my = m[1];
        const float sxx = m[2] - mx * mx, syy = m[3] - my * my, sxy = m[4] - mx * my;
        const float A1 = 2.0f * mx * my + C1, A2 = 2.0f * sxy + C2;
        const float B1 = mx * mx + my * my + C1, B2 = sxx + syy + C2;
        const float s = A1 * A2 / (B1 * B2);
        const float ds_dmx = (2.0f * my * A2) / (B1 * B2) - s * (2.0f * mx) / B1;
        const float ds_dsxx = -s / B2;
        const float ds_dsxy = 2.0f * A1 / (B1 * B2);
        const size_t P = (size_t)W * H, o = (size_t)gy * W + gx;
        partial[(ch * 3 + 0) * P + o] = ds_dmx + ds_dsxx * (-2.0f * mx) + ds_dsxy * (-my);
        partial[(ch * 3 + 1) * P + o] = ds_dsxx;
        partial[(ch * 3 + 2) * P + o] = ds_dsxy;
        ssim = s;
        l1 = fabsf(sx[r + kR][c + kR] - sy[r + kR][c + kR]);
    }
    for (int k = 16; k > 0; k >>= 1) {
        ssim += __shfl_xor_sync(0xffffffffu, ssim, k);
        l1 += __shfl_xor_sync(0xffffffffu, l1, k);
    }
    const int lane = tid & 31, warp = tid >> 5;
    if (lane == 0) { red[0][warp] = ssim; red[1][warp] = l1; }
    __syncthreads();
    if (warp == 0) {
        constexpr int kWarps = kTX * kTY / 32;
        float a = lane < kWarps ? red[0][lane] : 0.0f, b = lane < kWarps ? red[1][lane] : 0.0f;
        for (int k = 16; k > 0; k >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, k);
            b += __shfl_xor_sync(0xffffffffu, b, k);
        }
        if (lane == 0) {
            const size_t blk = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
            block_sums[2 * blk] = (double)a;
            block_sums[2 * blk + 1] = (double)b;
        }
    }
}

__global__ void __launch_bounds__(kTX * kTY) k_ssim_bwd(const float* __restrict__ partial, const float* __restrict__ x,
                                                        const float* __restrict__ y, uint32_t W, uint32_t H,
                                                        Window win, float lambda, float* __restrict__ dl) {
    __shared__ float sp[3][kHY][kHX];
    __shared__ float hp[3][kHY][kTX];
    const int ch = blockIdx.z;
    const int tx0 = blockIdx.x * kTX - kR, ty0 = blockIdx.y * kTY - kR;
    const int tid = threadIdx.y * kTX + threadIdx.x;
    const size_t P = (size_t)W * H;
    for (int i = tid; i < kHX * kHY; i += kTX * kTY) {
        const int lx = i % kHX, ly = i / kHX, gx = tx0 + lx, gy = ty0 + ly;
        const bool in = gx >= 0 && gx < (int)W && gy >= 0 && gy < (int)H;
        const size_t o = in ? (size_t)gy * W + gx : 0;
#pragma unroll
        for (int q = 0; q < 3; ++q) sp[q][ly][lx] = in ? partial[(ch * 3 + q) * P + o] : 0.0f;
    }
    __syncthreads();
    for (int i = tid; i < kTX * kHY; i += kTX * kTY) {
        const int c = i % kTX, r = i / kTX;
        float s[3] = {0, 0, 0};
#pragma unroll
        for (int k = 0; k < 11; ++k) {
            const float w = win.w[k];
#pragma unroll
            for (int q = 0; q < 3; ++q) s[q] += w * sp[q][r][c + k];
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) hp[q][r][c] = s[q];
    }
    __syncthreads();
    const int c = threadIdx.x, r = threadIdx.y;
    const int gx = blockIdx.x * kTX + c, gy = blockIdx.y * kTY + r;
    if (gx >= (int)W || gy >= (int)H) return;
    float b[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < 11; ++k) {
        const float w = win.w[k];
#pragma unroll
        for (int q = 0; q < 3; ++q) b[q] += w * hp[q][r + k][c];
    }
    const size_t q = ((size_t)gy * W + gx) * 3 + ch;
    const float xv = x[q], yv = y[q], d = xv - yv;
    const float inv = 1.0f / (float)(3 * P);
    const float g_l1 = (d > 0.0f ? inv : (d < 0.0f ? -inv : 0.0f));
    dl[q] = g_l1 - lambda * inv * (b[0] + 2.0f * xv * b[1] + yv * b[2]);
}

// sums[0..1] = column sums of the per-block partials that follow them
__global__ void k_reduce_sums(double* __restrict__ sums, size_t blocks) {
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
    return dim3((width + kTX - 1) / kTX, (height + kTY - 1) / kTY, 3);
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
    const dim3 grid = loss_grid(width, height), block(kTX, kTY);
    k_ssim_fwd<<<grid, block, 0, s>>>(x, y, width, height, win, scratch, sums + 2);
    k_reduce_sums<<<1, 1024, 0, s>>>(sums, (size_t)grid.x * grid.y * grid.z);
    if (dl) k_ssim_bwd<<<grid, block, 0, s>>>(scratch, x, y, width, height, win, lambda, dl);
}

}  // namespace gs
