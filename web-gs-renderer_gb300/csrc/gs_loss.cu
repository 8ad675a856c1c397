// gs_loss.cu -- L = mean|x - y| + lambda * (1 - mean SSIM) and dL/dx on the device, for the
// differentiation workload (no counterpart in the reference). SSIM is per channel with an 11x11
// Gaussian window (sigma 1.5, normalised, separable), zero padding, C1 = 0.01^2, C2 = 0.03^2. With
// the filtered moments m1 = G*x, m2 = G*x^2, mxy = G*(xy) the gradient is
//   dSSIM/dx = G*(dS/dm1) + 2x G*(dS/dm2) + y G*(dS/dmxy)
// (the window is symmetric), so the whole loss is four separable passes: horizontal and vertical
// blurs of the five moments (the vertical pass also forms the SSIM map and its three partials), then
// horizontal and vertical blurs of the partials combined with the L1 term. Images are H x W x 3.
#include <cmath>

#include "gs_kernels.h"

namespace gs {
namespace {

struct Window {
    float w[11];
};

// one thread per (pixel, channel): horizontal 11-tap sums of x, y, x^2, y^2, xy
__global__ void k_moments_h(const float* __restrict__ x, const float* __restrict__ y, uint32_t W, uint32_t H,
                            Window win, float* __restrict__ out /* 15 planes: (ch*5 + k) */) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y, ch = blockIdx.z;
    if (px >= W) return;
    float s[5] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int i = -5; i <= 5; ++i) {
        const int xx = (int)px + i;
        if (xx < 0 || xx >= (int)W) continue;
        const size_t q = ((size_t)py * W + xx) * 3 + ch;
        const float a = x[q], b = y[q], w = win.w[i + 5];
        s[0] += w * a;
        s[1] += w * b;
        s[2] += w * a * a;
        s[3] += w * b * b;
        s[4] += w * a * b;
    }
    const size_t P = (size_t)W * H, o = (size_t)py * W + px;
#pragma unroll
    for (int k = 0; k < 5; ++k) out[(ch * 5 + k) * P + o] = s[k];
}

// vertical sums -> SSIM map partials (3 planes per channel) and the SSIM / L1 sums
__global__ void k_moments_v(const float* __restrict__ hm, const float* __restrict__ x, const float* __restrict__ y,
                            uint32_t W, uint32_t H, Window win, float* __restrict__ partial /* 9 planes */,
                            double* __restrict__ sums /* [ssim, l1] */) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y, ch = blockIdx.z;
    const float C1 = 0.01f * 0.01f, C2 = 0.03f * 0.03f;
    float ssim = 0.0f, l1 = 0.0f;
    if (px < W) {
        const size_t P = (size_t)W * H;
        float m[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int i = -5; i <= 5; ++i) {
            const int yy = (int)py + i;
            if (yy < 0 || yy >= (int)H) continue;
            const size_t o = (size_t)yy * W + px;
            const float w = win.w[i + 5];
#pragma unroll
            for (int k = 0; k < 5; ++k) m[k] += w * hm[(ch * 5 + k) * P + o];
        }
        const float mx = m[0], my = m[1];
        const float sxx = m[2] - mx * mx, syy = m[3] - my * my, sxy = m[4] - mx * my;
        const float A1 = 2.0f * mx * my + C1, A2 = 2.0f * sxy + C2;
        const float B1 = mx * mx + my * my + C1, B2 = sxx + syy + C2;
        const float s = A1 * A2 / (B1 * B2);
        const float ds_dmx = (2.0f * my * A2) / (B1 * B2) - s * (2.0f * mx) / B1;
        const float ds_dsxx = -s / B2;
        const float ds_dsxy = 2.0f * A1 / (B1 * B2);
        const size_t o = (size_t)py * W + px;
        partial[(ch * 3 + 0) * P + o] = ds_dmx + ds_dsxx * (-2.0f * mx) + ds_dsxy * (-my);
        partial[(ch * 3 + 1) * P + o] = ds_dsxx;
        partial[(ch * 3 + 2) * P + o] = ds_dsxy;
        ssim = s;
        const size_t q = o * 3 + ch;
        l1 = fabsf(x[q] - y[q]);
    }
    // block reduction, one double atomic per block and quantity
    __shared__ float red[2][32];
    float a = ssim, b = l1;
    for (int k = 16; k > 0; k >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, k);
        b += __shfl_xor_sync(0xffffffffu, b, k);
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0) { red[0][warp] = a; red[1][warp] = b; }
    __syncthreads();
    if (warp == 0) {
        const uint32_t nw = blockDim.x >> 5;
        a = lane < nw ? red[0][lane] : 0.0f;
        b = lane < nw ? red[1][lane] : 0.0f;
        for (int k = 16; k > 0; k >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, k);
            b += __shfl_xor_sync(0xffffffffu, b, k);
        }
        if (lane == 0) {  // one partial per block; k_reduce_sums adds them (no contended atomics)
            const size_t blk = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
            sums[2 * blk] = (double)a;
            sums[2 * blk + 1] = (double)b;
        }
    }
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

__global__ void k_partial_h(const float* __restrict__ partial, uint32_t W, uint32_t H, Window win,
                            float* __restrict__ out /* 9 planes */) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y, plane = blockIdx.z;
    if (px >= W) return;
    const size_t P = (size_t)W * H;
    const float* src = partial + plane * P + (size_t)py * W;
    float s = 0.0f;
#pragma unroll
    for (int i = -5; i <= 5; ++i) {
        const int xx = (int)px + i;
        if (xx >= 0 && xx < (int)W) s += win.w[i + 5] * src[xx];
    }
    out[plane * P + (size_t)py * W + px] = s;
}

__global__ void k_partial_v(const float* __restrict__ hp, const float* __restrict__ x, const float* __restrict__ y,
                            uint32_t W, uint32_t H, Window win, float lambda, float* __restrict__ dl) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y, ch = blockIdx.z;
    if (px >= W) return;
    const size_t P = (size_t)W * H;
    float b[3] = {0, 0, 0};
#pragma unroll
    for (int i = -5; i <= 5; ++i) {
        const int yy = (int)py + i;
        if (yy < 0 || yy >= (int)H) continue;
        const size_t o = (size_t)yy * W + px;
        const float w = win.w[i + 5];
#pragma unroll
        for (int k = 0; k < 3; ++k) b[k] += w * hp[(ch * 3 + k) * P + o];
    }
    const size_t q = ((size_t)py * W + px) * 3 + ch;
    const float xv = x[q], yv = y[q], d = xv - yv;
    const float inv = 1.0f / (float)(3 * P);
    const float g_l1 = (d > 0.0f ? inv : (d < 0.0f ? -inv : 0.0f));
    dl[q] = g_l1 - lambda * inv * (b[0] + 2.0f * xv * b[1] + yv * b[2]);
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

}  // namespace

size_t loss_scratch_floats(uint32_t width, uint32_t height) { return (size_t)width * height * (15 + 9 + 9); }

size_t loss_sum_doubles(uint32_t width, uint32_t height) {
    return 2 + 2 * (size_t)((width + 127u) / 128u) * height * 3;
}

void launch_loss_l1_ssim(const float* x, const float* y, uint32_t width, uint32_t height, float lambda,
                         float* scratch, double* sums, float* dl, cudaStream_t s) {
    const Window win = make_window();
    const size_t P = (size_t)width * height;
    float* hm = scratch;
    float* partial = hm + 15 * P;
    float* hp = partial + 9 * P;
    const dim3 block(128);
    const uint32_t bx = (width + 127u) / 128u;
    k_moments_h<<<dim3(bx, height, 3), block, 0, s>>>(x, y, width, height, win, hm);
    k_moments_v<<<dim3(bx, height, 3), block, 0, s>>>(hm, x, y, width, height, win, partial, sums + 2);
    k_reduce_sums<<<1, 1024, 0, s>>>(sums, (size_t)bx * height * 3);
    if (dl) {
        k_partial_h<<<dim3(bx, height, 9), block, 0, s>>>(partial, width, height, win, hp);
        k_partial_v<<<dim3(bx, height, 3), block, 0, s>>>(hp, x, y, width, height, win, lambda, dl);
    }
}

}  // namespace gs
