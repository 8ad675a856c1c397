// gs_camera.cu -- the uniform builder on the device: Camera.getUniform() (src/renderer/camera.js:87-98,
// lookAt / perspective of :135-142) for a batch of cameras, one thread per camera, with the same
// function the host's gs_camera_view runs (gs_camera.h), so the blocks are the same bits. A batch of
// orbit views then uploads 56-byte cameras instead of 176-byte blocks, and the blocks are built inside
// the batch's captured graph.
#include "gs_camera.h"
#include "gs_kernels.h"

namespace gs {
namespace {

__global__ void k_camera_views(const gs_camera* __restrict__ cams, uint32_t n, ViewBlock* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float block[44];
    gs_cam::camera_block(cams[i], block);
    float4* dst = reinterpret_cast<float4*>(out + i);  // 176 = 11 x 16 bytes; blocks are 16-byte aligned
#pragma unroll
    for (int k = 0; k < 11; ++k) dst[k] = make_float4(block[4 * k], block[4 * k + 1], block[4 * k + 2], block[4 * k + 3]);
}

}  // namespace

void launch_camera_views(const gs_camera* cams, uint32_t n, ViewBlock* out, cudaStream_t s) {
    if (n == 0) return;
    k_camera_views<<<(n + 63u) / 64u, 64, 0, s>>>(cams, n, out);
}

}  // namespace gs
