// gs_camera.h -- Camera.getUniform() (src/renderer/camera.js:87-98) with the lookAt and 0..1-depth
// perspective of camera.js:135-142 (wgpu-matrix 3.4.2, not vendored; restated from its published
// definitions), as one function compiled for both the host (gs_camera_view, gs_host.cpp) and the
// device (k_camera_views, gs_camera.cu), so the two give the same bits by construction.
//
// Everything is evaluated in IEEE double (correctly rounded + - * / and sqrt; no contraction: the host
// code is built with -ffp-contract=off and the device code with -fmad=false) and each stored element is
// rounded to f32 once, as the reference's Float32Array stores round it. The tangent is this file's own
// series in plain double arithmetic (no libm, no device math library), so host and device agree.
#pragma once
#include <cmath>
#include <cstdint>

#include "../../include/gs.h"

#ifdef __CUDACC__
#define GS_HD __host__ __device__ __forceinline__
#else
#define GS_HD inline
#endif

namespace gs_cam {

struct D3 {
    double x, y, z;
};
GS_HD D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
GS_HD D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
GS_HD double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GS_HD D3 normalize(D3 a) {
    const double l = sqrt(dot(a, a));
    if (l > 0) return D3{a.x / l, a.y / l, a.z / l};
    return D3{0, 0, 0};
}

// sin and cos of x in [0, pi/4] by their Taylor series (22 terms: the truncation is far below one
// double ulp there).
GS_HD double sin_series(double x) {
    const double x2 = x * x;
    double term = x, sum = 0.0;
    for (int k = 0; k < 11; ++k) {
        sum = sum + term;
        term = -term * x2 / (double)((2 * k + 2) * (2 * k + 3));
    }
    return sum;
}
GS_HD double cos_series(double x) {
    const double x2 = x * x;
    double term = 1.0, sum = 0.0;
    for (int k = 0; k < 11; ++k) {
        sum = sum + term;
        term = -term * x2 / (double)((2 * k + 1) * (2 * k + 2));
    }
    return sum;
}
// tan(x) for x in (0, pi/2): sin/cos on [0, pi/4], cot(pi/2 - x) above it.
GS_HD double tan_half_open(double x) {
    const double kQuarterPi = 0.78539816339744831, kHalfPi = 1.5707963267948966;
    if (x <= kQuarterPi) return sin_series(x) / cos_series(x);
    const double y = kHalfPi - x;
    return cos_series(y) / sin_series(y);
}

GS_HD bool camera_valid(const gs_camera& c) {
    return c.width > 0u && c.height > 0u && c.fovy_deg > 0.0f && c.fovy_deg < 180.0f && c.z_near > 0.0f &&
           c.z_far > c.z_near;
}

// The 176-byte GlobalUniforms block (preprocess.wgsl:2-12) as packed by renderer.js:773-797, written
// into out[44] (the count word stays 0: the scene's count is used). The camera must be valid.
GS_HD void camera_block(const gs_camera& c, float out[44]) {
    for (int i = 0; i < 44; ++i) out[i] = 0.0f;
    const D3 e{c.eye[0], c.eye[1], c.eye[2]}, t{c.target[0], c.target[1], c.target[2]}, u{c.up[0], c.up[1], c.up[2]};
    // lookAt: the camera's z axis points from the target to the eye; the view matrix (column-major)
    // is the inverse of the camera frame
    const D3 zA = normalize(sub(e, t));
    const D3 xA = normalize(cross(u, zA));
    const D3 yA = normalize(cross(zA, xA));
    float* view = out;
    view[0] = (float)xA.x; view[1] = (float)yA.x; view[2] = (float)zA.x;
    view[4] = (float)xA.y; view[5] = (float)yA.y; view[6] = (float)zA.y;
    view[8] = (float)xA.z; view[9] = (float)yA.z; view[10] = (float)zA.z;
    view[12] = (float)-dot(xA, e); view[13] = (float)-dot(yA, e); view[14] = (float)-dot(zA, e);
    view[15] = 1.0f;
    // perspective: f = cot(fovy / 2), clip depth in [0, 1]
    const double aspect = (double)c.width / (double)c.height;
    const double fovy = (double)c.fovy_deg * 3.141592653589793 / 180.0;
    const double f = tan_half_open(3.141592653589793 * 0.5 - 0.5 * fovy);
    const double range_inv = 1.0 / ((double)c.z_near - (double)c.z_far);
    float proj[16];
    for (int i = 0; i < 16; ++i) proj[i] = 0.0f;
    proj[0] = (float)(f / aspect);
    proj[5] = (float)f;
    proj[10] = (float)((double)c.z_far * range_inv);
    proj[11] = -1.0f;
    proj[14] = (float)((double)c.z_far * (double)c.z_near * range_inv);
    // mat4.multiply(projection, view): each element a double dot product over k, rounded once
    float* view_proj = out + 16;
    for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 4; ++row) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += (double)proj[k * 4 + row] * (double)view[col * 4 + k];
            view_proj[col * 4 + row] = (float)s;
        }
    out[32] = c.eye[0];
    out[33] = c.eye[1];
    out[34] = c.eye[2];
    const double tan_y = tan_half_open(fovy / 2.0), tan_x = tan_y * aspect;
    out[36] = (float)((double)c.width / (2.0 * tan_x));
    out[37] = (float)((double)c.height / (2.0 * tan_y));
    out[38] = (float)tan_x;
    out[39] = (float)tan_y;
    out[40] = (float)c.width;
    out[41] = (float)c.height;
}

}  // namespace gs_cam
