// gs_host.cpp -- host utilities of libwebgs.so that need no GPU: the camera uniform builder and
// the seeded synthetic scene generator. Compiled with -ffp-contract=off so that results are
// bit-identical on x86-64 and aarch64 hosts.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/gs.h"

namespace {

// ---- camera: src/renderer/camera.js:87-98 and :135-142 ---------------------------------------
// wgpu-matrix (3.4.2, not vendored) lookAt builds the inverse of a camera frame whose z axis points
// from the target to the eye; perspective maps view depth [near, far] to clip depth [0, 1] (WebGPU
// convention). Both are restated here from their published definitions; the reference stores every
// matrix in a Float32Array, so each element is rounded to f32 once.
struct D3 { double x, y, z; };
D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
D3 normalize(D3 a) {
    const double l = std::sqrt(dot(a, a));
    return l > 0 ? D3{a.x / l, a.y / l, a.z / l} : D3{0, 0, 0};
}

// ---- deterministic normal draws ------------------------------------------------------------
// Counter-based: every (seed, stream, index) maps to its own 64-bit hash, so generation order and
// thread count never change the scene. log and cos are evaluated by series with basic IEEE double
// operations only, so no libm differences between hosts can leak into the data.
uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double uniform01(uint64_t seed, uint64_t stream, uint64_t counter) {
    uint64_t h = mix64(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull);
    h = mix64(h ^ (stream * 0xD1B54A32D192ED03ull));
    h = mix64(h ^ (counter * 0xA24BAED4963EE407ull + 0x2545F4914F6CDD1Dull));
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);  // (0, 1)
}
// ln(u), u in (0, 1]: u = m 2^e with m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(s), s = (m-1)/(m+1).
double det_log(double u) {
    int e = 0;
    double m = std::frexp(u, &e);  // exact
    if (m < 0.70710678118654752) { m *= 2.0; e -= 1; }
    const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
    double term = s, sum = 0.0;
    for (int k = 0; k < 14; ++k) {
        sum = sum + term / (double)(2 * k + 1);
        term = term * s2;
    }
    return (double)e * 0.6931471805599453 + 2.0 * sum;
}
// cos(2 pi u) for u in (0, 1) by octant reduction and Taylor series on |x| <= pi/4.
double det_cos2pi(double u) {
    double v = u - std::floor(u + 0.5);  // [-0.5, 0.5)
    if (v < 0) v = -v;                   // cos is even
    double sign = 1.0;
    if (v > 0.25) { v = 0.5 - v; sign = -1.0; }  // cos(pi - a) = -cos(a)
    const double kTwoPi = 6.283185307179586;
    double r;
    if (v <= 0.125) {
        const double x = kTwoPi * v, x2 = x * x;
        double term = 1.0, sum = 0.0;
        for (int k = 0; k < 12; ++k) {
            sum = sum + term;
            term = -term * x2 / (double)((2 * k + 1) * (2 * k + 2));
        }
        r = sum;
    } else {
        const double x = kTwoPi * (0.25 - v), x2 = x * x;  // cos(pi/2 - a) = sin(a)
        double term = x, sum = 0.0;
        for (int k = 0; k < 12; ++k) {
            sum = sum + term;
            term = -term * x2 / (double)((2 * k + 2) * (2 * k + 3));
        }
        r = sum;
    }
    return sign * r;
}
double normal01(uint64_t seed, uint64_t stream, uint64_t i) {
    const double u1 = uniform01(seed, stream, 2 * i), u2 = uniform01(seed, stream, 2 * i + 1);
    return std::sqrt(-2.0 * det_log(u1)) * det_cos2pi(u2);
}

enum Stream : uint64_t {
    kMean = 1, kScale = 2, kQuat = 3, kOpacity = 4, kDc = 5, kRest = 6,
    kCluster = 7, kClusterPick = 8, kPerturbMean = 9, kPerturbSh = 10
};

void quat_to_mat(const double q[4], double m[3][3]) {  // q = (w, x, y, z), unit
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    m[0][0] = 1 - 2 * (y * y + z * z); m[0][1] = 2 * (x * y - w * z);     m[0][2] = 2 * (x * z + w * y);
    m[1][0] = 2 * (x * y + w * z);     m[1][1] = 1 - 2 * (x * x + z * z); m[1][2] = 2 * (y * z - w * x);
    m[2][0] = 2 * (x * z - w * y);     m[2][1] = 2 * (y * z + w * x);     m[2][2] = 1 - 2 * (x * x + y * y);
}

void unit_quat(uint64_t seed, uint64_t stream, uint64_t i, double q[4]) {
    double l2 = 0;
    for (int k = 0; k < 4; ++k) {
        q[k] = normal01(seed, stream, 4 * i + k);
        l2 += q[k] * q[k];
    }
    const double l = std::sqrt(l2);
    for (int k = 0; k < 4; ++k) q[k] = l > 0 ? q[k] / l : (k == 0 ? 1.0 : 0.0);
}

}  // namespace

extern "C" int gs_camera_view(const float eye[3], const float target[3], const float up[3], float fovy_deg,
                              uint32_t width, uint32_t height, float z_near, float z_far, gs_view* out) {
    if (!eye || !target || !up || !out || width == 0 || height == 0 || !(fovy_deg > 0.0f) || !(fovy_deg < 180.0f) ||
        !(z_near > 0.0f) || !(z_far > z_near))
        return GS_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    const D3 e{eye[0], eye[1], eye[2]}, t{target[0], target[1], target[2]}, u{up[0], up[1], up[2]};
    const D3 zA = normalize(sub(e, t));
    const D3 xA = normalize(cross(u, zA));
    const D3 yA = normalize(cross(zA, xA));
    float view[16] = {(float)xA.x, (float)yA.x, (float)zA.x, 0.0f,
                      (float)xA.y, (float)yA.y, (float)zA.y, 0.0f,
                      (float)xA.z, (float)yA.z, (float)zA.z, 0.0f,
                      (float)-dot(xA, e), (float)-dot(yA, e), (float)-dot(zA, e), 1.0f};
    const double aspect = (double)width / (double)height;
    const double fovy = (double)fovy_deg * 3.141592653589793 / 180.0;
    const double f = std::tan(3.141592653589793 * 0.5 - 0.5 * fovy);
    const double rangeInv = 1.0 / ((double)z_near - (double)z_far);
    float proj[16] = {0};
    proj[0] = (float)(f / aspect);
    proj[5] = (float)f;
    proj[10] = (float)((double)z_far * rangeInv);
    proj[11] = -1.0f;
    proj[14] = (float)((double)z_far * (double)z_near * rangeInv);
    // mat4.multiply(projection, view): column-major product computed in double, stored as f32.
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += (double)proj[k * 4 + r] * (double)view[c * 4 + k];
            out->view_proj[c * 4 + r] = (float)s;
        }
    std::memcpy(out->view, view, sizeof(view));
    out->camera_pos[0] = eye[0];
    out->camera_pos[1] = eye[1];
    out->camera_pos[2] = eye[2];
    const double tanFovY = std::tan(fovy / 2.0), tanFovX = tanFovY * aspect;
    out->focal[0] = (float)((double)width / (2.0 * tanFovX));
    out->focal[1] = (float)((double)height / (2.0 * tanFovY));
    out->tan_fov[0] = (float)tanFovX;
    out->tan_fov[1] = (float)tanFovY;
    out->texture_size[0] = (float)width;
    out->texture_size[1] = (float)height;
    return GS_OK;
}

extern "C" int gs_synth_scene(uint32_t kind, uint32_t count, uint64_t seed, uint32_t clusters, float box,
                              float* packed) {
    if (!packed || kind > 1u || (kind == 1u && (clusters == 0u || !(box > 0.0f)))) return GS_ERR_INVALID;
    const uint64_t n = count;
    float* pos = packed;
    float* scale = pos + 3 * n;
    float* quat = scale + 3 * n;
    float* dc = quat + 4 * n;
    float* opac = dc + 3 * n;
    float* rest = opac + n;

    // Cluster table for kind 1: centres U(-box/2, box/2)^3, axis sigma U(0.3, 2.5), random rotation.
    const uint32_t K = kind == 1u ? clusters : 0u;
    double* ctab = K ? new double[(size_t)K * 15] : nullptr;  // centre(3) sigma(3) rot(9)
    for (uint32_t k = 0; k < K; ++k) {
        double* c = ctab + (size_t)k * 15;
        for (int a = 0; a < 3; ++a) c[a] = (uniform01(seed, kCluster, 16 * k + a) - 0.5) * (double)box;
        for (int a = 0; a < 3; ++a) c[3 + a] = 0.3 + 2.2 * uniform01(seed, kCluster, 16 * k + 3 + a);
        double q[4], m[3][3];
        unit_quat(seed, kCluster + 1000, k, q);
        quat_to_mat(q, m);
        for (int r = 0; r < 3; ++r)
            for (int s = 0; s < 3; ++s) c[6 + 3 * r + s] = m[r][s];
    }
    const double half = 0.5 * (double)box;

#pragma omp parallel for schedule(static)
    for (int64_t gi = 0; gi < (int64_t)n; ++gi) {
        const uint64_t g = (uint64_t)gi;
        double z[3];
        for (int a = 0; a < 3; ++a) z[a] = normal01(seed, kMean, 3 * g + a);
        if (K == 0u) {
            for (int a = 0; a < 3; ++a) pos[3 * g + a] = (float)z[a];
        } else {
            uint32_t k = (uint32_t)(uniform01(seed, kClusterPick, g) * (double)K);
            if (k >= K) k = K - 1u;
            const double* c = ctab + (size_t)k * 15;
            for (int r = 0; r < 3; ++r) {
                double v = c[r];
                for (int s = 0; s < 3; ++s) v += c[6 + 3 * r + s] * (c[3 + s] * z[s]);
                v = v < -half ? -half : (v > half ? half : v);
                pos[3 * g + r] = (float)v;
            }
        }
        for (int a = 0; a < 3; ++a) scale[3 * g + a] = (float)(-4.0 + 0.5 * normal01(seed, kScale, 3 * g + a));
        double q[4];
        unit_quat(seed, kQuat, g, q);
        for (int a = 0; a < 4; ++a) quat[4 * g + a] = (float)q[a];
        opac[g] = (float)(1.5 * normal01(seed, kOpacity, g));
        for (int a = 0; a < 3; ++a) dc[3 * g + a] = (float)(0.5 * normal01(seed, kDc, 3 * g + a));
        for (int a = 0; a < 45; ++a) rest[45 * g + a] = (float)(0.05 * normal01(seed, kRest, 45 * g + a));
    }
    delete[] ctab;
    return GS_OK;
}

extern "C" int gs_perturb_scene(float* packed, uint32_t count, uint64_t seed, float sigma_mean, float sigma_sh) {
    if (!packed) return GS_ERR_INVALID;
    const uint64_t n = count;
    float* pos = packed;
    float* dc = packed + 10 * n;
    float* rest = packed + 14 * n;
#pragma omp parallel for schedule(static)
    for (int64_t gi = 0; gi < (int64_t)n; ++gi) {
        const uint64_t g = (uint64_t)gi;
        for (int a = 0; a < 3; ++a)
            pos[3 * g + a] = (float)((double)pos[3 * g + a] + (double)sigma_mean * normal01(seed, kPerturbMean, 3 * g + a));
        for (int a = 0; a < 3; ++a)
            dc[3 * g + a] = (float)((double)dc[3 * g + a] + (double)sigma_sh * normal01(seed, kPerturbSh, 48 * g + a));
        for (int a = 0; a < 45; ++a)
            rest[45 * g + a] = (float)((double)rest[45 * g + a] + (double)sigma_sh * normal01(seed, kPerturbSh, 48 * g + 3 + a));
    }
    return GS_OK;
}
