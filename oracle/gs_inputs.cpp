// gs_inputs.cpp -- TEST INFRASTRUCTURE ONLY: the inputs of the benchmark configurations, built on
// the CPU without the product library, for the timed CPU baseline (bench.py --impl reference) and as
// an independent cross-check of the product's host utilities (tests/test_oracle_inputs.py).
//
//   oracle_camera_view   Camera.getUniform() (src/renderer/camera.js:87-98) with the lookAt and
//                        0..1-depth perspective of camera.js:135-142 (wgpu-matrix 3.4.2, not vendored;
//                        restated from its published definitions), evaluated in double and rounded to
//                        f32 once per stored element, packed as renderer.js:773-797 packs it.
//   oracle_synth_scene   the seeded synthetic scenes of the benchmark configurations: counter-based
//                        hashing to uniforms, Box-Muller normals with log and cos evaluated by series
//                        in plain IEEE double arithmetic (no libm), so every host makes the same bytes.
//   oracle_perturb_scene the target scene of the differentiation workload (means and SH perturbed).
// Built with -ffp-contract=off, like the product's host code.
#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

// ---- camera --------------------------------------------------------------------------------------
struct V3 {
    double x, y, z;
};
V3 v_sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
double v_dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 v_cross(const V3& a, const V3& b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V3 v_unit(const V3& a) {
    const double len = std::sqrt(v_dot(a, a));
    if (!(len > 0.0)) return {0.0, 0.0, 0.0};
    return {a.x / len, a.y / len, a.z / len};
}

constexpr double kPi = 3.141592653589793;

// ---- seeded draws --------------------------------------------------------------------------------
// splitmix64 finaliser
uint64_t finalize64(uint64_t v) {
    v ^= v >> 30;
    v *= 0xBF58476D1CE4E5B9ull;
    v ^= v >> 27;
    v *= 0x94D049BB133111EBull;
    return v ^ (v >> 31);
}

// uniform in (0, 1) for (seed, stream, counter): three rounds of the finaliser over the mixed words
double draw_uniform(uint64_t seed, uint64_t stream, uint64_t counter) {
    uint64_t h = finalize64(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull);
    h = finalize64(h ^ (stream * 0xD1B54A32D192ED03ull));
    h = finalize64(h ^ (counter * 0xA24BAED4963EE407ull + 0x2545F4914F6CDD1Dull));
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// natural log of u in (0, 1] via u = m * 2^e, m in [1/sqrt(2), sqrt(2)), ln m = 2 atanh((m-1)/(m+1))
double series_log(double u) {
    int e = 0;
    double m = std::frexp(u, &e);
    if (m < 0.70710678118654752) {
        m *= 2.0;
        e -= 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double power = s, acc = 0.0;
    for (int k = 0; k < 14; ++k) {
        acc = acc + power / (double)(2 * k + 1);
        power = power * s2;
    }
    return (double)e * 0.6931471805599453 + 2.0 * acc;
}

// cos(2 pi u): reduce to [0, 1/4] by symmetry, then a Taylor series of cos or of sin on |x| <= pi/4
double series_cos_turns(double u) {
    double v = u - std::floor(u + 0.5);
    if (v < 0) v = -v;
    double sign = 1.0;
    if (v > 0.25) {
        v = 0.5 - v;
        sign = -1.0;
    }
    const double two_pi = 6.283185307179586;
    double acc = 0.0;
    if (v <= 0.125) {
        const double x = two_pi * v, x2 = x * x;
        double term = 1.0;
        for (int k = 0; k < 12; ++k) {
            acc = acc + term;
            term = -term * x2 / (double)((2 * k + 1) * (2 * k + 2));
        }
    } else {
        const double x = two_pi * (0.25 - v), x2 = x * x;
        double term = x;
        for (int k = 0; k < 12; ++k) {
            acc = acc + term;
            term = -term * x2 / (double)((2 * k + 2) * (2 * k + 3));
        }
    }
    return sign * acc;
}

double draw_normal(uint64_t seed, uint64_t stream, uint64_t i) {
    const double a = draw_uniform(seed, stream, 2 * i);
    const double b = draw_uniform(seed, stream, 2 * i + 1);
    return std::sqrt(-2.0 * series_log(a)) * series_cos_turns(b);
}

// one independent stream per attribute
constexpr uint64_t kDrawMean = 1, kDrawScale = 2, kDrawQuat = 3, kDrawOpacity = 4, kDrawDc = 5, kDrawRest = 6,
                   kDrawCluster = 7, kDrawClusterPick = 8, kDrawPerturbMean = 9, kDrawPerturbSh = 10;

// N(0,1)^4 normalised; (w, x, y, z)
void draw_unit_quat(uint64_t seed, uint64_t stream, uint64_t i, double q[4]) {
    double sq = 0.0;
    for (int k = 0; k < 4; ++k) {
        q[k] = draw_normal(seed, stream, 4 * i + k);
        sq += q[k] * q[k];
    }
    const double len = std::sqrt(sq);
    for (int k = 0; k < 4; ++k) q[k] = len > 0 ? q[k] / len : (k == 0 ? 1.0 : 0.0);
}

// rotation matrix [row][col] of the unit quaternion (w, x, y, z)
void rotation_of(const double q[4], double r[3][3]) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    r[0][0] = 1 - 2 * (y * y + z * z);
    r[0][1] = 2 * (x * y - w * z);
    r[0][2] = 2 * (x * z + w * y);
    r[1][0] = 2 * (x * y + w * z);
    r[1][1] = 1 - 2 * (x * x + z * z);
    r[1][2] = 2 * (y * z - w * x);
    r[2][0] = 2 * (x * z - w * y);
    r[2][1] = 2 * (y * z + w * x);
    r[2][2] = 1 - 2 * (x * x + y * y);
}

}  // namespace

extern "C" {

// Writes the 176-byte GlobalUniforms block (preprocess.wgsl:2-12). Returns 0, or 1 for bad arguments.
int oracle_camera_view(const float eye[3], const float target[3], const float up[3], float fovy_deg, uint32_t width,
                       uint32_t height, float z_near, float z_far, void* out176) {
    if (!eye || !target || !up || !out176 || width == 0 || height == 0 || !(fovy_deg > 0.0f) ||
        !(fovy_deg < 180.0f) || !(z_near > 0.0f) || !(z_far > z_near))
        return 1;
    float block[44];
    std::memset(block, 0, sizeof(block));
    const V3 e{eye[0], eye[1], eye[2]};
    const V3 t{target[0], target[1], target[2]};
    const V3 u{up[0], up[1], up[2]};
    // lookAt: camera z axis from the target to the eye; the view matrix is the inverse camera frame
    const V3 az = v_unit(v_sub(e, t));
    const V3 ax = v_unit(v_cross(u, az));
    const V3 ay = v_unit(v_cross(az, ax));
    float* view = block;  // column-major
    const V3 axes[3] = {ax, ay, az};
    for (int r = 0; r < 3; ++r) {
        view[0 * 4 + r] = (float)(r == 0 ? ax.x : r == 1 ? ay.x : az.x);
        view[1 * 4 + r] = (float)(r == 0 ? ax.y : r == 1 ? ay.y : az.y);
        view[2 * 4 + r] = (float)(r == 0 ? ax.z : r == 1 ? ay.z : az.z);
        view[3 * 4 + r] = (float)(-v_dot(axes[r], e));
    }
    view[15] = 1.0f;
    // perspective with clip depth in [0, 1]: f = cot(fovy / 2)
    const double aspect = (double)width / (double)height;
    const double fovy = (double)fovy_deg * kPi / 180.0;
    const double f = std::tan(kPi * 0.5 - 0.5 * fovy);
    const double inv_range = 1.0 / ((double)z_near - (double)z_far);
    float proj[16];
    std::memset(proj, 0, sizeof(proj));
    proj[0] = (float)(f / aspect);
    proj[5] = (float)f;
    proj[10] = (float)((double)z_far * inv_range);
    proj[11] = -1.0f;
    proj[14] = (float)((double)z_far * (double)z_near * inv_range);
    // viewProj = proj * view (column-major), each element a double dot product rounded once
    float* view_proj = block + 16;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double acc = 0.0;
            for (int k = 0; k < 4; ++k) acc += (double)proj[k * 4 + r] * (double)view[c * 4 + k];
            view_proj[c * 4 + r] = (float)acc;
        }
    block[32] = eye[0];
    block[33] = eye[1];
    block[34] = eye[2];
    // count (offset 35) stays 0: the scene's count is used
    const double tan_y = std::tan(fovy / 2.0);
    const double tan_x = tan_y * aspect;
    block[36] = (float)((double)width / (2.0 * tan_x));
    block[37] = (float)((double)height / (2.0 * tan_y));
    block[38] = (float)tan_x;
    block[39] = (float)tan_y;
    block[40] = (float)width;
    block[41] = (float)height;
    std::memcpy(out176, block, 176);
    return 0;
}

// Seeded synthetic scene in the packed layout (59 * count floats). kind 0: N(0,1)^3 means; kind 1:
// a mixture of `clusters` anisotropic clusters (centres U(-box/2, box/2)^3, axis sigma U(0.3, 2.5),
// random rotation, uniform pick) clipped to the box. Log-scales N(-4, 0.5^2), quaternions N(0,1)^4
// normalised, opacity logits N(0, 1.5^2), DC N(0, 0.5^2), rest N(0, 0.05^2). Returns 0, or 1.
int oracle_synth_scene(uint32_t kind, uint32_t count, uint64_t seed, uint32_t clusters, float box, float* packed) {
    if (!packed || kind > 1u || (kind == 1u && (clusters == 0u || !(box > 0.0f)))) return 1;
    const uint64_t n = count;
    float* pos = packed;
    float* lsc = packed + 3 * n;
    float* rot = packed + 6 * n;
    float* dc = packed + 10 * n;
    float* opa = packed + 13 * n;
    float* rest = packed + 14 * n;
    const uint32_t nc = kind == 1u ? clusters : 0u;
    struct Cluster {
        double centre[3], sigma[3], r[3][3];
    };
    Cluster* tab = nc ? new Cluster[nc] : nullptr;
    for (uint32_t k = 0; k < nc; ++k) {
        for (int a = 0; a < 3; ++a) tab[k].centre[a] = (draw_uniform(seed, kDrawCluster, 16 * k + a) - 0.5) * (double)box;
        for (int a = 0; a < 3; ++a) tab[k].sigma[a] = 0.3 + 2.2 * draw_uniform(seed, kDrawCluster, 16 * k + 3 + a);
        double q[4];
        draw_unit_quat(seed, kDrawCluster + 1000, k, q);
        rotation_of(q, tab[k].r);
    }
    const double lim = 0.5 * (double)box;
#pragma omp parallel for schedule(static)
    for (int64_t gi = 0; gi < (int64_t)n; ++gi) {
        const uint64_t g = (uint64_t)gi;
        double z[3];
        for (int a = 0; a < 3; ++a) z[a] = draw_normal(seed, kDrawMean, 3 * g + a);
        if (nc == 0u) {
            for (int a = 0; a < 3; ++a) pos[3 * g + a] = (float)z[a];
        } else {
            uint32_t k = (uint32_t)(draw_uniform(seed, kDrawClusterPick, g) * (double)nc);
            if (k >= nc) k = nc - 1u;
            const Cluster& c = tab[k];
            for (int r = 0; r < 3; ++r) {
                double v = c.centre[r];
                for (int s = 0; s < 3; ++s) v += c.r[r][s] * (c.sigma[s] * z[s]);
                if (v < -lim) v = -lim;
                if (v > lim) v = lim;
                pos[3 * g + r] = (float)v;
            }
        }
        for (int a = 0; a < 3; ++a) lsc[3 * g + a] = (float)(-4.0 + 0.5 * draw_normal(seed, kDrawScale, 3 * g + a));
        double q[4];
        draw_unit_quat(seed, kDrawQuat, g, q);
        for (int a = 0; a < 4; ++a) rot[4 * g + a] = (float)q[a];
        opa[g] = (float)(1.5 * draw_normal(seed, kDrawOpacity, g));
        for (int a = 0; a < 3; ++a) dc[3 * g + a] = (float)(0.5 * draw_normal(seed, kDrawDc, 3 * g + a));
        for (int a = 0; a < 45; ++a) rest[45 * g + a] = (float)(0.05 * draw_normal(seed, kDrawRest, 45 * g + a));
    }
    delete[] tab;
    return 0;
}

// In place: means += N(0, sigma_mean^2), DC and rest += N(0, sigma_sh^2). Returns 0, or 1.
int oracle_perturb_scene(float* packed, uint32_t count, uint64_t seed, float sigma_mean, float sigma_sh) {
    if (!packed) return 1;
    const uint64_t n = count;
    float* pos = packed;
    float* dc = packed + 10 * n;
    float* rest = packed + 14 * n;
#pragma omp parallel for schedule(static)
    for (int64_t gi = 0; gi < (int64_t)n; ++gi) {
        const uint64_t g = (uint64_t)gi;
        for (int a = 0; a < 3; ++a)
            pos[3 * g + a] = (float)((double)pos[3 * g + a] + (double)sigma_mean * draw_normal(seed, kDrawPerturbMean, 3 * g + a));
        for (int a = 0; a < 3; ++a)
            dc[3 * g + a] = (float)((double)dc[3 * g + a] + (double)sigma_sh * draw_normal(seed, kDrawPerturbSh, 48 * g + a));
        for (int a = 0; a < 45; ++a)
            rest[45 * g + a] =
                (float)((double)rest[45 * g + a] + (double)sigma_sh * draw_normal(seed, kDrawPerturbSh, 48 * g + 3 + a));
    }
    return 0;
}

}  // extern "C"
