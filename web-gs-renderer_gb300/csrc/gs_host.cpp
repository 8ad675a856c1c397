// gs_host.cpp -- host utilities of libwebgs.so that need no GPU: the camera uniform builder and
// the seeded synthetic scene generator. Compiled with -ffp-contract=off so that results are
// bit-identical on x86-64 and aarch64 hosts.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gs.h"
#include "gs_camera.h"

namespace {

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
    if (!eye || !target || !up || !out) return GS_ERR_INVALID;
    gs_camera c;
    for (int k = 0; k < 3; ++k) {
        c.eye[k] = eye[k];
        c.target[k] = target[k];
        c.up[k] = up[k];
    }
    c.fovy_deg = fovy_deg;
    c.width = width;
    c.height = height;
    c.z_near = z_near;
    c.z_far = z_far;
    if (!gs_cam::camera_valid(c)) return GS_ERR_INVALID;
    float block[44];
    gs_cam::camera_block(c, block);  // the same function the device builder runs (gs_camera.h)
    static_assert(sizeof(block) == sizeof(gs_view), "the view block is 176 bytes");
    std::memcpy(out, block, sizeof(gs_view));
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

// ---- PLY ingest: src/loader/loader.js:56-213 restated -----------------------------------------------
namespace {

struct PlyProp {
    std::string name;
    int type;  // index into kPlyTypes
    uint32_t offset;
};
struct PlyType {
    const char* name;
    uint32_t size;
    int kind;  // 0 signed int, 1 unsigned int, 2 float32, 3 float64
};
const PlyType kPlyTypes[] = {
    {"char", 1, 0},   {"uchar", 1, 1},  {"int8", 1, 0},    {"uint8", 1, 1},   {"short", 2, 0},   {"ushort", 2, 1},
    {"int16", 2, 0},  {"uint16", 2, 1}, {"int", 4, 0},     {"uint", 4, 1},    {"int32", 4, 0},   {"uint32", 4, 1},
    {"float", 4, 2},  {"float32", 4, 2}, {"double", 8, 3}, {"float64", 8, 3},
};

// loader.js:3-11: the 59 properties, in the order of the packed layout (loader.js:75-110, 143-147)
std::vector<std::string> required_properties() {
    std::vector<std::string> r = {"x", "y", "z", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3",
                                  "f_dc_0", "f_dc_1", "f_dc_2", "opacity"};
    for (int i = 0; i < 45; ++i) r.push_back("f_rest_" + std::to_string(i));
    return r;
}

double read_le(const uint8_t* p, const PlyType& t) {  // DataView getters with littleEndian = true
    uint64_t u = 0;
    for (uint32_t i = 0; i < t.size; ++i) u |= (uint64_t)p[i] << (8 * i);
    switch (t.kind) {
        case 0: {
            const uint32_t bits = 8 * t.size;
            int64_t v = (int64_t)u;
            if (bits < 64 && (u >> (bits - 1)) & 1u) v = (int64_t)(u | (~0ull << bits));
            return (double)v;
        }
        case 1: return (double)u;
        case 2: { uint32_t b = (uint32_t)u; float f; std::memcpy(&f, &b, 4); return (double)f; }
        default: { double d; std::memcpy(&d, &u, 8); return d; }
    }
}

int ply_fail(char* err, size_t err_len, const std::string& msg) {
    if (err && err_len) {
        const size_t k = std::min(err_len - 1, msg.size());
        std::memcpy(err, msg.data(), k);
        err[k] = '\0';
    }
    return GS_ERR_INVALID;
}

}  // namespace

extern "C" int gs_ply_parse(const uint8_t* bytes, size_t size, uint32_t* count, float* packed, char* err,
                            size_t err_len) {
    if (!bytes || !count) return ply_fail(err, err_len, "Invalid PLY: null buffer");
    // findHeaderEnd (loader.js:118-136): "end_header", then an optional "\r" and an optional "\n"
    static const char kEnd[] = "end_header";
    const size_t kEndLen = sizeof(kEnd) - 1;
    size_t idx = size;
    for (size_t i = 0; i + kEndLen <= size; ++i)
        if (std::memcmp(bytes + i, kEnd, kEndLen) == 0) { idx = i; break; }
    if (idx == size) return ply_fail(err, err_len, "Invalid PLY: \"end_header\" not found");
    size_t body = idx + kEndLen;
    if (body < size && bytes[body] == '\r') ++body;
    if (body < size && bytes[body] == '\n') ++body;
    // parseHeader (loader.js:151-213)
    std::string header(reinterpret_cast<const char*>(bytes), body);
    long long vcount = 0;
    bool little = false, has_format = false;
    std::string element;
    std::vector<PlyProp> props;
    uint32_t stride = 0;
    size_t pos = 0;
    while (pos <= header.size()) {
        size_t nl = header.find('\n', pos);
        if (nl == std::string::npos) nl = header.size();
        std::vector<std::string> words;
        std::string w;
        for (size_t i = pos; i < nl; ++i) {
            const char ch = header[i];
            if (ch == ' ' || ch == '\t' || ch == '\r' || ch == '\v' || ch == '\f') {
                if (!w.empty()) words.push_back(w);
                w.clear();
            } else {
                w.push_back(ch);
            }
        }
        if (!w.empty()) words.push_back(w);
        pos = nl + 1;
        if (words.empty()) continue;
        if (words[0] == "format") {
            has_format = true;
            little = words.size() > 1 && words[1] == "binary_little_endian";
        }
        if (words[0] == "element") {
            element = words.size() > 1 ? words[1] : "";
            if (element == "vertex") vcount = words.size() > 2 ? std::atoll(words[2].c_str()) : 0;
        }
        if (words[0] == "property" && element == "vertex") {
            if (words.size() > 1 && words[1] == "list")
                return ply_fail(err, err_len, "Invalid PLY: list properties are not supported");
            const std::string type = words.size() > 1 ? words[1] : "";
            int t = -1;
            for (int k = 0; k < (int)(sizeof(kPlyTypes) / sizeof(kPlyTypes[0])); ++k)
                if (type == kPlyTypes[k].name) t = k;
            if (t < 0) return ply_fail(err, err_len, "Invalid PLY: unknown property type \"" + type + "\"");
            props.push_back({words.size() > 2 ? words[2] : "", t, stride});
            stride += kPlyTypes[t].size;
        }
    }
    if (!has_format) return ply_fail(err, err_len, "Invalid PLY: missing \"format\" line");
    if (!little) return ply_fail(err, err_len, "Invalid PLY: unsupported format");
    if (vcount <= 0) return ply_fail(err, err_len, "Invalid PLY: vertex count missing or zero");
    if (vcount > 0xFFFFFFFFll) return ply_fail(err, err_len, "Invalid PLY: vertex count exceeds 2^32-1");
    const std::vector<std::string> req = required_properties();
    std::vector<const PlyProp*> map(req.size(), nullptr);
    for (size_t r = 0; r < req.size(); ++r) {
        for (const PlyProp& p : props)
            if (p.name == req[r]) map[r] = &p;  // last definition wins, as Map(properties) does
        if (!map[r]) return ply_fail(err, err_len, "Invalid PLY: missing required property \"" + req[r] + "\"");
    }
    const uint64_t n = (uint64_t)vcount;
    if (body + n * stride > size) return ply_fail(err, err_len, "Invalid PLY: vertex data truncated");
    *count = (uint32_t)n;
    if (!packed) return GS_OK;
    // loader.js:80-110, 143-147: positions, scales, rotations, f_dc, opacity, f_rest blocks
    const uint64_t width[6] = {3, 3, 4, 3, 1, 45};
    uint64_t base[6];
    base[0] = 0;
    for (int b = 1; b < 6; ++b) base[b] = base[b - 1] + width[b - 1] * n;
#pragma omp parallel for schedule(static)
    for (int64_t gi = 0; gi < (int64_t)n; ++gi) {
        const uint8_t* rec = bytes + body + (uint64_t)gi * stride;
        size_t r = 0;
        for (int b = 0; b < 6; ++b)
            for (uint64_t c = 0; c < width[b]; ++c, ++r) {
                const PlyProp* p = map[r];
                packed[base[b] + (uint64_t)gi * width[b] + c] = (float)read_le(rec + p->offset, kPlyTypes[p->type]);
            }
    }
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

extern "C" int gs_write_ppm(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height) {
    if (!path || !rgba8 || width == 0 || height == 0) return GS_ERR_INVALID;
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return GS_ERR_INVALID;
    bool ok = std::fprintf(f, "P6\n%u %u\n255\n", width, height) > 0;
    std::vector<uint8_t> row((size_t)width * 3);
    for (uint32_t y = 0; ok && y < height; ++y) {
        const uint8_t* src = rgba8 + (size_t)y * width * 4;
        for (uint32_t x = 0; x < width; ++x) {
            row[3 * x + 0] = src[4 * x + 0];
            row[3 * x + 1] = src[4 * x + 1];
            row[3 * x + 2] = src[4 * x + 2];
        }
        ok = std::fwrite(row.data(), 1, row.size(), f) == row.size();
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? GS_OK : GS_ERR_INVALID;
}
