// addon.cc -- Node N-API binding of libwebgs.so for the reference's JavaScript Renderer.
//
// Exposes the C ABI of include/gs.h to JavaScript with the shape renderer.js uses: a native context
// object with uploadGsData / setGs / execute / timings. Status codes become thrown JS Errors, the
// way the reference's fail() (src/utils/utils.js:3-47) throws. Source only in this repository: the
// build image has no Node runtime or node_api.h.
#include <node_api.h>

#include <map>
#include <string>

#include "../../include/gs.h"

namespace {

struct Native {
    gs_ctx* ctx = nullptr;
    std::map<std::string, gs_scene*> scenes;  // uploadGsData name -> scene (renderer.js #gsBuffers)
    std::string current;                      // setGs name (renderer.js #currentGs)
};

napi_value throw_status(napi_env env, int rc, gs_ctx* ctx) {
    napi_throw_error(env, nullptr, gs_last_error(ctx));
    (void)rc;
    return nullptr;
}

Native* unwrap(napi_env env, napi_callback_info info, size_t* argc, napi_value* argv) {
    napi_value self;
    napi_get_cb_info(env, info, argc, argv, &self, nullptr);
    Native* n = nullptr;
    napi_unwrap(env, self, reinterpret_cast<void**>(&n));
    return n;
}

// new Native({tileSize, digitBits, rasterBatch, maxInstanceFactor, profile})
napi_value construct(napi_env env, napi_callback_info info) {
    size_t argc = 1;
    napi_value argv[1], self;
    napi_get_cb_info(env, info, &argc, argv, &self, nullptr);
    gs_config cfg;
    gs_config_default(&cfg);
    if (argc >= 1) {
        napi_value v;
        bool has = false;
        uint32_t u = 0;
        const char* keys[] = {"tileSize", "digitBits", "rasterBatch", "maxInstanceFactor"};
        uint32_t* dst[] = {&cfg.tile_size, &cfg.digit_bits, &cfg.raster_batch, &cfg.max_instance_factor};
        for (int i = 0; i < 4; ++i) {
            napi_has_named_property(env, argv[0], keys[i], &has);
            if (has && napi_get_named_property(env, argv[0], keys[i], &v) == napi_ok &&
                napi_get_value_uint32(env, v, &u) == napi_ok)
                *dst[i] = u;
        }
        napi_has_named_property(env, argv[0], "profile", &has);
        if (has) cfg.flags |= GS_FLAG_PROFILE;
    }
    Native* n = new Native();
    const int rc = gs_ctx_create(&cfg, &n->ctx);
    if (rc != GS_OK) {
        delete n;
        napi_throw_error(env, nullptr, "gs_ctx_create failed (no CUDA device or invalid configuration)");
        return nullptr;
    }
    napi_wrap(env, self, n, [](napi_env, void* data, void*) {
        Native* m = static_cast<Native*>(data);
        for (auto& kv : m->scenes) gs_scene_destroy(kv.second);
        gs_ctx_destroy(m->ctx);
        delete m;
    }, nullptr, nullptr);
    return self;
}

// uploadGsData({count, packed: Float32Array}, name)  -- renderer.js:468-479
napi_value upload_gs_data(napi_env env, napi_callback_info info) {
    size_t argc = 2;
    napi_value argv[2];
    Native* n = unwrap(env, info, &argc, argv);
    napi_value vcount, vpacked;
    uint32_t count = 0;
    napi_get_named_property(env, argv[0], "count", &vcount);
    napi_get_value_uint32(env, vcount, &count);
    napi_get_named_property(env, argv[0], "packed", &vpacked);
    napi_typedarray_type type;
    size_t length = 0;
    void* data = nullptr;
    napi_get_typedarray_info(env, vpacked, &type, &length, &data, nullptr, nullptr);
    if (type != napi_float32_array || length != (size_t)count * 59) {
        napi_throw_type_error(env, nullptr, "packed must be a Float32Array of 59 * count floats");
        return nullptr;
    }
    size_t name_len = 0;
    char name[256];
    napi_get_value_string_utf8(env, argv[1], name, sizeof(name), &name_len);
    gs_scene* scene = nullptr;
    const int rc = gs_scene_upload(n->ctx, static_cast<const float*>(data), count, GS_MEM_HOST, &scene);
    if (rc != GS_OK) return throw_status(env, rc, n->ctx);
    auto it = n->scenes.find(name);
    if (it != n->scenes.end()) gs_scene_destroy(it->second);
    n->scenes[name] = scene;
    return nullptr;
}

// setGs(name) -- renderer.js:461-466: an unknown name throws like fail()
napi_value set_gs(napi_env env, napi_callback_info info) {
    size_t argc = 1;
    napi_value argv[1];
    Native* n = unwrap(env, info, &argc, argv);
    char name[256];
    size_t len = 0;
    napi_get_value_string_utf8(env, argv[0], name, sizeof(name), &len);
    if (!n->scenes.count(name)) {
        napi_throw_error(env, nullptr, (std::string("Invalid Gs buffer for name \"") + name + "\"").c_str());
        return nullptr;
    }
    n->current = name;
    return nullptr;
}

// render(viewBlock: ArrayBuffer(176), image: Uint8Array(W*H*4)) -- the passes of renderer.js:822-932
napi_value render(napi_env env, napi_callback_info info) {
    size_t argc = 2;
    napi_value argv[2];
    Native* n = unwrap(env, info, &argc, argv);
    auto it = n->scenes.find(n->current);
    if (it == n->scenes.end()) return nullptr;  // nothing to draw until a PLY is uploaded (renderer.js:489)
    void* view = nullptr;
    size_t vlen = 0;
    napi_get_arraybuffer_info(env, argv[0], &view, &vlen);
    if (vlen != sizeof(gs_view)) {
        napi_throw_type_error(env, nullptr, "view block must be 176 bytes");
        return nullptr;
    }
    napi_typedarray_type type;
    size_t length = 0;
    void* pixels = nullptr;
    napi_get_typedarray_info(env, argv[1], &type, &length, &pixels, nullptr, nullptr);
    gs_image img{GS_MEM_HOST, static_cast<uint8_t*>(pixels), nullptr, nullptr, nullptr};
    const int rc = gs_forward(n->ctx, it->second, static_cast<const gs_view*>(view), &img);
    if (rc != GS_OK && rc != GS_ERR_OVERFLOW) return throw_status(env, rc, n->ctx);  // overflow truncates silently
    return nullptr;
}

// timings() -> {label: {ms}} like profiler.js:113-121
napi_value timings(napi_env env, napi_callback_info info) {
    size_t argc = 0;
    Native* n = unwrap(env, info, &argc, nullptr);
    gs_timing rows[16];
    int32_t count = 0;
    napi_value out;
    napi_create_object(env, &out);
    if (gs_get_timings(n->ctx, rows, 16, &count) != GS_OK) return out;
    for (int i = 0; i < count; ++i) {
        napi_value row, ms;
        napi_create_object(env, &row);
        napi_create_double(env, rows[i].ms, &ms);
        napi_set_named_property(env, row, "ms", ms);
        napi_set_named_property(env, out, rows[i].label, row);
    }
    return out;
}

napi_value init(napi_env env, napi_value exports) {
    napi_property_descriptor methods[] = {
        {"uploadGsData", nullptr, upload_gs_data, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"setGs", nullptr, set_gs, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"render", nullptr, render, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"timings", nullptr, timings, nullptr, nullptr, nullptr, napi_default, nullptr},
    };
    napi_value cls;
    napi_define_class(env, "Native", NAPI_AUTO_LENGTH, construct, nullptr, 4, methods, &cls);
    napi_set_named_property(env, exports, "Native", cls);
    return exports;
}

}  // namespace

NAPI_MODULE(NODE_GYP_MODULE_NAME, init)
