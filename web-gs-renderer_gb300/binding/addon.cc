// addon.cc -- Node N-API binding of libwebgs.so for the reference's JavaScript Renderer.
//
// Exposes the C ABI of include/gs.h to JavaScript with the shape renderer.js uses: a native context
// object with uploadGsData / setGs / render / timings, plus the differentiable pair (renderRgb /
// backward), the L1 + SSIM loss and the batched render. Status codes become thrown JS Errors, the
// way the reference's fail() (src/utils/utils.js:3-47) throws. Source only in this repository: the
// build image has no Node runtime or node_api.h.
#include <node_api.h>

#include <map>
#include <string>
#include <vector>

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

// new Native({tileSize, digitBits, rasterBatch, maxInstanceFactor, sortBlock, profile, differentiable})
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
        const char* keys[] = {"tileSize", "digitBits", "rasterBatch", "maxInstanceFactor", "sortBlock"};
        uint32_t* dst[] = {&cfg.tile_size, &cfg.digit_bits, &cfg.raster_batch, &cfg.max_instance_factor,
                           &cfg.sort_block};
        for (int i = 0; i < 5; ++i) {
            napi_has_named_property(env, argv[0], keys[i], &has);
            if (has && napi_get_named_property(env, argv[0], keys[i], &v) == napi_ok &&
                napi_get_value_uint32(env, v, &u) == napi_ok)
                *dst[i] = u;
        }
        napi_has_named_property(env, argv[0], "profile", &has);
        if (has) cfg.flags |= GS_FLAG_PROFILE;
        napi_has_named_property(env, argv[0], "differentiable", &has);
        if (has) cfg.flags |= GS_FLAG_DIFFERENTIABLE;
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
    const gs_view* vb = static_cast<const gs_view*>(view);
    if (type != napi_uint8_array || length != (size_t)vb->texture_size[0] * vb->texture_size[1] * 4) {
        napi_throw_type_error(env, nullptr, "image must be a Uint8Array of W*H*4 bytes");
        return nullptr;
    }
    gs_image img{GS_MEM_HOST, static_cast<uint8_t*>(pixels), nullptr, nullptr, nullptr};
    const int rc = gs_forward(n->ctx, it->second, static_cast<const gs_view*>(view), &img);
    if (rc != GS_OK && rc != GS_ERR_OVERFLOW) return throw_status(env, rc, n->ctx);  // overflow truncates silently
    return nullptr;
}

// Float32Array argument i of exactly `count` floats, or a thrown TypeError.
float* float_array(napi_env env, napi_value v, size_t count, const char* what) {
    napi_typedarray_type type;
    size_t length = 0;
    void* data = nullptr;
    if (napi_get_typedarray_info(env, v, &type, &length, &data, nullptr, nullptr) != napi_ok ||
        type != napi_float32_array || length != count) {
        napi_throw_type_error(env, nullptr, (std::string(what) + ": wrong Float32Array length").c_str());
        return nullptr;
    }
    return static_cast<float*>(data);
}

const gs_view* view_block(napi_env env, napi_value v) {
    void* view = nullptr;
    size_t vlen = 0;
    if (napi_get_arraybuffer_info(env, v, &view, &vlen) != napi_ok || vlen != sizeof(gs_view)) {
        napi_throw_type_error(env, nullptr, "view block must be a 176-byte ArrayBuffer");
        return nullptr;
    }
    return static_cast<const gs_view*>(view);
}

// renderRgb(viewBlock, rgb: Float32Array(W*H*3)) -- the forward of the differentiable op: fp32 colour
// before quantization; with {differentiable: true} the context keeps what backward needs
napi_value render_rgb(napi_env env, napi_callback_info info) {
    size_t argc = 2;
    napi_value argv[2];
    Native* n = unwrap(env, info, &argc, argv);
    auto it = n->scenes.find(n->current);
    if (it == n->scenes.end()) return nullptr;
    const gs_view* view = view_block(env, argv[0]);
    if (!view) return nullptr;
    const size_t pix = (size_t)view->texture_size[0] * view->texture_size[1];
    float* rgb = float_array(env, argv[1], pix * 3, "rgb");
    if (!rgb) return nullptr;
    gs_image img{GS_MEM_HOST, nullptr, rgb, nullptr, nullptr};
    const int rc = gs_forward(n->ctx, it->second, view, &img);
    if (rc != GS_OK && rc != GS_ERR_OVERFLOW) return throw_status(env, rc, n->ctx);
    return nullptr;
}

// backward(dLdRgb: Float32Array(W*H*3), grad: Float32Array(59*count)) -- gradients of the last
// renderRgb with respect to the packed attributes (the uploadGsData layout)
napi_value backward(napi_env env, napi_callback_info info) {
    size_t argc = 2;
    napi_value argv[2];
    Native* n = unwrap(env, info, &argc, argv);
    auto it = n->scenes.find(n->current);
    if (it == n->scenes.end()) {
        napi_throw_error(env, nullptr, "backward: no scene selected");
        return nullptr;
    }
    napi_typedarray_type type;
    size_t dl_len = 0;
    void* dl = nullptr;
    napi_get_typedarray_info(env, argv[0], &type, &dl_len, &dl, nullptr, nullptr);
    if (type != napi_float32_array) {
        napi_throw_type_error(env, nullptr, "dLdRgb must be a Float32Array");
        return nullptr;
    }
    float* grad = float_array(env, argv[1], (size_t)gs_scene_count(it->second) * 59, "grad");
    if (!grad) return nullptr;
    const int rc = gs_backward(n->ctx, it->second, static_cast<const float*>(dl), grad, GS_MEM_HOST);
    if (rc != GS_OK) return throw_status(env, rc, n->ctx);
    return nullptr;
}

// loss(rgb, target, width, height, lambda, dLdRgb) -> L1 + lambda (1 - SSIM); dLdRgb receives dL/drgb
napi_value loss(napi_env env, napi_callback_info info) {
    size_t argc = 6;
    napi_value argv[6];
    Native* n = unwrap(env, info, &argc, argv);
    uint32_t w = 0, h = 0;
    double lambda = 0.2;
    napi_get_value_uint32(env, argv[2], &w);
    napi_get_value_uint32(env, argv[3], &h);
    napi_get_value_double(env, argv[4], &lambda);
    const size_t count = (size_t)w * h * 3;
    float* rgb = float_array(env, argv[0], count, "rgb");
    float* target = rgb ? float_array(env, argv[1], count, "target") : nullptr;
    float* dl = target ? float_array(env, argv[5], count, "dLdRgb") : nullptr;
    if (!dl) return nullptr;
    double value = 0.0;
    const int rc = gs_loss_l1_ssim(n->ctx, rgb, target, w, h, (float)lambda, &value, dl, GS_MEM_HOST);
    if (rc != GS_OK) return throw_status(env, rc, n->ctx);
    napi_value out;
    napi_create_double(env, value, &out);
    return out;
}

// renderBatch([{name, view: ArrayBuffer(176), image: Uint8Array(W*H*4)}, ...]) -- many views and
// scenes in one launch
napi_value render_batch(napi_env env, napi_callback_info info) {
    size_t argc = 1;
    napi_value argv[1];
    Native* n = unwrap(env, info, &argc, argv);
    uint32_t count = 0;
    napi_get_array_length(env, argv[0], &count);
    std::vector<gs_batch_view> views(count);
    for (uint32_t i = 0; i < count; ++i) {
        napi_value item, vname, vview, vimage;
        napi_get_element(env, argv[0], i, &item);
        napi_get_named_property(env, item, "name", &vname);
        napi_get_named_property(env, item, "view", &vview);
        napi_get_named_property(env, item, "image", &vimage);
        char name[256];
        size_t len = 0;
        napi_get_value_string_utf8(env, vname, name, sizeof(name), &len);
        auto it = n->scenes.find(name);
        if (it == n->scenes.end()) {
            napi_throw_error(env, nullptr, (std::string("Invalid Gs buffer for name \"") + name + "\"").c_str());
            return nullptr;
        }
        const gs_view* view = view_block(env, vview);
        if (!view) return nullptr;
        napi_typedarray_type type;
        size_t length = 0;
        void* pixels = nullptr;
        napi_get_typedarray_info(env, vimage, &type, &length, &pixels, nullptr, nullptr);
        if (type != napi_uint8_array || length != (size_t)view->texture_size[0] * view->texture_size[1] * 4) {
            napi_throw_type_error(env, nullptr, "image must be a Uint8Array of W*H*4 bytes");
            return nullptr;
        }
        views[i].scene = it->second;
        views[i].view = *view;
        views[i].out = gs_image{GS_MEM_HOST, static_cast<uint8_t*>(pixels), nullptr, nullptr, nullptr};
    }
    const int rc = gs_forward_batch(n->ctx, views.data(), count);
    if (rc != GS_OK && rc != GS_ERR_OVERFLOW) return throw_status(env, rc, n->ctx);
    return nullptr;
}

// renderBatchCameras([{name, camera: {eye: [3], target: [3], up: [3], fovy, width, height, near, far},
// image: Uint8Array(W*H*4)}, ...]) -- a batch whose 176-byte blocks are built on the device from the
// cameras (the reference's Camera state, camera.js)
napi_value render_batch_cameras(napi_env env, napi_callback_info info) {
    size_t argc = 1;
    napi_value argv[1];
    Native* n = unwrap(env, info, &argc, argv);
    uint32_t count = 0;
    napi_get_array_length(env, argv[0], &count);
    std::vector<gs_batch_camera> views(count);
    auto number = [&](napi_value obj, const char* key) {
        napi_value v;
        double d = 0.0;
        napi_get_named_property(env, obj, key, &v);
        napi_get_value_double(env, v, &d);
        return d;
    };
    auto vec3 = [&](napi_value obj, const char* key, float out[3]) {
        napi_value arr, e;
        napi_get_named_property(env, obj, key, &arr);
        for (uint32_t k = 0; k < 3; ++k) {
            double d = 0.0;
            napi_get_element(env, arr, k, &e);
            napi_get_value_double(env, e, &d);
            out[k] = (float)d;
        }
    };
    for (uint32_t i = 0; i < count; ++i) {
        napi_value item, vname, vcam, vimage;
        napi_get_element(env, argv[0], i, &item);
        napi_get_named_property(env, item, "name", &vname);
        napi_get_named_property(env, item, "camera", &vcam);
        napi_get_named_property(env, item, "image", &vimage);
        char name[256];
        size_t len = 0;
        napi_get_value_string_utf8(env, vname, name, sizeof(name), &len);
        auto it = n->scenes.find(name);
        if (it == n->scenes.end()) {
            napi_throw_error(env, nullptr, (std::string("Invalid Gs buffer for name \"") + name + "\"").c_str());
            return nullptr;
        }
        gs_camera& c = views[i].camera;
        vec3(vcam, "eye", c.eye);
        vec3(vcam, "target", c.target);
        vec3(vcam, "up", c.up);
        c.fovy_deg = (float)number(vcam, "fovy");
        c.width = (uint32_t)number(vcam, "width");
        c.height = (uint32_t)number(vcam, "height");
        c.z_near = (float)number(vcam, "near");
        c.z_far = (float)number(vcam, "far");
        napi_typedarray_type type;
        size_t length = 0;
        void* pixels = nullptr;
        napi_get_typedarray_info(env, vimage, &type, &length, &pixels, nullptr, nullptr);
        if (type != napi_uint8_array || length != (size_t)c.width * c.height * 4) {
            napi_throw_type_error(env, nullptr, "image must be a Uint8Array of W*H*4 bytes");
            return nullptr;
        }
        views[i].scene = it->second;
        views[i].out = gs_image{GS_MEM_HOST, static_cast<uint8_t*>(pixels), nullptr, nullptr, nullptr};
    }
    const int rc = gs_forward_batch_cameras(n->ctx, views.data(), count);
    if (rc != GS_OK && rc != GS_ERR_OVERFLOW) return throw_status(env, rc, n->ctx);
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
        {"renderRgb", nullptr, render_rgb, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"backward", nullptr, backward, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"loss", nullptr, loss, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"renderBatch", nullptr, render_batch, nullptr, nullptr, nullptr, napi_default, nullptr},
        {"renderBatchCameras", nullptr, render_batch_cameras, nullptr, nullptr, nullptr, napi_default, nullptr},
    };
    napi_value cls;
    napi_define_class(env, "Native", NAPI_AUTO_LENGTH, construct, nullptr, sizeof(methods) / sizeof(methods[0]),
                      methods, &cls);
    napi_set_named_property(env, exports, "Native", cls);
    return exports;
}

}  // namespace

NAPI_MODULE(NODE_GYP_MODULE_NAME, init)
