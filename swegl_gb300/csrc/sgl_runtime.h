// sgl_runtime.h — host-side runtime objects behind the C ABI.
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sgl.h"
#include "sgl_internal.h"

namespace sgl {

// A grow-only device allocation.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf();
    cudaError_t ensure(size_t need);
    void release();
};

// Per-view scratch reused across frames: vertex NDC, visibility flags,
// per-pixel depth keys and the frame counters.
struct FrameScratch {
    DevBuf ndc, yes, key, prec, classes, cliptri, clippx, spans, counters;
};

struct Ctx;

// A scene resident in device memory.
struct Scene {
    DevBuf d_pos_u, d_nrm_v, d_vnode, d_tris, d_prims, d_mats, d_texs, d_texels, d_wpos, d_wnrm, d_uv,
        d_node_world, d_node_rs;
    SceneDev dev{};
    LightsDev lights{};
    std::vector<sgl_node_desc> nodes;
    uint32_t n_vertices = 0;
    uint32_t n_triangles = 0;
    size_t device_bytes = 0;

    sgl_status upload_desc(Ctx *ctx, const sgl_scene_desc *d);
    sgl_status refresh_nodes(Ctx *ctx);
    sgl_status set_lights(Ctx *ctx, float ambient, const float *sun, float sun_intensity, const sgl_point_light *pl,
                          int n);
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    std::map<int, std::unique_ptr<Scene>> scenes;
    int next_scene_id = 1;
    FrameScratch frame;
    DevBuf stage_pixels, stage_z, debug_flags;
    Profiler prof;

    void fail(const char *fmt, ...) __attribute__((format(printf, 2, 3)));
    Scene *find(int id)
    {
        auto it = scenes.find(id);
        return it == scenes.end() ? nullptr : it->second.get();
    }
};

ViewDev make_view(const sgl_view &v);
sgl_status check_view(Ctx *ctx, const sgl_view &v, const sgl_target &t);
sgl_status render_view_device(Ctx *ctx, Scene &s, const sgl_view &view, uint32_t *rect_pixels, int pitch_px,
                              float *zbuf, FrameScratch &fs, cudaStream_t st, uint8_t *slot_flags, int *launches,
                              Profiler *prof = nullptr);

} // namespace sgl
