// sgl_api.cpp — the C ABI of include/sgl.h: contexts, scenes, the plain
// one-frame-per-launch renderer, the batched renderer and its autotuner.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include <cuda_runtime.h>

#include "sgl.h"
#include "sgl_cull.h"
#include "sgl_internal.h"
#include "sgl_runtime.h"

namespace sgl {

ViewDev make_view(const sgl_view &v)
{
    ViewDev d;
    d.x = v.x;
    d.y = v.y;
    d.w = v.w;
    d.h = v.h;
    for (int i = 0; i < 12; i++) {
        d.view[i] = v.view[i];
        d.proj[i] = v.proj[i];
    }
    d.campos[0] = v.camera_pos[0];
    d.campos[1] = v.camera_pos[1];
    d.campos[2] = v.camera_pos[2];
    d.shader = v.shader;
    // viewport_t constructor (src/render/viewport.cpp:94-97): x+w/2.0f, w/2.0f, -h/2.0f
    d.vm00 = (float)v.w / 2.0f;
    d.vm03 = (float)v.x + (float)v.w / 2.0f;
    d.vm11 = (float)(-v.h) / 2.0f;
    d.vm13 = (float)v.y + (float)v.h / 2.0f;
    cull_planes(v, d.cull);
    return d;
}

sgl_status check_view(Ctx *ctx, const sgl_view &v, const sgl_target &t)
{
    if (v.shader < 0 || v.shader >= SGL_SHADER_COUNT) {
        ctx->fail("unknown pixel shader %d", v.shader);
        return SGL_ERR_INVALID;
    }
    if (v.layers < 0 || v.layers > SGL_MAX_LAYERS) {
        ctx->fail("transparency layers %d outside 0..%d", v.layers, SGL_MAX_LAYERS);
        return SGL_ERR_INVALID;
    }
    if (v.dof.enabled && !(v.dof.max_radius >= 0.0f && v.dof.max_radius <= 4096.0f)) {
        ctx->fail("depth-of-field max_radius %g outside 0..4096 pixels", (double)v.dof.max_radius);
        return SGL_ERR_INVALID;
    }
    if (v.w <= 0 || v.h <= 0 || v.x < 0 || v.y < 0 || (int64_t)v.w * v.h > (1ll << 28)) {
        ctx->fail("bad viewport %d,%d %dx%d", v.x, v.y, v.w, v.h);
        return SGL_ERR_INVALID;
    }
    if (!t.pixels || t.pitch < 4 * t.width || t.width <= 0 || t.height <= 0 || v.x + v.w > t.width ||
        v.y + v.h > t.height || (t.pitch & 3)) {
        ctx->fail("viewport %d,%d %dx%d does not fit its %dx%d surface (pitch %d)", v.x, v.y, v.w, v.h, t.width,
                  t.height, t.pitch);
        return SGL_ERR_INVALID;
    }
    return SGL_OK;
}

// The lane bound to a caller's stream (created on first use).
static sgl_status ext_lane(Ctx *ctx, cudaStream_t st, Lane **out)
{
    if (!ctx->ext_lane) {
        auto l = std::make_unique<Lane>();
        sgl_status r = l->init(ctx, kMaxBatch, st);
        if (r != SGL_OK)
            return r;
        ctx->ext_lane = std::move(l);
    }
    ctx->ext_lane->stream = st;
    *out = ctx->ext_lane.get();
    return SGL_OK;
}

// Entry points other than sgl_render take opaque views only.
sgl_status reject_layers(Ctx *ctx, const sgl_view &v)
{
    if (v.layers == 0)
        return SGL_OK;
    ctx->fail("views with transparency layers render through sgl_render only");
    return SGL_ERR_UNSUPPORTED;
}

// One view with transparency layers.  Its flatten and copy passes read and
// write the surface outside the viewport's rectangle (viewport.cpp:53-79,
// post_shaders.hpp:22-31), so a host surface is staged whole.  The call
// waits for the frame: the fragment pool is checked and, when it was too
// small (nothing was written then), grown and the view rendered again.
static sgl_status render_layered(Ctx *ctx, Lane *lane, BatchEntry &e, const sgl_target &t, bool device_buffers,
                                 int *launches, sgl_frame_stats *acc, bool want_stats)
{
    const sgl_view &v = e.view;
    const size_t surf_bytes = (size_t)t.pitch * t.height, px = (size_t)v.w * v.h;
    if (device_buffers) {
        e.surface = (uint32_t *)t.pixels;
    } else {
        CUDA_TRY(ctx->stage_pixels.ensure(surf_bytes));
        CUDA_TRY(ctx->stage_z.ensure(4 * px));
        CUDA_TRY(cudaMemcpyAsync(ctx->stage_pixels.ptr, t.pixels, surf_bytes, cudaMemcpyHostToDevice, lane->stream));
        e.surface = (uint32_t *)ctx->stage_pixels.ptr;
        e.zbuf = t.zbuffer ? (float *)ctx->stage_z.ptr : nullptr;
    }
    e.pitch_px = t.pitch / 4;
    e.rect_pixels = e.surface + (size_t)v.y * e.pitch_px + v.x;
    int slot = 0;
    bool fit = false;
    for (int attempt = 0; attempt < 3 && !fit; attempt++) {
        sgl_status r = lane->prepare(ctx, &e, 1, ctx->tile, ctx->inline_span, nullptr, &slot);
        if (r == SGL_OK)
            r = lane->launch(ctx, slot, ctx->tile, false, launches, &ctx->prof);
        if (r == SGL_OK)
            r = lane->layered_fit(ctx, slot, &fit);
        if (r != SGL_OK)
            return r;
    }
    if (!fit) {
        ctx->fail("the fragment pool did not fit after growing");
        return SGL_ERR_OOM;
    }
    if (!device_buffers) {
        // rows y .. y+h-1 hold every pixel the view wrote
        const size_t row0 = (size_t)v.y * t.pitch;
        CUDA_TRY(cudaMemcpyAsync((uint8_t *)t.pixels + row0, (uint8_t *)ctx->stage_pixels.ptr + row0,
                                 (size_t)v.h * t.pitch, cudaMemcpyDeviceToHost, lane->stream));
        if (t.zbuffer)
            CUDA_TRY(cudaMemcpyAsync(t.zbuffer, ctx->stage_z.ptr, 4 * px, cudaMemcpyDeviceToHost, lane->stream));
        CUDA_TRY(cudaStreamSynchronize(lane->stream));
    }
    if (want_stats) {
        unsigned long long d = 0, f = 0;
        sgl_status r = lane->read_counters(ctx, slot, &d, &f, nullptr);
        if (r != SGL_OK)
            return r;
        acc->drawn_triangles += d;
        acc->fragments += f;
    }
    acc->pixels += px;
    return SGL_OK;
}

static bool valid_tile(int t) { return t == 8 || t == 16 || t == 32; }
static bool valid_span_bin(int b) { return b >= 1 && b <= 64; }

} // namespace sgl

using namespace sgl;

extern "C" {

SGL_API int sgl_version(void) { return 2; }

SGL_API sgl_status sgl_host_alloc(size_t bytes, int write_combined, void **out)
{
    if (!out)
        return SGL_ERR_INVALID;
    *out = nullptr;
    if (bytes == 0)
        return SGL_ERR_INVALID;
    const unsigned flags = cudaHostAllocPortable | (write_combined ? cudaHostAllocWriteCombined : 0u);
    if (cudaHostAlloc(out, bytes, flags) != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return SGL_ERR_OOM;
    }
    return SGL_OK;
}

SGL_API sgl_status sgl_host_free(void *p)
{
    if (p && cudaFreeHost(p) != cudaSuccess) {
        cudaGetLastError();
        return SGL_ERR_CUDA;
    }
    return SGL_OK;
}

SGL_API const char *sgl_status_string(sgl_status s)
{
    switch (s) {
    case SGL_OK: return "ok";
    case SGL_ERR_INVALID: return "invalid argument";
    case SGL_ERR_OOM: return "out of memory";
    case SGL_ERR_CUDA: return "CUDA error";
    case SGL_ERR_NOT_FOUND: return "not found";
    case SGL_ERR_BUDGET: return "over the memory budget";
    case SGL_ERR_TIMEOUT: return "timed out";
    case SGL_ERR_NO_DEVICE: return "no CUDA device";
    case SGL_ERR_UNSUPPORTED: return "unsupported";
    case SGL_ERR_BUSY: return "not ready";
    default: return "unknown status";
    }
}

SGL_API sgl_status sgl_create(sgl_ctx **out, int device)
{
    if (!out)
        return SGL_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return SGL_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n)
        return SGL_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess || cudaFree(0) != cudaSuccess)
        return SGL_ERR_CUDA;
    Ctx *ctx = new (std::nothrow) Ctx();
    if (!ctx)
        return SGL_ERR_OOM;
    ctx->device = device;
    ctx->lane = std::make_unique<Lane>();
    if (ctx->lane->init(ctx, 1, nullptr) != SGL_OK) {
        delete ctx;
        return SGL_ERR_CUDA;
    }
    ctx->stream = ctx->lane->stream;
    *out = reinterpret_cast<sgl_ctx *>(ctx);
    return SGL_OK;
}

SGL_API void sgl_destroy(sgl_ctx *c)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    ctx->lane.reset();
    ctx->ext_lane.reset();
    ctx->scenes.clear();
    delete ctx;
}

SGL_API const char *sgl_last_error(const sgl_ctx *c)
{
    const Ctx *ctx = reinterpret_cast<const Ctx *>(c);
    return ctx ? ctx->last_error.c_str() : "null context";
}

SGL_API sgl_status sgl_scene_upload(sgl_ctx *c, const sgl_scene_desc *desc, int *scene_id)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || !desc || !scene_id)
        return SGL_ERR_INVALID;
    cudaSetDevice(ctx->device);
    auto s = std::make_unique<Scene>();
    sgl_status st = s->upload_desc(ctx, desc);
    if (st != SGL_OK)
        return st;
    const int id = ctx->next_scene_id++;
    ctx->scenes[id] = std::move(s);
    *scene_id = id;
    return SGL_OK;
}

SGL_API sgl_status sgl_scene_release(sgl_ctx *c, int scene_id)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx)
        return SGL_ERR_INVALID;
    auto it = ctx->scenes.find(scene_id);
    if (it == ctx->scenes.end())
        return SGL_ERR_NOT_FOUND;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    ctx->scenes.erase(it);
    return SGL_OK;
}

SGL_API sgl_status sgl_scene_set_nodes(sgl_ctx *c, int scene_id, const sgl_node_desc *nodes, int n_nodes)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || !nodes)
        return SGL_ERR_INVALID;
    Scene *s = ctx->find(scene_id);
    if (!s)
        return SGL_ERR_NOT_FOUND;
    if (n_nodes != (int)s->nodes.size()) {
        ctx->fail("scene has %zu nodes, got %d", s->nodes.size(), n_nodes);
        return SGL_ERR_INVALID;
    }
    for (int i = 0; i < n_nodes; i++)
        if (nodes[i].parent < -1 || nodes[i].parent >= n_nodes) {
            ctx->fail("node %d has bad parent %d", i, nodes[i].parent);
            return SGL_ERR_INVALID;
        }
    cudaSetDevice(ctx->device);
    std::vector<sgl_node_desc> saved = s->nodes;
    s->nodes.assign(nodes, nodes + n_nodes);
    sgl_status st = s->refresh_nodes(ctx);
    if (st != SGL_OK) {
        s->nodes = saved;
        s->refresh_nodes(ctx);
    }
    return st;
}

SGL_API sgl_status sgl_scene_set_lights(sgl_ctx *c, int scene_id, float ambient, const float sun_direction[3],
                                        float sun_intensity, const sgl_point_light *lights, int n_lights)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx)
        return SGL_ERR_INVALID;
    Scene *s = ctx->find(scene_id);
    if (!s)
        return SGL_ERR_NOT_FOUND;
    cudaSetDevice(ctx->device);
    return s->set_lights(ctx, ambient, sun_direction, sun_intensity, lights, n_lights);
}

SGL_API sgl_status sgl_scene_info(sgl_ctx *c, int scene_id, uint64_t *n_triangles, uint64_t *n_vertices,
                                  uint64_t *device_bytes)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx)
        return SGL_ERR_INVALID;
    Scene *s = ctx->find(scene_id);
    if (!s)
        return SGL_ERR_NOT_FOUND;
    if (n_triangles)
        *n_triangles = s->n_triangles;
    if (n_vertices)
        *n_vertices = s->n_vertices;
    if (device_bytes)
        *device_bytes = s->device_bytes;
    return SGL_OK;
}

SGL_API sgl_status sgl_render(sgl_ctx *c, int scene_id, const sgl_view *views, const sgl_target *targets, int n_views,
                              int device_buffers, void *stream, sgl_frame_stats *stats)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || !views || !targets || n_views <= 0)
        return SGL_ERR_INVALID;
    Scene *s = ctx->find(scene_id);
    if (!s) {
        ctx->fail("unknown scene %d", scene_id);
        return SGL_ERR_NOT_FOUND;
    }
    cudaSetDevice(ctx->device);
    for (int i = 0; i < n_views; i++) {
        sgl_status st = check_view(ctx, views[i], targets[i]);
        if (st != SGL_OK)
            return st;
    }
    Lane *lane = ctx->lane.get();
    if (device_buffers) {
        sgl_status r = ext_lane(ctx, (cudaStream_t)stream, &lane);
        if (r != SGL_OK)
            return r;
    }
    sgl_frame_stats acc{};
    int launches = 0;
    // one view per launch sequence, in order: views may share a surface (renderer.hpp:18-25)
    for (int i = 0; i < n_views; i++) {
        const sgl_view &v = views[i];
        const sgl_target &t = targets[i];
        BatchEntry e{s, v, nullptr, t.pitch / 4, t.zbuffer};
        const size_t px = (size_t)v.w * v.h;
        if (v.layers > 0) {
            sgl_status r = render_layered(ctx, lane, e, t, device_buffers != 0, &launches, &acc, stats != nullptr);
            if (r != SGL_OK)
                return r;
            continue;
        }
        if (device_buffers) {
            e.rect_pixels = (uint32_t *)t.pixels + (size_t)v.y * (t.pitch / 4) + v.x;
        } else {
            CUDA_TRY(ctx->stage_pixels.ensure(4 * px));
            CUDA_TRY(ctx->stage_z.ensure(4 * px));
            e.rect_pixels = (uint32_t *)ctx->stage_pixels.ptr;
            e.pitch_px = v.w;
            e.zbuf = (float *)ctx->stage_z.ptr;
        }
        int slot = 0;
        sgl_status r = lane->prepare(ctx, &e, 1, ctx->tile, ctx->inline_span, nullptr, &slot);
        if (r == SGL_OK) {
            // one CUDA graph launch per view (captured once per lane slot and
            // sequence variant); direct launches while per-kernel timing is on
            r = lane->launch(ctx, slot, ctx->tile, !ctx->prof.enabled, &launches, &ctx->prof);
        }
        if (r != SGL_OK)
            return r;
        if (!device_buffers) {
            uint8_t *dst = (uint8_t *)t.pixels + (size_t)v.y * t.pitch + 4 * (size_t)v.x;
            CUDA_TRY(cudaMemcpy2DAsync(dst, t.pitch, ctx->stage_pixels.ptr, 4 * (size_t)v.w, 4 * (size_t)v.w, v.h,
                                       cudaMemcpyDeviceToHost, lane->stream));
            if (t.zbuffer)
                CUDA_TRY(cudaMemcpyAsync(t.zbuffer, ctx->stage_z.ptr, 4 * px, cudaMemcpyDeviceToHost, lane->stream));
            CUDA_TRY(cudaStreamSynchronize(lane->stream));
        }
        if (stats) {
            unsigned long long d = 0, f = 0;
            r = lane->read_counters(ctx, slot, &d, &f, nullptr);
            if (r != SGL_OK)
                return r;
            acc.drawn_triangles += d;
            acc.fragments += f;
        }
        acc.pixels += px;
    }
    if (stats) {
        acc.triangles = s->n_triangles;
        acc.kernel_launches = (uint32_t)launches;
        *stats = acc;
    }
    return SGL_OK;
}

SGL_API sgl_status sgl_render_debug(sgl_ctx *c, int scene_id, const sgl_view *view, const sgl_target *target,
                                    uint32_t *winner, uint8_t *slot_flags, sgl_frame_stats *stats)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || !view || !target)
        return SGL_ERR_INVALID;
    Scene *s = ctx->find(scene_id);
    if (!s)
        return SGL_ERR_NOT_FOUND;
    cudaSetDevice(ctx->device);
    sgl_status r = check_view(ctx, *view, *target);
    if (r == SGL_OK)
        r = reject_layers(ctx, *view);
    if (r != SGL_OK)
        return r;
    Lane *lane = ctx->lane.get();
    cudaStream_t st = lane->stream;
    const size_t px = (size_t)view->w * view->h;
    const size_t nflags = 2 * (size_t)std::max<uint32_t>(s->n_triangles, 1);
    CUDA_TRY(ctx->stage_pixels.ensure(4 * px));
    CUDA_TRY(ctx->stage_z.ensure(4 * px));
    CUDA_TRY(ctx->debug_flags.ensure(nflags));
    CUDA_TRY(cudaMemsetAsync(ctx->debug_flags.ptr, 0, nflags, st));
    BatchEntry e{s, *view, (uint32_t *)ctx->stage_pixels.ptr, view->w, (float *)ctx->stage_z.ptr};
    int slot = 0, launches = 0;
    r = lane->prepare(ctx, &e, 1, ctx->tile, ctx->inline_span, (uint8_t *)ctx->debug_flags.ptr, &slot);
    if (r == SGL_OK)
        r = lane->launch(ctx, slot, ctx->tile, false, &launches, nullptr);
    if (r != SGL_OK)
        return r;
    const sgl_target &t = *target;
    uint8_t *dst = (uint8_t *)t.pixels + (size_t)view->y * t.pitch + 4 * (size_t)view->x;
    CUDA_TRY(cudaMemcpy2DAsync(dst, t.pitch, ctx->stage_pixels.ptr, 4 * (size_t)view->w, 4 * (size_t)view->w,
                               view->h, cudaMemcpyDeviceToHost, st));
    if (t.zbuffer)
        CUDA_TRY(cudaMemcpyAsync(t.zbuffer, ctx->stage_z.ptr, 4 * px, cudaMemcpyDeviceToHost, st));
    if (winner) {
        std::vector<unsigned long long> keys(px);
        CUDA_TRY(cudaMemcpyAsync(keys.data(), lane->key.ptr, 8 * px, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        for (size_t i = 0; i < px; i++)
            winner[i] = keys[i] == kEmptyKey ? 0xFFFFFFFFu : (uint32_t)(keys[i] & 0xFFFFFFFFu);
    }
    if (slot_flags)
        CUDA_TRY(cudaMemcpyAsync(slot_flags, ctx->debug_flags.ptr, 2 * (size_t)s->n_triangles,
                                 cudaMemcpyDeviceToHost, st));
    unsigned long long d = 0, f = 0;
    r = lane->read_counters(ctx, slot, &d, &f, nullptr);
    if (r != SGL_OK)
        return r;
    CUDA_TRY(cudaStreamSynchronize(st));
    if (stats) {
        sgl_frame_stats acc{};
        acc.triangles = s->n_triangles;
        acc.drawn_triangles = d;
        acc.fragments = f;
        acc.pixels = px;
        acc.kernel_launches = (uint32_t)launches;
        *stats = acc;
    }
    return SGL_OK;
}

static sgl_status batch_entries(Ctx *ctx, const sgl_batch_item *items, int n, std::vector<BatchEntry> &out)
{
    out.clear();
    out.reserve(n);
    for (int i = 0; i < n; i++) {
        Scene *s = ctx->find(items[i].scene_id);
        if (!s) {
            ctx->fail("batch item %d: unknown scene %d", i, items[i].scene_id);
            return SGL_ERR_NOT_FOUND;
        }
        sgl_status st = check_view(ctx, items[i].view, items[i].target);
        if (st != SGL_OK)
            return st;
        const sgl_target &t = items[i].target;
        const sgl_view &v = items[i].view;
        out.push_back(BatchEntry{s, v, (uint32_t *)t.pixels + (size_t)v.y * (t.pitch / 4) + v.x, t.pitch / 4,
                                 t.zbuffer});
    }
    return SGL_OK;
}

// Batch items with their own pose: the node matrices composed on the host (as
// sgl_scene_set_nodes does), then k_pose writes the item's world positions and
// normals (and k_box its primitives' boxes) into the lane's pose scratch on
// the lane's stream, and the item's entry points at them (the scene's own arrays and nodes are untouched).
static sgl_status pose_items(Ctx *ctx, Lane *lane, const sgl_batch_item *items, int n, std::vector<BatchEntry> &e)
{
    std::vector<std::vector<float>> mats((size_t)n);
    size_t total = 0;
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    for (int i = 0; i < n; i++) {
        if (!items[i].nodes)
            continue;
        const Scene *s = e[i].scene;
        if (items[i].n_nodes != (int)s->nodes.size()) {
            ctx->fail("batch item %d: a pose gives all %zu nodes of the scene, not %d", i, s->nodes.size(),
                      items[i].n_nodes);
            return SGL_ERR_INVALID;
        }
        std::vector<sgl_node_desc> nd(items[i].nodes, items[i].nodes + items[i].n_nodes);
        std::vector<float> world, rs;
        if (!node_matrices(nd, world, rs)) {
            ctx->fail("batch item %d: the pose's node hierarchy has a cycle or a bad parent index", i);
            return SGL_ERR_INVALID;
        }
        mats[i] = std::move(world);
        mats[i].insert(mats[i].end(), rs.begin(), rs.end());
        total += up(sizeof(float) * mats[i].size()) + up(2 * sizeof(float4) * std::max<size_t>(s->n_vertices, 1)) +
                 (s->dev.pbox ? up(2 * sizeof(float4) * s->dev.n_prims) : 0);
    }
    if (!total)
        return SGL_OK;
    CUDA_TRY(lane->poses.ensure(total));
    uint8_t *base = (uint8_t *)lane->poses.ptr;
    size_t off = 0;
    for (int i = 0; i < n; i++) {
        if (!items[i].nodes)
            continue;
        const Scene *s = e[i].scene;
        float *m = (float *)(base + off);
        off += up(sizeof(float) * mats[i].size());
        float4 *wpos = (float4 *)(base + off);
        float4 *wnrm = wpos + s->n_vertices;
        off += up(2 * sizeof(float4) * std::max<size_t>(s->n_vertices, 1));
        float4 *pbox = nullptr;
        if (s->dev.pbox) {
            pbox = (float4 *)(base + off);
            off += up(2 * sizeof(float4) * s->dev.n_prims);
        }
        const size_t nm = mats[i].size() / 2;
        // (from pageable memory: staged before the call returns)
        CUDA_TRY(cudaMemcpyAsync(m, mats[i].data(), sizeof(float) * mats[i].size(), cudaMemcpyHostToDevice,
                                 lane->stream));
        CUDA_TRY(launch_pose(s->dev, m, m + nm, wpos, wnrm, pbox, lane->stream));
        e[i].wpos = wpos;
        e[i].wnrm = wnrm;
        e[i].pbox = pbox;
        e[i].node_world = m;
        e[i].node_rs = m + nm;
    }
    return SGL_OK;
}

SGL_API sgl_status sgl_render_batch(sgl_ctx *c, const sgl_batch_item *items, int n_items,
                                    const sgl_batch_opts *opts, void *stream, sgl_frame_stats *stats)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || !items || n_items <= 0 || n_items > kMaxBatch)
        return SGL_ERR_INVALID;
    cudaSetDevice(ctx->device);
    const int tile = (opts && valid_tile(opts->tile)) ? opts->tile : ctx->tile;
    const int bin = (opts && valid_span_bin(opts->span_bin)) ? opts->span_bin : ctx->inline_span;
    const bool graph = opts ? opts->use_graph != 0 : true;
    std::vector<BatchEntry> all;
    sgl_status r = batch_entries(ctx, items, n_items, all);
    if (r != SGL_OK)
        return r;
    Lane *lane = nullptr;
    r = ext_lane(ctx, (cudaStream_t)stream, &lane);
    if (r != SGL_OK)
        return r;
    r = pose_items(ctx, lane, items, n_items, all);
    if (r != SGL_OK)
        return r;
    // items with transparency layers run after the others, each as its own
    // launch sequence, in item order (the call then waits for them)
    std::vector<BatchEntry> e;
    std::vector<int> layered;
    for (int i = 0; i < n_items; i++) {
        if (all[i].view.layers > 0)
            layered.push_back(i);
        else
            e.push_back(all[i]);
    }
    int slot = 0, launches = 0;
    sgl_frame_stats acc{};
    if (!e.empty()) {
        r = lane->prepare(ctx, e.data(), (int)e.size(), tile, bin, nullptr, &slot);
        if (r == SGL_OK)
            r = lane->launch(ctx, slot, tile, graph, &launches, graph ? nullptr : &ctx->prof);
        if (r != SGL_OK)
            return r;
        if (stats) {
            unsigned long long d = 0, f = 0;
            r = lane->read_counters(ctx, slot, &d, &f, nullptr);
            if (r != SGL_OK)
                return r;
            acc.drawn_triangles = d;
            acc.fragments = f;
        }
    }
    for (int i : layered) {
        r = render_layered(ctx, lane, all[i], items[i].target, true, &launches, &acc, stats != nullptr);
        if (r != SGL_OK)
            return r;
    }
    if (stats) {
        acc.triangles = 0;
        acc.pixels = 0;
        for (auto &en : all) {
            acc.triangles += en.scene->n_triangles;
            acc.pixels += (uint64_t)en.view.w * en.view.h;
        }
        acc.kernel_launches = (uint32_t)launches;
        *stats = acc;
    }
    return SGL_OK;
}

SGL_API sgl_status sgl_autotune(sgl_ctx *c, const sgl_batch_item *items, int n_items, sgl_batch_opts *chosen)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || !items || !chosen || n_items <= 0 || n_items > kMaxBatch)
        return SGL_ERR_INVALID;
    cudaSetDevice(ctx->device);
    std::vector<BatchEntry> e;
    sgl_status r = batch_entries(ctx, items, n_items, e);
    for (int i = 0; r == SGL_OK && i < n_items; i++)
        r = reject_layers(ctx, items[i].view); // the tuner times one launch sequence
    if (r != SGL_OK)
        return r;
    Lane *lane = nullptr;
    r = ext_lane(ctx, ctx->stream, &lane);
    if (r == SGL_OK)
        r = pose_items(ctx, lane, items, n_items, e);
    if (r != SGL_OK)
        return r;
    cudaEvent_t a = nullptr, b = nullptr;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    const int tiles[3] = {8, 16, 32}, bins[3] = {8, 16, 32};
    float best = 1e30f;
    sgl_batch_opts pick{16, 16, 1};
    for (int ti = 0; ti < 3 && r == SGL_OK; ti++)
        for (int bi = 0; bi < 3 && r == SGL_OK; bi++) {
            float total = 0.0f;
            for (int rep = 0; rep < 4 && r == SGL_OK; rep++) { // first run captures the graph, then 3 timed
                int slot = 0;
                r = lane->prepare(ctx, e.data(), n_items, tiles[ti], bins[bi], nullptr, &slot);
                if (r != SGL_OK)
                    break;
                cudaEventRecord(a, lane->stream);
                r = lane->launch(ctx, slot, tiles[ti], true, nullptr, nullptr);
                cudaEventRecord(b, lane->stream);
                if (cudaEventSynchronize(b) != cudaSuccess) {
                    r = SGL_ERR_CUDA;
                    break;
                }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, a, b);
                if (rep > 0)
                    total += ms;
            }
            if (r == SGL_OK && total < best) {
                best = total;
                pick = sgl_batch_opts{tiles[ti], bins[bi], 1};
            }
        }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (r != SGL_OK)
        return r;
    *chosen = pick;
    return SGL_OK;
}

SGL_API sgl_status sgl_dof(sgl_ctx *c, const sgl_view *view, const sgl_target *in, const sgl_target *out,
                           int device_buffers, void *stream)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || !view || !in || !out || !in->zbuffer)
        return SGL_ERR_INVALID;
    cudaSetDevice(ctx->device);
    sgl_status r = check_view(ctx, *view, *in);
    if (r == SGL_OK)
        r = check_view(ctx, *view, *out);
    if (r == SGL_OK && !(view->dof.max_radius >= 0.0f && view->dof.max_radius <= 4096.0f)) {
        ctx->fail("depth-of-field max_radius %g outside 0..4096 pixels", (double)view->dof.max_radius);
        r = SGL_ERR_INVALID;
    }
    if (r != SGL_OK)
        return r;
    const sgl_view &v = *view;
    const size_t px = (size_t)v.w * v.h;
    cudaStream_t st = device_buffers ? (cudaStream_t)stream : ctx->stream;
    uint32_t *src = nullptr, *dst = nullptr;
    int src_pitch = 0, dst_pitch = 0;
    float *z = nullptr;
    if (device_buffers) {
        src = (uint32_t *)in->pixels + (size_t)v.y * (in->pitch / 4) + v.x;
        dst = (uint32_t *)out->pixels + (size_t)v.y * (out->pitch / 4) + v.x;
        src_pitch = in->pitch / 4;
        dst_pitch = out->pitch / 4;
        z = in->zbuffer;
    } else {
        CUDA_TRY(ctx->dof_stage.ensure(12 * px));
        src = (uint32_t *)ctx->dof_stage.ptr;
        dst = src + px;
        z = (float *)(dst + px);
        src_pitch = dst_pitch = v.w;
        CUDA_TRY(cudaMemcpy2DAsync(src, 4 * (size_t)v.w, (const uint8_t *)in->pixels + (size_t)v.y * in->pitch +
                                                            4 * (size_t)v.x,
                                   in->pitch, 4 * (size_t)v.w, v.h, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(z, in->zbuffer, 4 * px, cudaMemcpyHostToDevice, st));
    }
    ItemDev it{};
    it.v = make_view(v);
    it.pixels = src;
    it.pitch_px = src_pitch;
    it.dof_src = src;
    it.dof_src_pitch = src_pitch;
    it.zbuf = z;
    it.dof = 1;
    it.dof_out = dst;
    it.dof_pitch = dst_pitch;
    const float k = v.dof.px_scale > 0.0f ? v.dof.px_scale : (v.proj[5] * (float)v.h) / 2.0f;
    it.dof_focus = v.dof.focus;
    it.dof_ka = k * v.dof.aperture;
    it.dof_rmax = v.dof.max_radius;
    it.p22 = v.proj[10];
    it.p23 = v.proj[11];
    it.dof_halo = dof_halo_of(v.dof.max_radius);
    it.dof_tiles_x = (v.w + kDofTile - 1) / kDofTile;
    const uint32_t dof_tiles = (uint32_t)it.dof_tiles_x * (uint32_t)((v.h + kDofTile - 1) / kDofTile);
    const size_t counters_at = (sizeof(ItemDev) + sizeof(BatchDev) + 4 * sizeof(uint32_t) + 15) & ~(size_t)15;
    CUDA_TRY(ctx->dof_desc.ensure(counters_at + sizeof(unsigned long long) * kCounterWords));
    uint8_t *dd = (uint8_t *)ctx->dof_desc.ptr;
    ItemDev *d_it = (ItemDev *)dd;
    BatchDev *d_b = (BatchDev *)(dd + sizeof(ItemDev));
    uint32_t *d_base = (uint32_t *)(dd + sizeof(ItemDev) + sizeof(BatchDev));
    BatchDev b{};
    b.items = d_it;
    b.counters = (unsigned long long *)(dd + counters_at); // the gather's tile counter
    b.px_base = d_base;
    b.dof_base = d_base + 2;
    b.n_items = 1;
    b.total_px = (uint32_t)px;
    b.total_dof_tiles = dof_tiles;
    const uint32_t base[4] = {0u, (uint32_t)px, 0u, dof_tiles};
    CUDA_TRY(cudaMemcpyAsync(d_it, &it, sizeof it, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_b, &b, sizeof b, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_base, base, sizeof base, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(b.counters, 0, sizeof(unsigned long long) * kCounterWords, st));
    CUDA_TRY(launch_dof(d_b, st));
    if (!device_buffers) {
        CUDA_TRY(cudaMemcpy2DAsync((uint8_t *)out->pixels + (size_t)v.y * out->pitch + 4 * (size_t)v.x, out->pitch,
                                   dst, 4 * (size_t)v.w, 4 * (size_t)v.w, v.h, cudaMemcpyDeviceToHost, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st)); // the descriptors above live on this call's stack
    return SGL_OK;
}

SGL_API sgl_status sgl_check_status(sgl_ctx *c, uint32_t *code, uint64_t *index, uint32_t *count, int reset)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || !code || !index || !count)
        return SGL_ERR_INVALID;
    cudaSetDevice(ctx->device);
    bool compiled = false;
    unsigned cd = 0, n = 0;
    unsigned long long ix = 0;
    CUDA_TRY(check_status(&cd, &ix, &n, reset != 0, &compiled));
    if (!compiled) {
        ctx->fail("this build has no device-side bounds checks (load libsgl_check.so)");
        return SGL_ERR_UNSUPPORTED;
    }
    *code = cd;
    *index = ix;
    *count = n;
    return SGL_OK;
}

SGL_API sgl_status sgl_profile(sgl_ctx *c, int enable)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx)
        return SGL_ERR_INVALID;
    prof_flush(&ctx->prof);
    ctx->prof.enabled = enable != 0;
    for (int k = 0; k < kProfKernels; k++) {
        ctx->prof.ms[k] = 0.0;
        ctx->prof.launches[k] = 0;
    }
    return SGL_OK;
}

SGL_API sgl_status sgl_profile_read(sgl_ctx *c, int kernel, const char **name, double *total_ms, uint64_t *launches)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || kernel < 0)
        return SGL_ERR_INVALID;
    if (kernel >= kProfKernels)
        return SGL_ERR_NOT_FOUND;
    prof_flush(&ctx->prof);
    if (name)
        *name = prof_kernel_name(kernel);
    if (total_ms)
        *total_ms = ctx->prof.ms[kernel];
    if (launches)
        *launches = ctx->prof.launches[kernel];
    return SGL_OK;
}

} // extern "C"
