// sgl_api.cpp — host runtime behind the C ABI of include/sgl.h: contexts,
// device-resident scenes, per-view frame setup and the launch sequence.
//
// Host arithmetic that feeds bit-exact results (node matrices, viewport
// matrix) repeats the reference's single-precision operation order; this file
// is compiled with -ffp-contract=off.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sgl.h"
#include "sgl_internal.h"
#include "sgl_runtime.h"

namespace sgl {

// ------------------------------------------------------------- utilities --

void Ctx::fail(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    last_error = buf;
}

DevBuf::~DevBuf() { release(); }

void DevBuf::release()
{
    if (ptr)
        cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

cudaError_t DevBuf::ensure(size_t need)
{
    if (need <= bytes && ptr)
        return cudaSuccess;
    release();
    size_t n = std::max<size_t>(need, 256);
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return e;
    }
    bytes = n;
    return cudaSuccess;
}

// scale(m, v) (src/projection/points.cpp:14-30)
static void scale_m(float *r, const float *m, const float *s)
{
    std::memcpy(r, m, 16 * sizeof(float));
    for (int row = 0; row < 4; row++)
        for (int c = 0; c < 3; c++)
            r[row * 4 + c] *= s[c];
}

// 4x4 product summed k = 0..3 left to right (the order of freon::Matrix as
// the reference is built here; every order gives the same bits for the
// identity parent of a root node)
static void matmul4(float *r, const float *a, const float *b)
{
    float t[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            float s = a[i * 4 + 0] * b[0 * 4 + j];
            for (int k = 1; k < 4; k++)
                s = s + a[i * 4 + k] * b[k * 4 + j];
            t[i * 4 + j] = s;
        }
    std::memcpy(r, t, sizeof t);
}

static const float kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

// node_t::get_local_world_matrix (swegl/data/model.hpp:56-61) composed with
// the parents as vertex_shader_t::original_to_world does (vertex_shaders.hpp:16-33)
static bool node_matrices(const std::vector<sgl_node_desc> &nodes, std::vector<float> &world, std::vector<float> &rs)
{
    const int n = (int)nodes.size();
    world.assign(16 * (size_t)std::max(n, 1), 0.0f);
    rs.assign(16 * (size_t)std::max(n, 1), 0.0f);
    std::vector<int> state(n, 0); // 0 todo, 1 in progress, 2 done
    std::vector<int> stack;
    for (int i = 0; i < n; i++) {
        if (state[i] == 2)
            continue;
        stack.push_back(i);
        while (!stack.empty()) {
            int k = stack.back();
            int p = nodes[k].parent;
            if (p >= 0 && state[p] != 2) {
                if (state[p] == 1 || p >= n)
                    return false; // cycle or bad parent
                state[k] = 1;
                stack.push_back(p);
                continue;
            }
            float local[16];
            scale_m(local, nodes[k].rotation, nodes[k].scale);
            std::memcpy(&rs[16 * (size_t)k], local, sizeof local);
            local[3] += nodes[k].translation[0];
            local[7] += nodes[k].translation[1];
            local[11] += nodes[k].translation[2];
            matmul4(&world[16 * (size_t)k], p >= 0 ? &world[16 * (size_t)p] : kIdentity, local);
            state[k] = 2;
            stack.pop_back();
        }
    }
    return true;
}

static uint32_t prim_triangles(const sgl_primitive_desc &p)
{
    if (p.mode == SGL_TRIANGLES)
        return p.index_count / 3;
    if (p.mode == SGL_TRIANGLE_STRIP || p.mode == SGL_TRIANGLE_FAN)
        return p.index_count >= 2 ? p.index_count - 2 : 0;
    return 0;
}

template <typename T>
static cudaError_t upload(DevBuf &b, const T *src, size_t n)
{
    cudaError_t e = b.ensure(sizeof(T) * std::max<size_t>(n, 1));
    if (e != cudaSuccess || n == 0)
        return e;
    return cudaMemcpy(b.ptr, src, sizeof(T) * n, cudaMemcpyHostToDevice);
}

#define CUDA_TRY(expr)                                                                                                 \
    do {                                                                                                               \
        cudaError_t _e = (expr);                                                                                       \
        if (_e != cudaSuccess) {                                                                                       \
            ctx->fail("%s: %s", #expr, cudaGetErrorString(_e));                                                        \
            return _e == cudaErrorMemoryAllocation ? SGL_ERR_OOM : SGL_ERR_CUDA;                                       \
        }                                                                                                              \
    } while (0)

// --------------------------------------------------------------- scenes --

sgl_status Scene::refresh_nodes(Ctx *ctx)
{
    std::vector<float> world, rs;
    if (!node_matrices(nodes, world, rs)) {
        ctx->fail("node hierarchy has a cycle or a bad parent index");
        return SGL_ERR_INVALID;
    }
    CUDA_TRY(upload(d_node_world, world.data(), world.size()));
    CUDA_TRY(upload(d_node_rs, rs.data(), rs.size()));
    dev.node_world = (const float *)d_node_world.ptr;
    dev.node_rs = (const float *)d_node_rs.ptr;
    CUDA_TRY(launch_world(dev, 0));
    CUDA_TRY(cudaStreamSynchronize(0));
    return SGL_OK;
}

sgl_status Scene::set_lights(Ctx *ctx, float ambient, const float *sun, float sun_intensity, const sgl_point_light *pl,
                             int n)
{
    if (n < 0 || (n > 0 && !pl) || !sun) {
        ctx->fail("bad light arguments");
        return SGL_ERR_INVALID;
    }
    if (n > kMaxPointLights) {
        ctx->fail("%d point lights; the GPU path supports at most %d", n, kMaxPointLights);
        return SGL_ERR_UNSUPPORTED;
    }
    lights.ambient = ambient;
    lights.sun[0] = sun[0];
    lights.sun[1] = sun[1];
    lights.sun[2] = sun[2];
    lights.sun_intensity = sun_intensity;
    lights.n = n;
    for (int i = 0; i < n; i++)
        lights.pl[i] = make_float4(pl[i].position[0], pl[i].position[1], pl[i].position[2], pl[i].intensity);
    return SGL_OK;
}

static sgl_status validate_scene(Ctx *ctx, const sgl_scene_desc *d)
{
    if (!d || d->n_nodes < 0 || d->n_primitives < 0 || d->n_materials < 0 || d->n_textures < 0 ||
        d->n_point_lights < 0) {
        ctx->fail("null or negative-sized scene description");
        return SGL_ERR_INVALID;
    }
    if ((d->n_nodes && !d->nodes) || (d->n_primitives && !d->primitives) ||
        (d->n_vertices && (!d->positions || !d->normals || !d->uvs)) || (d->n_indices && !d->indices) ||
        (d->n_materials && !d->materials) || (d->n_textures && !d->textures) ||
        (d->n_point_lights && !d->point_lights)) {
        ctx->fail("scene description has a null array with a non-zero count");
        return SGL_ERR_INVALID;
    }
    for (int i = 0; i < d->n_nodes; i++)
        if (d->nodes[i].parent < -1 || d->nodes[i].parent >= d->n_nodes) {
            ctx->fail("node %d has bad parent %d", i, d->nodes[i].parent);
            return SGL_ERR_INVALID;
        }
    for (int t = 0; t < d->n_textures; t++) {
        const sgl_texture_desc &td = d->textures[t];
        if (!td.texels || td.width <= 0 || td.height <= 0 || (int64_t)td.width * td.height > (1ll << 28)) {
            ctx->fail("texture %d: bad texels or size %dx%d", t, td.width, td.height);
            return SGL_ERR_INVALID;
        }
    }
    for (int m = 0; m < d->n_materials; m++)
        if (d->materials[m].texture < -1 || d->materials[m].texture >= d->n_textures ||
            d->materials[m].shininess < 0 || d->materials[m].shininess > 1024) {
            ctx->fail("material %d: bad texture index or shininess", m);
            return SGL_ERR_INVALID;
        }
    uint64_t tris = 0;
    for (int p = 0; p < d->n_primitives; p++) {
        const sgl_primitive_desc &pd = d->primitives[p];
        if (pd.node < 0 || pd.node >= d->n_nodes) {
            ctx->fail("primitive %d: bad node %d", p, pd.node);
            return SGL_ERR_INVALID;
        }
        if (pd.mode != SGL_TRIANGLES && pd.mode != SGL_TRIANGLE_STRIP && pd.mode != SGL_TRIANGLE_FAN) {
            ctx->fail("primitive %d: mode %d is not a triangle mode", p, pd.mode);
            return SGL_ERR_UNSUPPORTED;
        }
        if (pd.material < -1 || pd.material >= d->n_materials) {
            ctx->fail("primitive %d: bad material %d", p, pd.material);
            return SGL_ERR_INVALID;
        }
        if ((uint64_t)pd.vertex_offset + pd.vertex_count > d->n_vertices ||
            (uint64_t)pd.index_offset + pd.index_count > d->n_indices) {
            ctx->fail("primitive %d: vertex or index range outside the arrays", p);
            return SGL_ERR_INVALID;
        }
        for (uint32_t i = 0; i < pd.index_count; i++)
            if (d->indices[pd.index_offset + i] >= pd.vertex_count) {
                ctx->fail("primitive %d: index %u out of its %u vertices", p, d->indices[pd.index_offset + i],
                          pd.vertex_count);
                return SGL_ERR_INVALID;
            }
        tris += prim_triangles(pd);
    }
    if (tris >= (1ull << 31)) {
        ctx->fail("too many triangles (%llu)", (unsigned long long)tris);
        return SGL_ERR_UNSUPPORTED;
    }
    return SGL_OK;
}

sgl_status Scene::upload_desc(Ctx *ctx, const sgl_scene_desc *d)
{
    sgl_status st = validate_scene(ctx, d);
    if (st != SGL_OK)
        return st;
    nodes.assign(d->nodes, d->nodes + d->n_nodes);
    n_vertices = d->n_vertices;
    // Draw order: node by node, primitives of a node in description order
    // (renderer.cpp:83,191).
    std::vector<int> order;
    order.reserve(d->n_primitives);
    {
        std::vector<std::vector<int>> by_node(std::max(d->n_nodes, 1));
        for (int p = 0; p < d->n_primitives; p++)
            by_node[d->primitives[p].node].push_back(p);
        for (auto &v : by_node)
            order.insert(order.end(), v.begin(), v.end());
    }
    std::vector<PrimDesc> prims(order.size());
    std::vector<uint4> tris;
    std::vector<uint32_t> vnode(d->n_vertices, 0);
    uint64_t total = 0;
    for (int p : order)
        total += prim_triangles(d->primitives[p]);
    tris.reserve(total);
    for (size_t q = 0; q < order.size(); q++) {
        const sgl_primitive_desc &p = d->primitives[order[q]];
        prims[q].material = p.material;
        prims[q].node = p.node;
        for (uint32_t v = 0; v < p.vertex_count; v++)
            vnode[p.vertex_offset + v] = (uint32_t)p.node;
        const uint32_t *idx = d->indices + p.index_offset;
        const uint32_t base = p.vertex_offset;
        const uint32_t nt = prim_triangles(p);
        for (uint32_t t = 0; t < nt; t++) {
            uint32_t i0, i1, i2;
            if (p.mode == SGL_TRIANGLE_STRIP) { // renderer.cpp:198-207, with the parity swap
                const uint32_t i = t + 2;
                i0 = idx[i - 2];
                i1 = idx[i - 1 + (i & 1)];
                i2 = idx[i - (i & 1)];
            } else if (p.mode == SGL_TRIANGLE_FAN) { // :209-218
                const uint32_t i = t + 2;
                i0 = idx[0];
                i1 = idx[i - 1];
                i2 = idx[i];
            } else { // :220-229
                i0 = idx[3 * t];
                i1 = idx[3 * t + 1];
                i2 = idx[3 * t + 2];
            }
            tris.push_back(make_uint4(base + i0, base + i1, base + i2, (uint32_t)q));
        }
    }
    n_triangles = (uint32_t)tris.size();
    std::vector<float4> pos_u(d->n_vertices), nrm_v(d->n_vertices);
    for (uint32_t g = 0; g < d->n_vertices; g++) {
        pos_u[g] = make_float4(d->positions[3 * g], d->positions[3 * g + 1], d->positions[3 * g + 2], d->uvs[2 * g]);
        nrm_v[g] = make_float4(d->normals[3 * g], d->normals[3 * g + 1], d->normals[3 * g + 2], d->uvs[2 * g + 1]);
    }
    std::vector<MatDesc> mats(std::max(d->n_materials, 1));
    for (int m = 0; m < d->n_materials; m++)
        mats[m] = MatDesc{d->materials[m].color, d->materials[m].texture, d->materials[m].double_sided,
                          d->materials[m].shininess};
    // textures: one allocation, 256-byte aligned per texture
    std::vector<size_t> tex_off(d->n_textures);
    size_t tex_words = 0;
    for (int t = 0; t < d->n_textures; t++) {
        tex_off[t] = tex_words;
        tex_words += ((size_t)d->textures[t].width * d->textures[t].height + 63) & ~(size_t)63;
    }
    CUDA_TRY(d_texels.ensure(sizeof(uint32_t) * std::max<size_t>(tex_words, 1)));
    std::vector<TexDesc> texs(std::max(d->n_textures, 1));
    for (int t = 0; t < d->n_textures; t++) {
        const sgl_texture_desc &td = d->textures[t];
        uint32_t *dst = (uint32_t *)d_texels.ptr + tex_off[t];
        CUDA_TRY(cudaMemcpy(dst, td.texels, sizeof(uint32_t) * (size_t)td.width * td.height, cudaMemcpyHostToDevice));
        texs[t] = TexDesc{dst, td.width, td.height};
    }
    CUDA_TRY(upload(d_pos_u, pos_u.data(), pos_u.size()));
    CUDA_TRY(upload(d_nrm_v, nrm_v.data(), nrm_v.size()));
    CUDA_TRY(upload(d_vnode, vnode.data(), vnode.size()));
    CUDA_TRY(upload(d_tris, tris.data(), tris.size()));
    CUDA_TRY(upload(d_prims, prims.data(), std::max<size_t>(prims.size(), 1)));
    CUDA_TRY(upload(d_mats, mats.data(), mats.size()));
    CUDA_TRY(upload(d_texs, texs.data(), texs.size()));
    CUDA_TRY(d_wpos.ensure(sizeof(float4) * std::max<size_t>(n_vertices, 1)));
    CUDA_TRY(d_wnrm.ensure(sizeof(float4) * std::max<size_t>(n_vertices, 1)));
    CUDA_TRY(d_uv.ensure(sizeof(float2) * std::max<size_t>(n_vertices, 1)));
    dev = SceneDev{};
    dev.pos_u = (const float4 *)d_pos_u.ptr;
    dev.nrm_v = (const float4 *)d_nrm_v.ptr;
    dev.vnode = (const uint32_t *)d_vnode.ptr;
    dev.tris = (const uint4 *)d_tris.ptr;
    dev.prims = (const PrimDesc *)d_prims.ptr;
    dev.mats = (const MatDesc *)d_mats.ptr;
    dev.texs = (const TexDesc *)d_texs.ptr;
    dev.wpos = (float4 *)d_wpos.ptr;
    dev.wnrm = (float4 *)d_wnrm.ptr;
    dev.uv = (float2 *)d_uv.ptr;
    dev.n_vertices = n_vertices;
    dev.n_triangles = n_triangles;
    dev.n_mats = d->n_materials;
    dev.n_texs = d->n_textures;
    dev.default_mat = MatDesc{d->default_material.color, d->default_material.texture,
                              d->default_material.double_sided, d->default_material.shininess};
    if (dev.default_mat.texture >= d->n_textures)
        dev.default_mat.texture = -1;
    st = set_lights(ctx, d->ambient, d->sun_direction, d->sun_intensity, d->point_lights, d->n_point_lights);
    if (st != SGL_OK)
        return st;
    st = refresh_nodes(ctx);
    if (st != SGL_OK)
        return st;
    device_bytes = d_pos_u.bytes + d_nrm_v.bytes + d_vnode.bytes + d_tris.bytes + d_prims.bytes + d_mats.bytes +
                   d_texs.bytes + d_texels.bytes + d_wpos.bytes + d_wnrm.bytes + d_uv.bytes + d_node_world.bytes + d_node_rs.bytes;
    return SGL_OK;
}

// ---------------------------------------------------------------- views --

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
    // viewport_t constructor (src/render/viewport.cpp:94-97): x+w/2.0f, w/2.0f, -h/2.0f
    d.vm00 = (float)v.w / 2.0f;
    d.vm03 = (float)v.x + (float)v.w / 2.0f;
    d.vm11 = (float)(-v.h) / 2.0f;
    d.vm13 = (float)v.y + (float)v.h / 2.0f;
    return d;
}

sgl_status check_view(Ctx *ctx, const sgl_view &v, const sgl_target &t)
{
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

// Render one view into device buffers (surface rect + z) on `st`.
sgl_status render_view_device(Ctx *ctx, Scene &s, const sgl_view &view, uint32_t *rect_pixels, int pitch_px,
                              float *zbuf, FrameScratch &fs, cudaStream_t st, uint8_t *slot_flags, int *launches,
                              Profiler *prof)
{
    const size_t px = (size_t)view.w * view.h;
    const size_t span_cap = std::max<size_t>(65536, px / 8);
    CUDA_TRY(fs.ndc.ensure(sizeof(float4) * std::max<uint32_t>(s.n_vertices, 1)));
    CUDA_TRY(fs.yes.ensure(std::max<uint32_t>(s.n_vertices, 1)));
    CUDA_TRY(fs.key.ensure(sizeof(unsigned long long) * px));
    CUDA_TRY(fs.prec.ensure(sizeof(float4) * px));
    CUDA_TRY(fs.classes.ensure(sizeof(uint32_t) * kClasses * (size_t)std::max<uint32_t>(s.n_triangles, 1)));
    CUDA_TRY(fs.cliptri.ensure(sizeof(uint32_t) * std::max<uint32_t>(s.n_triangles, 1)));
    CUDA_TRY(fs.clippx.ensure(sizeof(uint32_t) * px));
    CUDA_TRY(fs.spans.ensure(sizeof(SpanRec) * span_cap));
    CUDA_TRY(fs.counters.ensure(kCounterWords * sizeof(unsigned long long)));
    FrameDev f;
    f.ndc = (float4 *)fs.ndc.ptr;
    f.yes = (uint8_t *)fs.yes.ptr;
    f.key = (unsigned long long *)fs.key.ptr;
    f.prec = (float4 *)fs.prec.ptr;
    f.classes = (uint32_t *)fs.classes.ptr;
    f.cliptri = (uint32_t *)fs.cliptri.ptr;
    f.clippx = (uint32_t *)fs.clippx.ptr;
    f.spans = (SpanRec *)fs.spans.ptr;
    f.span_cap = (uint32_t)std::min<size_t>(fs.spans.bytes / sizeof(SpanRec), 0xFFFFFFFFu);
    f.pixels = rect_pixels;
    f.pitch_px = pitch_px;
    f.zbuf = zbuf;
    f.counters = (unsigned long long *)fs.counters.ptr;
    f.counters32 = (uint32_t *)fs.counters.ptr;
    f.slot_flags = slot_flags;
    const ViewDev v = make_view(view);
    CUDA_TRY(launch_frame(s.dev, s.lights, v, f, st, launches, prof));
    return SGL_OK;
}

} // namespace sgl

using namespace sgl;

// ----------------------------------------------------------------- C ABI --

extern "C" {

SGL_API int sgl_version(void) { return 1; }

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
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return SGL_ERR_CUDA;
    }
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
    ctx->scenes.clear();
    if (ctx->stream)
        cudaStreamDestroy(ctx->stream);
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
    cudaSetDevice(ctx->device);
    std::vector<sgl_node_desc> saved = s->nodes;
    s->nodes.assign(nodes, nodes + n_nodes);
    sgl_status st = s->refresh_nodes(ctx);
    if (st != SGL_OK)
        s->nodes = saved;
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

static sgl_status read_stats(Ctx *ctx, FrameScratch &fs, cudaStream_t st, sgl_frame_stats *acc)
{
    unsigned long long h[2]; // [C_DRAWN], [C_FRAGMENTS]
    CUDA_TRY(cudaMemcpyAsync(h, fs.counters.ptr, sizeof h, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    acc->drawn_triangles += h[0];
    acc->fragments += h[1];
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
    cudaStream_t st = device_buffers ? (cudaStream_t)stream : ctx->stream;
    sgl_frame_stats acc{};
    int launches = 0;
    for (int i = 0; i < n_views; i++) {
        const sgl_view &v = views[i];
        const sgl_target &t = targets[i];
        const int pitch_px = t.pitch / 4;
        if (device_buffers) {
            uint32_t *rect = (uint32_t *)t.pixels + (size_t)v.y * pitch_px + v.x;
            sgl_status r = render_view_device(ctx, *s, v, rect, pitch_px, t.zbuffer, ctx->frame, st, nullptr,
                                              &launches, &ctx->prof);
            if (r != SGL_OK)
                return r;
        } else {
            const size_t px = (size_t)v.w * v.h;
            CUDA_TRY(ctx->stage_pixels.ensure(4 * px));
            CUDA_TRY(ctx->stage_z.ensure(4 * px));
            sgl_status r = render_view_device(ctx, *s, v, (uint32_t *)ctx->stage_pixels.ptr, v.w,
                                              (float *)ctx->stage_z.ptr, ctx->frame, st, nullptr, &launches,
                                              &ctx->prof);
            if (r != SGL_OK)
                return r;
            uint8_t *dst = (uint8_t *)t.pixels + (size_t)v.y * t.pitch + 4 * (size_t)v.x;
            CUDA_TRY(cudaMemcpy2DAsync(dst, t.pitch, ctx->stage_pixels.ptr, 4 * (size_t)v.w, 4 * (size_t)v.w, v.h,
                                       cudaMemcpyDeviceToHost, st));
            if (t.zbuffer)
                CUDA_TRY(cudaMemcpyAsync(t.zbuffer, ctx->stage_z.ptr, 4 * px, cudaMemcpyDeviceToHost, st));
            if (stats) {
                sgl_status r2 = read_stats(ctx, ctx->frame, st, &acc);
                if (r2 != SGL_OK)
                    return r2;
            }
            CUDA_TRY(cudaStreamSynchronize(st));
        }
        acc.pixels += (uint64_t)v.w * v.h;
    }
    if (stats) {
        if (device_buffers) {
            // per-view counters are not kept apart in the asynchronous mode: report the last view
            sgl_status r2 = read_stats(ctx, ctx->frame, st, &acc);
            if (r2 != SGL_OK)
                return r2;
        }
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
    if (r != SGL_OK)
        return r;
    cudaStream_t st = ctx->stream;
    const size_t px = (size_t)view->w * view->h;
    CUDA_TRY(ctx->stage_pixels.ensure(4 * px));
    CUDA_TRY(ctx->stage_z.ensure(4 * px));
    CUDA_TRY(ctx->debug_flags.ensure(2 * (size_t)std::max<uint32_t>(s->n_triangles, 1)));
    CUDA_TRY(cudaMemsetAsync(ctx->debug_flags.ptr, 0, 2 * (size_t)std::max<uint32_t>(s->n_triangles, 1), st));
    int launches = 0;
    r = render_view_device(ctx, *s, *view, (uint32_t *)ctx->stage_pixels.ptr, view->w, (float *)ctx->stage_z.ptr,
                           ctx->frame, st, (uint8_t *)ctx->debug_flags.ptr, &launches);
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
        CUDA_TRY(cudaMemcpyAsync(keys.data(), ctx->frame.key.ptr, 8 * px, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        for (size_t i = 0; i < px; i++)
            winner[i] = keys[i] == kEmptyKey ? 0xFFFFFFFFu : (uint32_t)(keys[i] & 0xFFFFFFFFu);
    }
    if (slot_flags)
        CUDA_TRY(cudaMemcpyAsync(slot_flags, ctx->debug_flags.ptr, 2 * (size_t)s->n_triangles,
                                 cudaMemcpyDeviceToHost, st));
    sgl_frame_stats acc{};
    r = read_stats(ctx, ctx->frame, st, &acc);
    if (r != SGL_OK)
        return r;
    CUDA_TRY(cudaStreamSynchronize(st));
    if (stats) {
        acc.triangles = s->n_triangles;
        acc.pixels = px;
        acc.kernel_launches = (uint32_t)launches;
        *stats = acc;
    }
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
