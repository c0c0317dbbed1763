// sgl_scene.cpp — device-resident scenes: validation, upload, node matrices
// and lights.
//
// Host arithmetic that feeds bit-exact results (node matrices) repeats the
// reference's single-precision operation order; compiled with -ffp-contract=off.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
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
    // A first allocation takes what is asked (scene arrays are allocated once).
    // A buffer that has to grow — a scratch pool meeting a larger batch —
    // takes half again its size, in 2 MB steps, so that a stream of batches of
    // varying size reallocates rarely: each reallocation frees the old block,
    // and cudaFree waits for the whole device, every stream included.
    const size_t want = std::max<size_t>(need, 256);
    size_t n = want;
    if (ptr) {
        constexpr size_t kStep = 2u << 20;
        n = std::max(n, bytes + bytes / 2);
        n = (n + kStep - 1) / kStep * kStep;
    }
    release();
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess && n > want) {
        cudaGetLastError(); // no room for the headroom: take what is needed
        n = want;
        e = cudaMalloc(&ptr, n);
    }
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
bool node_matrices(const std::vector<sgl_node_desc> &nodes, std::vector<float> &world, std::vector<float> &rs)
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
    CUDA_TRY(cudaDeviceSynchronize()); // in-flight frames read the world positions
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
    LightsDev l{};
    l.ambient = ambient;
    l.sun[0] = sun[0];
    l.sun[1] = sun[1];
    l.sun[2] = sun[2];
    l.sun_intensity = sun_intensity;
    l.n = n;
    for (int i = 0; i < n; i++)
        l.pl[i] = make_float4(pl[i].position[0], pl[i].position[1], pl[i].position[2], pl[i].intensity);
    // in-flight frames read the lights from device memory: wait for them first
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(upload(d_lights, &l, 1));
    dev.lights = (const LightsDev *)d_lights.ptr;
    lights = l;
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
    // every primitive owns its vertices (primitive_t::vertices): no two
    // vertex ranges overlap
    std::vector<std::pair<uint32_t, int>> ranges;
    ranges.reserve(d->n_primitives);
    for (int p = 0; p < d->n_primitives; p++)
        if (d->primitives[p].vertex_count)
            ranges.emplace_back(d->primitives[p].vertex_offset, p);
    std::sort(ranges.begin(), ranges.end());
    uint64_t end = 0;
    int end_prim = -1;
    for (const auto &r : ranges) {
        if (r.first < end) {
            ctx->fail("primitives %d and %d share vertices (each primitive owns its vertex range)", end_prim,
                      r.second);
            return SGL_ERR_INVALID;
        }
        end = (uint64_t)r.first + d->primitives[r.second].vertex_count;
        end_prim = r.second;
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
    std::vector<uint4> pgeo(order.size());
    std::vector<uint8_t> psmall(std::max<size_t>(order.size(), 1), 0);
    bool any_small = false, any_big = false;
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
        pgeo[q] = make_uint4(p.vertex_offset, p.vertex_count, (uint32_t)tris.size(), nt);
        psmall[q] = (p.vertex_count <= kFuseVerts && nt <= kFuseTris) ? 1 : 0;
        any_small |= psmall[q] != 0;
        any_big |= psmall[q] == 0;
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
    CUDA_TRY(upload(d_prims, prims.data(), prims.size()));
    CUDA_TRY(upload(d_pgeo, pgeo.data(), pgeo.size()));
    CUDA_TRY(upload(d_mats, mats.data(), mats.size()));
    CUDA_TRY(upload(d_texs, texs.data(), texs.size()));
    // per draw-order primitive: the material and texture the pixel shader binds
    const MatDesc def_mat{d->default_material.color,
                          d->default_material.texture < d->n_textures ? d->default_material.texture : -1,
                          d->default_material.double_sided, d->default_material.shininess};
    std::vector<PrimShade> pshade(std::max<size_t>(prims.size(), 1));
    for (size_t q = 0; q < prims.size(); q++) {
        const int mi = prims[q].material;
        const bool in_range = mi >= 0 && mi < d->n_materials;
        const MatDesc &m = in_range ? mats[mi] : def_mat;
        PrimShade ps{};
        ps.color = m.color;
        ps.shininess = m.shininess;
        ps.double_sided = in_range && mats[mi].double_sided ? 1 : 0;
        if (m.texture < 0 || m.texture >= d->n_textures) {
            ps.tex = nullptr;
            ps.tw = ps.th = 1;
        } else {
            ps.tex = texs[m.texture].texels;
            ps.tw = texs[m.texture].w;
            ps.th = texs[m.texture].h;
        }
        pshade[q] = ps;
    }
    CUDA_TRY(upload(d_pshade, pshade.data(), pshade.size()));
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
    dev.pgeo = (const uint4 *)d_pgeo.ptr;
    dev.pshade = (const PrimShade *)d_pshade.ptr;
    dev.n_prims = (uint32_t)pgeo.size();
    // Primitives within kFuseVerts / kFuseTris take the fused geometry pass.
    // A scene that also has larger ones runs the general passes as well, and
    // each pass skips the other's primitives: the general passes skip the
    // triangles of fused-pass primitives and the vertices that only those use
    // (a vertex that a larger primitive shares is transformed by both, to the
    // same value).
    dev.fused = any_small ? 1 : 0;
    dev.mixed = any_small && any_big ? 1 : 0;
    if (dev.mixed) {
        std::vector<uint8_t> vsmall(std::max<uint32_t>(n_vertices, 1), 0);
        for (size_t q = 0; q < pgeo.size(); q++)
            if (psmall[q])
                std::fill(vsmall.begin() + pgeo[q].x, vsmall.begin() + pgeo[q].x + pgeo[q].y, (uint8_t)1);
        for (size_t q = 0; q < pgeo.size(); q++)
            if (!psmall[q])
                std::fill(vsmall.begin() + pgeo[q].x, vsmall.begin() + pgeo[q].x + pgeo[q].y, (uint8_t)0);
        CUDA_TRY(upload(d_psmall, psmall.data(), psmall.size()));
        CUDA_TRY(upload(d_vsmall, vsmall.data(), vsmall.size()));
        dev.psmall = (const uint8_t *)d_psmall.ptr;
        dev.vsmall = (const uint8_t *)d_vsmall.ptr;
    }
    if (dev.fused) { // the primitives' boxes, written with the world positions
        CUDA_TRY(d_pbox.ensure(2 * sizeof(float4) * pgeo.size()));
        dev.pbox = (float4 *)d_pbox.ptr;
    }
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
                   d_texs.bytes + d_texels.bytes + d_wpos.bytes + d_wnrm.bytes + d_uv.bytes + d_node_world.bytes + d_node_rs.bytes + d_lights.bytes + d_pgeo.bytes + d_pshade.bytes + d_psmall.bytes + d_vsmall.bytes + d_pbox.bytes;
    return SGL_OK;
}

} // namespace sgl
