/*
 * ref_harness.cpp — drives gbizzotto/swegl's own, unmodified render path
 * (compiled from the reference sources by oracle/ref/Makefile) on a scene
 * given in the flat sgl_scene_desc layout, headless.
 *
 * TEST INFRASTRUCTURE ONLY.  Built into oracle/_ref/libswegl_ref.so, used by
 * tests/golden/make_golden.py to produce golden fixtures and to validate the
 * CPU restatement in oracle/sgl_oracle.c.  Nothing in the product links it.
 *
 * What it calls (paths inside the reference):
 *   vertex_shader_t::original_to_world   swegl/render/vertex_shaders.hpp:29-33
 *   _render(scene, viewport)             src/render/renderer.cpp:77-235
 * which is exactly render(scene, vp...) of swegl/render/renderer.hpp:27-34.
 *
 * Extra pixel shaders plug into the reference's own plug-in hooks
 * (swegl/render/pixel_shaders.hpp:15-29) to expose internal state:
 *   kind 1  ordinal of the fill_triangle_2 call that won the pixel
 *   kind 2  bits of the per-pixel perspective progress
 *   kind 3  the Phong light value (65536 * L, as the int the shader returns)
 *   kind 4  the bilinear texel colour alone
 * Kind 0 renders with the reference shader the view's `shader` field names
 * (SGL_SHADER_*, include/sgl.h).
 *
 * Also exported: matrix44_t::from_quaternion
 * (swegl/projection/matrix44.hpp:34-43) and scene_t::animate
 * (swegl/data/model.hpp:146-177) on flat inputs, which pin the glTF node and
 * animation arithmetic of the restatement.  The reference's glTF loader
 * itself is driven by ref_gltf.cpp (its nlohmann/json include resolves to
 * the stand-in in shim/json.hpp).
 */
#include <cstring>
#include <memory>
#include <vector>

#include <swegl/render/renderer.hpp>
#include <swegl/render/pixel_shaders.hpp>
#include <swegl/render/post_shaders.hpp>
#include <swegl/render/vertex_shaders.hpp>

#include "sgl.h"

namespace {

struct id_shader : swegl::pixel_shader_t {
    int calls = 0;
    void prepare_for_triangle(swegl::vertex_idx, swegl::vertex_idx, swegl::vertex_idx, bool) override { calls++; }
    int shade(float) override { return calls - 1; }
};

struct progress_shader : swegl::pixel_shader_t {
    int shade(float progress) override
    {
        int bits;
        std::memcpy(&bits, &progress, 4);
        return bits;
    }
};

// Counts prepare_for_triangle calls while forwarding to a reference shader.
struct counting_base {
    uint64_t calls = 0;
};
template <class S>
struct counting : S, counting_base {
    void prepare_for_triangle(swegl::vertex_idx i0, swegl::vertex_idx i1, swegl::vertex_idx i2, bool inv) override
    {
        calls++;
        S::prepare_for_triangle(i0, i1, i2, inv);
    }
};
using counting_full_shader =
    counting<swegl::pixel_shader_light_and_texture<swegl::pixel_shader_lights_phong, swegl::pixel_shader_texture_bilinear>>;

// The reference's own pixel shader for an SGL_SHADER_* mode (include/sgl.h).
std::shared_ptr<swegl::pixel_shader_t> shader_for_mode(int mode, counting_base **counter)
{
    using namespace swegl;
    std::shared_ptr<pixel_shader_t> p;
    counting_base *c = nullptr;
    auto make = [&](auto tag) {
        auto q = std::make_shared<counting<typename decltype(tag)::type>>();
        c = q.get();
        p = q;
    };
    struct phong_bil { using type = pixel_shader_light_and_texture<pixel_shader_lights_phong, pixel_shader_texture_bilinear>; };
    struct phong_near { using type = pixel_shader_light_and_texture<pixel_shader_lights_phong, pixel_shader_texture>; };
    struct flat_bil { using type = pixel_shader_light_and_texture<pixel_shader_lights_flat, pixel_shader_texture_bilinear>; };
    struct flat_near { using type = pixel_shader_light_and_texture<pixel_shader_lights_flat, pixel_shader_texture>; };
    struct color { using type = pixel_shader_t; };
    struct bil { using type = pixel_shader_texture_bilinear; };
    struct near { using type = pixel_shader_texture; };
    struct phong { using type = pixel_shader_lights_phong; };
    struct flat { using type = pixel_shader_lights_flat; };
    switch (mode) {
    case SGL_SHADER_PHONG_BILINEAR: make(phong_bil{}); break;
    case SGL_SHADER_PHONG_NEAREST: make(phong_near{}); break;
    case SGL_SHADER_FLAT_BILINEAR: make(flat_bil{}); break;
    case SGL_SHADER_FLAT_NEAREST: make(flat_near{}); break;
    case SGL_SHADER_COLOR: make(color{}); break;
    case SGL_SHADER_BILINEAR: make(bil{}); break;
    case SGL_SHADER_NEAREST: make(near{}); break;
    case SGL_SHADER_PHONG: make(phong{}); break;
    case SGL_SHADER_FLAT: make(flat{}); break;
    default: break;
    }
    *counter = c;
    return p;
}

swegl::matrix44_t to_matrix(const float *m)
{
    swegl::matrix44_t r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            r[i][j] = m[i * 4 + j];
    return r;
}

void set_bits(swegl::vector_t &dst, const float *src)
{
    dst.x() = src[0];
    dst.y() = src[1];
    dst.z() = src[2];
}

swegl::scene_t build_scene(const sgl_scene_desc *d)
{
    swegl::scene_t s;
    s.nodes.resize(d->n_nodes);
    for (int i = 0; i < d->n_nodes; i++) {
        const sgl_node_desc &nd = d->nodes[i];
        swegl::node_t &n = s.nodes[i];
        n.scale = swegl::vertex_t(nd.scale[0], nd.scale[1], nd.scale[2]);
        n.rotation = to_matrix(nd.rotation);
        n.translation = swegl::vertex_t(nd.translation[0], nd.translation[1], nd.translation[2]);
        if (nd.parent < 0)
            s.root_nodes.push_back(i);
        else
            s.nodes[nd.parent].children_idx.push_back(i);
    }
    for (int p = 0; p < d->n_primitives; p++) {
        const sgl_primitive_desc &pd = d->primitives[p];
        swegl::primitive_t prim;
        prim.mode = (swegl::primitive_t::index_mode_t)pd.mode;
        prim.material_id = pd.material;
        prim.vertices.resize(pd.vertex_count);
        prim.vertices.reserve(pd.vertex_count + 2); // room for the two near-clip vertices
        for (uint32_t v = 0; v < pd.vertex_count; v++) {
            const uint32_t g = pd.vertex_offset + v;
            swegl::mesh_vertex_t &mv = prim.vertices[v];
            mv.v = swegl::vertex_t(d->positions[3 * g], d->positions[3 * g + 1], d->positions[3 * g + 2]);
            mv.tex_coords = swegl::vec2f_t(d->uvs[2 * g], d->uvs[2 * g + 1]);
            set_bits(mv.normal, &d->normals[3 * g]); // exact bits, no renormalisation
            mv.yes = false;
        }
        prim.indices.assign(d->indices + pd.index_offset, d->indices + pd.index_offset + pd.index_count);
        s.nodes[pd.node].primitives.push_back(std::move(prim));
    }
    for (int m = 0; m < d->n_materials; m++) {
        swegl::material_t mat;
        mat.color = swegl::pixel_colors((unsigned int)d->materials[m].color);
        mat.texture_idx = d->materials[m].texture;
        mat.double_sided = d->materials[m].double_sided != 0;
        s.materials.push_back(mat);
    }
    for (int t = 0; t < d->n_textures; t++) {
        const sgl_texture_desc &td = d->textures[t];
        unsigned int *copy = new unsigned int[(size_t)td.width * td.height];
        std::memcpy(copy, td.texels, sizeof(unsigned int) * (size_t)td.width * td.height);
        s.images.emplace_back(copy, td.width, td.height);
    }
    for (int l = 0; l < d->n_point_lights; l++) {
        const sgl_point_light &pl = d->point_lights[l];
        s.point_source_lights.push_back(swegl::point_source_light{
            swegl::vertex_t(pl.position[0], pl.position[1], pl.position[2]), pl.intensity});
    }
    s.ambient_light_intensity = d->ambient;
    set_bits(s.sun_direction, d->sun_direction);
    s.sun_intensity = d->sun_intensity;
    s.default_material.color = swegl::pixel_colors((unsigned int)d->default_material.color);
    s.default_material.texture_idx = d->default_material.texture;
    s.default_material.double_sided = d->default_material.double_sided != 0;
    return s;
}

} // namespace

extern "C" {

/* Render `n_views` views of the scene with the reference, in order, exactly as
 * swegl::render(scene, vp0, vp1, ...) does.  `shader_kind` selects the pixel
 * shader (see the file header).  `triangle_calls[i]` receives the number of
 * fill_triangle_2 calls that reached prepare_for_triangle for view i (kinds 0
 * and 1).  Returns 0, or -1 on a bad argument. */
__attribute__((visibility("default"))) int ref_render(const sgl_scene_desc *desc, const sgl_view *views,
                                                      const sgl_target *targets, int n_views, int shader_kind,
                                                      uint64_t *triangle_calls)
{
    if (!desc || !views || !targets || n_views <= 0)
        return -1;
    for (int m = 0; m < desc->n_materials; m++)
        if (desc->materials[m].shininess != 32)
            return -1; // the reference hard-codes the exponent 32
    swegl::scene_t scene = build_scene(desc);

    std::vector<SDL_PixelFormat> formats(n_views, SDL_PixelFormat{4});
    std::vector<SDL_Surface> surfaces(n_views);
    std::vector<std::shared_ptr<swegl::pixel_shader_t>> shaders(n_views);
    std::vector<counting_base *> counters(n_views, nullptr);
    std::vector<std::unique_ptr<swegl::viewport_t>> vps;
    swegl::post_shader_t post_null;
    for (int i = 0; i < n_views; i++) {
        surfaces[i] = SDL_Surface{targets[i].width, targets[i].height, targets[i].pitch, targets[i].pixels,
                                  &formats[i]};
        switch (shader_kind) {
        case 0:
            shaders[i] = shader_for_mode(views[i].shader, &counters[i]);
            if (!shaders[i])
                return -1;
            break;
        case 1: shaders[i] = std::make_shared<id_shader>(); break;
        case 2: shaders[i] = std::make_shared<progress_shader>(); break;
        case 3: shaders[i] = std::make_shared<swegl::pixel_shader_lights_phong>(); break;
        case 4: shaders[i] = std::make_shared<swegl::pixel_shader_texture_bilinear>(); break;
        default: return -1;
        }
        const sgl_view &v = views[i];
        auto vp = std::make_unique<swegl::viewport_t>(v.x, v.y, v.w, v.h, &surfaces[i], shaders[i],
                                                      shader_kind == 0 ? v.layers : 0);
        vp->m_camera.m_viewmatrix = to_matrix(v.view);
        vp->m_camera.m_projectionmatrix = to_matrix(v.proj);
        vp->m_camera.m_center = swegl::vertex_t(v.camera_pos[0], v.camera_pos[1], v.camera_pos[2]);
        vp->set_post_shader(post_null);
        vps.push_back(std::move(vp));
    }

    // swegl::render(scene, vp...) == original_to_world once, then _render per viewport.
    swegl::vertex_shader_t::original_to_world(scene);
    for (int i = 0; i < n_views; i++) {
        swegl::_render(scene, *vps[i]);
        if (targets[i].zbuffer)
            std::memcpy(targets[i].zbuffer, vps[i]->zbuffer(), sizeof(float) * (size_t)views[i].w * views[i].h);
        if (triangle_calls) {
            if (shader_kind == 0)
                triangle_calls[i] = counters[i]->calls;
            else if (shader_kind == 1)
                triangle_calls[i] = (uint64_t) static_cast<id_shader *>(shaders[i].get())->calls;
            else
                triangle_calls[i] = 0;
        }
    }
    return 0;
}


/* matrix44_t::from_quaternion(q[0], q[1], q[2], q[3]), row-major into out[16]. */
__attribute__((visibility("default"))) void ref_from_quaternion(const float *q, float *out)
{
    const swegl::matrix44_t m = swegl::matrix44_t::from_quaternion(q[0], q[1], q[2], q[3]);
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            out[4 * i + j] = m[i][j];
}

/* scene_t::animate(seconds) on `nodes` (scale, rotation, translation are
 * read and written back).  Animation a has channels
 * [ch_first[a], ch_first[a + 1]); channel c targets node ch_node[c] on path
 * ch_path[c] (0 scale, 1 rotation, 2 translation, 3 other) with keyframes
 * [st_first[c], st_first[c + 1]) of times `times` and 4-float `values`, in
 * the order given (the loader sorts them by time).  Each animation's end
 * time is the largest last keyframe time of its channels (gltf.cpp:381). */
__attribute__((visibility("default"))) int ref_animate(sgl_node_desc *nodes, int n_nodes, int n_anims,
                                                       const int *ch_first, const int *ch_node,
                                                       const int *ch_path, const int *st_first,
                                                       const float *times, const float *values, float seconds)
{
    swegl::scene_t s;
    s.nodes.resize(n_nodes);
    for (int i = 0; i < n_nodes; i++) {
        s.nodes[i].scale = swegl::vertex_t(nodes[i].scale[0], nodes[i].scale[1], nodes[i].scale[2]);
        s.nodes[i].rotation = to_matrix(nodes[i].rotation);
        s.nodes[i].translation =
            swegl::vertex_t(nodes[i].translation[0], nodes[i].translation[1], nodes[i].translation[2]);
    }
    for (int a = 0; a < n_anims; a++) {
        swegl::animation_t &an = s.animations.emplace_back();
        for (int c = ch_first[a]; c < ch_first[a + 1]; c++) {
            if (ch_node[c] < 0 || ch_node[c] >= n_nodes || st_first[c + 1] <= st_first[c])
                return -1;
            swegl::animation_channel_t ch{ch_node[c], (swegl::animation_channel_t::path_t)ch_path[c], {}};
            for (int k = st_first[c]; k < st_first[c + 1]; k++)
                ch.steps.push_back(swegl::animation_step_t{
                    times[k], swegl::vec4f_t(values[4 * k], values[4 * k + 1], values[4 * k + 2], values[4 * k + 3])});
            an.end_time = std::max(an.end_time, ch.steps.back().time);
            an.channels.push_back(std::move(ch));
        }
    }
    s.animate(seconds);
    for (int i = 0; i < n_nodes; i++) {
        nodes[i].scale[0] = s.nodes[i].scale.x();
        nodes[i].scale[1] = s.nodes[i].scale.y();
        nodes[i].scale[2] = s.nodes[i].scale.z();
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++)
                nodes[i].rotation[4 * r + c] = s.nodes[i].rotation[r][c];
        nodes[i].translation[0] = s.nodes[i].translation.x();
        nodes[i].translation[1] = s.nodes[i].translation.y();
        nodes[i].translation[2] = s.nodes[i].translation.z();
    }
    return 0;
}

} // extern "C"
