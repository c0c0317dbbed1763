// Renders a scene dump through the drop-in C++ API (swegl_gb300/swegl.hpp)
// exactly as swegl code would: scene_t, viewport_t on one SDL surface, and
// swegl::render(scene, vp0, vp1, ...).  Used by tests/test_gpu_dropin.py.
//
// usage: dropin_render <scene dump> <output> [<scene.gltf|.glb> <seconds>]
// Output: the surface (h * w uint32), then each view's z-buffer.  With a glTF
// file the scene is swegl::load_scene(file) animated to <seconds>
// (scene_t::animate), with the dump's lights; the dump's geometry is unused.
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

#include "swegl_gb300/swegl.hpp"

namespace {
struct Reader {
    FILE *f;
    template <typename T>
    T get()
    {
        T v{};
        if (fread(&v, sizeof v, 1, f) != 1) {
            fprintf(stderr, "short read\n");
            exit(2);
        }
        return v;
    }
    void get(void *p, size_t n)
    {
        if (n && fread(p, 1, n, f) != n) {
            fprintf(stderr, "short read\n");
            exit(2);
        }
    }
};
// The swegl pixel shader of an SGL_SHADER_* mode, as an application builds it.
std::shared_ptr<swegl::pixel_shader_t> make_shader(int mode)
{
    using namespace swegl;
    switch (mode) {
    case SGL_SHADER_PHONG_NEAREST:
        return std::make_shared<pixel_shader_light_and_texture<pixel_shader_lights_phong, pixel_shader_texture>>();
    case SGL_SHADER_FLAT_BILINEAR:
        return std::make_shared<pixel_shader_light_and_texture<pixel_shader_lights_flat, pixel_shader_texture_bilinear>>();
    case SGL_SHADER_FLAT_NEAREST:
        return std::make_shared<pixel_shader_light_and_texture<pixel_shader_lights_flat, pixel_shader_texture>>();
    case SGL_SHADER_COLOR: return std::make_shared<pixel_shader_t>();
    case SGL_SHADER_BILINEAR: return std::make_shared<pixel_shader_texture_bilinear>();
    case SGL_SHADER_NEAREST: return std::make_shared<pixel_shader_texture>();
    case SGL_SHADER_PHONG: return std::make_shared<pixel_shader_lights_phong>();
    case SGL_SHADER_FLAT: return std::make_shared<pixel_shader_lights_flat>();
    default:
        return std::make_shared<pixel_shader_light_and_texture<pixel_shader_lights_phong, pixel_shader_texture_bilinear>>();
    }
}
} // namespace

int main(int argc, char **argv)
{
    if (argc != 3 && argc != 5)
        return 2;
    FILE *in = fopen(argv[1], "rb");
    if (!in)
        return 2;
    Reader r{in};
    swegl::scene_t scene;
    const int n_nodes = r.get<int>();
    scene.nodes.resize(n_nodes);
    for (int i = 0; i < n_nodes; i++) {
        swegl::node_t &n = scene.nodes[i];
        float s[3], rot[16], t[3];
        r.get(s, sizeof s);
        r.get(rot, sizeof rot);
        r.get(t, sizeof t);
        const int parent = r.get<int>();
        n.scale = swegl::vertex_t(s[0], s[1], s[2]);
        for (int k = 0; k < 16; k++)
            n.rotation[k / 4][k % 4] = rot[k];
        n.translation = swegl::vertex_t(t[0], t[1], t[2]);
        if (parent >= 0)
            scene.nodes[parent].children_idx.push_back(i);
        else
            scene.root_nodes.push_back(i);
    }
    const int n_prims = r.get<int>();
    for (int p = 0; p < n_prims; p++) {
        const int node = r.get<int>(), mode = r.get<int>(), material = r.get<int>();
        const int nv = r.get<int>(), ni = r.get<int>();
        swegl::primitive_t prim;
        prim.mode = (swegl::primitive_t::index_mode_t)mode;
        prim.material_id = material;
        prim.vertices.resize(nv);
        for (int v = 0; v < nv; v++) {
            float a[8];
            r.get(a, sizeof a);
            swegl::mesh_vertex_t &mv = prim.vertices[v];
            mv.v = swegl::vertex_t(a[0], a[1], a[2]);
            mv.normal.x() = a[3]; // exact bits, no renormalisation
            mv.normal.y() = a[4];
            mv.normal.z() = a[5];
            mv.tex_coords = swegl::vec2f_t(a[6], a[7]);
        }
        prim.indices.resize(ni);
        r.get(prim.indices.data(), sizeof(uint32_t) * ni);
        scene.nodes[node].primitives.push_back(std::move(prim));
    }
    const int n_mats = r.get<int>();
    for (int m = 0; m < n_mats; m++) {
        swegl::material_t mat;
        mat.color = swegl::pixel_colors(r.get<unsigned int>());
        mat.texture_idx = r.get<int>();
        mat.double_sided = r.get<int>() != 0;
        mat.shininess = r.get<int>();
        scene.materials.push_back(mat);
    }
    const int n_tex = r.get<int>();
    for (int t = 0; t < n_tex; t++) {
        const int w = r.get<int>(), h = r.get<int>();
        unsigned int *texels = new unsigned int[(size_t)w * h];
        r.get(texels, 4 * (size_t)w * h);
        scene.images.emplace_back(texels, w, h);
    }
    const int n_lights = r.get<int>();
    for (int l = 0; l < n_lights; l++) {
        float a[4];
        r.get(a, sizeof a);
        scene.point_source_lights.push_back(swegl::point_source_light{swegl::vertex_t(a[0], a[1], a[2]), a[3]});
    }
    scene.ambient_light_intensity = r.get<float>();
    float sun[3];
    r.get(sun, sizeof sun);
    scene.sun_direction.x() = sun[0];
    scene.sun_direction.y() = sun[1];
    scene.sun_direction.z() = sun[2];
    scene.sun_intensity = r.get<float>();
    if (argc == 5) {
        try {
            swegl::scene_t loaded = swegl::load_scene(argv[3]);
            loaded.point_source_lights = scene.point_source_lights;
            loaded.ambient_light_intensity = scene.ambient_light_intensity;
            loaded.sun_direction = scene.sun_direction;
            loaded.sun_intensity = scene.sun_intensity;
            loaded.animate((float)atof(argv[4]));
            scene = std::move(loaded);
        } catch (const swegl::render_error &e) {
            fprintf(stderr, "load_scene %d: %s\n", e.status, e.what());
            return 3;
        }
    }
    const int n_views = r.get<int>();
    const int sw = r.get<int>(), sh = r.get<int>();
    std::vector<uint32_t> pixels((size_t)sw * sh, 0);
    SDL_PixelFormat fmt{4};
    SDL_Surface surface{sw, sh, 4 * sw, pixels.data(), &fmt};
    std::vector<std::shared_ptr<swegl::pixel_shader_t>> shaders;
    std::vector<std::unique_ptr<swegl::viewport_t>> vps;
    swegl::post_shader_t post_null;
    for (int i = 0; i < n_views; i++) {
        const int x = r.get<int>(), y = r.get<int>(), w = r.get<int>(), h = r.get<int>();
        float view[16], proj[16], cam[3];
        r.get(view, sizeof view);
        r.get(proj, sizeof proj);
        r.get(cam, sizeof cam);
        shaders.push_back(make_shader(r.get<int>()));
        const int layers = r.get<int>();
        auto vp = std::make_unique<swegl::viewport_t>(x, y, w, h, &surface, shaders.back(), layers);
        for (int k = 0; k < 16; k++) {
            vp->m_camera.m_viewmatrix[k / 4][k % 4] = view[k];
            vp->m_camera.m_projectionmatrix[k / 4][k % 4] = proj[k];
        }
        vp->m_camera.m_center = swegl::vertex_t(cam[0], cam[1], cam[2]);
        vp->set_post_shader(post_null);
        vps.push_back(std::move(vp));
    }
    fclose(in);
    try {
        if (n_views == 1)
            swegl::render(scene, *vps[0]);
        else if (n_views == 2)
            swegl::render(scene, *vps[0], *vps[1]);
        else
            for (auto &vp : vps)
                swegl::render(scene, *vp);
        // a second frame with a moved node re-uses the resident scene
        swegl::render(scene, *vps[0]);
    } catch (const swegl::render_error &e) {
        fprintf(stderr, "render_error %d: %s\n", e.status, e.what());
        return 3;
    }
    FILE *out = fopen(argv[2], "wb");
    if (!out)
        return 2;
    fwrite(pixels.data(), 4, pixels.size(), out);
    for (auto &vp : vps)
        fwrite(vp->zbuffer(), 4, (size_t)vp->m_w * vp->m_h, out);
    fclose(out);
    return 0;
}
