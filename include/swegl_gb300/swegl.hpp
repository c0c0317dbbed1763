// swegl.hpp — drop-in C++ API of the GB300 renderer.
//
// Mirrors the public interface of gbizzotto/swegl's render path so that code
// written against it compiles unchanged and renders on the GPU: the same
// namespace, type names and data members (scene_t, node_t, primitive_t,
// mesh_vertex_t, material_t, texture_t, point_source_light, camera_t,
// viewport_t, the pixel-shader plug-in types, post_shader_t) and the variadic
// render(scene, viewport...).  Reference files: swegl/data/model.hpp,
// swegl/data/texture.hpp, swegl/projection/*.hpp, swegl/render/viewport.hpp,
// swegl/render/pixel_shaders.hpp, swegl/render/post_shaders.hpp,
// swegl/render/renderer.hpp.
//
// render() uploads a scene once (device-resident, keyed by the scene's
// address and its structure), refreshes node transforms and lights on every
// call, renders each viewport in order through the C ABI (include/sgl.h) and
// writes the viewport rectangle of its SDL surface and its z-buffer, as the
// reference does.  Differences, all explicit:
//   * the reference's pixel shaders (pixel_shader_t, the flat and Phong light
//     shaders, the nearest and bilinear texture shaders and their
//     pixel_shader_light_and_texture<L, T> combinations) and viewports with
//     0 to SGL_MAX_LAYERS transparency layers run on the GPU, with or without
//     the depth-of-field post shader; more layers throw swegl::render_error
//     (there is no CPU fallback);
//   * the scene is not mutated (v_world, v_viewport, normal_world, yes and
//     the temporary clip vertices of the reference are not written back);
//   * errors throw swegl::render_error instead of undefined behaviour;
//   * after editing vertex data without changing any count, call
//     swegl::gpu::invalidate(scene) so the next render re-uploads it.
// Link with swegl_gb300/_build/libsgl.so.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../sgl.h"

#ifndef SDL_h_
// The two SDL2 structs the render path touches, for headless use; include
// <SDL.h> first to use SDL's own.
struct SDL_PixelFormat {
    uint8_t BytesPerPixel;
};
struct SDL_Surface {
    int w, h;
    int pitch;
    void *pixels;
    SDL_PixelFormat *format;
};
#endif

namespace swegl {

struct render_error : std::runtime_error {
    int status;
    render_error(int st, const std::string &what) : std::runtime_error(what), status(st) {}
};

// --------------------------------------------------------------------- math --

class vertex_t {
    float _x = 0, _y = 0, _z = 0;

public:
    vertex_t() = default;
    vertex_t(float x, float y, float z) : _x(x), _y(y), _z(z) {}
    float &x() { return _x; }
    float x() const { return _x; }
    float &y() { return _y; }
    float y() const { return _y; }
    float &z() { return _z; }
    float z() const { return _z; }
};

class vector_t {
    float _x = 0, _y = 0, _z = 0;

public:
    vector_t() = default;
    vector_t(float x, float y, float z) : _x(x), _y(y), _z(z) {}
    float &x() { return _x; }
    float x() const { return _x; }
    float &y() { return _y; }
    float y() const { return _y; }
    float &z() { return _z; }
    float z() const { return _z; }
    float len_squared() const { return _x * _x + _y * _y + _z * _z; }
    float len() const { return std::sqrt(len_squared()); }
    vector_t &normalize()
    {
        const float l = len();
        if (l != 0) {
            _x /= l;
            _y /= l;
            _z /= l;
        }
        return *this;
    }
    float dot(const vector_t &o) const { return _x * o._x + _y * o._y + _z * o._z; }
};

// A vector normalised on construction and assignment.
class normal_t : public vector_t {
public:
    normal_t() = default;
    normal_t(float x, float y, float z) : vector_t(x, y, z) { normalize(); }
    normal_t(const vector_t &v) : vector_t(v) { normalize(); }
    normal_t &operator=(const vector_t &v)
    {
        vector_t::operator=(v);
        normalize();
        return *this;
    }
};

class vec2f_t {
    float _x = 0, _y = 0;

public:
    vec2f_t() = default;
    vec2f_t(float x, float y) : _x(x), _y(y) {}
    float &x() { return _x; }
    float x() const { return _x; }
    float &y() { return _y; }
    float y() const { return _y; }
};

// Row-major 4x4 matrix with the transforms of matrix44_t.
struct matrix44_t {
    float m[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    static const matrix44_t Identity;
    float *operator[](int i) { return m[i]; }
    const float *operator[](int i) const { return m[i]; }
    // rotations compose on the left; rows (a, b) <- (c*a + s*b, -s*a + c*b)
    void rotate_rows(int a, int b, float angle)
    {
        const float c = (float)std::cos(angle), s = (float)std::sin(angle);
        for (int k = 0; k < 4; k++) {
            const float ra = m[a][k], rb = m[b][k];
            m[a][k] = c * ra + s * rb;
            m[b][k] = -s * ra + c * rb;
        }
    }
    void rotate_x(float a) { rotate_rows(1, 2, a); }
    void rotate_y(float a) { rotate_rows(0, 2, a); }
    void rotate_z(float a) { rotate_rows(0, 1, a); }
    void translate(float x, float y, float z)
    {
        m[0][3] += x;
        m[1][3] += y;
        m[2][3] += z;
    }
};
inline const matrix44_t matrix44_t::Identity{};

inline vertex_t operator+(const vertex_t &a, const vector_t &b) { return {a.x() + b.x(), a.y() + b.y(), a.z() + b.z()}; }
inline vector_t operator-(const vertex_t &a, const vertex_t &b) { return {a.x() - b.x(), a.y() - b.y(), a.z() - b.z()}; }
inline vector_t operator*(const vector_t &a, float s) { return {a.x() * s, a.y() * s, a.z() * s}; }
inline vector_t operator+(const vector_t &a, const vector_t &b) { return {a.x() + b.x(), a.y() + b.y(), a.z() + b.z()}; }

inline normal_t cross(const vector_t &a, const vector_t &b)
{
    return normal_t(a.y() * b.z() - a.z() * b.y(), a.z() * b.x() - a.x() * b.z(), a.x() * b.y() - a.y() * b.x());
}

// camera_t (swegl/projection/camera.hpp): the view starts looking down -z;
// the projection is the reference's fixed one (n = 0.5, f = 10) until the
// caller writes m_projectionmatrix.
class camera_t {
public:
    float m_xfov = 0, m_yfov = 0;
    vertex_t m_center{0, 0, 0};
    matrix44_t m_viewmatrix;
    matrix44_t m_projectionmatrix;

    explicit camera_t(float aspect_ratio)
    {
        m_viewmatrix[2][2] = -1;
        const float n = 0.5f, f = 10.0f;
        if (aspect_ratio > 1) {
            m_projectionmatrix[0][0] = 2 * n;
            m_projectionmatrix[1][1] = aspect_ratio * 2 * n;
        } else {
            m_projectionmatrix[0][0] = (1.0f / aspect_ratio) * 2 * n;
            m_projectionmatrix[1][1] = 2 * n;
        }
        m_projectionmatrix[2][2] = f / (f - n);
        m_projectionmatrix[2][3] = -f * n / (f - n);
        m_projectionmatrix[3][2] = 1;
    }
    void rotate_x(float a) { m_viewmatrix.rotate_x(-a); }
    void rotate_y(float a) { m_viewmatrix.rotate_y(-a); }
    void rotate_z(float a) { m_viewmatrix.rotate_z(-a); }
    // moves in the camera's own axes
    void translate(float x, float y, float z)
    {
        m_viewmatrix.translate(-x, -y, -z);
        const auto &m = m_viewmatrix;
        m_center.x() += x * m[0][0] + y * m[1][0] + z * m[2][0];
        m_center.y() += x * m[0][1] + y * m[1][1] + z * m[2][1];
        m_center.z() += x * m[0][2] + y * m[1][2] + z * m[2][2];
    }
    vertex_t position() const { return m_center; }
};

// ------------------------------------------------------------------- colours --

struct pixel_colors {
    union {
        struct {
            unsigned char b, g, r, a;
        } o;
        int i;
    };
    pixel_colors() : i(0) {}
    pixel_colors(unsigned char b, unsigned char g, unsigned char r, unsigned char a) : o{b, g, r, a} {}
    pixel_colors(int v) : i(v) {}
    pixel_colors(unsigned int v) : i((int)v) {}
    int to_int() const { return i; }
};

// --------------------------------------------------------------------- scene --

using vertex_idx = std::uint32_t;

struct mesh_vertex_t {
    vertex_t v;
    vertex_t v_world;     // not written by the GPU renderer
    vertex_t v_viewport;  // not written by the GPU renderer
    vec2f_t tex_coords;
    normal_t normal;
    normal_t normal_world; // not written by the GPU renderer
    bool yes = false;
};

struct primitive_t {
    enum index_mode_t { POINTS = 0, LINES = 1, LINE_LOOP = 2, LINE_STRIP = 3, TRIANGLES = 4, TRIANGLE_STRIP = 5,
                        TRIANGLE_FAN = 6 };
    std::vector<mesh_vertex_t> vertices;
    std::vector<vertex_idx> indices;
    index_mode_t mode = TRIANGLES;
    int material_id = -1;
};

struct node_t {
    vertex_t scale = vertex_t(1, 1, 1);
    matrix44_t rotation = matrix44_t::Identity;
    vertex_t translation = vertex_t(0, 0, 0);
    matrix44_t original_to_world_matrix = matrix44_t::Identity;
    std::vector<primitive_t> primitives;
    std::vector<int> children_idx;
    bool root = true;
};

struct point_source_light {
    vertex_t position;
    float intensity;
};

struct material_t {
    pixel_colors color = pixel_colors(255, 255, 255, 255);
    float metallic = 1;
    float roughness = 1;
    int texture_idx = -1;
    bool double_sided = false;
    int shininess = 32; // point-light specular exponent (the reference's constant)
};

struct mipmap_t {
    unsigned int *m_bitmap = nullptr;
    unsigned int m_width = 0, m_height = 0;
    mipmap_t(unsigned int *b, unsigned int w, unsigned int h) : m_bitmap(b), m_width(w), m_height(h) {}
    ~mipmap_t() { delete[] m_bitmap; }
    mipmap_t(const mipmap_t &) = delete;
    mipmap_t &operator=(const mipmap_t &) = delete;
};

// texture_t: takes ownership of a new[]'d 0xAARRGGBB bitmap (texture.hpp:29-38).
class texture_t {
public:
    std::vector<std::shared_ptr<mipmap_t>> m_mipmaps;
    explicit texture_t(unsigned int rgb) { m_mipmaps.push_back(std::make_shared<mipmap_t>(new unsigned int[1]{rgb}, 1, 1)); }
    texture_t(unsigned int *data, int w, int h)
    {
        m_mipmaps.push_back(std::make_shared<mipmap_t>(data, (unsigned)w, (unsigned)h));
    }
};

struct scene_t {
    std::vector<node_t> nodes;
    std::vector<int> root_nodes;
    float ambient_light_intensity = 0;
    normal_t sun_direction;
    float sun_intensity = 0;
    material_t default_material;
    std::vector<point_source_light> point_source_lights;
    std::vector<material_t> materials;
    std::vector<texture_t> images;
    // the animations of a scene from load_scene (scene_t::animations)
    std::shared_ptr<sgl_gltf> animation_source;

    // scene_t::animate (model.hpp:146-177): the nodes' scale, rotation and
    // translation at `elapsed_seconds`, for scenes from load_scene.
    inline void animate(float elapsed_seconds);
};

// -------------------------------------------------------- procedural meshes --

// make_tri (model.hpp:233-252): one triangle in the xy plane.
inline node_t make_tri(float size, int material_idx)
{
    node_t n;
    primitive_t p;
    p.vertices = {mesh_vertex_t{vertex_t{0, 0, 0}, {}, {}, vec2f_t{0, 0}, normal_t(0, 0, 1), {}},
                  mesh_vertex_t{vertex_t{size, 0, 0}, {}, {}, vec2f_t{0, 1}, normal_t(0, 0, 1), {}},
                  mesh_vertex_t{vertex_t{0, size, 0}, {}, {}, vec2f_t{1, 0}, normal_t(0, 0, 1), {}}};
    p.indices = {0, 1, 2};
    p.mode = primitive_t::TRIANGLES;
    p.material_id = material_idx;
    n.primitives.push_back(std::move(p));
    return n;
}

// make_cube (model.hpp:254-325): six fans of four vertices, faces laid out in
// a 2 x 3 texture atlas (the same vertex data as the reference).
inline node_t make_cube(float size, int material_idx)
{
    const float h = size / 2.0f;
    struct Face {
        float p[4][3];
        float t[4][2];
        float n[3];
    };
    const Face faces[6] = {
        {{{-h, h, h}, {h, h, h}, {h, h, -h}, {-h, h, -h}}, {{0.0f, 0.0f}, {0.5f, 0.0f}, {0.5f, 0.333f}, {0.0f, 0.333f}}, {0, 1, 0}},
        {{{-h, -h, h}, {h, -h, h}, {h, h, h}, {-h, h, h}}, {{0.5f, 0.0f}, {1.0f, 0.0f}, {1.0f, 0.333f}, {0.5f, 0.333f}}, {0, 0, 1}},
        {{{h, -h, h}, {h, -h, -h}, {h, h, -h}, {h, h, h}}, {{0.0f, 0.333f}, {0.5f, 0.333f}, {0.5f, 0.667f}, {0.0f, 0.667f}}, {1, 0, 0}},
        {{{h, -h, -h}, {-h, -h, -h}, {-h, h, -h}, {h, h, -h}}, {{0.5f, 0.667f}, {1.0f, 0.667f}, {1.0f, 1.0f}, {0.5f, 1.0f}}, {0, 0, -1}},
        {{{-h, -h, -h}, {-h, -h, h}, {-h, h, h}, {-h, h, -h}}, {{0.5f, 0.333f}, {1.0f, 0.333f}, {1.0f, 0.667f}, {0.5f, 0.667f}}, {-1, 0, 0}},
        {{{-h, -h, -h}, {h, -h, -h}, {h, -h, h}, {-h, -h, h}}, {{0.0f, 0.667f}, {0.5f, 0.667f}, {0.5f, 1.0f}, {0.0f, 1.0f}}, {0, -1, 0}},
    };
    node_t n;
    for (const Face &f : faces) {
        primitive_t p;
        for (int k = 0; k < 4; k++)
            p.vertices.push_back(mesh_vertex_t{vertex_t(f.p[k][0], f.p[k][1], f.p[k][2]), {}, {},
                                               vec2f_t(f.t[k][0], f.t[k][1]), normal_t(f.n[0], f.n[1], f.n[2]), {}});
        p.indices = {0, 1, 2, 3};
        p.mode = primitive_t::TRIANGLE_FAN;
        p.material_id = material_idx;
        n.primitives.push_back(std::move(p));
    }
    return n;
}

// A UV sphere in the strip layout of make_sphere (model.hpp:393-446): one
// TRIANGLE_STRIP per longitude slice (slice k spans longitudes k and k + 1 of
// `slice_angle`), 2 * (stacks + 1) vertices from the north pole down, indices
// (stacks + 1 + s, s).  Positions come straight from sin/cos, so their last
// bits may differ from the reference's accumulated rotations.
inline node_t make_uv_sphere(unsigned slices, unsigned stacks, float radius, int material_idx, double slice_angle = 0)
{
    const double pi = 3.14159265358979323846;
    if (slice_angle == 0)
        slice_angle = 2.0 * pi / slices;
    node_t n;
    for (unsigned k = 0; k < slices; k++) {
        primitive_t p;
        p.mode = primitive_t::TRIANGLE_STRIP;
        p.material_id = material_idx;
        for (unsigned row = 0; row < 2; row++)
            for (unsigned s = 0; s <= stacks; s++) {
                const double th = s * pi / stacks, ph = (k + row) * slice_angle;
                const vertex_t v((float)(radius * std::sin(th) * std::cos(ph)), (float)(radius * std::cos(th)),
                                 (float)(-radius * std::sin(th) * std::sin(ph)));
                p.vertices.push_back(mesh_vertex_t{v, {}, {}, vec2f_t((float)s / stacks, (float)(k + row) / slices),
                                                   normal_t(v.x(), v.y(), v.z()), {}});
            }
        for (unsigned s = 0; s <= stacks; s++) {
            p.indices.push_back(stacks + 1 + s);
            p.indices.push_back(s);
        }
        n.primitives.push_back(std::move(p));
    }
    return n;
}

// make_sphere(precision, radius, material) as the reference lays it out:
// precision + 1 slices of 2*pi/precision (the last one repeats the first).
inline node_t make_sphere(unsigned precision, float radius, int material_idx)
{
    const double pi = 3.14159265358979323846;
    node_t n = make_uv_sphere(precision + 1, precision, radius, material_idx, 2.0 * pi / precision);
    for (unsigned k = 0; k < n.primitives.size(); k++)
        for (unsigned row = 0; row < 2; row++)
            for (unsigned s = 0; s <= precision; s++)
                n.primitives[k].vertices[row * (precision + 1) + s].tex_coords =
                    vec2f_t((float)s / precision, (float)(k + row) / precision);
    return n;
}

// ------------------------------------------------------------ shader plug-ins --

// The pixel-shader plug-ins of swegl/render/pixel_shaders.hpp.  On the GPU they
// are tags naming one of the shaders of sgl.h (SGL_SHADER_*): the material
// colour of pixel_shader_t, the two light shaders, the two texture shaders and
// their pixel_shader_light_and_texture<L, T> combinations.  A shader of the
// caller's own (another subclass) has no GPU counterpart.
struct pixel_shader_t {
    virtual ~pixel_shader_t() = default;
    virtual int gpu_shader() const { return SGL_SHADER_COLOR; }
};
struct pixel_shader_lights_flat : pixel_shader_t {
    int gpu_shader() const override { return SGL_SHADER_FLAT; }
};
struct pixel_shader_lights_phong : pixel_shader_t {
    int gpu_shader() const override { return SGL_SHADER_PHONG; }
};
struct pixel_shader_texture : pixel_shader_t {
    int gpu_shader() const override { return SGL_SHADER_NEAREST; }
};
struct pixel_shader_texture_bilinear : pixel_shader_t {
    int gpu_shader() const override { return SGL_SHADER_BILINEAR; }
};
template <typename L, typename T>
struct pixel_shader_light_and_texture : pixel_shader_t {
    int gpu_shader() const override
    {
        constexpr bool phong = std::is_same<L, pixel_shader_lights_phong>::value;
        constexpr bool flat = std::is_same<L, pixel_shader_lights_flat>::value;
        constexpr bool bil = std::is_same<T, pixel_shader_texture_bilinear>::value;
        constexpr bool near = std::is_same<T, pixel_shader_texture>::value;
        static_assert((phong || flat) && (bil || near), "a light shader and a texture shader of swegl");
        return phong ? (bil ? SGL_SHADER_PHONG_BILINEAR : SGL_SHADER_PHONG_NEAREST)
                     : (bil ? SGL_SHADER_FLAT_BILINEAR : SGL_SHADER_FLAT_NEAREST);
    }
};

// post_shader_t (post_shaders.hpp:15-48): the opaque copy-back is a no-op.
struct post_shader_t {
    virtual ~post_shader_t() = default;
    virtual sgl_dof_desc dof() const { return sgl_dof_desc{0, 0, 0, 0, 0}; }
};

// The depth-of-field gather of the GB300 renderer (see sgl_dof in sgl.h),
// standing in for post_shader_depth_box.
struct post_shader_dof : post_shader_t {
    float focus, aperture, max_radius, px_scale;
    post_shader_dof(float focus_, float aperture_, float max_radius_ = 16.0f, float px_scale_ = 0.0f)
        : focus(focus_), aperture(aperture_), max_radius(max_radius_), px_scale(px_scale_)
    {
    }
    sgl_dof_desc dof() const override { return sgl_dof_desc{1, focus, aperture, max_radius, px_scale}; }
};

// ------------------------------------------------------------------ viewport --

struct viewport_t {
    int m_x, m_y, m_w, m_h;
    SDL_Surface *m_screen;
    std::unique_ptr<float[]> m_zbuffer;
    matrix44_t m_viewportmatrix;
    camera_t m_camera;
    std::shared_ptr<pixel_shader_t> m_pixel_shader;
    post_shader_t *m_post_shader = nullptr;
    int m_transparency_layer_count;
    bool m_got_transparency;

    viewport_t(int x, int y, int w, int h, SDL_Surface *screen, std::shared_ptr<pixel_shader_t> &pixel_shader,
               int transparency_layer_count)
        : m_x(x), m_y(y), m_w(w), m_h(h), m_screen(screen), m_zbuffer(new float[(size_t)w * h]),
          m_camera((float)(1.0 * w / h)), m_pixel_shader(pixel_shader),
          m_transparency_layer_count(transparency_layer_count), m_got_transparency(transparency_layer_count > 0)
    {
        m_viewportmatrix[0][3] = x + w / 2.0f;
        m_viewportmatrix[1][3] = y + h / 2.0f;
        m_viewportmatrix[0][0] = w / 2.0f;
        m_viewportmatrix[1][1] = -h / 2.0f;
    }
    void set_post_shader(post_shader_t &p) { m_post_shader = &p; }
    float *zbuffer() { return m_zbuffer.get(); }
    const float *zbuffer() const { return m_zbuffer.get(); }
    camera_t &camera() { return m_camera; }
    const camera_t &camera() const { return m_camera; }
};

// ---------------------------------------------------------------- GPU glue --

namespace gpu {

namespace detail {

struct Cached {
    int id = 0;
    std::vector<uint64_t> shape; // counts that must not change without a re-upload
};

struct State {
    sgl_ctx *ctx = nullptr;
    std::map<const scene_t *, Cached> scenes;
    ~State()
    {
        if (ctx)
            sgl_destroy(ctx);
    }
};

inline State &state()
{
    static State s;
    return s;
}

inline void check(int st, const char *what)
{
    if (st != SGL_OK) {
        const char *msg = state().ctx ? sgl_last_error(state().ctx) : "";
        throw render_error(st, std::string(what) + ": " + sgl_status_string(st) + " (" + msg + ")");
    }
}

inline sgl_ctx *context()
{
    State &s = state();
    if (!s.ctx)
        check(sgl_create(&s.ctx, 0), "sgl_create");
    return s.ctx;
}

inline void copy_m(float *dst, const matrix44_t &m) { std::memcpy(dst, m.m, sizeof m.m); }

inline std::vector<sgl_node_desc> nodes_of(const scene_t &s)
{
    std::vector<sgl_node_desc> out(s.nodes.size());
    for (size_t i = 0; i < s.nodes.size(); i++) {
        const node_t &n = s.nodes[i];
        out[i].scale[0] = n.scale.x();
        out[i].scale[1] = n.scale.y();
        out[i].scale[2] = n.scale.z();
        copy_m(out[i].rotation, n.rotation);
        out[i].translation[0] = n.translation.x();
        out[i].translation[1] = n.translation.y();
        out[i].translation[2] = n.translation.z();
        out[i].parent = -1;
    }
    for (size_t i = 0; i < s.nodes.size(); i++)
        for (int c : s.nodes[i].children_idx)
            if (c >= 0 && (size_t)c < out.size())
                out[c].parent = (int)i;
    return out;
}

inline std::vector<uint64_t> shape_of(const scene_t &s)
{
    std::vector<uint64_t> v{s.nodes.size(), s.materials.size(), s.images.size()};
    for (const node_t &n : s.nodes) {
        v.push_back(n.primitives.size());
        for (const primitive_t &p : n.primitives) {
            v.push_back(p.vertices.size());
            v.push_back(p.indices.size());
            v.push_back((uint64_t)p.mode);
            v.push_back((uint64_t)(int64_t)p.material_id);
        }
    }
    for (const texture_t &t : s.images)
        v.push_back((uint64_t)(uintptr_t)t.m_mipmaps.at(0)->m_bitmap);
    return v;
}

inline int upload(const scene_t &s)
{
    std::vector<sgl_node_desc> nodes = nodes_of(s);
    std::vector<sgl_primitive_desc> prims;
    std::vector<float> pos, nrm, uv;
    std::vector<uint32_t> idx;
    for (size_t ni = 0; ni < s.nodes.size(); ni++)
        for (const primitive_t &p : s.nodes[ni].primitives) {
            sgl_primitive_desc d{};
            d.node = (int)ni;
            d.mode = (int)p.mode;
            d.material = p.material_id;
            d.vertex_offset = (uint32_t)(pos.size() / 3);
            d.vertex_count = (uint32_t)p.vertices.size();
            d.index_offset = (uint32_t)idx.size();
            d.index_count = (uint32_t)p.indices.size();
            for (const mesh_vertex_t &mv : p.vertices) {
                pos.insert(pos.end(), {mv.v.x(), mv.v.y(), mv.v.z()});
                nrm.insert(nrm.end(), {mv.normal.x(), mv.normal.y(), mv.normal.z()});
                uv.insert(uv.end(), {mv.tex_coords.x(), mv.tex_coords.y()});
            }
            idx.insert(idx.end(), p.indices.begin(), p.indices.end());
            prims.push_back(d);
        }
    std::vector<sgl_material_desc> mats;
    for (const material_t &m : s.materials)
        mats.push_back(sgl_material_desc{(uint32_t)m.color.to_int(), m.texture_idx, m.double_sided ? 1 : 0,
                                         m.shininess});
    std::vector<sgl_texture_desc> texs;
    for (const texture_t &t : s.images) {
        const mipmap_t &mm = *t.m_mipmaps.at(0);
        texs.push_back(sgl_texture_desc{mm.m_bitmap, (int)mm.m_width, (int)mm.m_height});
    }
    std::vector<sgl_point_light> lights;
    for (const point_source_light &l : s.point_source_lights)
        lights.push_back(sgl_point_light{{l.position.x(), l.position.y(), l.position.z()}, l.intensity});
    sgl_scene_desc d{};
    d.n_nodes = (int)nodes.size();
    d.nodes = nodes.data();
    d.n_primitives = (int)prims.size();
    d.primitives = prims.data();
    d.n_vertices = (uint32_t)(pos.size() / 3);
    d.positions = pos.data();
    d.normals = nrm.data();
    d.uvs = uv.data();
    d.n_indices = (uint32_t)idx.size();
    d.indices = idx.data();
    d.n_materials = (int)mats.size();
    d.materials = mats.data();
    d.n_textures = (int)texs.size();
    d.textures = texs.data();
    d.n_point_lights = (int)lights.size();
    d.point_lights = lights.data();
    d.ambient = s.ambient_light_intensity;
    d.sun_direction[0] = s.sun_direction.x();
    d.sun_direction[1] = s.sun_direction.y();
    d.sun_direction[2] = s.sun_direction.z();
    d.sun_intensity = s.sun_intensity;
    const material_t &dm = s.default_material;
    d.default_material = sgl_material_desc{(uint32_t)dm.color.to_int(), dm.texture_idx, dm.double_sided ? 1 : 0,
                                           dm.shininess};
    int id = 0;
    check(sgl_scene_upload(context(), &d, &id), "sgl_scene_upload");
    return id;
}

// The resident copy of `s`, uploaded or refreshed as needed.
inline int resident(const scene_t &s)
{
    State &st = state();
    std::vector<uint64_t> shape = shape_of(s);
    auto it = st.scenes.find(&s);
    if (it != st.scenes.end() && it->second.shape != shape) {
        sgl_scene_release(context(), it->second.id);
        st.scenes.erase(it);
        it = st.scenes.end();
    }
    if (it == st.scenes.end()) {
        Cached c;
        c.id = upload(s);
        c.shape = std::move(shape);
        it = st.scenes.emplace(&s, std::move(c)).first;
        return it->second.id;
    }
    // node transforms and lights may change every frame (scene_t::animate)
    std::vector<sgl_node_desc> nodes = nodes_of(s);
    check(sgl_scene_set_nodes(context(), it->second.id, nodes.data(), (int)nodes.size()), "sgl_scene_set_nodes");
    std::vector<sgl_point_light> lights;
    for (const point_source_light &l : s.point_source_lights)
        lights.push_back(sgl_point_light{{l.position.x(), l.position.y(), l.position.z()}, l.intensity});
    const float sun[3] = {s.sun_direction.x(), s.sun_direction.y(), s.sun_direction.z()};
    check(sgl_scene_set_lights(context(), it->second.id, s.ambient_light_intensity, sun, s.sun_intensity,
                               lights.data(), (int)lights.size()),
          "sgl_scene_set_lights");
    return it->second.id;
}

inline void render_one(int scene_id, viewport_t &vp)
{
    if (!vp.m_pixel_shader)
        throw render_error(SGL_ERR_INVALID, "viewport without a pixel shader");
    if (!vp.m_screen || !vp.m_screen->format || vp.m_screen->format->BytesPerPixel != 4)
        throw render_error(SGL_ERR_INVALID, "viewport surface must be 32-bit");
    sgl_view v{};
    v.x = vp.m_x;
    v.y = vp.m_y;
    v.w = vp.m_w;
    v.h = vp.m_h;
    copy_m(v.view, vp.m_camera.m_viewmatrix);
    copy_m(v.proj, vp.m_camera.m_projectionmatrix);
    v.camera_pos[0] = vp.m_camera.m_center.x();
    v.camera_pos[1] = vp.m_camera.m_center.y();
    v.camera_pos[2] = vp.m_camera.m_center.z();
    v.dof = vp.m_post_shader ? vp.m_post_shader->dof() : sgl_dof_desc{0, 0, 0, 0, 0};
    v.shader = vp.m_pixel_shader->gpu_shader();
    v.layers = vp.m_got_transparency ? vp.m_transparency_layer_count : 0;
    sgl_target t{vp.m_screen->pixels, vp.m_screen->pitch, vp.m_screen->w, vp.m_screen->h, vp.m_zbuffer.get()};
    check(sgl_render(context(), scene_id, &v, &t, 1, 0, nullptr, nullptr), "sgl_render");
}

} // namespace detail

// Forget the resident copy of `s` (after editing its vertex data in place).
inline void invalidate(const scene_t &s)
{
    auto &st = detail::state();
    auto it = st.scenes.find(&s);
    if (it != st.scenes.end()) {
        sgl_scene_release(detail::context(), it->second.id);
        st.scenes.erase(it);
    }
}

} // namespace gpu

// load_scene (src/data/gltf.cpp:455-464): a .gltf or .glb file through the
// library's loader (sgl_gltf_load, which follows the reference loader's
// rules); like the reference's, the scene has no lights.
inline scene_t load_scene(const std::string &filename)
{
    sgl_gltf *g = nullptr;
    char err[512] = {0};
    const sgl_status st = sgl_gltf_load(filename.c_str(), &g, err, sizeof err);
    if (st != SGL_OK)
        throw render_error(st, err);
    std::shared_ptr<sgl_gltf> hold(g, sgl_gltf_free);
    const sgl_scene_desc &d = *sgl_gltf_scene(g);
    scene_t s;
    s.nodes.resize((size_t)d.n_nodes);
    for (int i = 0; i < d.n_nodes; i++) {
        const sgl_node_desc &nd = d.nodes[i];
        node_t &n = s.nodes[(size_t)i];
        n.scale = vertex_t(nd.scale[0], nd.scale[1], nd.scale[2]);
        for (int k = 0; k < 16; k++)
            n.rotation[k / 4][k % 4] = nd.rotation[k];
        n.translation = vertex_t(nd.translation[0], nd.translation[1], nd.translation[2]);
    }
    for (int i = 0; i < d.n_nodes; i++) {
        const int p = d.nodes[i].parent;
        if (p >= 0) {
            s.nodes[(size_t)p].children_idx.push_back(i);
            s.nodes[(size_t)i].root = false;
        }
    }
    for (int i = 0; i < d.n_nodes; i++)
        if (s.nodes[(size_t)i].root)
            s.root_nodes.push_back(i);
    for (int k = 0; k < d.n_primitives; k++) {
        const sgl_primitive_desc &pd = d.primitives[k];
        primitive_t pr;
        pr.mode = (primitive_t::index_mode_t)pd.mode;
        pr.material_id = pd.material;
        pr.vertices.resize(pd.vertex_count);
        for (uint32_t v = 0; v < pd.vertex_count; v++) {
            const size_t g3 = 3 * (size_t)(pd.vertex_offset + v), g2 = 2 * (size_t)(pd.vertex_offset + v);
            mesh_vertex_t &mv = pr.vertices[v];
            mv.v = vertex_t(d.positions[g3], d.positions[g3 + 1], d.positions[g3 + 2]);
            mv.normal.x() = d.normals[g3]; // as loaded, not normalised (gltf.cpp:170-174)
            mv.normal.y() = d.normals[g3 + 1];
            mv.normal.z() = d.normals[g3 + 2];
            mv.tex_coords = vec2f_t(d.uvs[g2], d.uvs[g2 + 1]);
        }
        pr.indices.assign(d.indices + pd.index_offset, d.indices + pd.index_offset + pd.index_count);
        s.nodes[(size_t)pd.node].primitives.push_back(std::move(pr));
    }
    for (int m = 0; m < d.n_materials; m++) {
        material_t mt;
        mt.color = pixel_colors((unsigned int)d.materials[m].color);
        mt.texture_idx = d.materials[m].texture;
        mt.double_sided = d.materials[m].double_sided != 0;
        mt.shininess = d.materials[m].shininess;
        s.materials.push_back(mt);
    }
    for (int t = 0; t < d.n_textures; t++) {
        const sgl_texture_desc &td = d.textures[t];
        unsigned int *copy = new unsigned int[(size_t)td.width * td.height];
        std::memcpy(copy, td.texels, sizeof(unsigned int) * (size_t)td.width * td.height);
        s.images.emplace_back(copy, td.width, td.height);
    }
    s.animation_source = std::move(hold);
    return s;
}

inline void scene_t::animate(float elapsed_seconds)
{
    if (!animation_source)
        return;
    std::vector<sgl_node_desc> nd(nodes.size());
    const sgl_status st = sgl_gltf_animate(animation_source.get(), elapsed_seconds, nd.data());
    if (st != SGL_OK)
        throw render_error(st, "sgl_gltf_animate");
    for (size_t i = 0; i < nodes.size() && i < nd.size(); i++) {
        nodes[i].scale = vertex_t(nd[i].scale[0], nd[i].scale[1], nd[i].scale[2]);
        for (int k = 0; k < 16; k++)
            nodes[i].rotation[k / 4][k % 4] = nd[i].rotation[k];
        nodes[i].translation = vertex_t(nd[i].translation[0], nd[i].translation[1], nd[i].translation[2]);
    }
}

// render(scene, vp...) (swegl/render/renderer.hpp:27-34): the world transform
// once, then every viewport in order.
template <typename... T>
void render(scene_t &scene, T &...viewports)
{
    const int id = gpu::detail::resident(scene);
    (gpu::detail::render_one(id, viewports), ...);
}

} // namespace swegl
