// raster.cu — sm_103a kernels of the swegl render path (one view per launch
// sequence): world transform, vertex stage, visibility flags, depth-key
// rasterisation, winner shading and resolve.
//
// Depth test semantics.  The reference draws triangles in order and keeps a
// fragment when z < zbuffer (strict, src/render/renderer.cpp:489-499), so the
// earliest-drawn of equal-depth fragments wins.  Here every fragment folds
// the 64-bit key (float bits of z << 32 | draw slot) into the pixel with
// atomicMin: depth is > 0.001 so its bits order like the floats, and the
// draw slot (2 * draw-order triangle + clip sub-triangle) breaks ties in draw
// order.  A second walk shades exactly the fragment whose key won, with the
// edge and span state the reference had for it.
#include <cstdint>

#include "sgl_device.cuh"
#include "sgl_internal.h"

namespace sgl {

// ---------------------------------------------------------------- vertices --

// vertex_shader_t::original_to_world (swegl/render/vertex_shaders.hpp:16-33) and
// the view-independent normal of camera_to_frustum (:63): rotate() normalises,
// .normalize() again, and the normal_t assignment a third time.
__global__ void k_world(SceneDev s)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= s.n_vertices)
        return;
    const uint32_t n = s.vnode[g];
    const float *M = s.node_world + 16 * n;
    const float *RS = s.node_rs + 16 * n;
    const float4 p = s.pos_u[g];
    const float4 q = s.nrm_v[g];
    const V3 w = transform3(mk3(p.x, p.y, p.z), M);
    const V3 nw = normalize3(normalize3(rotate_n(mk3(q.x, q.y, q.z), RS)));
    s.wpos[g] = make_float4(w.x, w.y, w.z, 0.0f);
    s.wnrm[g] = make_float4(nw.x, nw.y, nw.z, 0.0f);
}

// world_to_camera_or_frustum (vertex_shaders.hpp:35-52): view, projection
// (rows 0-2), x and y divided by |z'|; also clears the visibility flag.
__global__ void k_vertex(SceneDev s, ViewDev v, FrameDev f)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= s.n_vertices)
        return;
    const float4 w = s.wpos[g];
    V3 p = transform3(mk3(w.x, w.y, w.z), v.view);
    p = transform3(p, v.proj);
    if (p.z != 0.0f) {
        p.x = p.x / fabsf(p.z);
        p.y = p.y / fabsf(p.z);
    }
    f.ndc[g] = make_float4(p.x, p.y, p.z, 0.0f);
    f.yes[g] = 0;
}

// inside_camera_frustum (src/render/renderer.cpp:58-70)
__device__ __forceinline__ bool inside_frustum(V3 a, V3 b, V3 c)
{
    return (a.x >= -1.0f || b.x >= -1.0f || c.x >= -1.0f) && (a.y >= -1.0f || b.y >= -1.0f || c.y >= -1.0f) &&
           (a.x < 1.0f || b.x < 1.0f || c.x < 1.0f) && (a.y < 1.0f || b.y < 1.0f || c.y < 1.0f) &&
           (at_or_past_near(a.z) || at_or_past_near(b.z) || at_or_past_near(c.z)) && (a.x != b.x || a.x != c.x) &&
           (a.y != b.y || a.y != c.y);
}

__device__ __forceinline__ V3 ld3(const float4 *a, uint32_t i)
{
    const float4 t = a[i];
    return mk3(t.x, t.y, t.z);
}

// Visibility flags of the triangles of a primitive (renderer.cpp:86-185):
// inside the frustum and (double sided or front facing, front_face_visible
// :72-75, on the draw-order vertex triple).
__global__ void k_flags(SceneDev s, FrameDev f)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= s.n_triangles)
        return;
    const uint4 tri = s.tris[t];
    const V3 a = ld3(f.ndc, tri.x), b = ld3(f.ndc, tri.y), c = ld3(f.ndc, tri.z);
    if (!inside_frustum(a, b, c))
        return;
    const int m = s.prims[tri.w].material;
    const int ds = (m >= 0 && m < s.n_mats) ? s.mats[m].double_sided : 0;
    if (ds || cross_n(sub3(b, a), sub3(c, a)).z > 0.0f) {
        f.yes[tri.x] = 1;
        f.yes[tri.y] = 1;
        f.yes[tri.z] = 1;
    }
}

// ------------------------------------------------------------ triangle walk --

// A vertex as the triangle stage sees it (mesh_vertex_t, swegl/data/model.hpp:20-29).
struct TV {
    V3 vp;      // v_viewport: screen x, y and z'
    V3 world;   // v_world
    V3 normal;  // object-space normal (needed for near-clip vertices)
    V3 nworld;  // normal_world
    V2 uv;
};

// The state of pixel_shader_light_and_texture<lights_phong, texture_bilinear>
// (swegl/render/pixel_shaders.hpp:76-97,125-150,121-179).
struct Shader {
    V3 v0, v1, v2, n0, n1, n2;
    V3 vleft, vright, vleftdir, vrightdir, nleft, nright, nleftdir, nrightdir;
    V3 v, vdir, n, ndir;
    V2 t0, t1, t2, side_long_t_dir, side_short_t, side_short_t_dir, t_left, t_dir;
    bool llr;
    bool scan_ready;
    const uint32_t *tex;
    uint32_t color;
    int tw, th, shininess;
};

enum Mode { MODE_DEPTH = 0, MODE_SHADE = 1 };

struct Walk {
    SceneDev s;
    LightsDev L;
    ViewDev v;
    FrameDev f;
    uint32_t slot;
    unsigned long long fragments;
    unsigned long long drawn;
    Shader sh;
};

// pixel_shader_*::prepare_for_triangle (src/render/pixel_shaders.cpp:88-105,304-318)
__device__ __forceinline__ void sh_prepare_triangle(Shader &sh, const TV &a, const TV &b, const TV &c, bool inverted)
{
    sh.v0 = a.world;
    sh.v1 = b.world;
    sh.v2 = c.world;
    if (!inverted) {
        sh.n0 = a.nworld;
        sh.n1 = b.nworld;
        sh.n2 = c.nworld;
    } else {
        sh.n0 = neg3(a.nworld);
        sh.n1 = neg3(b.nworld);
        sh.n2 = neg3(c.nworld);
    }
    const float tw = (float)sh.tw, th = (float)sh.th;
    sh.t0 = mk2(a.uv.x * tw, a.uv.y * th);
    sh.t1 = mk2(b.uv.x * tw, b.uv.y * th);
    sh.t2 = mk2(c.uv.x * tw, c.uv.y * th);
    sh.side_long_t_dir = sub2(sh.t2, sh.t0);
}

// pixel_shaders.cpp:106-126,320-325
__device__ __forceinline__ void sh_prepare_upper(Shader &sh, bool llr)
{
    sh.vleft = sh.v0;
    sh.vright = sh.v0;
    sh.vleftdir = llr ? sub3(sh.v1, sh.v0) : sub3(sh.v2, sh.v0);
    sh.vrightdir = llr ? sub3(sh.v2, sh.v0) : sub3(sh.v1, sh.v0);
    sh.nleft = sh.n0;
    sh.nright = sh.n0;
    sh.nleftdir = llr ? sub3(sh.n1, sh.n0) : sub3(sh.n2, sh.n0);
    sh.nrightdir = llr ? sub3(sh.n2, sh.n0) : sub3(sh.n1, sh.n0);
    sh.llr = llr;
    sh.side_short_t = sh.t0;
    sh.side_short_t_dir = sub2(sh.t1, sh.t0);
}

// pixel_shaders.cpp:127-151,327-332
__device__ __forceinline__ void sh_prepare_lower(Shader &sh, bool llr)
{
    if (llr) {
        sh.vright = sh.v0;
        sh.vrightdir = sub3(sh.v2, sh.v0);
        sh.vleft = sh.v1;
        sh.vleftdir = sub3(sh.v2, sh.v1);
        sh.nright = sh.n0;
        sh.nrightdir = sub3(sh.n2, sh.n0);
        sh.nleft = sh.n1;
        sh.nleftdir = sub3(sh.n2, sh.n1);
    } else {
        sh.vleft = sh.v0;
        sh.vleftdir = sub3(sh.v2, sh.v0);
        sh.vright = sh.v1;
        sh.vrightdir = sub3(sh.v2, sh.v1);
        sh.nleft = sh.n0;
        sh.nleftdir = sub3(sh.n2, sh.n0);
        sh.nright = sh.n1;
        sh.nrightdir = sub3(sh.n2, sh.n1);
    }
    sh.llr = llr;
    sh.side_short_t = sh.t1;
    sh.side_short_t_dir = sub2(sh.t2, sh.t1);
}

// pixel_shaders.cpp:152-158,334-346
__device__ __forceinline__ void sh_prepare_scanline(Shader &sh, float pl, float pr)
{
    sh.v = add3(sh.vleft, mul3(sh.vleftdir, pl));
    sh.vdir = sub3(add3(sh.vright, mul3(sh.vrightdir, pr)), sh.v);
    sh.n = add3(sh.nleft, mul3(sh.nleftdir, pl));
    sh.ndir = sub3(add3(sh.nright, mul3(sh.nrightdir, pr)), sh.n);
    if (sh.llr) {
        sh.t_left = add2(sh.side_short_t, mul2(sh.side_short_t_dir, pl));
        sh.t_dir = sub2(add2(sh.t0, mul2(sh.side_long_t_dir, pr)), sh.t_left);
    } else {
        sh.t_left = add2(sh.t0, mul2(sh.side_long_t_dir, pl));
        sh.t_dir = sub2(add2(sh.side_short_t, mul2(sh.side_short_t_dir, pr)), sh.t_left);
    }
}

// pixel_shader_lights_phong::shade (src/render/pixel_shaders.cpp:159-205)
__device__ int sh_phong(const Shader &sh, const LightsDev &L, const ViewDev &v, float progress)
{
    const V3 center = add3(sh.v, mul3(sh.vdir, progress));
    const V3 normal = normalize3(add3(sh.n, mul3(sh.ndir, progress)));
    const V3 camvec = normalize3(sub3(mk3(v.campos[0], v.campos[1], v.campos[2]), center));
    float face_sun = -dot3(normal, mk3(L.sun[0], L.sun[1], L.sun[2]));
    if (face_sun < 0.0f)
        face_sun = 0.0f;
    else
        face_sun = face_sun * L.sun_intensity;
    float dyn = 0.0f;
    for (int l = 0; l < L.n; l++) {
        const float4 pl = L.pl[l];
        V3 ld = sub3(center, mk3(pl.x, pl.y, pl.z));
        const float d2 = ld.x * ld.x + ld.y * ld.y + ld.z * ld.z;
        float diffuse = pl.w / d2;
        if (diffuse < 0.05f) // (double)diffuse < 0.05, see sgl_device.cuh
            continue;
        ld = normalize3(ld);
        const float alignment = -dot3(normal, ld);
        if (alignment < 0.0f)
            continue;
        diffuse = diffuse * alignment;
        const V3 reflection = add3(ld, mul3(normal, alignment * 2.0f));
        float specular = dot3(reflection, camvec);
        if (specular > 0.0f) {
            specular = spec_pow(specular, sh.shininess);
            specular = specular * (float)sh.shininess / 2.0f;
            dyn = dyn + (diffuse + specular / d2);
        } else {
            dyn = dyn + diffuse;
        }
    }
    return f2i(65536.0f * (L.ambient + face_sun + dyn));
}

// pixel_shader_texture_bilinear::shade (src/render/pixel_shaders.cpp:348-384)
// with the pixel_colors_f sums of src/render/colors.cpp:11-30.  v comes from
// t.x and u from t.y, as in the reference.
__device__ uint32_t sh_bilinear(const Shader &sh, float progress)
{
    const V2 t = add2(sh.t_left, mul2(sh.t_dir, progress));
    float v = t.x;
    float u = t.y;
    // (float)(u - 0.5) in double equals u - 0.5f in float: 0.5 is exact and
    // double rounding is innocuous for a single subtraction.
    const float u1 = u - 0.5f, u2 = u + 0.5f, v1 = v - 0.5f, v2 = v + 0.5f;
    u = floorf(u2);
    v = floorf(v2);
    const int tw = sh.tw, th = sh.th;
    int v1m = (f2i(v1) + th) % th;
    int v2m = v1m + 1;
    if (v2m == th)
        v2m = 0;
    v1m *= tw;
    v2m *= tw;
    const int u1m = (f2i(u1) + tw) % tw;
    int u2m = u1m + 1;
    if (u2m == tw)
        u2m = 0;
    const long long n = (long long)tw * th;
    const long long i11 = (long long)v1m + u1m, i21 = (long long)v2m + u1m, i12 = (long long)v1m + u2m,
                    i22 = (long long)v2m + u2m;
    if (i11 < 0 || i11 >= n || i21 < 0 || i21 >= n || i12 < 0 || i12 >= n || i22 < 0 || i22 >= n)
        return 0u; // the reference reads outside the texture here
    const float w11 = (u - u1) * (v - v1), w21 = (u - u1) * (v2 - v), w12 = (u2 - u) * (v - v1),
                w22 = (u2 - u) * (v2 - v);
    uint32_t c11 = sh.color, c21 = sh.color, c12 = sh.color, c22 = sh.color; // untextured: 1x1 of the colour
    if (sh.tex) {
        c11 = __ldg(sh.tex + i11);
        c21 = __ldg(sh.tex + i21);
        c12 = __ldg(sh.tex + i12);
        c22 = __ldg(sh.tex + i22);
    }
    uint32_t out = 0;
#pragma unroll
    for (int ch = 0; ch < 4; ch++) {
        const int sft = 8 * ch;
        float acc = (float)((c11 >> sft) & 0xFFu) * w11;
        acc = acc + (float)((c21 >> sft) & 0xFFu) * w21;
        acc = acc + (float)((c12 >> sft) & 0xFFu) * w12;
        acc = acc + (float)((c22 >> sft) & 0xFFu) * w22;
        out |= ((uint32_t)f2i(roundf(acc)) & 0xFFu) << sft;
    }
    return out;
}

// pixel_shader_light_and_texture::shade (swegl/render/pixel_shaders.hpp:159-178)
__device__ uint32_t sh_shade(const Shader &sh, const LightsDev &L, const ViewDev &v, float progress)
{
    uint32_t color = sh_bilinear(sh, progress);
    // (float)(i / 65536.0): the int rounded to float, then an exact power-of-two scale
    float light = __int2float_rn(sh_phong(sh, L, v, progress)) * (1.0f / 65536.0f);
    uint32_t out = color & 0xFF000000u;
    if (light < 1.0f) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint32_t c = (color >> (8 * k)) & 0xFFu;
            out |= ((uint32_t)f2i((float)c * light) & 0xFFu) << (8 * k);
        }
    } else {
        light = sqrtf(light);
        light = sqrtf(light);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint32_t c = (color >> (8 * k)) & 0xFFu;
            const uint32_t q = (uint32_t)f2i((float)(255u - c) / light) & 0xFFu;
            out |= ((255u - q) & 0xFFu) << (8 * k);
        }
    }
    return out;
}

// fill_half_triangle (src/render/renderer.cpp:462-558), opaque branch
template <int MODE>
__device__ void fill_half(Walk &w, int y, int y_end, Side &Ls, Side &Rs)
{
    const ViewDev &v = w.v;
    for (; y < y_end; y++) {
        int x1 = f2i(ceilf(Ls.x));
        if (x1 < v.x)
            x1 = v.x;
        int x2 = f2i(ceilf(Rs.x));
        if (x2 > v.x + v.w)
            x2 = v.x + v.w;
        if (x1 < x2) {
            Interp q;
            q.init_self(Rs.x - Ls.x, Ls.it.value(), Rs.it.value());
            q.displace((float)x1 - Ls.x);
            const long long row = (long long)(y - v.y) * v.w - v.x;
            if (MODE == MODE_DEPTH)
                w.fragments += (unsigned long long)(x2 - x1);
            w.sh.scan_ready = false;
            for (; x1 < x2; x1++, q.step()) {
                const float z = q.value();
                if (below_near(z)) // (double)z <= 0.001
                    continue;
                const uint32_t zb = __float_as_uint(z);
                if (zb >= kMaxZBits)
                    continue; // never nearer than the cleared depth
                const unsigned long long key = ((unsigned long long)zb << 32) | w.slot;
                unsigned long long *kp = w.f.key + (row + x1);
                if (MODE == MODE_DEPTH) {
                    if (key < *kp)
                        atomicMin(kp, key);
                } else {
                    if (*kp == key) {
                        if (!w.sh.scan_ready) {
                            sh_prepare_scanline(w.sh, Ls.it.alpha, Rs.it.alpha);
                            w.sh.scan_ready = true;
                        }
                        w.f.pixels[(long long)(y - v.y) * w.f.pitch_px + (x1 - v.x)] = sh_shade(w.sh, w.L, w.v, q.alpha);
                    }
                }
            }
        }
        Ls.x = Ls.x + Ls.ratio;
        Rs.x = Rs.x + Rs.ratio;
        Ls.it.step();
        Rs.it.step();
    }
}

// fill_triangle_2 (src/render/renderer.cpp:361-460)
template <int MODE>
__device__ void fill_triangle_2(Walk &w, const TV *a, const TV *b, const TV *c, bool front_face_visible)
{
    const ViewDev &v = w.v;
    const TV *t;
    const bool inverted = !front_face_visible;
    if (b->vp.y < a->vp.y) { t = a; a = b; b = t; }
    if (c->vp.y < b->vp.y) { t = b; b = c; c = t; }
    if (b->vp.y < a->vp.y) { t = a; a = b; b = t; }
    const V3 v0 = a->vp, v1 = b->vp, v2 = c->vp;
    const int y0 = f2i(ceilf(v0.y));
    const int y1 = f2i(ceilf(v1.y));
    const int y2 = f2i(ceilf(v2.y));
    if (y0 == y2)
        return;
    Side lng, sht;
    lng.ratio = (v2.x - v0.x) / (v2.y - v0.y);
    lng.it.init_self(v2.y - v0.y, v0.z, v2.z);
    if (y0 < v.y) {
        lng.it.displace((float)v.y - v0.y);
        lng.x = v0.x + lng.ratio * ((float)v.y - v0.y);
    } else {
        lng.it.displace((float)y0 - v0.y);
        lng.x = v0.x + lng.ratio * ((float)y0 - v0.y);
    }
    if (MODE == MODE_DEPTH) {
        w.drawn++;
        if (w.f.slot_flags)
            w.f.slot_flags[w.slot] = 1;
    } else {
        sh_prepare_triangle(w.sh, *a, *b, *c, inverted);
    }
    if (y1 >= v.y) {
        sht.ratio = (v1.x - v0.x) / (v1.y - v0.y);
        sht.it.init_self(v1.y - v0.y, v0.z, v1.z);
        const int y = y0 > v.y ? y0 : v.y;
        const int y_end = y1 < v.y + v.h ? y1 : v.y + v.h;
        sht.it.displace((float)y - v0.y);
        sht.x = v0.x + sht.ratio * ((float)y - v0.y);
        const bool llr = lng.ratio > sht.ratio;
        if (MODE == MODE_SHADE)
            sh_prepare_upper(w.sh, llr);
        if (llr)
            fill_half<MODE>(w, y, y_end, sht, lng);
        else
            fill_half<MODE>(w, y, y_end, lng, sht);
    }
    if (y1 < v.y + v.h) {
        sht.ratio = (v2.x - v1.x) / (v2.y - v1.y);
        sht.it.init_self(v2.y - v1.y, v1.z, v2.z);
        const int y = y1 > v.y ? y1 : v.y;
        const int y_end = y2 < v.y + v.h ? y2 : v.y + v.h;
        sht.it.displace((float)y - v1.y);
        sht.x = v1.x + sht.ratio * ((float)y - v1.y);
        const bool llr = lng.ratio < sht.ratio;
        if (MODE == MODE_SHADE)
            sh_prepare_lower(w.sh, llr);
        if (llr)
            fill_half<MODE>(w, y, y_end, sht, lng);
        else
            fill_half<MODE>(w, y, y_end, lng, sht);
    }
}

// world_to_viewport (vertex_shaders.hpp:54-59) of a near-clip vertex
__device__ __forceinline__ void world_to_viewport(const Walk &w, TV &o, const float *rs)
{
    V3 p = transform3(o.world, w.v.view);
    o.nworld = normalize3(normalize3(rotate_n(o.normal, rs)));
    p = transform3(p, w.v.proj);
    if (p.z != 0.0f) {
        p.x = p.x / fabsf(p.z);
        p.y = p.y / fabsf(p.z);
    }
    p.x = w.v.vm00 * p.x + w.v.vm03;
    p.y = w.v.vm11 * p.y + w.v.vm13;
    o.vp = p;
}

// near-clip vertex a + (b - a) * cut (renderer.cpp:290-297)
__device__ __forceinline__ void clip_vertex(const Walk &w, TV &o, const TV &a, const TV &b, float cut, const float *rs)
{
    o.world = add3(a.world, mul3(sub3(b.world, a.world), cut));
    o.uv = add2(a.uv, mul2(sub2(b.uv, a.uv), cut));
    if (b.normal.x == a.normal.x && b.normal.y == a.normal.y && b.normal.z == a.normal.z)
        o.normal = a.normal;
    else
        o.normal = normalize3(add3(a.normal, mul3(sub3(b.normal, a.normal), cut)));
    world_to_viewport(w, o, rs);
}

// fill_triangle (src/render/renderer.cpp:240-359)
template <int MODE>
__device__ void fill_triangle(Walk &w, const TV *a, const TV *b, const TV *c, const float *rs, uint32_t tri)
{
    V3 v0 = a->vp, v1 = b->vp, v2 = c->vp;
    bool ffv = cross_n(sub3(v1, v0), sub3(v2, v0)).z < 0.0f;
    bool inverted_order = false;
    const TV *t;
    V3 tv;
    if (v1.z > v0.z) { tv = v0; v0 = v1; v1 = tv; t = a; a = b; b = t; inverted_order = !inverted_order; }
    if (v2.z > v1.z) { tv = v1; v1 = v2; v2 = tv; t = b; b = c; c = t; inverted_order = !inverted_order; }
    if (v1.z > v0.z) { tv = v0; v0 = v1; v1 = tv; t = a; a = b; b = t; inverted_order = !inverted_order; }
    if (at_or_past_near(v2.z)) {
        w.slot = 2 * tri;
        fill_triangle_2<MODE>(w, a, b, c, ffv);
    } else if (below_near(v1.z)) {
        TV n1, n2;
        clip_vertex(w, n1, *a, *b, (v0.z - 0.001f) / (v0.z - v1.z), rs);
        clip_vertex(w, n2, *a, *c, (v0.z - 0.001f) / (v0.z - v2.z), rs);
        ffv = cross_n(sub3(n1.vp, v0), sub3(n2.vp, v0)).z < 0.0f;
        if (inverted_order)
            ffv = !ffv;
        w.slot = 2 * tri;
        fill_triangle_2<MODE>(w, a, &n1, &n2, ffv);
    } else {
        TV n1, n2;
        clip_vertex(w, n1, *a, *c, (v0.z - 0.001f) / (v0.z - v2.z), rs);
        clip_vertex(w, n2, *b, *c, (v1.z - 0.001f) / (v1.z - v2.z), rs);
        ffv = cross_n(sub3(v1, v0), sub3(n2.vp, v0)).z < 0.0f;
        if (inverted_order)
            ffv = !ffv;
        w.slot = 2 * tri;
        fill_triangle_2<MODE>(w, a, b, &n2, ffv);
        ffv = cross_n(sub3(n2.vp, v0), sub3(n1.vp, v0)).z < 0.0f;
        if (inverted_order)
            ffv = !ffv;
        w.slot = 2 * tri + 1;
        fill_triangle_2<MODE>(w, a, &n2, &n1, ffv);
    }
}

__device__ __forceinline__ void load_tv(const SceneDev &s, const ViewDev &v, const FrameDev &f, uint32_t g, TV &o)
{
    const float4 n = f.ndc[g];
    o.vp = mk3(v.vm00 * n.x + v.vm03, v.vm11 * n.y + v.vm13, n.z); // frustum_to_viewport (viewport.cpp:123-129)
    const float4 w = s.wpos[g];
    o.world = mk3(w.x, w.y, w.z);
    const float4 pu = s.pos_u[g];
    const float4 nv = s.nrm_v[g];
    o.normal = mk3(nv.x, nv.y, nv.z);
    o.uv = mk2(pu.w, nv.w);
    const float4 nw = s.wnrm[g];
    o.nworld = mk3(nw.x, nw.y, nw.z);
}

__device__ __forceinline__ void warp_add(unsigned long long *dst, unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0 && v)
        atomicAdd(dst, v);
}

// One thread per draw-order triangle: the fill_triangle of renderer.cpp:191-230.
template <int MODE>
__global__ void __launch_bounds__(128) k_raster(SceneDev s, LightsDev L, ViewDev v, FrameDev f)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    Walk w;
    w.fragments = 0;
    w.drawn = 0;
    if (t < s.n_triangles) {
        const uint4 tri = s.tris[t];
        if (f.yes[tri.x] && f.yes[tri.y] && f.yes[tri.z]) {
            w.s = s;
            w.L = L;
            w.v = v;
            w.f = f;
            const PrimDesc pd = s.prims[tri.w];
            if (MODE == MODE_SHADE) {
                const MatDesc m = (pd.material >= 0 && pd.material < s.n_mats) ? s.mats[pd.material] : s.default_mat;
                w.sh.shininess = m.shininess;
                if (m.texture < 0 || m.texture >= s.n_texs) {
                    w.sh.color = m.color;
                    w.sh.tex = nullptr;
                    w.sh.tw = w.sh.th = 1;
                } else {
                    const TexDesc td = s.texs[m.texture];
                    w.sh.tex = td.texels;
                    w.sh.tw = td.w;
                    w.sh.th = td.h;
                }
            }
            TV tv[3];
            load_tv(s, v, f, tri.x, tv[0]);
            load_tv(s, v, f, tri.y, tv[1]);
            load_tv(s, v, f, tri.z, tv[2]);
            fill_triangle<MODE>(w, &tv[0], &tv[1], &tv[2], s.node_rs + 16 * pd.node, t);
        }
    }
    if (MODE == MODE_DEPTH) {
        warp_add(&f.counters[0], w.drawn);
        warp_add(&f.counters[1], w.fragments);
    }
}

// Background of the viewport (viewport_t::clear, viewport.cpp:88-113) and
// the depth of every pixel.
__global__ void k_resolve(ViewDev v, FrameDev f)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.w * v.h)
        return;
    const unsigned long long k = f.key[i];
    float z;
    if (k == kEmptyKey) {
        const int y = i / v.w, x = i - y * v.w;
        f.pixels[(long long)y * f.pitch_px + x] = 0u;
        z = __uint_as_float(kMaxZBits);
    } else {
        z = __uint_as_float((uint32_t)(k >> 32));
    }
    if (f.zbuf)
        f.zbuf[i] = z;
}

static inline unsigned grid_for(uint64_t n, int block) { return (unsigned)((n + block - 1) / block); }

cudaError_t launch_world(const SceneDev &s, cudaStream_t st)
{
    if (s.n_vertices == 0)
        return cudaSuccess;
    k_world<<<grid_for(s.n_vertices, 256), 256, 0, st>>>(s);
    return cudaGetLastError();
}

cudaError_t launch_frame(const SceneDev &s, const LightsDev &l, const ViewDev &v, const FrameDev &f, cudaStream_t st,
                         int *launches)
{
    int n = 0;
    cudaError_t e = cudaMemsetAsync(f.key, 0xFF, sizeof(unsigned long long) * (size_t)v.w * v.h, st);
    if (e != cudaSuccess)
        return e;
    if (s.n_vertices) {
        k_vertex<<<grid_for(s.n_vertices, 256), 256, 0, st>>>(s, v, f);
        n++;
    }
    if (s.n_triangles) {
        k_flags<<<grid_for(s.n_triangles, 256), 256, 0, st>>>(s, f);
        k_raster<MODE_DEPTH><<<grid_for(s.n_triangles, 128), 128, 0, st>>>(s, l, v, f);
        k_raster<MODE_SHADE><<<grid_for(s.n_triangles, 128), 128, 0, st>>>(s, l, v, f);
        n += 3;
    }
    k_resolve<<<grid_for((uint64_t)v.w * v.h, 256), 256, 0, st>>>(v, f);
    n++;
    if (launches)
        *launches += n;
    return cudaGetLastError();
}

} // namespace sgl
