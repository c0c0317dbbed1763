// sgl_shade.cuh — the pixel shaders of the swegl render path on the device:
// pixel_shader_lights_phong, pixel_shader_lights_flat, pixel_shader_texture
// (nearest), pixel_shader_texture_bilinear, the material colour of
// pixel_shader_t, and their pixel_shader_light_and_texture<L, T>
// combinations (swegl/render/pixel_shaders.hpp:15-179,
// src/render/pixel_shaders.cpp:14-384), with the reference's single-precision
// operation order.
#pragma once

#include "sgl_device.cuh"
#include "sgl_internal.h"

namespace sgl {

// The state of pixel_shader_light_and_texture<lights_phong, texture_bilinear>
// (swegl/render/pixel_shaders.hpp:76-97,125-150,121-179).
struct Shader {
    V3 v0, v1, v2, n0, n1, n2;
    V3 vleft, vright, vleftdir, vrightdir, nleft, nright, nleftdir, nrightdir;
    V3 v, vdir, n, ndir;
    V2 t0, t1, t2, side_long_t_dir, side_short_t, side_short_t_dir, t_left, t_dir;
    bool llr;
    const uint32_t *tex;
    uint32_t color;
    int tw, th, shininess;
    int flat_light; // pixel_shader_lights_flat::light as shade() returns it
};

// pixel_shader_*::prepare_for_triangle (src/render/pixel_shaders.cpp:88-105,304-318)
__device__ __forceinline__ void sh_prepare_triangle(Shader &sh, const V3 w[3], const V3 n[3], const V2 uv[3],
                                                    bool inverted)
{
    sh.v0 = w[0];
    sh.v1 = w[1];
    sh.v2 = w[2];
    if (!inverted) {
        sh.n0 = n[0];
        sh.n1 = n[1];
        sh.n2 = n[2];
    } else {
        sh.n0 = neg3(n[0]);
        sh.n1 = neg3(n[1]);
        sh.n2 = neg3(n[2]);
    }
    const float tw = (float)sh.tw, th = (float)sh.th;
    sh.t0 = mk2(uv[0].x * tw, uv[0].y * th);
    sh.t1 = mk2(uv[1].x * tw, uv[1].y * th);
    sh.t2 = mk2(uv[2].x * tw, uv[2].y * th);
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

// The sun and point-light sum of the Phong and the flat light shaders
// (src/render/pixel_shaders.cpp:159-205 per pixel, :33-84 per triangle): the
// same expressions at a point with a normal.
//
// A point light whose direction the reference would find behind the surface
// (alignment < 0, the light skipped) is skipped here before its division and
// normalisation when the unnormalised dot product already shows it with a
// margin that rounding cannot cross: with a_i = n_i * d_i (d = center minus
// the light), the float sum of the a_i is within 3 * 2^-24 * sum |a_i| of the
// exact dot product, and the reference's dot product of n with the
// normalised d (three IEEE divisions by the same length, three products, two
// sums) is within 2^-22 * sum |a_i| / length of the exact one divided by
// that length.  A float sum above 2^-20 * sum |a_i| therefore makes both
// positive, and the reference skips the light too (its test on the
// intensity / distance^2 ratio only skips more).  Sums below 2^-100 (where
// products could be subnormal), squared distances from 2^100 up (where the
// length could overflow) and NaNs take the full path.
__host__ __device__ __forceinline__ float light_sum(const LightsDev &L, V3 center, V3 normal, V3 camvec,
                                                    int shininess)
{
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
        const float ax = normal.x * ld.x, ay = normal.y * ld.y, az = normal.z * ld.z;
        const float mag = fabsf(ax) + fabsf(ay) + fabsf(az);
        if (ax + ay + az > 0x1p-20f * mag && mag > 0x1p-100f && d2 < 0x1p100f)
            continue; // behind the surface
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
            specular = spec_pow(specular, shininess);
            specular = specular * (float)shininess / 2.0f;
            dyn = dyn + (diffuse + specular / d2);
        } else {
            dyn = dyn + diffuse;
        }
    }
    return L.ambient + face_sun + dyn;
}

// pixel_shader_lights_phong::shade (src/render/pixel_shaders.cpp:159-205)
__device__ __forceinline__ int sh_phong(const Shader &sh, const LightsDev &L, const ViewDev &v, float progress)
{
    const V3 center = add3(sh.v, mul3(sh.vdir, progress));
    const V3 normal = normalize3(add3(sh.n, mul3(sh.ndir, progress)));
    const V3 camvec = normalize3(sub3(mk3(v.campos[0], v.campos[1], v.campos[2]), center));
    return f2i(65536.0f * light_sum(L, center, normal, camvec, sh.shininess));
}

// pixel_shader_lights_flat::prepare_for_triangle (src/render/pixel_shaders.cpp:
// 33-84) on fill_triangle_2's vertex order: the face normal (cross()
// normalises; the unary minus of a normal_t builds a normal_t, normalised
// again), the centroid (v0 + v1 + v2) / 3 and the same light sum; shade()
// returns light * 65536 converted to int.
__device__ __forceinline__ int flat_light(const V3 w[3], bool inverted, const LightsDev &L, const ViewDev &v,
                                          int shininess)
{
    V3 normal = cross_n(sub3(w[1], w[0]), sub3(w[2], w[0]));
    if (inverted)
        normal = normalize3(neg3(normal));
    const V3 sum = add3(add3(w[0], w[1]), w[2]);
    const V3 center = mk3(sum.x / 3.0f, sum.y / 3.0f, sum.z / 3.0f);
    const V3 camvec = normalize3(sub3(mk3(v.campos[0], v.campos[1], v.campos[2]), center));
    float light = light_sum(L, center, normal, camvec, shininess);
    light = light * 65536.0f;
    return f2i(light);
}

// pixel_shader_texture::shade (src/render/pixel_shaders.cpp:276-281): the
// texel at (int)t % size, the int converted to unsigned by the unsigned width
// and height.
__device__ __forceinline__ uint32_t sh_nearest(const Shader &sh, float progress)
{
    const V2 t = add2(sh.t_left, mul2(sh.t_dir, progress));
    const uint32_t tw = (uint32_t)sh.tw, th = (uint32_t)sh.th;
    const uint32_t u = (uint32_t)f2i(t.x) % tw;
    const uint32_t vv = (uint32_t)f2i(t.y) % th;
    if (sh.tex && !in_bounds(u < tw && vv < th, CHK_TEXEL, (unsigned long long)vv * tw + u))
        return 0u;
    return sh.tex ? __ldg(sh.tex + vv * tw + u) : sh.color; // untextured: 1x1 of the colour
}

// pixel_shader_texture_bilinear::shade (src/render/pixel_shaders.cpp:348-384)
// with the pixel_colors_f sums of src/render/colors.cpp:11-30.  v comes from
// t.x and u from t.y, as in the reference.
__device__ __forceinline__ uint32_t sh_bilinear(const Shader &sh, float progress)
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
        // the two texels of a row are neighbours unless the column wraps: one
        // 8-byte load when the pair starts on an even texel (textures start
        // 256-byte aligned), else two 4-byte loads
        const bool pair = u2m == u1m + 1;
        if (pair && (i11 & 1) == 0) {
            const uint2 t = __ldg(reinterpret_cast<const uint2 *>(sh.tex + i11));
            c11 = t.x;
            c12 = t.y;
        } else {
            c11 = __ldg(sh.tex + i11);
            c12 = __ldg(sh.tex + i12);
        }
        if (pair && (i21 & 1) == 0) {
            const uint2 t = __ldg(reinterpret_cast<const uint2 *>(sh.tex + i21));
            c21 = t.x;
            c22 = t.y;
        } else {
            c21 = __ldg(sh.tex + i21);
            c22 = __ldg(sh.tex + i22);
        }
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

// The view's pixel shader (SGL_SHADER_*, include/sgl.h); the combinations are
// pixel_shader_light_and_texture::shade (swegl/render/pixel_shaders.hpp:159-178).
// ALL_MODES = false compiles the default Phong + bilinear shader alone.
template <bool ALL_MODES = true>
__device__ __forceinline__ uint32_t sh_shade(const Shader &sh, const LightsDev &L, const ViewDev &v, float progress)
{
    const int mode = ALL_MODES ? v.shader : SGL_SHADER_PHONG_BILINEAR;
    if (mode >= SGL_SHADER_COLOR) {
        switch (mode) {
        case SGL_SHADER_COLOR: return sh.color;
        case SGL_SHADER_BILINEAR: return sh_bilinear(sh, progress);
        case SGL_SHADER_NEAREST: return sh_nearest(sh, progress);
        case SGL_SHADER_PHONG: return (uint32_t)sh_phong(sh, L, v, progress);
        default: return (uint32_t)sh.flat_light; // SGL_SHADER_FLAT
        }
    }
    const bool nearest = mode == SGL_SHADER_PHONG_NEAREST || mode == SGL_SHADER_FLAT_NEAREST;
    const bool flat = mode == SGL_SHADER_FLAT_BILINEAR || mode == SGL_SHADER_FLAT_NEAREST;
    uint32_t color = nearest ? sh_nearest(sh, progress) : sh_bilinear(sh, progress);
    // (float)(i / 65536.0): the int rounded to float, then an exact power-of-two scale
    float light = __int2float_rn(flat ? sh.flat_light : sh_phong(sh, L, v, progress)) * (1.0f / 65536.0f);
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


} // namespace sgl
