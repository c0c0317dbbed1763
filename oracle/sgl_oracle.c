/*
 * sgl_oracle.c — CPU restatement of gbizzotto/swegl's render path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg use it, as the checker / the timed CPU
 * reference; the product never links or calls it.
 *
 * Parity is pinned: tests/golden holds outputs of the reference itself
 * (compiled headless from its own sources by oracle/ref), and the tests check
 * this restatement against them bit for bit (colour, depth, winner ordinal,
 * per-pixel progress).
 *
 * Each function follows the reference function cited beside it (paths inside
 * gbizzotto/swegl) with the same single-precision operation order.  Compile
 * with -ffp-contract=off: fused multiply-adds change the reference's bits.
 * Values the reference converts with an out-of-range (int) cast take the x86-64
 * result (INT_MIN), which is what the reference's own x86 build produces.
 *
 * One extension: the point-light specular exponent comes from the material
 * (sgl_material_desc::shininess); the reference hard-codes 32
 * (src/render/pixel_shaders.cpp:192) and golden scenes use 32.
 *
 * The depth-of-field gather (orc_dof) is not the reference's: its
 * post_shader_depth_box (swegl/render/post_shaders.hpp:51-132) reads a
 * z-buffer the opaque path never writes and indexes past its source row.  It
 * is the CPU oracle of the gather specified in include/sgl.h (sgl_dof) with
 * the tap table of include/sgl_dof_taps.h.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sgl.h"
#include "sgl_dof_taps.h"

#define ORC_API __attribute__((visibility("default")))

typedef struct { float x, y, z; } v3;
typedef struct { float x, y; } v2;

static inline v3 mk3(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
static inline v3 neg3(v3 a) { return mk3(-a.x, -a.y, -a.z); }
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }   /* points.hpp:91-94 */
static inline v2 mk2(float x, float y) { v2 r; r.x = x; r.y = y; return r; }
static inline v2 add2(v2 a, v2 b) { return mk2(a.x + b.x, a.y + b.y); }          /* vec2f.hpp:150-153 */
static inline v2 sub2(v2 a, v2 b) { return mk2(a.x - b.x, a.y - b.y); }          /* vec2f.hpp:146-149 */
static inline v2 mul2(v2 a, float s) { return mk2(a.x * s, a.y * s); }           /* vec2f.hpp:154-158 */

/* vector_t::normalize (swegl/projection/points.hpp:71-90) */
static inline v3 normalize3(v3 v)
{
    float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    if (l != 0) {
        v.x /= l;
        v.y /= l;
        v.z /= l;
    }
    return v;
}

/* cross() returns a normal_t, normalised by its constructor (src/projection/points.cpp:32-37) */
static inline v3 cross_n(v3 a, v3 b)
{
    return normalize3(mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x));
}

/* transform(vertex, m): rows 0-2 of m only (src/projection/points.cpp:8-13) */
static inline v3 transform3(v3 v, const float *m)
{
    return mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3],
               m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7],
               m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11]);
}

/* rotate(normal, m): upper 3x3, then the normal_t constructor normalises (points.cpp:44-49) */
static inline v3 rotate_n(v3 v, const float *m)
{
    return normalize3(mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z,
                          m[4] * v.x + m[5] * v.y + m[6] * v.z,
                          m[8] * v.x + m[9] * v.y + m[10] * v.z));
}

/* (int)f as the reference's x86-64 build computes it (cvttss2si): values
 * outside the int range, and NaN, give INT_MIN. */
static inline int f2i(float f)
{
    if (f >= -2147483648.0f && f < 2147483648.0f)
        return (int)f;
    return INT32_MIN;
}

/* ------------------------------------------------------------------ scene -- */

typedef struct {
    float world[16]; /* original_to_world_matrix */
    float rs[16];    /* scale(rotation, scale): the normal matrix */
    int done;
} onode;

typedef struct {
    const sgl_scene_desc *d;
    onode *nodes;
    int *prim_order;   /* draw order: node by node, then desc order */
    uint32_t *tri_base; /* first global triangle index of each primitive (desc index) */
    uint64_t n_triangles;
    v3 *world;          /* v_world per vertex */
    v3 *nworld;         /* normal_world per vertex */
} oscene;

/* scale(m, v) (src/projection/points.cpp:14-30) */
static void scale_m(float *r, const float *m, const float *s)
{
    memcpy(r, m, 16 * sizeof(float));
    for (int row = 0; row < 4; row++)
        for (int c = 0; c < 3; c++)
            r[row * 4 + c] *= s[c];
}

/* 4x4 product summed k = 0..3 left to right */
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
    memcpy(r, t, sizeof t);
}

static const float IDENTITY[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

/* node_t::get_local_world_matrix (swegl/data/model.hpp:56-61) and the
 * recursion of vertex_shader_t::original_to_world (vertex_shaders.hpp:16-33) */
static int node_world(oscene *s, int i, int depth)
{
    onode *n = &s->nodes[i];
    if (n->done)
        return 0;
    if (depth > s->d->n_nodes)
        return -1;
    const sgl_node_desc *nd = &s->d->nodes[i];
    float local[16];
    scale_m(local, nd->rotation, nd->scale);
    memcpy(n->rs, local, sizeof local);
    local[3] += nd->translation[0];
    local[7] += nd->translation[1];
    local[11] += nd->translation[2];
    const float *parent = IDENTITY;
    if (nd->parent >= 0) {
        if (nd->parent >= s->d->n_nodes || node_world(s, nd->parent, depth + 1))
            return -1;
        parent = s->nodes[nd->parent].world;
    }
    matmul4(n->world, parent, local);
    n->done = 1;
    return 0;
}

static void scene_free(oscene *s)
{
    free(s->nodes);
    free(s->prim_order);
    free(s->tri_base);
    free(s->world);
    free(s->nworld);
    memset(s, 0, sizeof *s);
}

static uint32_t prim_triangles(const sgl_primitive_desc *p)
{
    if (p->mode == SGL_TRIANGLES)
        return p->index_count / 3;
    if (p->mode == SGL_TRIANGLE_STRIP || p->mode == SGL_TRIANGLE_FAN)
        return p->index_count >= 2 ? p->index_count - 2 : 0;
    return 0;
}

static int scene_prepare(oscene *s, const sgl_scene_desc *d)
{
    memset(s, 0, sizeof *s);
    s->d = d;
    s->nodes = (onode *)calloc((size_t)(d->n_nodes > 0 ? d->n_nodes : 1), sizeof(onode));
    s->prim_order = (int *)malloc(sizeof(int) * (size_t)(d->n_primitives > 0 ? d->n_primitives : 1));
    s->tri_base = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(d->n_primitives > 0 ? d->n_primitives : 1));
    s->world = (v3 *)malloc(sizeof(v3) * (size_t)(d->n_vertices ? d->n_vertices : 1));
    s->nworld = (v3 *)malloc(sizeof(v3) * (size_t)(d->n_vertices ? d->n_vertices : 1));
    if (!s->nodes || !s->prim_order || !s->tri_base || !s->world || !s->nworld)
        return -1;
    for (int i = 0; i < d->n_nodes; i++)
        if (node_world(s, i, 0))
            return -1;
    /* draw order: nodes in order, primitives of a node in desc order (renderer.cpp:83,191) */
    int k = 0;
    for (int n = 0; n < d->n_nodes; n++)
        for (int p = 0; p < d->n_primitives; p++)
            if (d->primitives[p].node == n)
                s->prim_order[k++] = p;
    if (k != d->n_primitives)
        return -1;
    uint64_t t = 0;
    for (int q = 0; q < k; q++) {
        int p = s->prim_order[q];
        s->tri_base[p] = (uint32_t)t;
        t += prim_triangles(&d->primitives[p]);
    }
    s->n_triangles = t;
    for (int p = 0; p < d->n_primitives; p++) {
        const sgl_primitive_desc *pd = &d->primitives[p];
        const onode *n = &s->nodes[pd->node];
        for (uint32_t v = 0; v < pd->vertex_count; v++) {
            uint32_t g = pd->vertex_offset + v;
            v3 pos = mk3(d->positions[3 * g], d->positions[3 * g + 1], d->positions[3 * g + 2]);
            v3 nrm = mk3(d->normals[3 * g], d->normals[3 * g + 1], d->normals[3 * g + 2]);
            s->world[g] = transform3(pos, n->world);                       /* vertex_shaders.hpp:22-23 */
            /* camera_to_frustum (vertex_shaders.hpp:63): rotate() normalises,
             * .normalize() again, and the normal_t assignment a third time */
            s->nworld[g] = normalize3(normalize3(rotate_n(nrm, n->rs)));
        }
    }
    return 0;
}

/* ----------------------------------------------------------- interpolator -- */

/* interpolator_g<1> (swegl/render/interpolator.hpp:52-104) */
typedef struct { float top, tstep, alpha, bottom, bstep, v0, dv; } interp;

static inline void interp_init_self(interp *it, float dist, float z1, float z2)
{
    it->v0 = z1;
    it->dv = z2 - z1;
    float alphastep = 1.0f / dist;
    it->bottom = 1.0f / z1;
    float invz2 = 1.0f / z2;
    it->alpha = 0.0f;
    it->top = it->alpha;
    it->top *= it->bottom;
    it->tstep = (1.0f * invz2 - it->top) * alphastep;
    it->bstep = (invz2 - it->bottom) * alphastep;
}
static inline void interp_displace(interp *it, float move)
{
    it->top += it->tstep * move;
    it->bottom += it->bstep * move;
    it->alpha = it->top / it->bottom;
}
static inline void interp_step(interp *it)
{
    it->top += it->tstep;
    it->bottom += it->bstep;
    it->alpha = it->top / it->bottom;
}
static inline float interp_value(const interp *it) { return it->v0 + it->dv * it->alpha; }

typedef struct { interp it; float ratio; float x; } line_side; /* renderer.cpp:21-26 */

/* ----------------------------------------------------------- pixel shader -- */

/* A vertex as the triangle stage sees it (mesh_vertex_t, model.hpp:20-29). */
typedef struct { v3 world, normal, nworld, vp; v2 uv; } tvert;

typedef struct {
    /* pixel_shader_lights_phong state (pixel_shaders.hpp:76-97) */
    v3 v0, v1, v2, vleft, vright, vleftdir, vrightdir, v, vdir;
    v3 n0, n1, n2, nleft, nright, nleftdir, nrightdir, n, ndir;
    /* pixel_shader_texture_bilinear state (pixel_shaders.hpp:125-150) */
    v2 t0, t1, t2, side_long_t_dir, side_short_t, side_short_t_dir, t_left, t_dir;
    int llr;
    const uint32_t *tex;
    uint32_t default_bitmap;
    int tw, th;
    int shininess;
    /* pixel_shader_t::color (pixel_shaders.hpp:20), pixel_shader_lights_flat::light */
    uint32_t color;
    int flat_light;
    /* scene / viewport inputs */
    const sgl_scene_desc *d;
    v3 campos;
    int kind;
    int mode; /* SGL_SHADER_* of the view */
    int calls;
} shader;

static int mode_flat(int m) { return m == SGL_SHADER_FLAT_BILINEAR || m == SGL_SHADER_FLAT_NEAREST || m == SGL_SHADER_FLAT; }

/* pixel_shader_texture_bilinear::prepare_for_primitive (pixel_shaders.cpp:284-302) */
static void sh_prepare_primitive(shader *sh, const sgl_primitive_desc *p)
{
    const sgl_scene_desc *d = sh->d;
    const sgl_material_desc *m = (p->material >= 0 && p->material < d->n_materials) ? &d->materials[p->material]
                                                                                    : &d->default_material;
    sh->shininess = m->shininess;
    sh->color = m->color; /* pixel_shader_t::prepare_for_primitive (pixel_shaders.cpp:14-31) */
    if (m->texture < 0 || m->texture >= d->n_textures) {
        sh->default_bitmap = m->color;
        sh->tex = &sh->default_bitmap;
        sh->tw = sh->th = 1;
    } else {
        sh->tex = d->textures[m->texture].texels;
        sh->tw = d->textures[m->texture].width;
        sh->th = d->textures[m->texture].height;
    }
}

static int sh_flat_light(const shader *sh, const tvert *a, const tvert *b, const tvert *c, int inverted);

/* prepare_for_triangle of the phong and the bilinear shaders (pixel_shaders.cpp:88-105,304-318) */
static void sh_prepare_triangle(shader *sh, const tvert *a, const tvert *b, const tvert *c, int inverted)
{
    sh->calls++;
    sh->v0 = a->world;
    sh->v1 = b->world;
    sh->v2 = c->world;
    if (!inverted) {
        sh->n0 = a->nworld;
        sh->n1 = b->nworld;
        sh->n2 = c->nworld;
    } else {
        sh->n0 = neg3(a->nworld);
        sh->n1 = neg3(b->nworld);
        sh->n2 = neg3(c->nworld);
    }
    sh->t0 = a->uv;
    sh->t1 = b->uv;
    sh->t2 = c->uv;
    sh->t0.x *= (float)sh->tw;
    sh->t0.y *= (float)sh->th;
    sh->t1.x *= (float)sh->tw;
    sh->t1.y *= (float)sh->th;
    sh->t2.x *= (float)sh->tw;
    sh->t2.y *= (float)sh->th;
    sh->side_long_t_dir = sub2(sh->t2, sh->t0);
    if (sh->kind == 0 && mode_flat(sh->mode))
        sh->flat_light = sh_flat_light(sh, a, b, c, inverted);
}

/* pixel_shaders.cpp:106-126 and 320-325 */
static void sh_prepare_upper(shader *sh, int llr)
{
    sh->vleft = sh->v0;
    sh->vright = sh->v0;
    if (llr) {
        sh->vleftdir = sub3(sh->v1, sh->v0);
        sh->vrightdir = sub3(sh->v2, sh->v0);
    } else {
        sh->vleftdir = sub3(sh->v2, sh->v0);
        sh->vrightdir = sub3(sh->v1, sh->v0);
    }
    sh->nleft = sh->n0;
    sh->nright = sh->n0;
    if (llr) {
        sh->nleftdir = sub3(sh->n1, sh->n0);
        sh->nrightdir = sub3(sh->n2, sh->n0);
    } else {
        sh->nleftdir = sub3(sh->n2, sh->n0);
        sh->nrightdir = sub3(sh->n1, sh->n0);
    }
    sh->llr = llr;
    sh->side_short_t = sh->t0;
    sh->side_short_t_dir = sub2(sh->t1, sh->t0);
}

/* pixel_shaders.cpp:127-151 and 327-332 */
static void sh_prepare_lower(shader *sh, int llr)
{
    if (llr) {
        sh->vright = sh->v0;
        sh->vrightdir = sub3(sh->v2, sh->v0);
        sh->vleft = sh->v1;
        sh->vleftdir = sub3(sh->v2, sh->v1);
        sh->nright = sh->n0;
        sh->nrightdir = sub3(sh->n2, sh->n0);
        sh->nleft = sh->n1;
        sh->nleftdir = sub3(sh->n2, sh->n1);
    } else {
        sh->vleft = sh->v0;
        sh->vleftdir = sub3(sh->v2, sh->v0);
        sh->vright = sh->v1;
        sh->vrightdir = sub3(sh->v2, sh->v1);
        sh->nleft = sh->n0;
        sh->nleftdir = sub3(sh->n2, sh->n0);
        sh->nright = sh->n1;
        sh->nrightdir = sub3(sh->n2, sh->n1);
    }
    sh->llr = llr;
    sh->side_short_t = sh->t1;
    sh->side_short_t_dir = sub2(sh->t2, sh->t1);
}

/* pixel_shaders.cpp:152-158 and 334-346 */
static void sh_prepare_scanline(shader *sh, float pl, float pr)
{
    sh->v = add3(sh->vleft, mul3(sh->vleftdir, pl));
    sh->vdir = sub3(add3(sh->vright, mul3(sh->vrightdir, pr)), sh->v);
    sh->n = add3(sh->nleft, mul3(sh->nleftdir, pl));
    sh->ndir = sub3(add3(sh->nright, mul3(sh->nrightdir, pr)), sh->n);
    if (sh->llr) {
        sh->t_left = add2(sh->side_short_t, mul2(sh->side_short_t_dir, pl));
        sh->t_dir = sub2(add2(sh->t0, mul2(sh->side_long_t_dir, pr)), sh->t_left);
    } else {
        sh->t_left = add2(sh->t0, mul2(sh->side_long_t_dir, pl));
        sh->t_dir = sub2(add2(sh->side_short_t, mul2(sh->side_short_t_dir, pr)), sh->t_left);
    }
}

/* The sun and point-light sum of the Phong and the flat light shaders
 * (pixel_shaders.cpp:159-205 per pixel, :33-84 per triangle): both evaluate
 * the same expressions at a point with a normal. */
static float light_sum(const sgl_scene_desc *d, v3 center, v3 normal, v3 camvec, int shininess)
{
    v3 sun = mk3(d->sun_direction[0], d->sun_direction[1], d->sun_direction[2]);
    float face_sun = -dot3(normal, sun);
    if (face_sun < 0.0f)
        face_sun = 0.0f;
    else
        face_sun *= d->sun_intensity;
    float dyn = 0.0f;
    for (int l = 0; l < d->n_point_lights; l++) {
        const sgl_point_light *pl = &d->point_lights[l];
        v3 ld = sub3(center, mk3(pl->position[0], pl->position[1], pl->position[2]));
        float d2 = ld.x * ld.x + ld.y * ld.y + ld.z * ld.z;
        float diffuse = pl->intensity / d2;
        if ((double)diffuse < 0.05)
            continue;
        ld = normalize3(ld);
        float alignment = -dot3(normal, ld);
        if (alignment < 0.0f)
            continue;
        diffuse *= alignment;
        v3 reflection = add3(ld, mul3(normal, alignment * 2));
        float specular = dot3(reflection, camvec);
        if (specular > 0) {
            specular = (float)pow((double)specular, (double)shininess);
            specular = specular * (float)shininess / 2;
            dyn += diffuse + specular / d2;
        } else {
            dyn += diffuse;
        }
    }
    return d->ambient + face_sun + dyn;
}

/* pixel_shader_lights_phong::shade (src/render/pixel_shaders.cpp:159-205) */
static int sh_phong(const shader *sh, float progress)
{
    v3 center = add3(sh->v, mul3(sh->vdir, progress));
    v3 normal = normalize3(add3(sh->n, mul3(sh->ndir, progress)));
    v3 camvec = normalize3(sub3(sh->campos, center));
    return f2i(65536 * light_sum(sh->d, center, normal, camvec, sh->shininess));
}

/* pixel_shader_lights_flat::prepare_for_triangle (pixel_shaders.cpp:33-84):
 * the face normal (cross() normalises; the unary minus of a normal_t builds a
 * normal_t, normalised again), the centroid (v0 + v1 + v2) / 3 and the same
 * light sum; shade() returns light * 65536 converted to int. */
static int sh_flat_light(const shader *sh, const tvert *a, const tvert *b, const tvert *c, int inverted)
{
    v3 normal = cross_n(sub3(b->world, a->world), sub3(c->world, a->world));
    if (inverted)
        normal = normalize3(neg3(normal));
    v3 sum = add3(add3(a->world, b->world), c->world);
    v3 center = mk3(sum.x / 3, sum.y / 3, sum.z / 3);
    v3 camvec = normalize3(sub3(sh->campos, center));
    float light = light_sum(sh->d, center, normal, camvec, sh->shininess);
    light *= 65536;
    return f2i(light);
}

static inline uint8_t u8_of(float f) { return (uint8_t)f2i(f); }

/* pixel_shader_texture_bilinear::shade (src/render/pixel_shaders.cpp:348-384)
 * with pixel_colors / pixel_colors_f arithmetic (src/render/colors.cpp:11-30).
 * Note the reference's axis use: v comes from t.x, u from t.y. */
static uint32_t sh_bilinear(const shader *sh, float progress)
{
    v2 t = add2(sh->t_left, mul2(sh->t_dir, progress));
    float v = t.x;
    float u = t.y;
    float u1 = (float)((double)u - 0.5);
    float u2 = (float)((double)u + 0.5);
    float v1 = (float)((double)v - 0.5);
    float v2f = (float)((double)v + 0.5);
    u = floorf(u2);
    v = floorf(v2f);
    const int tw = sh->tw, th = sh->th;
    int v1m = (f2i(v1) + th) % th;
    int v2m = v1m + 1;
    if (v2m == th)
        v2m = 0;
    v1m *= tw;
    v2m *= tw;
    int u1m = (f2i(u1) + tw) % tw;
    int u2m = u1m + 1;
    if (u2m == tw)
        u2m = 0;
    const long n = (long)tw * th;
    long i11 = (long)v1m + u1m, i21 = (long)v2m + u1m, i12 = (long)v1m + u2m, i22 = (long)v2m + u2m;
    if (i11 < 0 || i11 >= n || i21 < 0 || i21 >= n || i12 < 0 || i12 >= n || i22 < 0 || i22 >= n)
        return 0; /* the reference reads outside the texture here */
    const float w11 = (u - u1) * (v - v1), w21 = (u - u1) * (v2f - v), w12 = (u2 - u) * (v - v1),
                w22 = (u2 - u) * (v2f - v);
    const uint32_t c[4] = {sh->tex[i11], sh->tex[i21], sh->tex[i12], sh->tex[i22]};
    const float w[4] = {w11, w21, w12, w22};
    uint32_t out = 0;
    for (int ch = 0; ch < 4; ch++) {
        float acc = (float)((c[0] >> (8 * ch)) & 0xFF) * w[0];
        for (int k = 1; k < 4; k++)
            acc = acc + (float)((c[k] >> (8 * ch)) & 0xFF) * w[k];
        out |= (uint32_t)u8_of(roundf(acc)) << (8 * ch);
    }
    return out;
}

/* pixel_shader_texture::shade (src/render/pixel_shaders.cpp:276-281): the
 * texel at (int)t % size, the int converted to unsigned by the unsigned
 * texture width and height. */
static uint32_t sh_nearest(const shader *sh, float progress)
{
    v2 t = add2(sh->t_left, mul2(sh->t_dir, progress));
    const uint32_t tw = (uint32_t)sh->tw, th = (uint32_t)sh->th;
    const uint32_t u = (uint32_t)f2i(t.x) % tw;
    const uint32_t v = (uint32_t)f2i(t.y) % th;
    return sh->tex[v * tw + u];
}

/* The view's pixel shader; the combinations are
 * pixel_shader_light_and_texture::shade (swegl/render/pixel_shaders.hpp:159-178). */
static uint32_t sh_shade(shader *sh, float progress, int ordinal)
{
    switch (sh->kind) {
    case 1: return (uint32_t)ordinal;
    case 2: { uint32_t b; memcpy(&b, &progress, 4); return b; }
    case 3: return (uint32_t)sh_phong(sh, progress);
    case 4: return sh_bilinear(sh, progress);
    default: break;
    }
    switch (sh->mode) {
    case SGL_SHADER_COLOR: return sh->color;
    case SGL_SHADER_BILINEAR: return sh_bilinear(sh, progress);
    case SGL_SHADER_NEAREST: return sh_nearest(sh, progress);
    case SGL_SHADER_PHONG: return (uint32_t)sh_phong(sh, progress);
    case SGL_SHADER_FLAT: return (uint32_t)sh->flat_light;
    default: break;
    }
    const int nearest = sh->mode == SGL_SHADER_PHONG_NEAREST || sh->mode == SGL_SHADER_FLAT_NEAREST;
    uint32_t color = nearest ? sh_nearest(sh, progress) : sh_bilinear(sh, progress);
    const int li = mode_flat(sh->mode) ? sh->flat_light : sh_phong(sh, progress);
    float light = (float)((double)li / 65536.0);
    uint8_t ch[4];
    memcpy(ch, &color, 4);
    if (light < 1) {
        for (int k = 0; k < 3; k++)
            ch[k] = u8_of((float)ch[k] * light);
    } else {
        light = sqrtf(light);
        light = sqrtf(light);
        for (int k = 0; k < 3; k++)
            ch[k] = (uint8_t)(255 - u8_of((float)(255 - ch[k]) / light));
    }
    memcpy(&color, ch, 4);
    return color;
}

/* ------------------------------------------------------------- rasteriser -- */

typedef struct {
    const sgl_view *view;
    const sgl_target *target;
    float *zb;
    float vm00, vm03, vm11, vm13; /* viewport_t::m_viewportmatrix (viewport.cpp:94-99) */
    shader sh;
    uint32_t *winner_slot;
    uint32_t slot;
    uint64_t fragments;
    uint64_t drawn;
    uint64_t clip_one, clip_two; /* triangles through the near-clip branches */
    /* transparency layers (viewport_t::m_transparency_layers): layer k of
     * view pixel p at [k * w * h + p]; 0 = opaque view */
    int n_layers;
    float *lz;
    uint32_t *lc;
} raster;

static const union { int32_t i; float f; } MAX_Z = {0x7F7F7F7F}; /* max_z, renderer.cpp:15-19 */

/* blend (src/render/colors.cpp:39-57) on 0xAARRGGBB pixels */
static uint32_t blend_px(uint32_t back, uint32_t front)
{
    const int alpha = (int)(front >> 24), balpha = (int)(back >> 24);
    const int new_alpha = 255 - ((255 - alpha) * (255 - balpha) / 255);
    if (alpha == 255)
        return (front & 0x00FFFFFFu) | ((uint32_t)(uint8_t)new_alpha << 24);
    if (alpha == 0)
        return (back & 0x00FFFFFFu) | ((uint32_t)(uint8_t)new_alpha << 24);
    uint32_t out = (uint32_t)(uint8_t)new_alpha << 24;
    for (int c = 0; c < 3; c++) {
        const int b = (int)((back >> (8 * c)) & 0xFF), f = (int)((front >> (8 * c)) & 0xFF);
        out |= (uint32_t)(uint8_t)(b * ((256 - alpha) / 256.0) + f * (alpha / 256.0)) << (8 * c);
    }
    return out;
}

/* A fragment that passed the depth test of a view with transparency layers
 * (renderer.cpp:500-550): an opaque colour is drawn and drops the layers
 * behind it; a transparent one is inserted among the layers, in front of
 * those farther away, pushing the others up (or, when every layer is used,
 * down, losing the farthest). */
static void layer_insert(raster *r, long off, uint32_t *video, float z, uint32_t color)
{
    const int n = r->n_layers;
    const long px = (long)r->view->w * r->view->h;
    float *lz = r->lz + off;
    uint32_t *lc = r->lc + off;
    int li;
    for (li = 0; li < n; li++)
        if (lz[li * px] == MAX_Z.f || lz[li * px] < z)
            break;
    if ((color >> 24) == 255) {
        *video = color;
        r->zb[off] = z;
        int i, k;
        for (i = 0, k = li; k < n; i++, k++) {
            lz[i * px] = lz[k * px];
            lc[i * px] = lc[k * px];
        }
        for (; i < n; i++) {
            lz[i * px] = MAX_Z.f;
            lc[i * px] = 0;
        }
    } else if (lz[(n - 1) * px] != MAX_Z.f) {
        while (li-- > 0) {
            const float tz = lz[li * px];
            const uint32_t tc = lc[li * px];
            lz[li * px] = z;
            lc[li * px] = color;
            z = tz;
            color = tc;
        }
    } else {
        for (; li < n; li++) {
            const float tz = lz[li * px];
            const uint32_t tc = lc[li * px];
            lz[li * px] = z;
            lc[li * px] = color;
            z = tz;
            color = tc;
            if (z == MAX_Z.f)
                break;
        }
    }
}

/* viewport_t::flatten (viewport.cpp:43-86), then post_shader_t::shade's copy
 * of the first layer to the screen (post_shaders.hpp:22-47).  As in the
 * reference, the screen pixels read and written are those of surface row j
 * (flatten) and row j + y (copy), column i, for view pixel (i, j). */
static void layers_resolve(raster *r)
{
    const sgl_view *v = r->view;
    const long px = (long)v->w * v->h;
    uint32_t *screen = (uint32_t *)r->target->pixels;
    const int pitch_px = r->target->pitch / 4;
    for (int k = 1; k < r->n_layers; k++)
        for (long p = 0; p < px; p++)
            if (r->lc[k * px + p] >> 24)
                r->lc[p] = blend_px(r->lc[p], r->lc[k * px + p]);
    for (int j = 0; j < v->h; j++)
        for (int i = 0; i < v->w; i++) {
            const uint32_t back = screen[(long)j * pitch_px + i];
            uint32_t *f = &r->lc[(long)j * v->w + i];
            *f = (*f >> 24) ? blend_px(back, *f) : back;
        }
    for (int j = 0; j < v->h; j++)
        for (int i = 0; i < v->w; i++)
            screen[(long)(j + v->y) * pitch_px + i] = r->lc[(long)j * v->w + i];
}

/* fill_half_triangle (src/render/renderer.cpp:462-558), opaque branch */
static void fill_half(raster *r, int y, int y_end, line_side *L, line_side *R)
{
    const sgl_view *vp = r->view;
    uint32_t *pixels = (uint32_t *)r->target->pixels;
    const int pitch_px = r->target->pitch / 4;
    for (; y < y_end; y++) {
        int x1 = f2i(ceilf(L->x));
        if (x1 < vp->x)
            x1 = vp->x;
        int x2 = f2i(ceilf(R->x));
        if (x2 > vp->x + vp->w)
            x2 = vp->x + vp->w;
        if (x1 < x2) {
            sh_prepare_scanline(&r->sh, L->it.alpha, R->it.alpha);
            interp q;
            interp_init_self(&q, R->x - L->x, interp_value(&L->it), interp_value(&R->it));
            interp_displace(&q, (float)x1 - L->x);
            long zoff = (long)(y - vp->y) * vp->w + (x1 - vp->x);
            for (; x1 < x2; x1++, zoff++, interp_step(&q)) {
                float z = interp_value(&q);
                r->fragments++;
                if ((double)z <= 0.001)
                    continue;
                if (z >= r->zb[zoff])
                    continue;
                const uint32_t color = sh_shade(&r->sh, q.alpha, r->sh.calls - 1);
                if (r->n_layers) {
                    layer_insert(r, zoff, &pixels[(long)y * pitch_px + x1], z, color);
                    continue;
                }
                pixels[(long)y * pitch_px + x1] = color;
                r->zb[zoff] = z;
                if (r->winner_slot)
                    r->winner_slot[zoff] = r->slot;
            }
        }
        L->x += L->ratio;
        R->x += R->ratio;
        interp_step(&L->it);
        interp_step(&R->it);
    }
}

/* fill_triangle_2 (src/render/renderer.cpp:361-460) */
static void fill_triangle_2(raster *r, const tvert *a, const tvert *b, const tvert *c, int front_face_visible)
{
    const sgl_view *vp = r->view;
    const tvert *t;
    int inverted = !front_face_visible;
    if (b->vp.y < a->vp.y) { t = a; a = b; b = t; }
    if (c->vp.y < b->vp.y) { t = b; b = c; c = t; }
    if (b->vp.y < a->vp.y) { t = a; a = b; b = t; }
    const v3 v0 = a->vp, v1 = b->vp, v2 = c->vp;
    int y0 = f2i(ceilf(v0.y));
    int y1 = f2i(ceilf(v1.y));
    int y2 = f2i(ceilf(v2.y));
    if (y0 == y2)
        return;
    line_side lng, sht;
    lng.ratio = (v2.x - v0.x) / (v2.y - v0.y);
    interp_init_self(&lng.it, v2.y - v0.y, v0.z, v2.z);
    if (y0 < vp->y) {
        interp_displace(&lng.it, (float)vp->y - v0.y);
        lng.x = v0.x + lng.ratio * ((float)vp->y - v0.y);
    } else {
        interp_displace(&lng.it, (float)y0 - v0.y);
        lng.x = v0.x + lng.ratio * ((float)y0 - v0.y);
    }
    r->drawn++;
    sh_prepare_triangle(&r->sh, a, b, c, inverted);
    int y, y_end;
    if (y1 >= vp->y) {
        sht.ratio = (v1.x - v0.x) / (v1.y - v0.y);
        interp_init_self(&sht.it, v1.y - v0.y, v0.z, v1.z);
        y = y0 > vp->y ? y0 : vp->y;
        y_end = y1 < vp->y + vp->h ? y1 : vp->y + vp->h;
        interp_displace(&sht.it, (float)y - v0.y);
        sht.x = v0.x + sht.ratio * ((float)y - v0.y);
        int llr = lng.ratio > sht.ratio;
        sh_prepare_upper(&r->sh, llr);
        if (llr)
            fill_half(r, y, y_end, &sht, &lng);
        else
            fill_half(r, y, y_end, &lng, &sht);
    }
    if (y1 < vp->y + vp->h) {
        sht.ratio = (v2.x - v1.x) / (v2.y - v1.y);
        interp_init_self(&sht.it, v2.y - v1.y, v1.z, v2.z);
        y = y1 > vp->y ? y1 : vp->y;
        y_end = y2 < vp->y + vp->h ? y2 : vp->y + vp->h;
        interp_displace(&sht.it, (float)y - v1.y);
        sht.x = v1.x + sht.ratio * ((float)y - v1.y);
        int llr = lng.ratio < sht.ratio;
        sh_prepare_lower(&r->sh, llr);
        if (llr)
            fill_half(r, y, y_end, &sht, &lng);
        else
            fill_half(r, y, y_end, &lng, &sht);
    }
}

typedef struct {
    const float *view, *proj;
} cam;

/* world_to_viewport (vertex_shaders.hpp:54-59): view, projection and |z'|
 * divide (camera_to_frustum, :61-71), then the viewport transform (viewport.cpp:123-129) */
static void world_to_viewport(const raster *r, tvert *v, const float *rs)
{
    v3 p = transform3(v->world, r->view->view);
    v->nworld = normalize3(normalize3(rotate_n(v->normal, rs)));
    p = transform3(p, r->view->proj);
    if (p.z != 0) {
        p.x /= fabsf(p.z);
        p.y /= fabsf(p.z);
    }
    p.x = r->vm00 * p.x + r->vm03;
    p.y = r->vm11 * p.y + r->vm13;
    v->vp = p;
}

/* near-clip vertex: a + (b - a) * cut on position, texture coordinates and
 * normal; the normal is copied when equal (renderer.cpp:290-297) */
static void clip_vertex(const raster *r, tvert *out, const tvert *a, const tvert *b, float cut, const float *rs)
{
    out->world = add3(a->world, mul3(sub3(b->world, a->world), cut));
    out->uv = add2(a->uv, mul2(sub2(b->uv, a->uv), cut));
    if (b->normal.x == a->normal.x && b->normal.y == a->normal.y && b->normal.z == a->normal.z)
        out->normal = a->normal;
    else
        out->normal = normalize3(add3(a->normal, mul3(sub3(b->normal, a->normal), cut)));
    world_to_viewport(r, out, rs);
}

/* fill_triangle (src/render/renderer.cpp:240-359) */
static void fill_triangle(raster *r, const tvert *a, const tvert *b, const tvert *c, const float *rs, uint32_t tri)
{
    v3 v0 = a->vp, v1 = b->vp, v2 = c->vp;
    int ffv = cross_n(sub3(v1, v0), sub3(v2, v0)).z < 0;
    int inverted_order = 0;
    const tvert *t;
    v3 tv;
    if (v1.z > v0.z) { tv = v0; v0 = v1; v1 = tv; t = a; a = b; b = t; inverted_order = !inverted_order; }
    if (v2.z > v1.z) { tv = v1; v1 = v2; v2 = tv; t = b; b = c; c = t; inverted_order = !inverted_order; }
    if (v1.z > v0.z) { tv = v0; v0 = v1; v1 = tv; t = a; a = b; b = t; inverted_order = !inverted_order; }
    if ((double)v2.z >= 0.001) {
        r->slot = 2 * tri;
        fill_triangle_2(r, a, b, c, ffv);
    } else if ((double)v1.z < 0.001) {
        tvert n1, n2;
        r->clip_one++;
        float cut_1 = (v0.z - 0.001f) / (v0.z - v1.z);
        clip_vertex(r, &n1, a, b, cut_1, rs);
        float cut_2 = (v0.z - 0.001f) / (v0.z - v2.z);
        clip_vertex(r, &n2, a, c, cut_2, rs);
        ffv = cross_n(sub3(n1.vp, v0), sub3(n2.vp, v0)).z < 0;
        if (inverted_order)
            ffv = !ffv;
        r->slot = 2 * tri;
        fill_triangle_2(r, a, &n1, &n2, ffv);
    } else {
        tvert n1, n2;
        r->clip_two++;
        float cut_0 = (v0.z - 0.001f) / (v0.z - v2.z);
        clip_vertex(r, &n1, a, c, cut_0, rs);
        float cut_1 = (v1.z - 0.001f) / (v1.z - v2.z);
        clip_vertex(r, &n2, b, c, cut_1, rs);
        ffv = cross_n(sub3(v1, v0), sub3(n2.vp, v0)).z < 0;
        if (inverted_order)
            ffv = !ffv;
        r->slot = 2 * tri;
        fill_triangle_2(r, a, b, &n2, ffv);
        ffv = cross_n(sub3(n2.vp, v0), sub3(n1.vp, v0)).z < 0;
        if (inverted_order)
            ffv = !ffv;
        r->slot = 2 * tri + 1;
        fill_triangle_2(r, a, &n2, &n1, ffv);
    }
}

/* inside_camera_frustum (renderer.cpp:58-70) */
static int inside_frustum(v3 a, v3 b, v3 c)
{
    return (a.x >= -1 || b.x >= -1 || c.x >= -1) && (a.y >= -1 || b.y >= -1 || c.y >= -1) &&
           (a.x < 1 || b.x < 1 || c.x < 1) && (a.y < 1 || b.y < 1 || c.y < 1) &&
           ((double)a.z >= 0.001 || (double)b.z >= 0.001 || (double)c.z >= 0.001) &&
           (a.x != b.x || a.x != c.x) && (a.y != b.y || a.y != c.y);
}

/* front_face_visible (renderer.cpp:72-75) */
static int front_visible(v3 a, v3 b, v3 c) { return cross_n(sub3(b, a), sub3(c, a)).z > 0; }

/* Draw-order vertex triple of triangle t of a primitive (renderer.cpp:198-229). */
static void tri_indices(const sgl_primitive_desc *p, const uint32_t *idx, uint32_t t, uint32_t *i0, uint32_t *i1,
                        uint32_t *i2)
{
    if (p->mode == SGL_TRIANGLE_STRIP) {
        uint32_t i = t + 2;
        *i0 = idx[i - 2];
        *i1 = idx[i - 1 + (i & 1)];
        *i2 = idx[i - (i & 1)];
    } else if (p->mode == SGL_TRIANGLE_FAN) {
        uint32_t i = t + 2;
        *i0 = idx[0];
        *i1 = idx[i - 1];
        *i2 = idx[i];
    } else {
        *i0 = idx[3 * t];
        *i1 = idx[3 * t + 1];
        *i2 = idx[3 * t + 2];
    }
}

typedef struct {
    uint64_t drawn;      /* fill_triangle_2 calls that reached prepare_for_triangle */
    uint64_t fragments;  /* covered (triangle, pixel) pairs of all spans */
    uint64_t clip_one;   /* triangles with only one vertex in front of the near plane */
    uint64_t clip_two;   /* triangles with two vertices in front of the near plane */
} view_stats;

/* _render (src/render/renderer.cpp:77-235) for one viewport, opaque path. */
static int render_view(const oscene *s, const sgl_view *view, const sgl_target *target, int kind,
                       uint32_t *winner_slot, view_stats *st)
{
    const sgl_scene_desc *d = s->d;
    const uint32_t nv = d->n_vertices;
    v3 *vpos = (v3 *)malloc(sizeof(v3) * (size_t)(nv ? nv : 1));
    uint8_t *yes = (uint8_t *)calloc(nv ? nv : 1, 1);
    float *zb = (float *)malloc(sizeof(float) * (size_t)view->w * (size_t)view->h);
    if (!vpos || !yes || !zb) {
        free(vpos);
        free(yes);
        free(zb);
        return -1;
    }
    /* world_to_camera_or_frustum (vertex_shaders.hpp:35-52) */
    for (uint32_t g = 0; g < nv; g++) {
        v3 p = transform3(s->world[g], view->view);
        p = transform3(p, view->proj);
        if (p.z != 0) {
            p.x /= fabsf(p.z);
            p.y /= fabsf(p.z);
        }
        vpos[g] = p;
    }
    /* viewport_t::clear (viewport.cpp:88-113) */
    uint32_t *pixels = (uint32_t *)target->pixels;
    const int pitch_px = target->pitch / 4;
    for (int y = view->y; y < view->y + view->h; y++)
        memset(&pixels[(long)y * pitch_px + view->x], 0, 4 * (size_t)view->w);
    memset(zb, 0x7F, sizeof(float) * (size_t)view->w * view->h);
    if (winner_slot)
        memset(winner_slot, 0xFF, sizeof(uint32_t) * (size_t)view->w * view->h);

    raster r;
    memset(&r, 0, sizeof r);
    r.view = view;
    r.target = target;
    r.zb = zb;
    r.vm00 = (float)view->w / 2.0f;
    r.vm03 = (float)view->x + (float)view->w / 2.0f;
    r.vm11 = -(float)view->h / 2.0f;
    r.vm13 = (float)view->y + (float)view->h / 2.0f;
    r.winner_slot = winner_slot;
    r.sh.d = d;
    r.sh.campos = mk3(view->camera_pos[0], view->camera_pos[1], view->camera_pos[2]);
    r.sh.kind = kind;
    r.sh.mode = view->shader;
    if (view->layers > 0 && kind == 0) {
        const size_t lpx = (size_t)view->layers * view->w * view->h;
        r.n_layers = view->layers;
        r.lz = (float *)malloc(sizeof(float) * lpx);
        r.lc = (uint32_t *)calloc(lpx, sizeof(uint32_t));
        if (!r.lz || !r.lc) {
            free(r.lz);
            free(r.lc);
            free(vpos);
            free(yes);
            free(zb);
            return -1;
        }
        memset(r.lz, 0x7F, sizeof(float) * lpx); /* viewport_t::clear (viewport.cpp:107-112) */
    }

    int q0 = 0;
    for (int n = 0; n < d->n_nodes; n++) {
        int q1 = q0;
        while (q1 < d->n_primitives && d->primitives[s->prim_order[q1]].node == n)
            q1++;
        /* flags of visible triangles (renderer.cpp:86-185) */
        for (int q = q0; q < q1; q++) {
            const sgl_primitive_desc *p = &d->primitives[s->prim_order[q]];
            const uint32_t *idx = d->indices + p->index_offset;
            const sgl_material_desc *m =
                (p->material >= 0 && p->material < d->n_materials) ? &d->materials[p->material] : NULL;
            const int double_sided = m && m->double_sided;
            const uint32_t nt = prim_triangles(p);
            for (uint32_t t = 0; t < nt; t++) {
                uint32_t i0, i1, i2;
                tri_indices(p, idx, t, &i0, &i1, &i2);
                uint32_t g0 = p->vertex_offset + i0, g1 = p->vertex_offset + i1, g2 = p->vertex_offset + i2;
                if (inside_frustum(vpos[g0], vpos[g1], vpos[g2]) &&
                    (double_sided || front_visible(vpos[g0], vpos[g1], vpos[g2])))
                    yes[g0] = yes[g1] = yes[g2] = 1;
            }
        }
        /* frustum_to_viewport (vertex_shaders.hpp:72-84) */
        for (int q = q0; q < q1; q++) {
            const sgl_primitive_desc *p = &d->primitives[s->prim_order[q]];
            for (uint32_t v = 0; v < p->vertex_count; v++) {
                uint32_t g = p->vertex_offset + v;
                if (yes[g]) {
                    vpos[g].x = r.vm00 * vpos[g].x + r.vm03;
                    vpos[g].y = r.vm11 * vpos[g].y + r.vm13;
                }
            }
        }
        /* painting (renderer.cpp:191-230) */
        for (int q = q0; q < q1; q++) {
            const int pi = s->prim_order[q];
            const sgl_primitive_desc *p = &d->primitives[pi];
            const uint32_t *idx = d->indices + p->index_offset;
            const float *rs = s->nodes[p->node].rs;
            sh_prepare_primitive(&r.sh, p);
            const uint32_t nt = prim_triangles(p);
            for (uint32_t t = 0; t < nt; t++) {
                uint32_t i0, i1, i2;
                tri_indices(p, idx, t, &i0, &i1, &i2);
                uint32_t g[3] = {p->vertex_offset + i0, p->vertex_offset + i1, p->vertex_offset + i2};
                if (!yes[g[0]] || !yes[g[1]] || !yes[g[2]])
                    continue;
                tvert tv[3];
                for (int k = 0; k < 3; k++) {
                    tv[k].world = s->world[g[k]];
                    tv[k].normal = mk3(d->normals[3 * g[k]], d->normals[3 * g[k] + 1], d->normals[3 * g[k] + 2]);
                    tv[k].nworld = s->nworld[g[k]];
                    tv[k].vp = vpos[g[k]];
                    tv[k].uv = mk2(d->uvs[2 * g[k]], d->uvs[2 * g[k] + 1]);
                }
                fill_triangle(&r, &tv[0], &tv[1], &tv[2], rs, s->tri_base[pi] + t);
            }
        }
        q0 = q1;
    }
    if (r.n_layers) {
        layers_resolve(&r);
        free(r.lz);
        free(r.lc);
    }
    if (target->zbuffer)
        memcpy(target->zbuffer, zb, sizeof(float) * (size_t)view->w * view->h);
    if (st) {
        st->drawn = r.drawn;
        st->fragments = r.fragments;
        st->clip_one = r.clip_one;
        st->clip_two = r.clip_two;
    }
    free(vpos);
    free(yes);
    free(zb);
    return 0;
}

/* --------------------------------------------------------- depth of field -- */

/* The depth-of-field gather of include/sgl.h (sgl_dof): src/out are the view's
 * colour (pitches in pixels), z its z-buffer (w*h). */
static void dof_gather(const sgl_view *view, const uint32_t *src, int src_pitch, const float *z, uint32_t *out,
                       int out_pitch)
{
    const int w = view->w, h = view->h;
    const float k = view->dof.px_scale > 0.0f ? view->dof.px_scale : (view->proj[5] * (float)h) / 2.0f;
    const float ka = k * view->dof.aperture;
    const float p22 = view->proj[10], p23 = view->proj[11];
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const float zp = z[(long)y * w + x];
            const float zv = (zp - p23) / p22;
            float r = (ka * fabsf(zv - view->dof.focus)) / zv;
            if (!(r >= 0.0f && r <= view->dof.max_radius))
                r = view->dof.max_radius;
            uint32_t sb = 0, sg = 0, sr = 0;
            for (int t = 0; t < SGL_DOF_TAPS; t++) {
                int sx = x + (int)lrintf(r * sgl_dof_taps[t][0]); /* nearest, ties to even */
                int sy = y + (int)lrintf(r * sgl_dof_taps[t][1]);
                sx = sx < 0 ? 0 : (sx >= w ? w - 1 : sx);
                sy = sy < 0 ? 0 : (sy >= h ? h - 1 : sy);
                const uint32_t c = src[(long)sy * src_pitch + sx];
                sb += c & 0xFFu;
                sg += (c >> 8) & 0xFFu;
                sr += (c >> 16) & 0xFFu;
            }
            const uint32_t centre = src[(long)y * src_pitch + x];
            out[(long)y * out_pitch + x] = (centre & 0xFF000000u) | (((sr + 16u) / 32u) << 16) |
                                           (((sg + 16u) / 32u) << 8) | ((sb + 16u) / 32u);
        }
}

/* The gather alone on host buffers: `in` holds the view's colour rectangle and
 * z-buffer, `out` receives the result in its rectangle. */
ORC_API int orc_dof(const sgl_view *view, const sgl_target *in, const sgl_target *out)
{
    if (!view || !in || !out || !in->zbuffer || view->w <= 0 || view->h <= 0)
        return -1;
    const int ip = in->pitch / 4, op = out->pitch / 4;
    const uint32_t *src = (const uint32_t *)in->pixels + (long)view->y * ip + view->x;
    uint32_t *dst = (uint32_t *)out->pixels + (long)view->y * op + view->x;
    dof_gather(view, src, ip, in->zbuffer, dst, op);
    return 0;
}

/* After render_view: the gather over the view's own rectangle when enabled. */
static int apply_dof(const sgl_view *view, const sgl_target *target)
{
    if (!view->dof.enabled || !target->zbuffer)
        return 0;
    const int p = target->pitch / 4;
    const size_t px = (size_t)view->w * view->h;
    uint32_t *tmp = (uint32_t *)malloc(4 * px);
    if (!tmp)
        return -1;
    uint32_t *rect = (uint32_t *)target->pixels + (long)view->y * p + view->x;
    for (int y = 0; y < view->h; y++)
        memcpy(tmp + (size_t)y * view->w, rect + (long)y * p, 4 * (size_t)view->w);
    dof_gather(view, tmp, view->w, target->zbuffer, rect, p);
    free(tmp);
    return 0;
}

/* ------------------------------------------------------------------- API -- */

/* Render views in order, as swegl::render(scene, vp0, vp1, ...) does.
 * kind: 0 Phong + bilinear (then the depth-of-field gather of views that
 * enable it), 1 winner ordinal, 2 progress bits, 3 Phong light int, 4
 * bilinear texel.  winner_slot (view 0, may be NULL) receives
 * 2 * triangle + sub-triangle of the pixel's winner.  stats (may be NULL)
 * receives [drawn, fragments, clip_one, clip_two] per view. */
ORC_API int orc_render(const sgl_scene_desc *desc, const sgl_view *views, const sgl_target *targets, int n_views,
                       int kind, uint32_t *winner_slot, uint64_t *stats)
{
    if (!desc || !views || !targets || n_views <= 0)
        return -1;
    oscene s;
    if (scene_prepare(&s, desc)) {
        scene_free(&s);
        return -1;
    }
    int rc = 0;
    for (int i = 0; i < n_views && rc == 0; i++) {
        view_stats st;
        rc = render_view(&s, &views[i], &targets[i], kind, i == 0 ? winner_slot : NULL, &st);
        if (rc == 0 && kind == 0)
            rc = apply_dof(&views[i], &targets[i]);
        if (stats) {
            stats[4 * i] = st.drawn;
            stats[4 * i + 1] = st.fragments;
            stats[4 * i + 2] = st.clip_one;
            stats[4 * i + 3] = st.clip_two;
        }
    }
    scene_free(&s);
    return rc;
}

ORC_API uint64_t orc_triangle_count(const sgl_scene_desc *desc)
{
    oscene s;
    uint64_t n = 0;
    if (scene_prepare(&s, desc) == 0)
        n = s.n_triangles;
    scene_free(&s);
    return n;
}

typedef struct {
    const oscene *s;
    const sgl_view *views;
    const sgl_target *targets;
    int n;
    int next;
    pthread_mutex_t mu;
    int rc;
} par_job;

static void *par_worker(void *arg)
{
    par_job *j = (par_job *)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int i = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (i >= j->n)
            return NULL;
        if (render_view(j->s, &j->views[i], &j->targets[i], 0, NULL, NULL) || apply_dof(&j->views[i], &j->targets[i]))
            j->rc = -1;
    }
}

/* Render independent views (each into its own target) on `threads` host
 * threads: the CPU-throughput baseline.  The scene is prepared once. */
ORC_API int orc_render_parallel(const sgl_scene_desc *desc, const sgl_view *views, const sgl_target *targets,
                                int n_views, int threads)
{
    if (!desc || !views || !targets || n_views <= 0 || threads <= 0)
        return -1;
    oscene s;
    if (scene_prepare(&s, desc)) {
        scene_free(&s);
        return -1;
    }
    par_job j;
    j.s = &s;
    j.views = views;
    j.targets = targets;
    j.n = n_views;
    j.next = 0;
    j.rc = 0;
    pthread_mutex_init(&j.mu, NULL);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    int started = 0;
    for (int t = 0; t < threads; t++)
        if (pthread_create(&th[t], NULL, par_worker, &j) == 0)
            started++;
    if (started == 0)
        par_worker(&j);
    for (int t = 0; t < started; t++)
        pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&j.mu);
    scene_free(&s);
    return j.rc;
}
